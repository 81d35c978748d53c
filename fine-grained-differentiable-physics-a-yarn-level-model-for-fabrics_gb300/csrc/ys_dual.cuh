// ys_dual.cuh -- forward-mode dual numbers for the step's sensitivities.
//
// Dual<K> carries a value and K tangents (directional derivatives along K
// seeded directions: parameters and/or initial state). Every element routine
// of the step is written once over a scalar type T; instantiated with
// T = double it is the plain step, with T = Dual<K> it also propagates the
// tangents of everything it computes, by the chain rule of each operation
// (the derivatives of sqrt, acos, sin, cos, tanh and exp below are the
// textbook ones). Comparisons and branches look at the value only. Where a
// function is not differentiable -- sqrt at 0 (the length of a zero vector),
// acos at +-1 (the angle of a straight yarn, whose bending energy theta^2 is
// smooth there) -- the tangent taken is 0, the subgradient that keeps the
// derivative of theta^2 exact.
#pragma once

#include <math.h>

#include "ys_common.cuh"

namespace ys {

// the double versions stay visible next to the Dual overloads below
using ::acos;
using ::cos;
using ::exp;
using ::fabs;
using ::sin;
using ::sqrt;
using ::tanh;

// Number of tangent directions a forward-mode step carries. Four keeps the
// dual element kernels within reach of the register file. With eight, the
// dual gather k_gather<Dual<8>> computes wrong values on sm_103a (CUDA 13.0)
// whenever the compiler front end optimises it (-Xcicc -O1 and above; every
// ptxas level alike), while its -Xcicc -O0 build, the -G build and the host
// build under address and undefined-behaviour sanitizers are right; so more
// directions are carried by more passes or by copies of a cloth in one
// batch, each with its own seeds.
constexpr int kTangents = 4;

template <int K>
struct Dual {
  double v;
  double d[K];
  YS_HD Dual() : v(0.0) {
    for (int k = 0; k < K; ++k) d[k] = 0.0;
  }
  YS_HD Dual(double x) : v(x) {
    for (int k = 0; k < K; ++k) d[k] = 0.0;
  }
  YS_HD Dual& operator+=(const Dual& b) {
    v += b.v;
    for (int k = 0; k < K; ++k) d[k] += b.d[k];
    return *this;
  }
  YS_HD Dual& operator-=(const Dual& b) {
    v -= b.v;
    for (int k = 0; k < K; ++k) d[k] -= b.d[k];
    return *this;
  }
  YS_HD Dual& operator*=(const Dual& b) {
    for (int k = 0; k < K; ++k) d[k] = d[k] * b.v + v * b.d[k];
    v *= b.v;
    return *this;
  }
  YS_HD Dual& operator/=(const Dual& b) {
    const double r = 1.0 / b.v, q = v * r;
    for (int k = 0; k < K; ++k) d[k] = (d[k] - q * b.d[k]) * r;
    v = q;
    return *this;
  }
  YS_HD Dual& operator+=(double b) { v += b; return *this; }
  YS_HD Dual& operator-=(double b) { v -= b; return *this; }
  YS_HD Dual& operator*=(double b) {
    v *= b;
    for (int k = 0; k < K; ++k) d[k] *= b;
    return *this;
  }
  YS_HD Dual& operator/=(double b) {
    v /= b;
    for (int k = 0; k < K; ++k) d[k] /= b;
    return *this;
  }
};

// value of a scalar of either kind
YS_HD double val(double x) { return x; }
template <int K>
YS_HD double val(const Dual<K>& x) { return x.v; }
// the same number with its tangents dropped (a detached copy)
template <class T>
YS_HD T detach(const T& x) { return T(val(x)); }

template <int K>
YS_HD Dual<K> operator-(const Dual<K>& a) {
  Dual<K> r;
  r.v = -a.v;
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K>
YS_HD Dual<K> operator+(Dual<K> a, const Dual<K>& b) { return a += b; }
template <int K>
YS_HD Dual<K> operator-(Dual<K> a, const Dual<K>& b) { return a -= b; }
template <int K>
YS_HD Dual<K> operator*(Dual<K> a, const Dual<K>& b) { return a *= b; }
template <int K>
YS_HD Dual<K> operator/(Dual<K> a, const Dual<K>& b) { return a /= b; }
template <int K>
YS_HD Dual<K> operator+(Dual<K> a, double b) { return a += b; }
template <int K>
YS_HD Dual<K> operator-(Dual<K> a, double b) { return a -= b; }
template <int K>
YS_HD Dual<K> operator*(Dual<K> a, double b) { return a *= b; }
template <int K>
YS_HD Dual<K> operator/(Dual<K> a, double b) { return a /= b; }
template <int K>
YS_HD Dual<K> operator+(double a, Dual<K> b) { return b += a; }
template <int K>
YS_HD Dual<K> operator-(double a, const Dual<K>& b) {
  Dual<K> r = -b;
  r.v += a;
  return r;
}
template <int K>
YS_HD Dual<K> operator*(double a, Dual<K> b) { return b *= a; }
template <int K>
YS_HD Dual<K> operator/(double a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a / b.v;
  const double s = -r.v / b.v;
  for (int k = 0; k < K; ++k) r.d[k] = s * b.d[k];
  return r;
}

#define YS_DUAL_CMP(op)                                                                           \
  template <int K>                                                                                \
  YS_HD bool operator op(const Dual<K>& a, const Dual<K>& b) { return a.v op b.v; }              \
  template <int K>                                                                                \
  YS_HD bool operator op(const Dual<K>& a, double b) { return a.v op b; }                        \
  template <int K>                                                                                \
  YS_HD bool operator op(double a, const Dual<K>& b) { return a op b.v; }
YS_DUAL_CMP(<)
YS_DUAL_CMP(>)
YS_DUAL_CMP(<=)
YS_DUAL_CMP(>=)
YS_DUAL_CMP(==)
YS_DUAL_CMP(!=)
#undef YS_DUAL_CMP

// f(a) with f' = dfa
template <int K>
YS_HD Dual<K> chain(const Dual<K>& a, double fa, double dfa) {
  Dual<K> r;
  r.v = fa;
  for (int k = 0; k < K; ++k) r.d[k] = dfa * a.d[k];
  return r;
}
template <int K>
YS_HD Dual<K> sqrt(const Dual<K>& a) {
  const double s = ::sqrt(a.v);
  return chain(a, s, s > 0.0 ? 0.5 / s : 0.0);
}
template <int K>
YS_HD Dual<K> acos(const Dual<K>& a) {
  const double q = 1.0 - a.v * a.v;
  return chain(a, ::acos(a.v), q > 0.0 ? -1.0 / ::sqrt(q) : 0.0);
}
template <int K>
YS_HD Dual<K> sin(const Dual<K>& a) { return chain(a, ::sin(a.v), ::cos(a.v)); }
template <int K>
YS_HD Dual<K> cos(const Dual<K>& a) { return chain(a, ::cos(a.v), -::sin(a.v)); }
template <int K>
YS_HD Dual<K> tanh(const Dual<K>& a) {
  const double t = ::tanh(a.v);
  return chain(a, t, 1.0 - t * t);
}
template <int K>
YS_HD Dual<K> exp(const Dual<K>& a) {
  const double e = ::exp(a.v);
  return chain(a, e, e);
}
template <int K>
YS_HD Dual<K> fabs(const Dual<K>& a) { return a.v < 0 ? -a : a; }

}  // namespace ys
