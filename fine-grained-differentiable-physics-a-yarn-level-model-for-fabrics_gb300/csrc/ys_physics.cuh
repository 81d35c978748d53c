// ys_physics.cuh -- per-element yarn forces and Jacobians of one implicit step.
//
// Each routine handles one element (edge, bend segment, crossing, shear
// segment, face) and returns its contribution to the step's system
//     A = M - h^2 dF/dx - h dF/dv,   b = h (F - (dF/dv)^T v) + M v
// (src/TrainHelper.cpp:19-20). The record producers (ys_elem_kernels.cuh)
// write each element's contribution to its own record, and the per-node
// gathers (ys_items.cuh) sum a node's records in a fixed order into the
// structured stencil layout of ys_common.cuh, so the accumulation is
// deterministic without atomics.
//
// The arithmetic restates the reference's hand-derived expressions term by
// term, including the places where they differ from exact derivatives; every
// routine names the reference lines it follows. The edge kinetic-energy terms
// are evaluated in closed form: with qdot = (a0, e0, a1, e1) and the 8x8 edge
// mass matrix built from 4x4 blocks B = [[z I, p], [q^T, s]] as
// [[2B, B], [B, 2B]], every quadratic form reduces to
//     qdot^T [[2B,B],[B,2B]] qdot = z Saa + p.Sae + q.Sea + s See
// and every product [[2B,B],[B,2B]] qdot = (B m0, B m1) with m0 = 2v0 + v1,
// m1 = v0 + 2v1, so no 8x8 matrix is ever formed.
#pragma once

#include <math.h>

#include "ys_common.cuh"
#include "ys_dual.cuh"

namespace ys {

// ---------------------------------------------------------------- helpers
template <class T>
YS_HD T dot3(const T* a, const T* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <class T>
YS_HD T norm3(const T* a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
template <class T>
YS_HD void cross3(const T* a, const T* b, T* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
template <class T>
YS_HD void proj3(const T* d, T P[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P[i][j] = (i == j ? 1.0 : 0.0) - d[i] * d[j];
}
template <class T>
YS_HD void matvec3(const T P[3][3], const T* a, T* o) {
  for (int i = 0; i < 3; ++i) o[i] = P[i][0] * a[0] + P[i][1] * a[1] + P[i][2] * a[2];
}
template <class T>
YS_HD void outer3(const T* a, const T* b, T O[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) O[i][j] = a[i] * b[j];
}
template <class T>
YS_HD void matmul3(const T A[3][3], const T B[3][3], T O[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) O[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}
YS_HD double ld(const double* p, int comp, int ntot, int node) { return p[(int64_t)comp * ntot + node]; }
YS_HD double& st(double* p, int comp, int ntot, int node) { return p[(int64_t)comp * ntot + node]; }

// Scalar-generic loads and stores. A per-node array p holds comp c of node i
// at p[c * ntot + i]; its tangent array dp (forward-mode runs only) holds
// tangent k at dp[(c * K + k) * ntot + i]. Record buffers use the same rule
// with c = field * nslot + slot. With T = double the tangent arrays are
// never touched.
YS_HD void lds(const double* p, const double* dp, int c, int ntot, int i, double& x) {
  (void)dp;
  x = p[(int64_t)c * ntot + i];
}
template <int K>
YS_HD void lds(const double* p, const double* dp, int c, int ntot, int i, Dual<K>& x) {
  x.v = p[(int64_t)c * ntot + i];
  for (int k = 0; k < K; ++k) x.d[k] = dp ? dp[((int64_t)c * K + k) * ntot + i] : 0.0;
}
template <class T>
YS_HD T ldT(const double* p, const double* dp, int c, int ntot, int i) {
  T x;
  lds(p, dp, c, ntot, i, x);
  return x;
}
YS_HD void stT(double* p, double* dp, int c, int ntot, int i, const double& x) {
  (void)dp;
  p[(int64_t)c * ntot + i] = x;
}
template <int K>
YS_HD void stT(double* p, double* dp, int c, int ntot, int i, const Dual<K>& x) {
  p[(int64_t)c * ntot + i] = x.v;
  if (dp)
    for (int k = 0; k < K; ++k) dp[((int64_t)c * K + k) * ntot + i] = x.d[k];
}
// a parameter of index i in a table of n entries (tangent k at dp[k * n + i])
YS_HD void ldp(const double* p, const double* dp, int i, int n, double& x) {
  (void)dp;
  (void)n;
  x = p[i];
}
template <int K>
YS_HD void ldp(const double* p, const double* dp, int i, int n, Dual<K>& x) {
  x.v = p[i];
  for (int k = 0; k < K; ++k) x.d[k] = dp ? dp[(int64_t)k * n + i] : 0.0;
}
template <class T>
YS_HD T ldpT(const double* p, const double* dp, int i, int n) {
  T x;
  ldp(p, dp, i, n, x);
  return x;
}
// per-cloth parameters S and mu (values in ClothParams, tangents [K][ncloth])
template <class T>
YS_HD T cloth_S(const View& v, int c) { return ldpT<T>(&v.cp[c].S, v.dS ? v.dS + c : nullptr, 0, v.ncloth); }
template <class T>
YS_HD T cloth_mu(const View& v, int c) { return ldpT<T>(&v.cp[c].mu, v.dmu ? v.dmu + c : nullptr, 0, v.ncloth); }

// ------------------------------------------------------------ edge element
// Local DOFs of an edge: x0 (0..2), e0 (3), x1 (4..6), e1 (7), where e is the
// Eulerian coordinate along the edge's yarn (u for warp, v for weft).
// Every node-node 3x3 block an edge produces is a I + b P with P = I - d d^T
// (mass, inertia and dM/dt blocks are multiples of I, stretch adds P), so an
// edge's contribution to A is held as 4 (a, b) pairs plus the Eulerian
// couplings; block index p = 2*(row node) + (column node).
template <class T>
struct EdgeOut {
  T llI[4], llP[4];  // A[x(n_a)][x(n_b)] = llI I + llP P
  T d[3];            // edge direction (defines P)
  T le[4][3];        // A[x(n_a)][e(n_b)]
  T el[4][3];        // A[e(n_a)][x(n_b)]
  T ee[4];           // A[e(n_a)][e(n_b)]
  T b[8];            // contribution to b
  T fe[2], kee[2], dee[2];  // F_E, dF_E/dE (position, velocity) before friction
  T cl[2][3], cle[2][3];    // crimp-compression accumulators
  T V[8];            // the step's velocity vector restricted to the edge (not stored)
  double h, h2;
  bool in[2];
  bool trunc;        // tangents of b through F and v only (M and D held constant)
};
constexpr int kEdgeFields = 65;

enum Mat { kM = 0, kK = 1, kD = 2 };

template <class T>
YS_HD double wt(const EdgeOut<T>& o, int X) { return X == kM ? 1.0 : X == kK ? -o.h2 : -o.h; }
// a matrix coefficient as it enters b = h F + (M - h D^T) v: detached when
// the tangents follow the reference's autograd, where M and D are built
// without a graph (src/MatrixMp.cpp:40-99)
template <class T>
YS_HD T mcoef(const EdgeOut<T>& o, const T& x) { return o.trunc ? detach(x) : x; }

// block (a, b) += val I of matrix X; b receives M V and -h D^T V
// (src/TrainHelper.cpp:19-20). LL blocks of X_LL[find_index(f, d, "LL")] are
// written transposed by To_Sparse_Mat (src/MatrixMp.cpp:54-65); a I + b P is
// symmetric, so the transpose changes nothing here.
template <class T>
YS_HD void acc_LLi(EdgeOut<T>& o, int X, int a, int b, const T& val) {
  o.llI[2 * a + b] += wt(o, X) * val;
  if (X == kM) {
    const T m = mcoef(o, val);
    for (int r = 0; r < 3; ++r) o.b[4 * a + r] += m * o.V[4 * b + r];
  } else if (X == kD) {
    const T m = mcoef(o, val);
    for (int r = 0; r < 3; ++r) o.b[4 * b + r] -= o.h * m * o.V[4 * a + r];
  }
}
template <class T>
YS_HD void acc_LLp(EdgeOut<T>& o, int a, int b, const T& val) { o.llP[2 * a + b] += -o.h2 * val; }  // stiffness only
// A[x(n_a)][e(n_b)] (X_LE[find_index(n_a, n_b, "EL") + k])
template <class T>
YS_HD void acc_LE(EdgeOut<T>& o, int X, int a, int b, const T* vec) {
  const double w = wt(o, X);
  T s = 0.0;
  for (int r = 0; r < 3; ++r) {
    o.le[2 * a + b][r] += w * vec[r];
    if (X == kM) o.b[4 * a + r] += mcoef(o, vec[r]) * o.V[4 * b + 3];
    if (X == kD) s += mcoef(o, vec[r]) * o.V[4 * a + r];
  }
  if (X == kD) o.b[4 * b + 3] -= o.h * s;
}
// A[e(n_a)][x(n_b)] (X_EL[find_index(n_b, n_a, "EL") + k])
template <class T>
YS_HD void acc_EL(EdgeOut<T>& o, int X, int a, int b, const T* vec) {
  const double w = wt(o, X);
  T s = 0.0;
  for (int c = 0; c < 3; ++c) {
    o.el[2 * a + b][c] += w * vec[c];
    if (X == kM) s += mcoef(o, vec[c]) * o.V[4 * b + c];
    if (X == kD) o.b[4 * b + c] -= o.h * mcoef(o, vec[c]) * o.V[4 * a + 3];
  }
  if (X == kM) o.b[4 * a + 3] += s;
}
template <class T>
YS_HD void acc_EE(EdgeOut<T>& o, int X, int a, int b, const T& val) {
  o.ee[2 * a + b] += wt(o, X) * val;
  if (X == kM) o.b[4 * a + 3] += mcoef(o, val) * o.V[4 * b + 3];
  else if (X == kD) o.b[4 * b + 3] -= o.h * mcoef(o, val) * o.V[4 * a + 3];
  if (a == b) {
    if (X == kK) o.kee[a] += val;
    else if (X == kD) o.dee[a] += val;
  }
}
template <class T>
YS_HD void acc_F(EdgeOut<T>& o, int dof, const T& f) {
  o.b[dof] += o.h * f;
  if ((dof & 3) == 3) o.fe[dof >> 2] += f;
}

// One node-pair block p = 2a + b of an edge Jacobian written with the
// pattern shared by Inertia_D_Pos, Inertia_D_Vel, MDotVDot_D_Pos and
// MDotVDot_D_Vel (src/PhysicsCloth.cpp:1544-1600, 1848-1900, 2226-2308,
// 2505-2577): C(i, j) = d(force DOF i)/d(DOF j) in edge-local order, given as
// the isotropic node-node factor iso, the (x, e) column lec[r] = C(4a+r,
// 4b+3), the (e, x) row elr[c] = C(4a+3, 4b+c) and eev = C(4a+3, 4b+3), added
// with sign s under the reference's interior tests. Each section adds a
// block as soon as it is formed, so no section holds all four blocks.
template <class T>
YS_HD void acc_jac_p(EdgeOut<T>& o, int X, double s, int p, const T& iso, const T* lec, const T* elr, const T& eev) {
  const int a = p >> 1, b = p & 1;
  acc_LLi(o, X, a, b, s * iso);
  const bool ok = (a == b) ? o.in[a] : (o.in[0] && o.in[1]);
  if (!ok) return;
  T t[3];
  for (int r = 0; r < 3; ++r) t[r] = s * lec[r];
  acc_LE(o, X, a, b, t);
  for (int c = 0; c < 3; ++c) t[c] = s * elr[c];
  acc_EL(o, X, a, b, t);
  acc_EE(o, X, a, b, s * eev);
}

template <class T>
YS_HD void edge_store_groups(const View& v, double* buf, double* dbuf, int n0, int k, const EdgeOut<T>& o,
                             bool early, bool late);

// All terms of one edge (src/PhysicsCloth.cpp:64-80): Mass, Gravity, Stretch,
// Inertia, MDotVDot, ParaColli; forces and both Jacobians. With ebuf given,
// the fields that are final once ParaColli is done (the stretch projector's
// factors and direction, the crimp accumulators) are stored to the record
// there, so they hold no registers through the kinetic-energy terms; the
// caller then stores the rest with edge_store_groups(..., false, true).
template <class T>
YS_HD void edge_element(const View& v, int n0, int n1, int k, EdgeOut<T>& o, double* ebuf = nullptr,
                        double* edbuf = nullptr) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n0]];
  const uint8_t f0 = v.flags[n0], f1 = v.flags[n1];
  o.in[0] = (f0 & YS_INTERIOR) != 0;
  o.in[1] = (f1 & YS_INTERIOR) != 0;
  const int line = (k == 0) ? P.warp_line_off + v.node_v[n0] : P.weft_line_off + v.node_u[n0];
  const T rho = ldpT<T>(v.line_rho, v.dline_rho, line, v.nlines), ks = ldpT<T>(v.line_ks, v.dline_ks, line, v.nlines);
  o.h = v.h;
  o.h2 = v.h * v.h;
  o.trunc = v.trunc != 0;
  for (int p = 0; p < 4; ++p) {
    o.llI[p] = o.llP[p] = o.ee[p] = 0.0;
    for (int r = 0; r < 3; ++r) o.le[p][r] = o.el[p][r] = 0.0;
  }
  for (int i = 0; i < 8; ++i) o.b[i] = 0.0;
  for (int t = 0; t < 2; ++t) {
    o.fe[t] = o.kee[t] = o.dee[t] = 0.0;
    for (int i = 0; i < 3; ++i) o.cl[t][i] = o.cle[t][i] = 0.0;
  }
  // geometry (src/ClothUnit.h:134-154)
  T x0[3], x1[3], a0[3], a1[3], dx[3], w[3], d[3];
  for (int i = 0; i < 3; ++i) {
    x0[i] = ldT<T>(v.X, v.dX, i, nt, n0); x1[i] = ldT<T>(v.X, v.dX, i, nt, n1);
    a0[i] = ldT<T>(v.V, v.dV, i, nt, n0); a1[i] = ldT<T>(v.V, v.dV, i, nt, n1);
  }
  const T du = ldT<T>(v.UV, v.dUV, k, nt, n1) - ldT<T>(v.UV, v.dUV, k, nt, n0);
  const T e0 = ldT<T>(v.UVD, v.dUVD, k, nt, n0), e1 = ldT<T>(v.UVD, v.dUVD, k, nt, n1);
  // reciprocals of the Eulerian length and of the length: one division each,
  // the terms below multiply by them
  const T idu = 1.0 / du, idu2 = idu * idu, idu3 = idu2 * idu;
  for (int i = 0; i < 3; ++i) { dx[i] = x1[i] - x0[i]; w[i] = dx[i] * idu; }
  const T l = norm3(dx);
  const T il = 1.0 / l;
  for (int i = 0; i < 3; ++i) { d[i] = dx[i] * il; o.d[i] = d[i]; }
  for (int i = 0; i < 3; ++i) { o.V[i] = a0[i]; o.V[4 + i] = a1[i]; }
  o.V[3] = o.in[0] ? e0 : 0.0;
  o.V[7] = o.in[1] ? e1 : 0.0;
  const T wTw = dot3(w, w);
  const T nw = norm3(w);
  T t3[3];

  // ---- Mass (src/PhysicsCloth.cpp:250-338)
  {
    const T coeff = (1.0 / 6.0) * rho * du;
    acc_LLi(o, kM, 0, 0, 2.0 * coeff);
    acc_LLi(o, kM, 1, 0, coeff);
    acc_LLi(o, kM, 0, 1, coeff);
    acc_LLi(o, kM, 1, 1, 2.0 * coeff);
    T LE2[3], LE1[3];
    for (int r = 0; r < 3; ++r) { LE2[r] = -2.0 * coeff * w[r]; LE1[r] = -1.0 * coeff * w[r]; }
    const T EE2 = 2.0 * coeff * wTw, EE1 = 0.5 * EE2;
    if (o.in[0]) { acc_LE(o, kM, 0, 0, LE2); acc_EL(o, kM, 0, 0, LE2); acc_EE(o, kM, 0, 0, EE2); }
    if (o.in[1]) { acc_LE(o, kM, 1, 1, LE2); acc_EL(o, kM, 1, 1, LE2); acc_EE(o, kM, 1, 1, EE2); }
    if (o.in[0] && o.in[1]) {
      acc_LE(o, kM, 1, 0, LE1);
      acc_LE(o, kM, 0, 1, LE1);
      acc_EL(o, kM, 0, 1, LE1);  // M_EL[find_index(n1, n0)] = E0L1
      acc_EL(o, kM, 1, 0, LE1);  // M_EL[find_index(n0, n1)] = E1L0
      acc_EE(o, kM, 0, 1, EE1);
      acc_EE(o, kM, 1, 0, EE1);
    }
  }
  // ---- Gravity_F / Gravity_D (src/PhysicsCloth.cpp:340-425)
  {
    for (int i = 0; i < 3; ++i) {
      const T g = 0.5 * rho * P.G[i] * du;
      acc_F(o, i, -g);
      acc_F(o, 4 + i, -g);
    }
    T sx[3] = {x0[0] + x1[0], x0[1] + x1[1], x0[2] + x1[2]};
    const T gx = P.G[0] * sx[0] + P.G[1] * sx[1] + P.G[2] * sx[2];
    if (o.in[0]) acc_F(o, 3, -((-0.5) * rho * gx));
    if (o.in[1]) acc_F(o, 7, -(0.5 * rho * gx));
    T g0[3], g1[3];
    for (int r = 0; r < 3; ++r) { g0[r] = 0.5 * rho * P.G[r]; g1[r] = -g0[r]; }
    if (o.in[0]) { acc_EL(o, kK, 0, 0, g0); acc_LE(o, kK, 0, 0, g0); }
    if (o.in[1]) { acc_EL(o, kK, 1, 1, g1); acc_LE(o, kK, 1, 1, g1); }
    if (o.in[0] && o.in[1]) {
      acc_LE(o, kK, 1, 0, g0);  // L1E0
      acc_LE(o, kK, 0, 1, g1);  // L0E1
      acc_EL(o, kK, 0, 1, g0);  // E0L1
      acc_EL(o, kK, 1, 0, g1);  // E1L0
    }
  }
  // ---- Stretch_F / Stretch_D (src/PhysicsCloth.cpp:427-577)
  {
    const double sgn = (k == 0) ? 1.0 : -1.0;
    for (int i = 0; i < 3; ++i) {
      const T f = ks * (nw - 1) * d[i];
      acc_F(o, i, f);
      acc_F(o, 4 + i, -f);
      o.cl[0][i] += sgn * f;
      o.cl[1][i] -= sgn * f;
    }
    const T fe = 0.5 * ks * (nw * nw - 1);
    if (o.in[0]) acc_F(o, 3, -fe);
    if (o.in[1]) acc_F(o, 7, fe);
    // LL = (ks / l) P - (ks / du) I, +LL on (0,0), (1,1) and -LL across
    const T cP = ks * il, cI = -(ks * idu);
    acc_LLp(o, 0, 0, cP); acc_LLp(o, 1, 0, -cP); acc_LLp(o, 0, 1, -cP); acc_LLp(o, 1, 1, cP);
    acc_LLi(o, kK, 0, 0, cI); acc_LLi(o, kK, 1, 0, -cI); acc_LLi(o, kK, 0, 1, -cI); acc_LLi(o, kK, 1, 1, cI);
    const T EE = -ks * ((nw * nw) * idu);
    T LE[3], EL[3], nLE[3], nEL[3];
    for (int r = 0; r < 3; ++r) {
      LE[r] = ks * (nw * idu) * d[r];
      EL[r] = ks * idu * w[r];
      nLE[r] = -LE[r];
      nEL[r] = -EL[r];
    }
    if (o.in[0]) {
      acc_LE(o, kK, 0, 0, LE); acc_EL(o, kK, 0, 0, EL); acc_EE(o, kK, 0, 0, EE);
      for (int i = 0; i < 3; ++i) o.cle[0][i] += sgn * LE[i];
    }
    if (o.in[1]) {
      acc_LE(o, kK, 1, 1, LE); acc_EL(o, kK, 1, 1, EL); acc_EE(o, kK, 1, 1, EE);
      for (int i = 0; i < 3; ++i) o.cle[1][i] += sgn * LE[i];
    }
    if (o.in[0] && o.in[1]) {
      acc_LE(o, kK, 1, 0, nLE); acc_LE(o, kK, 0, 1, nLE);
      acc_EL(o, kK, 0, 1, nEL); acc_EL(o, kK, 1, 0, nEL);
      acc_EE(o, kK, 0, 1, -EE); acc_EE(o, kK, 1, 0, -EE);
    }
  }
  // ---- ParaColli_F / ParaColli_D (src/PhysicsCloth.cpp:989-1069)
  {
    const T dd = (((f0 & YS_FLIP) != 0) != ((f1 & YS_FLIP) != 0)) ? 4.0 * P.R : 2.0 * P.R;
    T rl = dd - du;
    if (rl < 0) rl = 0.0;
    const T fu0 = P.kc * P.L * rl;
    if (o.in[0]) acc_F(o, 3, fu0);
    if (o.in[1]) acc_F(o, 7, -fu0);
    const T ee = -P.kc * P.L * rl;
    if (o.in[0]) acc_EE(o, kK, 0, 0, ee);
    if (o.in[1]) acc_EE(o, kK, 1, 1, ee);
    if (o.in[0] && o.in[1]) { acc_EE(o, kK, 0, 1, ee); acc_EE(o, kK, 1, 0, ee); }
  }
  if (ebuf) edge_store_groups(v, ebuf, edbuf, n0, k, o, true, false);

  // ---- kinetic-energy terms: shared sums
  T m0a[3], m1a[3];
  for (int i = 0; i < 3; ++i) { m0a[i] = 2.0 * a0[i] + a1[i]; m1a[i] = a0[i] + 2.0 * a1[i]; }
  const T m0e = 2.0 * e0 + e1, m1e = e0 + 2.0 * e1;
  const T Saa = dot3(a0, m0a) + dot3(a1, m1a);
  T Sae[3], Sea[3];
  for (int i = 0; i < 3; ++i) { Sae[i] = a0[i] * m0e + a1[i] * m1e; Sea[i] = e0 * m0a[i] + e1 * m1a[i]; }
  const T See = e0 * m0e + e1 * m1e;
  const T r6 = (1.0 / 6.0) * rho;
  const T sc = 1.0 / 6.0 * rho * du;
  const T wSae = dot3(w, Sae), wSea = dot3(w, Sea);
  const T pj = -(-idu);  // (-w_x0)_j for the active component j

  // ---- Inertia_F (src/PhysicsCloth.cpp:1071-1186)
  {
    for (int j = 0; j < 3; ++j) {
      const T sj = (-2.0 * idu2 * dx[j]);
      const T T0 = 0.5 * (sc * (pj * Sae[j] + pj * Sea[j] + sj * See));
      acc_F(o, j, T0);
      acc_F(o, 4 + j, -T0);
    }
    const T QM = Saa - wSae - wSea + wTw * See;
    const T Quv = (-idu) * wSae + (-idu) * wSea + (2.0 * idu) * wTw * See;
    const T Tuv0 = 0.5 * (-(1.0 / 6.0) * rho * QM + (1.0 / 6.0) * rho * du * Quv);
    if (o.in[0]) acc_F(o, 3, Tuv0);
    if (o.in[1]) acc_F(o, 7, -Tuv0);
  }
  // ---- Inertia_D_Pos (src/PhysicsCloth.cpp:1188-1601)
  {
    const T T00 = 0.5 * (r6 * ((2.0 * idu2) * See));
    T Tx0uv0[3], Tuv0x0[3];
    for (int j = 0; j < 3; ++j) {
      const T Qx0 = pj * Sae[j] + pj * Sea[j] + (-2.0 * idu2 * dx[j]) * See;
      const T c2 = idu2;
      // the sign-asymmetric mixed block of src/PhysicsCloth.cpp:1357-1361
      const T Qx0uv0 = (-c2) * Sae[j] + (-(-c2)) * Sea[j] + ((-4.0 * idu2) * w[j]) * See;
      Tx0uv0[j] = 0.5 * ((-1.0 / 6.0) * rho * Qx0 + (1.0 / 6.0) * rho * du * Qx0uv0);
      Tuv0x0[j] = 0.5 * ((-1.0 / 6.0) * rho * Qx0 + (1.0 / 6.0) * rho * du * (-Qx0uv0));
    }
    const T Quv0 = (-idu) * wSae + (-idu) * wSea + (2.0 * idu) * wTw * See;
    const T c6 = 2.0 * idu2;
    const T Quvuv = (-c6) * wSae + (-c6) * wSea + (6.0 * idu2) * wTw * See;
    const T Tuu = 0.5 * ((-1.0 / 6.0) * rho * Quv0 - (1.0 / 6.0) * rho * Quv0 + (1.0 / 6.0) * rho * du * Quvuv);
    for (int p = 0; p < 4; ++p) {
      const double sgn = ((p >> 1) == (p & 1)) ? 1.0 : -1.0;
      T lec[3], elr[3];
      for (int r = 0; r < 3; ++r) { lec[r] = sgn * Tx0uv0[r]; elr[r] = sgn * Tuv0x0[r]; }
      acc_jac_p(o, kK, 1.0, p, sgn * T00, lec, elr, sgn * Tuu);
    }
  }
  // ---- Inertia_D_Vel (src/PhysicsCloth.cpp:1602-1901): row x_j of C = M_xj qdot
  {
    const T me_[2] = {m0e, m1e};
    const T* ma_[2] = {m0a, m1a};
    for (int b = 0; b < 2; ++b) {
      const T iso = sc * (pj * me_[b]);
      T lec[3], elr[3];
      const T wm = dot3(w, ma_[b]);
      for (int r = 0; r < 3; ++r) {
        lec[r] = sc * (pj * ma_[b][r] + (-2.0 * idu2 * dx[r]) * me_[b]);
        elr[r] = -(1.0 / 6.0) * rho * (ma_[b][r] - w[r] * me_[b]) + (1.0 / 6.0) * rho * du * ((-idu) * w[r] * me_[b]);
      }
      const T eev = -(1.0 / 6.0) * rho * (-wm + wTw * me_[b]) +
                         (1.0 / 6.0) * rho * du * ((-idu) * wm + (2.0 * idu) * wTw * me_[b]);
      for (int a = 0; a < 2; ++a) {
        const double sgn = a == 0 ? 1.0 : -1.0;  // rows of x1 / uv1 are the negated rows of x0 / uv0
        T lp[3], ep[3];
        for (int r = 0; r < 3; ++r) { lp[r] = sgn * lec[r]; ep[r] = sgn * elr[r]; }
        acc_jac_p(o, kD, 1.0, 2 * a + b, sgn * iso, lp, ep, sgn * eev);
      }
    }
  }
  // ---- MDotVDot (src/PhysicsCloth.cpp:1903-2577)
  {
    const T dud = e1 - e0;
    T wd[3];
    for (int i = 0; i < 3; ++i) wd[i] = ((a1[i] - a0[i]) * du - dx[i] * dud) * idu2;
    const T wTwd = dot3(w, wd) + dot3(wd, w);
    // B_M m and B_dot m for m = m0, m1 (4-vectors); M_dot qdot = r6 dud (B_M m) + r6 du (B_dot m)
    T BMm[2][4], Bdm[2][4], r[8];
    for (int b = 0; b < 2; ++b) {
      const T* ma = b == 0 ? m0a : m1a;
      const T me = b == 0 ? m0e : m1e;
      for (int i = 0; i < 3; ++i) { BMm[b][i] = ma[i] + (-w[i]) * me; Bdm[b][i] = (-wd[i]) * me; }
      BMm[b][3] = (-w[0]) * ma[0] + (-w[1]) * ma[1] + (-w[2]) * ma[2] + wTw * me;
      Bdm[b][3] = (-wd[0]) * ma[0] + (-wd[1]) * ma[1] + (-wd[2]) * ma[2] + wTwd * me;
      for (int i = 0; i < 4; ++i) r[4 * b + i] = r6 * dud * BMm[b][i] + r6 * du * Bdm[b][i];
    }
    // MDotVDot_F: F -= M_dot qdot
    for (int i = 0; i < 3; ++i) { acc_F(o, i, -r[i]); acc_F(o, 4 + i, -r[4 + i]); }
    if (o.in[0]) acc_F(o, 3, -r[3]);
    if (o.in[1]) acc_F(o, 7, -r[7]);
    // MDotVDot_D_Pos, added (src/PhysicsCloth.cpp:2154-2234)
    for (int t = 0; t < 2; ++t) {
      const double sw = t == 0 ? -1.0 : 1.0;
      const T wxj = sw * idu;
      const T P1 = -wxj;
      const T wdxj = t == 0 ? (dud * idu2) : -(dud * idu2);
      const T P2 = -wdxj;
      T wuv[3], wduv[3];
      for (int i = 0; i < 3; ++i) wuv[i] = (sw * w[i]) * idu;
      const T wTwuv = sw * (2.0 * idu) * wTw;
      for (int i = 0; i < 3; ++i) {
        wduv[i] = (a1[i] - a0[i]) * idu2 - (4 * dx[i] * dud) * idu3;
        if (t == 1) wduv[i] = -wduv[i];
      }
      const T wTwduv = 2 * dot3(wuv, wd) + 2 * dot3(wduv, w);
      for (int b = 0; b < 2; ++b) {
        const T* ma = b == 0 ? m0a : m1a;
        const T me = b == 0 ? m0e : m1e;
        const T iso = r6 * dud * (P1 * me) + r6 * du * (P2 * me);
        T elr[3], lec[3];
        for (int j = 0; j < 3; ++j) {
          const T S1 = (sw * 2.0 * idu2 * dx[j]);
          const T S2 = 2 * (wxj * wd[j]) + 2 * (w[j] * wdxj);
          elr[j] = r6 * dud * (P1 * ma[j] + S1 * me) + r6 * du * (P2 * ma[j] + S2 * me);
          lec[j] = r6 * dud * (wuv[j] * me) - r6 * r[4 * b + j] + r6 * du * (-wduv[j] * me);
        }
        const T eev = r6 * dud * (dot3(wuv, ma) + wTwuv * me) - r6 * r[4 * b + 3] +
                      r6 * du * (-dot3(wduv, ma) + wTwduv * me);
        acc_jac_p(o, kK, 1.0, 2 * b + t, iso, lec, elr, eev);
      }
    }
    // MDotVDot_D_Vel, subtracted (src/PhysicsCloth.cpp:2342-2577)
    for (int t = 0; t < 2; ++t) {
      const double sw = t == 0 ? -1.0 : 1.0;
      const T wdj = sw * idu;
      const T P1 = -wdj;
      T wdv[3];
      for (int i = 0; i < 3; ++i) wdv[i] = (t == 0 ? idu : -idu) * w[i];
      const T wtwd = 2 * dot3(w, wdv);
      const T cm = (t == 0 ? -1.0 : 1.0) * (1.0 / 6.0) * rho;
      for (int b = 0; b < 2; ++b) {
        const T* ma = b == 0 ? m0a : m1a;
        const T me = b == 0 ? m0e : m1e;
        const double f = (b == t) ? 2.0 : 1.0;  // [[2B, B], [B, 2B]] block factor of M_dot
        const T iso = (1.0 / 6.0) * rho * du * (P1 * me) + (r6 * dud * (f * 1.0) + r6 * du * (f * 0.0));
        T elr[3], lec[3];
        for (int j = 0; j < 3; ++j) {
          const T S1 = 2 * (w[j] * wdj);
          elr[j] = (1.0 / 6.0) * rho * du * (P1 * ma[j] + S1 * me) +
                   (r6 * dud * (f * -w[j]) + r6 * du * (f * -wd[j]));
          lec[j] = cm * BMm[b][j] + (1.0 / 6.0) * rho * du * (-wdv[j] * me) +
                   (r6 * dud * (f * -w[j]) + r6 * du * (f * -wd[j]));
        }
        const T eev = cm * BMm[b][3] + (1.0 / 6.0) * rho * du * (-dot3(wdv, ma) + wtwd * me) +
                      (r6 * dud * (f * wTw) + r6 * du * (f * wTwd));
        acc_jac_p(o, kD, -1.0, 2 * b + t, iso, lec, elr, eev);
      }
    }
  }
  (void)t3;
}

// record layout of an edge in the per-element buffer (field-major over the
// 2 * ntot edge slots: slot = k * ntot + n0; tangents in dbuf)
// `early`: llP, d, cl, cle (final after the stretch and contact terms);
// `late`: every other field
template <class T>
YS_HD void edge_store_groups(const View& v, double* buf, double* dbuf, int n0, int k, const EdgeOut<T>& o,
                             bool early, bool late) {
  const int nt = v.ntot;
  int f = 0;
  auto put = [&](const T& x, bool g) {
    if (g) stT(buf, dbuf, 2 * f + k, nt, n0, x);
    ++f;
  };
  for (int p = 0; p < 4; ++p) put(o.llI[p], late);
  for (int p = 0; p < 4; ++p) put(o.llP[p], early);
  for (int i = 0; i < 3; ++i) put(o.d[i], early);
  for (int p = 0; p < 4; ++p) for (int r = 0; r < 3; ++r) put(o.le[p][r], late);
  for (int p = 0; p < 4; ++p) for (int r = 0; r < 3; ++r) put(o.el[p][r], late);
  for (int p = 0; p < 4; ++p) put(o.ee[p], late);
  for (int i = 0; i < 8; ++i) put(o.b[i], late);
  for (int t = 0; t < 2; ++t) { put(o.fe[t], late); put(o.kee[t], late); put(o.dee[t], late); }
  for (int t = 0; t < 2; ++t) for (int i = 0; i < 3; ++i) put(o.cl[t][i], early);
  for (int t = 0; t < 2; ++t) for (int i = 0; i < 3; ++i) put(o.cle[t][i], early);
}
template <class T>
YS_HD void edge_store(const View& v, double* buf, double* dbuf, int n0, int k, const EdgeOut<T>& o) {
  edge_store_groups(v, buf, dbuf, n0, k, o, true, true);
}
// field offsets of the layout above
constexpr int kE_llI = 0, kE_llP = 4, kE_d = 8, kE_le = 11, kE_el = 23, kE_ee = 35, kE_b = 39, kE_fkd = 47,
              kE_cl = 53, kE_cle = 59;

// ------------------------------------------------------------ bend element
template <class T>
struct BendGeom {
  T du, l1, l2, d1[3], d2[3], P1[3][3], P2[3][3], theta;
  T c;  // cos(theta), the clamped argument of the acos
};
// src/ClothUnit.h:197-210; the theta clamp uses EPS = DBL_MIN
// (src/Constants.h:25) and so never changes a finite value.
template <class T>
YS_HD void bend_geom(const T* x2, const T* x0, const T* x1, T du, BendGeom<T>& g) {
  T a1[3], a2[3];
  for (int i = 0; i < 3; ++i) { a1[i] = x1[i] - x0[i]; a2[i] = x2[i] - x0[i]; }
  g.du = du;
  g.l1 = norm3(a1);
  g.l2 = norm3(a2);
  for (int i = 0; i < 3; ++i) { g.d1[i] = a1[i] / g.l1; g.d2[i] = a2[i] / g.l2; }
  proj3(g.d1, g.P1);
  proj3(g.d2, g.P2);
  T c = -dot3(g.d1, g.d2);
  const double lo = -1.0 + 2.2250738585072014e-308, hi = 1.0 - 2.2250738585072014e-308;
  if (c < lo) c = lo;
  if (c > hi) c = hi;
  g.c = c;
  g.theta = acos(c);
}

// Bending force and Hessian blocks shared by Bending_* and Crimp_Bending_*
// (src/PhysicsCloth.cpp:579-822, 824-987).
template <class T>
struct BendTerms {
  T Fx1[3], Fx2[3];
  T L11[3][3], L12[3][3], L21[3][3], L22[3][3];
  T L1E1[3], L2E1[3];
  bool active;
};
template <class T>
YS_HD void bend_terms(const BendGeom<T>& g, const T& kb, BendTerms<T>& t) {
  for (int i = 0; i < 3; ++i) {
    t.Fx1[i] = t.Fx2[i] = t.L1E1[i] = t.L2E1[i] = 0.0;
    for (int j = 0; j < 3; ++j) t.L11[i][j] = t.L12[i][j] = t.L21[i][j] = t.L22[i][j] = 0.0;
  }
  // sin and cos of theta = acos(c) from c itself: sin = sqrt((1 - c)(1 + c))
  // (zero exactly where sin(acos(c)) is: c = +-1), cos = c
  const T th = g.theta, s = sqrt((1.0 - g.c) * (1.0 + g.c));
  t.active = (s != 0.0);
  if (!t.active) return;
  const T co = g.c, du = g.du;
  T a[3], b[3];
  matvec3(g.P1, g.d2, a);
  matvec3(g.P2, g.d1, b);
  const T il1 = 1.0 / g.l1, il2 = 1.0 / g.l2, idu = 1.0 / du, is = 1.0 / s;  // one division each
  const T c1 = (-2 * kb * th) * (il1 * idu * is), c2 = (-2 * kb * th) * (il2 * idu * is);
  for (int i = 0; i < 3; ++i) { t.Fx1[i] = c1 * a[i]; t.Fx2[i] = c2 * b[i]; }
  const T k11 = (2 * kb) * ((il1 * il1) * idu * is), k12 = (-2 * kb) * (il1 * il2 * idu * is);
  const T k22 = (2 * kb) * ((il2 * il2) * idu * is);
  const T cs2 = co * (is * is);
  T Tm[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const T ad1 = a[i] * g.d1[j], aa = a[i] * a[j], d1a = g.d1[i] * a[j];
      const T bd2 = b[i] * g.d2[j], bb = b[i] * b[j], d2b = g.d2[i] * b[j];
      t.L11[i][j] = k11 * (th * (ad1 + cs2 * aa + co * g.P1[i][j] + d1a) - is * aa);
      t.L22[i][j] = k22 * (th * (bd2 + cs2 * bb + co * g.P2[i][j] + d2b) - is * bb);
      Tm[i][j] = th * (g.P1[i][j] - cs2 * ad1) + is * ad1;
    }
  matmul3(Tm, g.P2, t.L12);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t.L12[i][j] *= k12;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const T bd2 = b[i] * g.d2[j];
      Tm[i][j] = th * (g.P2[i][j] - cs2 * bd2) + is * bd2;
    }
  matmul3(Tm, g.P1, t.L21);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t.L21[i][j] *= k12;
  const T e1 = (2 * kb * th) * (il1 * (idu * idu) * is), e2 = (2 * kb * th) * (il2 * (idu * idu) * is);
  for (int i = 0; i < 3; ++i) { t.L1E1[i] = e1 * a[i]; t.L2E1[i] = e2 * b[i]; }
}

// Bend segment record (one per middle node and yarn direction): the four
// independent Hessian blocks of Bending_D and its Eulerian couplings, the
// forces of Bending_F, and the crimp-bending forces / couplings that feed the
// compression estimate (Crimp_Bending_F/D). The other blocks follow from
// these as in src/PhysicsCloth.cpp:705-727 and are formed by the gather.
constexpr int kBendFields = 62;
constexpr int kB_L11 = 0, kB_L12 = 9, kB_L21 = 18, kB_L22 = 27, kB_L1E1 = 36, kB_L2E1 = 39, kB_E1E1 = 42,
              kB_Fx1 = 43, kB_Fx2 = 46, kB_Fu2 = 49, kB_cFx1 = 50, kB_cFx2 = 53, kB_cL1E1 = 56, kB_cL2E1 = 59;

// Bending_F / Bending_D on the real nodes (src/PhysicsCloth.cpp:579-822) and
// Crimp_Bending_F / Crimp_Bending_D on the crimp-offset centre lines
// (src/PhysicsCloth.cpp:824-987) for the segment n2 - n0 - n1 along yarn
// direction k; written to the bend buffer at slot k * ntot + n0.
template <class T>
YS_HD void bend_element(const View& v, double* buf, double* dbuf, int n2, int n0, int n1, int k, int line) {
  const int nt = v.ntot;
  const int64_t stride = 2LL * nt, base = (int64_t)k * nt + n0;
  (void)stride;
  (void)base;
  const T kb = ldpT<T>(v.line_kb, v.dline_kb, line, v.nlines);
  auto put = [&](int f, const T& x) { stT(buf, dbuf, 2 * f + k, nt, n0, x); };
  {
    T x2[3], x0[3], x1[3];
    for (int i = 0; i < 3; ++i) {
      x2[i] = ldT<T>(v.X, v.dX, i, nt, n2);
      x0[i] = ldT<T>(v.X, v.dX, i, nt, n0);
      x1[i] = ldT<T>(v.X, v.dX, i, nt, n1);
    }
    BendGeom<T> g;
    bend_geom(x2, x0, x1, ldT<T>(v.UV, v.dUV, k, nt, n1) - ldT<T>(v.UV, v.dUV, k, nt, n2), g);
    BendTerms<T> t;
    bend_terms(g, kb, t);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        put(kB_L11 + 3 * i + j, t.L11[i][j]);
        put(kB_L12 + 3 * i + j, t.L12[i][j]);
        put(kB_L21 + 3 * i + j, t.L21[i][j]);
        put(kB_L22 + 3 * i + j, t.L22[i][j]);
      }
    for (int i = 0; i < 3; ++i) {
      put(kB_L1E1 + i, t.L1E1[i]);
      put(kB_L2E1 + i, t.L2E1[i]);
      put(kB_Fx1 + i, t.Fx1[i]);
      put(kB_Fx2 + i, t.Fx2[i]);
    }
    const T th = g.theta, idu = 1.0 / g.du;
    put(kB_E1E1, (-2 * kb * (th * th)) * (idu * idu * idu));
    put(kB_Fu2, (-kb * th) * (idu * idu));
  }
  {
    const double R = v.cp[v.node_cloth[n0]].R;
    const double sg = k == 0 ? -1.0 : 1.0;  // warp: x - R n, weft: x + R n
    T x[3][3];
    const int nd[3] = {n2, n0, n1};
    for (int m = 0; m < 3; ++m) {
      const bool in = (v.flags[nd[m]] & YS_INTERIOR) != 0;
      for (int i = 0; i < 3; ++i)
        x[m][i] = in ? ldT<T>(v.X, v.dX, i, nt, nd[m]) + sg * (R * ldT<T>(v.NRM, v.dNRM, i, nt, nd[m]))
                     : ldT<T>(v.X, v.dX, i, nt, nd[m]);
    }
    // crimp segments keep the EPos of the build (src/Cloth.cpp:107)
    BendGeom<T> g;
    bend_geom(x[0], x[1], x[2], T(ld(v.UV0, k, nt, n1) - ld(v.UV0, k, nt, n2)), g);
    BendTerms<T> t;
    bend_terms(g, kb, t);
    for (int i = 0; i < 3; ++i) {
      put(kB_cFx1 + i, t.Fx1[i]);
      put(kB_cFx2 + i, t.Fx2[i]);
      put(kB_cL1E1 + i, t.L1E1[i]);
      put(kB_cL2E1 + i, t.L2E1[i]);
    }
  }
}

// ------------------------------------------------------------ wind (faces)
// Wind_F (src/PhysicsCloth.cpp:3091-3107), face geometry src/ClothUnit.h:268-273;
// returns wind_force / 3, the share of each of the face's three nodes.
template <class T>
YS_HD void wind_face(const View& v, const ClothParams& P, int n1, int n2, int n3, T* f3) {
  const int nt = v.ntot;
  T e1[3], e2[3], cr[3], n[3], fv[3], rel[3];
  for (int i = 0; i < 3; ++i) {
    const T xa = ldT<T>(v.X, v.dX, i, nt, n1);
    e1[i] = ldT<T>(v.X, v.dX, i, nt, n2) - xa;
    e2[i] = ldT<T>(v.X, v.dX, i, nt, n3) - xa;
  }
  cross3(e1, e2, cr);
  const T nc = norm3(cr), area = 0.5 * nc;
  for (int i = 0; i < 3; ++i) n[i] = (nc == 0.0) ? cr[i] : cr[i] / nc;
  for (int i = 0; i < 3; ++i) {
    fv[i] = (ldT<T>(v.V, v.dV, i, nt, n1) + ldT<T>(v.V, v.dV, i, nt, n2) + ldT<T>(v.V, v.dV, i, nt, n3)) / 3.0;
    rel[i] = P.wind[i] - fv[i];
  }
  const T vn = dot3(n, rel);
  for (int i = 0; i < 3; ++i) {
    const T tang = rel[i] - vn * n[i];
    const T f = P.wind_rho * area * fabs(vn) * vn * n[i] + P.wind_drag * area * tang;
    f3[i] = f / 3.0;
  }
}

// cell with top-left node tl: faces (src/Cloth.cpp:271-287) written to the
// face buffer [6][ntot] (face A then face B, each wind_force / 3)
template <class T>
YS_HD void cell_faces(const View& v, double* buf, double* dbuf, int tl) {
  const ClothParams& P = v.cp[v.node_cloth[tl]];
  const int tr = tl + 1, bl = tl + P.W, br = tl + P.W + 1;
  T fa[3], fb[3];
  if (((v.node_u[tl] + v.node_v[tl]) & 1) == 0) {
    wind_face(v, P, tl, tr, br, fa);
    wind_face(v, P, tl, br, bl, fb);
  } else {
    wind_face(v, P, tl, tr, bl, fa);
    wind_face(v, P, tr, br, bl, fb);
  }
  for (int i = 0; i < 3; ++i) {
    stT(buf, dbuf, i, v.ntot, tl, fa[i]);
    stT(buf, dbuf, 3 + i, v.ntot, tl, fb[i]);
  }
}

// ------------------------------------------------------------ crossing node
// Node normal (src/Cloth.cpp:440-463): smallest right singular vector of the
// centred 5-point stencil = eigenvector of the smallest eigenvalue of its 3x3
// scatter matrix (cyclic Jacobi rotations), signed by warp x weft and the
// weave's flip flag.
// a <- diagonalised S, V <- its eigenvectors (columns)
YS_HD void sym3_jacobi(const double S[3][3], double a[3][3], double V[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) a[i][j] = S[i][j];
  // off-diagonal entries below 1e-24 of the diagonal scale move the
  // eigenvectors by less than 1e-24 and are treated as zero
  const double tiny = 1e-24 * (fabs(S[0][0]) + fabs(S[1][1]) + fabs(S[2][2]));
  for (int sweep = 0; sweep < 50; ++sweep) {
    if (fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]) <= tiny) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (fabs(a[p][q]) <= tiny) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < 3; ++k) {
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = cs * akp - sn * akq;
          a[k][q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = cs * apk - sn * aqk;
          a[q][k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = cs * vkp - sn * vkq;
          V[k][q] = sn * vkp + cs * vkq;
        }
      }
  }
}
YS_HD int sym3_argmin(const double a[3][3]) {
  int m = 0;
  if (a[1][1] < a[m][m]) m = 1;
  if (a[2][2] < a[m][m]) m = 2;
  return m;
}
YS_HD void sym3_min_eigvec(const double S[3][3], double* out) {
  double a[3][3], V[3][3];
  sym3_jacobi(S, a, V);
  const int m = sym3_argmin(a);
  for (int k = 0; k < 3; ++k) out[k] = V[k][m];
}

// Eigenvector of the smallest eigenvalue of a symmetric 3x3 S by Rayleigh-
// quotient iteration from a guess close to it: x <- adj(S - mu I) x / |.|,
// mu = x^T S x (the adjugate solves the shifted system up to scale without a
// division and stays exact when mu hits the eigenvalue). Converges cubically;
// returns false (out untouched) unless the result is an eigenvector of the
// smallest eigenvalue to 1e-12 relative, for the caller to fall back on the
// Jacobi solver.
YS_HD bool sym3_min_eigvec_rqi(const double S[3][3], const double* guess, double* out) {
  double x[3] = {guess[0], guess[1], guess[2]};
  double nx = norm3(x);
  if (!(nx > 0.0)) return false;
  for (int i = 0; i < 3; ++i) x[i] /= nx;
  double mu = 0.0;
  for (int it = 0; it < 4; ++it) {
    double Sx[3];
    for (int i = 0; i < 3; ++i) Sx[i] = S[i][0] * x[0] + S[i][1] * x[1] + S[i][2] * x[2];
    mu = dot3(x, Sx);
    const double m00 = S[0][0] - mu, m11 = S[1][1] - mu, m22 = S[2][2] - mu;
    const double m01 = S[0][1], m02 = S[0][2], m12 = S[1][2];
    // adjugate of the symmetric M = S - mu I
    const double c00 = m11 * m22 - m12 * m12, c01 = m02 * m12 - m01 * m22, c02 = m01 * m12 - m02 * m11;
    const double c11 = m00 * m22 - m02 * m02, c12 = m01 * m02 - m00 * m12, c22 = m00 * m11 - m01 * m01;
    double y[3] = {c00 * x[0] + c01 * x[1] + c02 * x[2], c01 * x[0] + c11 * x[1] + c12 * x[2],
                   c02 * x[0] + c12 * x[1] + c22 * x[2]};
    const double ny = norm3(y);
    if (!(ny > 0.0) || !isfinite(ny)) break;  // x is already exact
    const double iy = 1.0 / ny;
    for (int i = 0; i < 3; ++i) x[i] = y[i] * iy;
  }
  double Sx[3];
  for (int i = 0; i < 3; ++i) Sx[i] = S[i][0] * x[0] + S[i][1] * x[1] + S[i][2] * x[2];
  mu = dot3(x, Sx);
  const double sc = fabs(S[0][0]) + fabs(S[1][1]) + fabs(S[2][2]) + 1e-300;
  double r2 = 0.0;
  for (int i = 0; i < 3; ++i) r2 += (Sx[i] - mu * x[i]) * (Sx[i] - mu * x[i]);
  if (!(r2 <= 1e-24 * sc * sc)) return false;
  // mu is the smallest eigenvalue iff the other two, l2 + l3 = tr - mu and
  // l2 l3 = e2 - mu (tr - mu), are both >= mu
  const double tr = S[0][0] + S[1][1] + S[2][2];
  const double e2 = S[0][0] * S[1][1] + S[0][0] * S[2][2] + S[1][1] * S[2][2] - S[0][1] * S[0][1] -
                    S[0][2] * S[0][2] - S[1][2] * S[1][2];
  const double sum = tr - mu, prod = e2 - mu * sum;
  if (!(sum >= 2.0 * mu && prod - mu * sum + mu * mu >= -1e-12 * sc * sc)) return false;
  for (int i = 0; i < 3; ++i) out[i] = x[i];
  return true;
}

YS_HD void node_normal(const View& v, int n, int W) {
  const int nt = v.ntot;
  const int ids[5] = {n, n - 1, n + 1, n - W, n + W};
  double p[5][3], mean[3] = {0, 0, 0}, S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int m = 0; m < 5; ++m)
    for (int i = 0; i < 3; ++i) { p[m][i] = ld(v.X, i, nt, ids[m]); mean[i] += p[m][i]; }
  for (int i = 0; i < 3; ++i) mean[i] /= 5.0;
  for (int m = 0; m < 5; ++m) {
    double r[3] = {p[m][0] - mean[0], p[m][1] - mean[1], p[m][2] - mean[2]};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] += r[i] * r[j];
  }
  double vw[3], vf[3], cr[3];
  for (int i = 0; i < 3; ++i) { vw[i] = p[2][i] - p[1][i]; vf[i] = p[4][i] - p[3][i]; }
  cross3(vw, vf, cr);
  // the smallest right singular vector of the centred positions (the
  // reference's torch::svd, src/Cloth.cpp:440-463) is the smallest
  // eigenvector of their scatter S; warp x weft is a close starting guess
  double nn[3];
  if (!sym3_min_eigvec_rqi(S, cr, nn)) sym3_min_eigvec(S, nn);
  const double len = norm3(nn);
  for (int i = 0; i < 3; ++i) nn[i] /= len;
  if (dot3(cr, nn) / (norm3(cr) * norm3(nn)) < 0)
    for (int i = 0; i < 3; ++i) nn[i] = -nn[i];
  if (v.flags[n] & YS_FLIP)
    for (int i = 0; i < 3; ++i) nn[i] = -nn[i];
  for (int i = 0; i < 3; ++i) st(v.NRM, i, nt, n) = nn[i];
}

// node_normal with tangents: the value as above; the tangent of the unit
// eigenvector n of the smallest eigenvalue l_m of the scatter S along dS is
// sum_{j != m} (v_j . dS n) / (l_m - l_j) v_j (first-order perturbation of a
// symmetric eigenproblem with simple eigenvalues, the derivative autograd
// takes through the SVD of src/Cloth.cpp:446). Values go to NRM, tangents
// to dNRM.
template <int K>
YS_HD void node_normal_dual(const View& v, int n, int W) {
  typedef Dual<K> D;
  const int nt = v.ntot;
  const int ids[5] = {n, n - 1, n + 1, n - W, n + W};
  D p[5][3], mean[3], S[3][3];
  for (int m = 0; m < 5; ++m)
    for (int i = 0; i < 3; ++i) { p[m][i] = ldT<D>(v.X, v.dX, i, nt, ids[m]); mean[i] += p[m][i]; }
  for (int i = 0; i < 3; ++i) mean[i] /= 5.0;
  for (int m = 0; m < 5; ++m) {
    D r[3] = {p[m][0] - mean[0], p[m][1] - mean[1], p[m][2] - mean[2]};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] += r[i] * r[j];
  }
  double Sv[3][3], a[3][3], V[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Sv[i][j] = S[i][j].v;
  sym3_jacobi(Sv, a, V);
  const int mm = sym3_argmin(a);
  D nn[3];
  for (int i = 0; i < 3; ++i) nn[i] = D(V[i][mm]);
  for (int jj = 0; jj < 3; ++jj) {
    if (jj == mm) continue;
    const double gap = a[mm][mm] - a[jj][jj];
    for (int k = 0; k < K; ++k) {
      double c = 0.0;  // v_j . dS_k n
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) c += V[r][jj] * S[r][q].d[k] * V[q][mm];
      for (int i = 0; i < 3; ++i) nn[i].d[k] += (c / gap) * V[i][jj];
    }
  }
  const D len = norm3(nn);
  for (int i = 0; i < 3; ++i) nn[i] /= len;
  double vw[3], vf[3], cr[3], nv[3];
  for (int i = 0; i < 3; ++i) {
    vw[i] = p[2][i].v - p[1][i].v;
    vf[i] = p[4][i].v - p[3][i].v;
    nv[i] = nn[i].v;
  }
  cross3(vw, vf, cr);
  if (dot3(cr, nv) / (norm3(cr) * norm3(nv)) < 0)
    for (int i = 0; i < 3; ++i) nn[i] = -nn[i];
  if (v.flags[n] & YS_FLIP)
    for (int i = 0; i < 3; ++i) nn[i] = -nn[i];
  for (int i = 0; i < 3; ++i) stT(v.NRM, v.dNRM, i, nt, n, nn[i]);
}

// ConSlideFriction (src/PhysicsCloth.cpp:2579-2641) for interior node n from
// its gathered no-slide force fe, dF_E/dE diagonals kee / dee and the crimp
// compression sums cl / cle; returns the A and b contributions of the E rows
// and stores COMP and SLIDE.
template <class T>
YS_HD void friction_node(const View& v, int n, const T* fe, const T* kee, const T* dee,
                         const T* cl, const T* cle, T* aEE, T* bE) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  T nrm[3];
  for (int i = 0; i < 3; ++i) nrm[i] = ldT<T>(v.NRM, v.dNRM, i, nt, n);
  T comp = 0.5 * dot3(nrm, cl);
  if (comp < 0) comp = 0.0;
  const T compEE[2] = {0.5 * dot3(nrm, cle), 0.5 * dot3(nrm, cle + 3)};
  stT(v.COMP, v.dCOMP, 0, nt, n, comp);
  const T mu = cloth_mu<T>(v, v.node_cloth[n]);
  const double kf = P.kf, df = P.df, h = v.h, h2 = v.h * v.h;
  const T lim = 1.0 * comp * mu;
  for (int k = 0; k < 2; ++k) {
    const T uvm = ldT<T>(v.UV, v.dUV, k, nt, n) - ldT<T>(v.UVB, v.dUVB, k, nt, n);
    const T FEns = fe[k], EEp = kee[k], EEv = dee[k];
    const T slide = 1.0 / (1.0 + exp(-(1e4 * (fabs(FEns) - lim))));
    const T t = tanh(10 * uvm), tl = tanh(10 * (lim - FEns));
    const T uvdot = ldT<T>(v.UVD, v.dUVD, k, nt, n);
    const T force = (-0.5 * (kf * uvm - t * comp * mu) * tl + 0.5 * (kf * uvm + t * comp * mu)) - df * uvdot;
    const T pos = (-0.5 * (kf - (1.0 - t * t) * mu * comp - t * mu * compEE[k])) * tl -
                       (0.5 * (kf * uvm - t * mu * comp)) * (1.0 - tl * tl) * (EEp - mu * compEE[k]) -
                       (0.5 * (kf + (1.0 - t * t) * mu * comp + t * mu * compEE[k]));
    // tanh(10 * fric_lim - F) as written at src/PhysicsCloth.cpp:2630-2631
    const T tq = tanh(10 * lim - FEns);
    const T vel = (-0.5 * (kf * uvm - t * mu * comp)) * (1.0 - tq * tq) * EEv - df;
    stT(v.SLIDE, v.dSLIDE, k, nt, n, slide);
    aEE[k] = -h2 * pos - h * vel;
    // D enters b without a graph in the reference (src/MatrixMp.cpp:40-99)
    bE[k] = h * (force - (v.trunc ? detach(vel) : vel) * uvdot);
  }
}

// ------------------------------------------------------------ shear
// Shear segment record (one per crossing and segment type): the forces on the
// warp and weft neighbours and the four independent Hessian blocks; the
// crossing's own force and blocks follow from them (src/PhysicsCloth.cpp:2710,
// 3033-3037) and are formed by the gather.
constexpr int kShearFields = 42;
constexpr int kS_F1 = 0, kS_F3 = 3, kS_J11 = 6, kS_J13 = 15, kS_J31 = 24, kS_J33 = 33;
// segment types in the order of src/Cloth.cpp:178-181: (warp, weft) offsets
YS_HD int shear_du(int seg) { return seg < 2 ? -1 : 1; }
YS_HD int shear_dv(int seg) { return (seg & 1) ? -1 : 1; }

// Shear_F / Shear_D (src/PhysicsCloth.cpp:2643-3089) for crossing n0 with warp
// neighbour n1 = n0 + (shear_du, 0) and weft neighbour n3 = n0 + (0, shear_dv),
// written to the shear buffer at slot seg * ntot + n0.
template <class T>
YS_HD void shear_element(const View& v, double* buf, double* dbuf, int n0, int seg) {
  const ClothParams& P = v.cp[v.node_cloth[n0]];
  const int n1 = n0 + shear_du(seg), n3 = n0 + shear_dv(seg) * P.W;
  const int nt = v.ntot;
  const double Lc = P.L, R = P.R;
  const T S = cloth_S<T>(v, v.node_cloth[n0]);
  const T comp = ldT<T>(v.COMP, v.dCOMP, 0, nt, n0);
  T a1v[3], a3v[3], d1[3], d3[3], P1[3][3], P3[3][3];
  for (int i = 0; i < 3; ++i) {
    const T x0 = ldT<T>(v.X, v.dX, i, nt, n0);
    a1v[i] = ldT<T>(v.X, v.dX, i, nt, n1) - x0;
    a3v[i] = ldT<T>(v.X, v.dX, i, nt, n3) - x0;
  }
  const T l1 = norm3(a1v), l3 = norm3(a3v);
  const T il1 = 1.0 / l1, il3 = 1.0 / l3;  // reciprocals, one division each
  for (int i = 0; i < 3; ++i) { d1[i] = a1v[i] * il1; d3[i] = a3v[i] * il3; }
  proj3(d1, P1);
  proj3(d3, P3);
  // the crossing angle, and its sine and cosine from its cosine c:
  // sin = sqrt((1 - c)(1 + c)), cos = c (phi in [0, pi])
  const T cph = dot3(d1, d3);
  const T phi = acos(cph);
  const T s = sqrt((1.0 - cph) * (1.0 + cph)), co = cph;
  T a3[3], a1[3];  // a3 = P1 d3, a1 = P3 d1
  matvec3(P1, d3, a3);
  matvec3(P3, d1, a1);
  const uint8_t f0 = v.flags[n0], f1 = v.flags[n1], f3 = v.flags[n3];
  const bool jam = (((f0 & YS_FLIP) != 0) != ((f1 & YS_FLIP) != 0)) && (((f0 & YS_FLIP) != 0) != ((f3 & YS_FLIP) != 0));
  T Fx1[3], Fx3[3], J11[3][3], J13[3][3], J31[3][3], J33[3][3];
  const T is = 1.0 / s, cs2 = co * (is * is);
  if (!jam) {
    const T kx = (comp + 1.0) * S * R * R * kPi;
    const T ph = phi - kPi / 2;
    // Shear_F takes phi.item() in (phi - PI/2) (src/PhysicsCloth.cpp:2720-2721):
    // that factor carries no derivative along the reference's gradient path
    const T phf = v.trunc ? detach(phi) - kPi / 2 : ph;
    const T cf1 = (kx * Lc * phf) * (il1 * is), cf3 = (kx * Lc * phf) * (il3 * is);
    for (int i = 0; i < 3; ++i) { Fx1[i] = cf1 * a3[i]; Fx3[i] = cf3 * a1[i]; }
    const T k11 = (kx * Lc) * ((il1 * il1) * is), k33 = (kx * Lc) * ((il3 * il3) * is);
    const T k13 = (kx * Lc) * (il3 * il1 * is), k31 = (kx * Lc) * (il1 * il3 * is);
    // src/PhysicsCloth.cpp:2715-2751 per block:
    //   J11 = k11 (ph (-a3 d1^T + cs2 a3 a3^T - co P1 - d1 a3^T) - a3 a3^T / s)
    //   J13 = k13 ph (cs2 - 1/s) (a3 d1^T) P3 = k13 ph (cs2 - 1/s) a3 a1^T, as a1 = P3 d1
    // (J33, J31 likewise with 1 <-> 3)
    const T kA1 = k11 * (ph * cs2 - is), kS1 = -k11 * ph, kP1 = kS1 * co;
    const T kA3 = k33 * (ph * cs2 - is), kS3 = -k33 * ph, kP3 = kS3 * co;
    const T kx13 = k13 * ph * (cs2 - is), kx31 = k31 * ph * (cs2 - is);
    for (int i = 0; i < 3; ++i) {
      const T al1 = kA1 * a3[i] + kS1 * d1[i], be1 = kS1 * a3[i];
      const T al3 = kA3 * a1[i] + kS3 * d3[i], be3 = kS3 * a1[i];
      for (int j = 0; j < 3; ++j) {
        J11[i][j] = al1 * a3[j] + be1 * d1[j] + kP1 * P1[i][j];
        J33[i][j] = al3 * a1[j] + be3 * d3[j] + kP3 * P3[i][j];
        J13[i][j] = kx13 * (a3[i] * a1[j]);
        J31[i][j] = kx31 * (a1[i] * a3[j]);
      }
    }
  } else {
    // jamming: smooth shear lock (src/PhysicsCloth.cpp:2656-2713, 2753-3031).
    // Every first derivative in those expressions is a multiple of
    // phi_x = -P d / (l sin phi) -- phi_s_x = sigma phi_x, con_func_x_x =
    // mu phi_x, gamma_x = kappa phi_x -- except kx_x, whose "1 - cf^2 cfx"
    // broadcasts a scalar 1 and so equals beta0 (1,1,1) + beta1 phi_x. With
    // the scalars below each Hessian entry is a short combination of rank-1
    // products; the arithmetic is the reference's, regrouped.
    const double pb = kPi / 2, pl = P.jam, sig = 0.6;
    const double cc = 3.0;
    const double LR = Lc / R;
    const T rl1s = il1 * is, rl3s = il3 * is;
    T px1[3], px3[3];
    for (int i = 0; i < 3; ++i) { px1[i] = -a3[i] * rl1s; px3[i] = -a1[i] * rl3s; }
    // half-angle sine and cosine: sqrt((1 -+ c) / 2), both >= 0 for phi in [0, pi]
    const T sh = sqrt(0.5 * (1.0 - cph)), ch = sqrt(0.5 * (1.0 + cph));
    const T gamma = (Lc * sqrt(2.0) - 2 * Lc * sh) / R;
    const T kap = -LR * ch;                       // gamma_x = kap * phi_x
    const T Aq = phi - pl, Bq = phi - pb;
    const T phs = phi * Aq * Bq;
    const T sgm = Aq * Bq + phi * Bq + phi * Aq;  // phi_s_x = sgm * phi_x
    const T omg = 2.0 * (Aq + Bq + phi);
    const double pb5 = P.pb5, pb4 = P.pb4;
    const T num = pb5 * Aq, den = phs * phs + pb4 * sig * sig;
    const T cf = tanh(num / den);
    const T den2 = den * den, rden2 = 1.0 / den2, rden22 = rden2 * rden2;
    const T tau = pb5 * den - num * (2 * phs * sgm);  // con_func_x_x numerator / phi_x
    const T muc = tau * rden2;                         // con_func_x_x = muc * phi_x
    const T g3 = gamma * gamma * gamma, g2 = gamma * gamma;
    const T base = 0.5 * (comp + 1.0) * S * kPi * (R * R);
    const T kx = base * ((1 + g3) + (1 - g3) * cf);
    const T beta0 = base * (1 - g3);
    const T beta1 = base * (cc * g2 * kap * (1 - cf) - (1 - g3) * cf * cf * muc);
    const T Bq2 = Bq * Bq;
    const T cf1 = (kx * Lc * Bq) * rl1s, cf3 = (kx * Lc * Bq) * rl3s;
    for (int i = 0; i < 3; ++i) {
      Fx1[i] = -0.5 * (beta0 + beta1 * px1[i]) * Lc * Bq2 + cf1 * a3[i];
      Fx3[i] = -0.5 * (beta0 + beta1 * px3[i]) * Lc * Bq2 + cf3 * a1[i];
    }
    // The Hessian entries of src/PhysicsCloth.cpp:2753-3031 are, for each
    // block, one fixed linear map (scalars below) applied to a few per-entry
    // quantities: pxx (phi_x_x), O = phi_xa phi_xb^T, Ob = its mirror, Rg
    // (the gamma_x_x remainder), fo (the kx-constant term), plus the scalar 1
    // broadcast by "1 - cf^2 cfx" (x1x1, x3x3 only) and kx_x's beta0 (1,1,1)
    // rows/columns. Those quantities are in turn combinations of a handful of
    // rank-1 matrices (a3 a3^T, a3 d1^T + d1 a3^T, P1, ...), so each block is
    // J = sum_k c_k B_k with c_k computed once per block.
    T P1P3[3][3], e3[3];
    matmul3(P1, P3, P1P3);  // P3 P1 is its transpose (both projectors symmetric)
    matvec3(P3, d3, e3);    // P3 d3: src/PhysicsCloth.cpp:2775-2777 multiplies outer(P3 d1, d3) by P3
    const T cfq = -2 * cf * (1 - cf * cf);
    const T c1 = cc * (cc - 1) * gamma, c2 = cc * g2;
    const T base2 = 0.5 * (comp + 1.0) * S * (R * R);
    const T kO = c1 * kap * kap * (1 - cf) - 2 * c2 * kap * (1 - cf * cf) * muc;
    const T kG = c2 * (1 - cf);
    const T cfqm2 = cfq * muc * muc;
    const T X4 = 4 * tau * den * phs * sgm;
    const T tns2 = 2 * num * sgm * sgm, tnp = 2 * num * phs, pb5den = pb5 * den;
    const T cross = 2 * phs * pb5 * sgm;
    const T hLB2 = 0.5 * Lc * Bq2, LB = Lc * Bq;
    const T kL = kx * Lc;
    const T r11 = (il1 * il1) * is, r33 = (il3 * il3) * is, r13 = il1 * il3 * is;
    const T qR11 = 0.5 * LR * sh * (rl1s * rl1s), qR33 = 0.5 * LR * sh * (rl3s * rl3s);
    const T qR13 = 0.5 * LR * sh * (il1 * il3 * (is * is));
    const T rho1 = rl1s * rl1s, rho3 = rl3s * rl3s, rho13 = rl1s * rl3s;
    // J = cP*pxx + cO*O + cOb*Ob + cR*Rg + fo (+ cOne*1 + row/column terms)
    const T hb = hLB2 * base2, g3c = 1 - g3;
    const T cR = -hb * kG;
    const T cnx_p = pb5den - tnp * sgm;  // nx = cnx_p pxx + ...
    // x1x1 and x3x3: psx = sgm pxx + omg O, cfdd = cfqm2 O + 1 - cf^2 cfx
    const T eD = -cf * cf;
    const T cPd = -hb * (kG * kap + g3c * eD * rden2 * cnx_p);
    const T cOd = -hb * (kO + g3c * (eD * (rden2 * (-tns2 - tnp * omg) - rden22 * X4) + cfqm2)) - 2 * LB * beta1;
    const T cOne = -hb * g3c;
    // x1x3 (psx = sgm pxx + omg (O + Ob) / 2) and x3x1 (psx = sgm pxx + omg O);
    // both: nx += cross (O - Ob), cfdd = cfqm2 Ob + (1 - cf^2) cfx
    const T eX = 1 - cf * cf;
    const T cPx = -hb * (kG * kap + g3c * eX * rden2 * cnx_p);
    const T cO13 = -hb * (kO + g3c * eX * (rden2 * (-tns2 - tnp * 0.5 * omg + cross) - rden22 * X4)) -
                        2 * LB * beta1;
    const T cOb13 = -hb * g3c * (eX * rden2 * (-tnp * 0.5 * omg - cross) + cfqm2);
    const T cO31 = -hb * (kO + g3c * eX * (rden2 * (-tns2 - tnp * omg + cross) - rden22 * X4)) - 2 * LB * beta1;
    const T cOb31 = -hb * g3c * (eX * rden2 * (-cross) + cfqm2);
    const T kq = Bq * cs2 - is;
    // x1x1: pxx = r11 (S - cs2 A + co P1), O = Ob = rho1 A, Rg = qR11 A,
    //       fo = kL r11 (-Bq S + kq A - Bq co P1); A = a3 a3^T, S = a3 d1^T + d1 a3^T
    {
      const T kA = cPd * (-cs2 * r11) + cOd * rho1 + cR * qR11 + kL * r11 * kq;
      const T kS = (cPd - kL * Bq) * r11;
      const T kP = (cPd - kL * Bq) * r11 * co;
      for (int i = 0; i < 3; ++i) {
        const T al = kA * a3[i] + kS * d1[i], be = kS * a3[i];
        for (int j = 0; j < 3; ++j)
          J11[i][j] = al * a3[j] + be * d1[j] + kP * P1[i][j] + (cOne - 2 * LB * beta0 * px1[j]);
      }
    }
    // x3x3: the same with (a1, d3, P3, r33, qR33, rho3, px3)
    {
      const T kA = cPd * (-cs2 * r33) + cOd * rho3 + cR * qR33 + kL * r33 * kq;
      const T kS = (cPd - kL * Bq) * r33;
      const T kP = (cPd - kL * Bq) * r33 * co;
      for (int i = 0; i < 3; ++i) {
        const T al = kA * a1[i] + kS * d3[i], be = kS * a1[i];
        for (int j = 0; j < 3; ++j)
          J33[i][j] = al * a1[j] + be * d3[j] + kP * P3[i][j] + (cOne - 2 * LB * beta0 * px3[j]);
      }
    }
    // x1x3: pxx = -r13 (cs2 A + M), O = rho13 A, Ob = rho13 B, Rg = qR13 A,
    //       fo = kL r13 (kq A + Bq M); A = a3 a1^T, B = a1 a3^T, M = P1 P3
    {
      const T kA = -cPx * r13 * cs2 + cO13 * rho13 + cR * qR13 + kL * r13 * kq;
      const T kB = cOb13 * rho13;
      const T kM = (-cPx + kL * Bq) * r13;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          J13[i][j] = kA * (a3[i] * a1[j]) + kB * (a1[i] * a3[j]) + kM * P1P3[i][j] - LB * beta0 * (px3[j] + px1[i]);
    }
    // x3x1: pxx = -r13 (cs2 E + M^T), O = rho13 A, Ob = rho13 B, Rg = qR13 A,
    //       fo = kL r13 (kq A + Bq M^T); A = a1 a3^T, B = a3 a1^T, E = a1 e3^T
    {
      const T kA = cO31 * rho13 + cR * qR13 + kL * r13 * kq;
      const T kB = cOb31 * rho13;
      const T kE = -cPx * r13 * cs2;
      const T kM = (-cPx + kL * Bq) * r13;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          J31[i][j] = kA * (a1[i] * a3[j]) + kB * (a3[i] * a1[j]) + kE * (a1[i] * e3[j]) + kM * P1P3[j][i] -
                      LB * beta0 * (px1[j] + px3[i]);
    }
  }
  int f = 0;
  auto put = [&](const T& x) { stT(buf, dbuf, 4 * (f++) + seg, nt, n0, x); };
  for (int i = 0; i < 3; ++i) put(Fx1[i]);
  for (int i = 0; i < 3; ++i) put(Fx3[i]);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) put(J11[i][j]);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) put(J13[i][j]);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) put(J31[i][j]);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) put(J33[i][j]);
}

}  // namespace ys
