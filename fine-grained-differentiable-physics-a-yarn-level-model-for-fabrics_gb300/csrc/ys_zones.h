// ys_zones.h -- impact-zone collision response on the host: the reference's
// Collision::collision_response loop (src/Collision.cpp:73-156) around the
// GPU detection, and the backward of its zone projections
// (src/Collision.cpp:496-682, InelasticProjection).
//
// Every round detects impacts (the caller's functor; after the first round
// only face pairs with an active face, update_active and the traversal's
// active test, src/Collision.cpp:158-182, 289-310), sorts them by time
// (operator<, src/Collision.cpp:255-257), keeps a greedy independent subset
// (src/Collision.cpp:259-283), adds it to impact zones with merging
// (src/Collision.cpp:438-476) and projects every zone that gained impacts:
//
//   min  1/2 sum_i a_i |x_i - x_old_i|^2
//   s.t. sum_k w_jk n_j . x_k >= thickness   for every impact j of the zone
//
// (NormalOpt, src/Collision.cpp:684-740, src/Collision.h:139-165: a_i =
// inv_m m_i with inv_m the zone's mean inverse mass, x_old the positions at
// the start of the response, obstacle nodes constant). The reference runs an
// augmented Lagrangian over Alglib's nonlinear CG (src/AugLag.cpp:13-43),
// which stops at its tolerances; here the projection is solved exactly as a
// least-distance programme (Lawson and Hanson, "Solving Least Squares
// Problems", 1974, ch. 23) through their non-negative least squares
// (ch. 23, algorithm NNLS), both restated below, for zones of up to
// exact_zone_impacts impacts, and by Hildreth's dual coordinate ascent on the
// same programme to 1e-13 relative for larger zones. Ties in time, which the
// reference leaves to its threads' emission order and std::sort, are broken
// by type, nodes, weights and normal so the result does not depend on the
// order of detection.
//
// The backward follows the reference's derivative of one projection
// (precompute_derivative and compute_derivative, src/Collision.cpp:478-524,
// 602-674): constraints within 1e-6 of active, a QR of their gradients in
// the sqrt(1 / a) metric truncated at the first |R_ii| < 1e-6, the
// multipliers moved onto the kept constraints, then dL/dx_in, dL/dw and
// dL/dn. As in the reference's autograd, the gradient of a projection's
// anchor goes to the zone's positions at the time of the projection.
#pragma once

#include "ys_pool.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace ys {

struct ZImpact {
  int type;     // 0 vertex-face, 1 edge-edge
  int node[4];  // cloth node id, or -1 - id for an obstacle node
  double t;
  double w[4];
  double n[3];
};

inline bool zimpact_less(const ZImpact& a, const ZImpact& b) {
  if (a.t != b.t) return a.t < b.t;
  if (a.type != b.type) return a.type < b.type;
  for (int k = 0; k < 4; ++k)
    if (a.node[k] != b.node[k]) return a.node[k] < b.node[k];
  for (int k = 0; k < 4; ++k)
    if (a.w[k] != b.w[k]) return a.w[k] < b.w[k];
  for (int k = 0; k < 3; ++k)
    if (a.n[k] != b.n[k]) return a.n[k] < b.n[k];
  return false;
}

namespace zone_detail {

// In-place Householder QR of A [m][p] (column-major, A[c * m + r]), no
// pivoting: R in the upper triangle, reflector j in V[j * m + j ..] with
// H_j = I - beta_j v v^T.
inline void qr(int m, int p, double* A, std::vector<double>& V, std::vector<double>& beta) {
  const int q = std::min(m, p);
  V.assign((size_t)m * std::max(q, 1), 0.0);
  beta.assign(std::max(q, 1), 0.0);
  for (int j = 0; j < q; ++j) {
    double* a = A + (size_t)j * m;
    double nx = 0.0;
    for (int r = j; r < m; ++r) nx += a[r] * a[r];
    nx = std::sqrt(nx);
    if (nx == 0.0) continue;
    const double alpha = a[j] >= 0.0 ? -nx : nx;
    double* v = V.data() + (size_t)j * m;
    double vv = 0.0;
    for (int r = j; r < m; ++r) v[r] = a[r];
    v[j] -= alpha;
    for (int r = j; r < m; ++r) vv += v[r] * v[r];
    if (vv == 0.0) continue;
    beta[j] = 2.0 / vv;
    for (int c = j + 1; c < p; ++c) {
      double* ac = A + (size_t)c * m;
      double s = 0.0;
      for (int r = j; r < m; ++r) s += v[r] * ac[r];
      s *= beta[j];
      for (int r = j; r < m; ++r) ac[r] -= s * v[r];
    }
    a[j] = alpha;
    for (int r = j + 1; r < m; ++r) a[r] = 0.0;
  }
}

// y <- Q^T y with the reflectors of qr()
inline void apply_qt(int m, int q, const std::vector<double>& V, const std::vector<double>& beta, double* y) {
  for (int j = 0; j < q; ++j) {
    if (beta[j] == 0.0) continue;
    const double* v = V.data() + (size_t)j * m;
    double s = 0.0;
    for (int r = j; r < m; ++r) s += v[r] * y[r];
    s *= beta[j];
    for (int r = j; r < m; ++r) y[r] -= s * v[r];
  }
}

// y <- Q y
inline void apply_q(int m, int q, const std::vector<double>& V, const std::vector<double>& beta, double* y) {
  for (int j = q - 1; j >= 0; --j) {
    if (beta[j] == 0.0) continue;
    const double* v = V.data() + (size_t)j * m;
    double s = 0.0;
    for (int r = j; r < m; ++r) s += v[r] * y[r];
    s *= beta[j];
    for (int r = j; r < m; ++r) y[r] -= s * v[r];
  }
}

// back substitution R z = y, R the leading p x p block of A [m][p]
inline bool back_solve(int m, int p, const double* R, const double* y, double* z) {
  for (int i = p - 1; i >= 0; --i) {
    double s = y[i];
    for (int c = i + 1; c < p; ++c) s -= R[(size_t)c * m + i] * z[c];
    const double d = R[(size_t)i * m + i];
    if (d == 0.0) return false;
    z[i] = s / d;
  }
  return true;
}

}  // namespace zone_detail

// Non-negative least squares min |E x - f|, x >= 0 (E [m][k] column-major),
// Lawson and Hanson's active-set algorithm. The QR of the passive columns is
// extended by one Householder reflector per added column and rebuilt only
// when columns leave. Returns 0, or 1 if an iteration cap was reached (x is
// then the last feasible iterate).
inline int nnls(int m, int k, const double* E, const double* f, double* x) {
  using namespace zone_detail;
  std::vector<char> inP(k, 0);
  std::vector<int> P;                  // passive columns, factorisation order
  std::vector<double> A, V, beta, y(m), r(m), zp;
  for (int j = 0; j < k; ++j) x[j] = 0.0;
  for (int i = 0; i < m; ++i) y[i] = f[i];  // Q^T f with no columns yet
  double enorm = 0.0;
  for (int j = 0; j < k; ++j) {
    double s = 0.0;
    for (int i = 0; i < m; ++i) s += E[(size_t)j * m + i] * E[(size_t)j * m + i];
    enorm = std::max(enorm, std::sqrt(s));
  }
  const double tol = 1e-13 * std::max(enorm, 1.0);
  // nonzero rows of every column (the zone constraints touch few nodes)
  std::vector<int> nzo(k + 1, 0), nzr;
  for (int j = 0; j < k; ++j) {
    for (int i = 0; i < m; ++i)
      if (E[(size_t)j * m + i] != 0.0) nzr.push_back(i);
    nzo[j + 1] = (int)nzr.size();
  }
  auto rebuild = [&]() {
    const int p = (int)P.size();
    A.assign((size_t)m * std::max(p, 1), 0.0);
    for (int c = 0; c < p; ++c) std::memcpy(A.data() + (size_t)c * m, E + (size_t)P[c] * m, sizeof(double) * m);
    qr(m, p, A.data(), V, beta);
    V.resize((size_t)m * std::max(p, 1));
    beta.resize(std::max(p, 1));
    for (int i = 0; i < m; ++i) y[i] = f[i];
    apply_qt(m, std::min(m, p), V, beta, y.data());
  };
  // appends column j (needs P.size() < m)
  auto add = [&](int j) {
    const int p = (int)P.size();
    A.resize((size_t)m * (p + 1));
    V.resize((size_t)m * (p + 1), 0.0);
    beta.resize(p + 1, 0.0);
    double* a = A.data() + (size_t)p * m;
    std::memcpy(a, E + (size_t)j * m, sizeof(double) * m);
    apply_qt(m, p, V, beta, a);
    double* v = V.data() + (size_t)p * m;
    for (int i = 0; i < m; ++i) v[i] = 0.0;
    beta[p] = 0.0;
    double nx = 0.0;
    for (int i = p; i < m; ++i) nx += a[i] * a[i];
    nx = std::sqrt(nx);
    if (nx > 0.0) {
      const double alpha = a[p] >= 0.0 ? -nx : nx;
      double vv = 0.0;
      for (int i = p; i < m; ++i) v[i] = a[i];
      v[p] -= alpha;
      for (int i = p; i < m; ++i) vv += v[i] * v[i];
      if (vv > 0.0) {
        beta[p] = 2.0 / vv;
        double s = 0.0;
        for (int i = p; i < m; ++i) s += v[i] * y[i];
        s *= beta[p];
        for (int i = p; i < m; ++i) y[i] -= s * v[i];
        a[p] = alpha;
        for (int i = p + 1; i < m; ++i) a[i] = 0.0;
      }
    }
    P.push_back(j);
  };
  // removes the last column (its reflector is its own inverse)
  auto pop = [&]() {
    const int p = (int)P.size() - 1;
    if (beta[p] != 0.0) {
      const double* v = V.data() + (size_t)p * m;
      double s = 0.0;
      for (int i = p; i < m; ++i) s += v[i] * y[i];
      s *= beta[p];
      for (int i = p; i < m; ++i) y[i] -= s * v[i];
    }
    P.pop_back();
    A.resize((size_t)m * std::max(p, 1));
    V.resize((size_t)m * std::max(p, 1));
    beta.resize(std::max(p, 1));
  };
  const int cap = 3 * k + 30;
  int blocked = -1;
  for (int outer = 0; outer < cap; ++outer) {
    for (int i = 0; i < m; ++i) r[i] = f[i];
    for (int j = 0; j < k; ++j)
      if (x[j] != 0.0)
        for (int e = nzo[j]; e < nzo[j + 1]; ++e) r[nzr[e]] -= E[(size_t)j * m + nzr[e]] * x[j];
    int jmax = -1;
    double best = tol;
    for (int j = 0; j < k; ++j) {
      if (inP[j] || j == blocked) continue;
      double s = 0.0;
      for (int e = nzo[j]; e < nzo[j + 1]; ++e) s += E[(size_t)j * m + nzr[e]] * r[nzr[e]];
      if (s > best) {
        best = s;
        jmax = j;
      }
    }
    if (jmax < 0) return 0;
    if ((int)P.size() >= m) return 1;  // cannot happen in exact arithmetic
    inP[jmax] = 1;
    add(jmax);
    bool first = true;
    for (int inner = 0; inner < cap; ++inner) {
      const int p = (int)P.size();
      zp.assign(p, 0.0);
      const bool ok = back_solve(m, p, A.data(), y.data(), zp.data());
      if (first && (!ok || !(zp[p - 1] > 0.0))) {
        // the column just added gave no positive step (rounding): leave it
        // out until the iterate changes
        pop();
        inP[jmax] = 0;
        blocked = jmax;
        break;
      }
      first = false;
      bool pos = ok;
      for (int c = 0; c < p && pos; ++c) pos = zp[c] > 0.0;
      if (pos) {
        for (int c = 0; c < p; ++c) x[P[c]] = zp[c];
        blocked = -1;
        break;
      }
      // step back to the boundary of x >= 0 and drop the variables it zeroes
      double alpha = 2.0;
      int cmin = -1;
      for (int c = 0; c < p; ++c)
        if (!(zp[c] > 0.0)) {
          const double xc = x[P[c]];
          const double d = xc - zp[c];
          const double a = d > 0.0 ? xc / d : 0.0;
          if (a < alpha) {
            alpha = a;
            cmin = c;
          }
        }
      if (cmin < 0) alpha = 0.0;
      for (int c = 0; c < p; ++c) {
        double& xc = x[P[c]];
        xc += alpha * (zp[c] - xc);
      }
      if (cmin >= 0) x[P[cmin]] = 0.0;
      std::vector<int> keep;
      for (int c = 0; c < p; ++c) {
        if (!(x[P[c]] > 0.0)) {
          x[P[c]] = 0.0;
          inP[P[c]] = 0;
        } else {
          keep.push_back(P[c]);
        }
      }
      P.swap(keep);
      rebuild();
      blocked = -1;
    }
  }
  return 1;
}

// Least-distance programme min |u| s.t. G u >= h (G [k][n] row-major) via
// NNLS on E = [G^T; h^T], f = e_n (Lawson and Hanson ch. 23). u [n] and the
// multipliers lam [k] (u = G^T lam, lam >= 0). h is scaled to unit maximum
// first. Returns 0, 1 if the constraints admit no solution (u = 0), 2 if the
// NNLS hit its cap (u from its last iterate).
inline int ldp(int n, int k, const double* G, const double* h, double* u, double* lam) {
  double s = 0.0;
  for (int j = 0; j < k; ++j) s = std::max(s, h[j]);
  for (int i = 0; i < n; ++i) u[i] = 0.0;
  for (int j = 0; j < k; ++j) lam[j] = 0.0;
  if (!(s > 0.0)) return 0;  // the anchor is feasible
  const int m = n + 1;
  std::vector<double> E((size_t)m * k), f(m, 0.0), x(k), r(m);
  for (int j = 0; j < k; ++j) {
    for (int i = 0; i < n; ++i) E[(size_t)j * m + i] = G[(size_t)j * n + i];
    E[(size_t)j * m + n] = h[j] / s;
  }
  f[n] = 1.0;
  const int st = nnls(m, k, E.data(), f.data(), x.data());
  for (int i = 0; i < m; ++i) r[i] = -f[i];
  for (int j = 0; j < k; ++j)
    if (x[j] != 0.0)
      for (int i = 0; i < m; ++i) r[i] += E[(size_t)j * m + i] * x[j];
  if (!(r[n] < -1e-12)) return 1;
  const double inv = -1.0 / r[n];
  for (int i = 0; i < n; ++i) u[i] = s * (r[i] * inv);
  for (int j = 0; j < k; ++j) lam[j] = s * (x[j] * inv);
  return st ? 2 : 0;
}

// The same least-distance programme for a large zone, with G sparse: row j
// has up to 4 blocks (column block cols[4 j + q] of 3 entries
// coef[12 j + 3 q + c]; cols < 0: unused). Hildreth's method (C. Hildreth,
// "A quadratic programming procedure", Naval Research Logistics Quarterly,
// 1957): coordinate ascent on the dual max_{lam >= 0} h^T lam - |G^T lam|^2 / 2
// with u = G^T lam kept current, rows swept in order, until a sweep changes no
// multiplier by more than tol relative and no constraint is violated by more
// than tol (h scaled to unit maximum). Each sweep costs O(rows); the exact
// NNLS costs O(n k^2). Returns 0, or 2 if max_sweeps passed without
// convergence (u and lam from the last sweep).
inline int ldp_sparse(int n, int k, const int* cols, const double* coef, const double* h, double* u, double* lam,
                      double tol = 1e-13, int max_sweeps = 200000) {
  double s = 0.0;
  for (int j = 0; j < k; ++j) s = std::max(s, h[j]);
  for (int i = 0; i < n; ++i) u[i] = 0.0;
  for (int j = 0; j < k; ++j) lam[j] = 0.0;
  if (!(s > 0.0)) return 0;
  std::vector<double> g2(k, 0.0), hs(k);
  for (int j = 0; j < k; ++j) {
    hs[j] = h[j] / s;
    for (int q = 0; q < 4; ++q)
      if (cols[4 * j + q] >= 0)
        for (int c = 0; c < 3; ++c) g2[j] += coef[12 * j + 3 * q + c] * coef[12 * j + 3 * q + c];
  }
  auto row_dot = [&](int j) {
    double d = 0.0;
    for (int q = 0; q < 4; ++q) {
      const int b = cols[4 * j + q];
      if (b < 0) continue;
      for (int c = 0; c < 3; ++c) d += coef[12 * j + 3 * q + c] * u[3 * b + c];
    }
    return d;
  };
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    double change = 0.0, lmax = 0.0;
    for (int j = 0; j < k; ++j) {
      if (!(g2[j] > 0.0)) continue;
      const double nl = std::max(0.0, lam[j] + (hs[j] - row_dot(j)) / g2[j]);
      const double dl = nl - lam[j];
      if (dl != 0.0) {
        for (int q = 0; q < 4; ++q) {
          const int b = cols[4 * j + q];
          if (b < 0) continue;
          for (int c = 0; c < 3; ++c) u[3 * b + c] += dl * coef[12 * j + 3 * q + c];
        }
        lam[j] = nl;
      }
      change = std::max(change, std::fabs(dl) * std::sqrt(g2[j]));
      lmax = std::max(lmax, nl * std::sqrt(g2[j]));
    }
    double viol = 0.0;
    for (int j = 0; j < k; ++j)
      if (g2[j] > 0.0) viol = std::max(viol, hs[j] - row_dot(j));
    if (change <= tol * std::max(lmax, 1.0) && viol <= tol) break;
  }
  for (int i = 0; i < n; ++i) u[i] *= s;
  for (int j = 0; j < k; ++j) lam[j] *= s;
  return sweep < max_sweeps ? 0 : 2;
}

struct ZoneRecord {  // one zone projection
  int round = 0;
  std::vector<int> nodes;    // the zone's cloth nodes, zone order
  std::vector<int> imps;     // its constraints: indices of accepted impacts
  std::vector<double> a;     // objective weight inv_m m of each node
  std::vector<double> xout;  // [3 nodes] projected positions
  std::vector<double> lam;   // multiplier of each constraint
  int status = 0;            // ldp() status; 3: reverted to the start of the step (see revert_factor)
};

struct ZoneResponse {
  // inputs
  int n_nodes = 0, n_faces = 0;
  const int* faces = nullptr;     // cloth faces [F][3]
  const double* obs_x = nullptr;  // obstacle node positions [No][3]
  const double* xprev = nullptr;  // cloth and obstacle positions at the start of the step
  const double* obs_xprev = nullptr;
  double thickness = 0.0;
  int max_iter = 100;
  // zones of up to this many impacts are projected exactly (LDP through
  // NNLS, cost O(n k^2)); larger ones -- a contact patch of a cloth lying on
  // an obstacle chains its impacts into one zone through shared nodes -- by
  // Hildreth's iterations on sparse rows (ldp_sparse)
  int exact_zone_impacts = 64;
  // a zone that gathers more impacts than this stops the response (a bound
  // on the time and memory of one projection; layers tangled beyond what a
  // step's detection separates keep merging zones)
  int max_zone_impacts = 65536;
  // A zone holds the constraints of every round it received impacts in,
  // each linearised where it was found; on a crumpling cloth two of them can
  // constrain one edge pair with nearly opposite normals, and the exact
  // projection then lies far away (nodes moved by centimetres; the
  // reference's inexact augmented Lagrangian stops long before). When the
  // projection would move a node by more than revert_factor times (its own
  // displacement in the step + thickness), the zone's nodes go back to their
  // positions at the start of the step instead (needs xprev; <= 0: off).
  double revert_factor = 4.0;
  // results
  std::vector<ZImpact> accepted;  // every impact a zone received, in order
  std::vector<int> accepted_round;
  std::vector<double> accepted_x;  // [accepted][4][3] its nodes' positions when it was found
  std::vector<double> accepted_xp;  // [accepted][4][3] and at the start of the step
  std::vector<ZoneRecord> tape;   // every projection, in order
  int rounds = 0, converged = 0, changed = 0, zones = 0, infeasible = 0, reverted = 0;
  int zone_overflow = 0;  // stopped at a zone larger than max_zone_impacts
};

namespace zone_detail {

inline double node_x(const double* x, const double* obs_x, int nd, int c) {
  return nd >= 0 ? x[3 * (size_t)nd + c] : obs_x[3 * (size_t)(-1 - nd) + c];
}

// projects one zone in place (x: all cloth positions), records it
// one zone's projection into rec; it writes x and local at the zone's own
// nodes only, so zones with disjoint nodes can be projected at once
inline void project_zone(const ZoneResponse& R, const std::vector<int>& nodes, const std::vector<int>& imps,
                         const double* mass, const double* xold, double* x, std::vector<int>& local, int round,
                         ZoneRecord& rec) {
  const int m = (int)nodes.size(), nv = 3 * m, k = (int)imps.size();
  rec.round = round;
  rec.nodes = nodes;
  rec.imps = imps;
  double inv_m = 0.0;
  for (int i = 0; i < m; ++i) inv_m += 1.0 / (mass ? mass[nodes[i]] : 1.0);
  inv_m /= (double)m;
  rec.a.resize(m);
  std::vector<double> isa(m);
  for (int i = 0; i < m; ++i) {
    rec.a[i] = inv_m * (mass ? mass[nodes[i]] : 1.0);
    isa[i] = 1.0 / std::sqrt(rec.a[i]);
    local[nodes[i]] = i;
  }
  const bool dense = k <= R.exact_zone_impacts;
  std::vector<double> G(dense ? (size_t)k * nv : 0, 0.0), h(k), u(nv);
  std::vector<int> cols(dense ? 0 : 4 * (size_t)k, -1);
  std::vector<double> coef(dense ? 0 : 12 * (size_t)k, 0.0);
  rec.lam.assign(k, 0.0);
  for (int j = 0; j < k; ++j) {
    const ZImpact& im = R.accepted[imps[j]];
    double hj = R.thickness;
    for (int q = 0; q < 4; ++q) {
      const int nd = im.node[q];
      if (nd >= 0) {
        const int li = local[nd];
        if (!dense) cols[4 * (size_t)j + q] = li;
        for (int c = 0; c < 3; ++c) {
          const double g = im.w[q] * im.n[c] * isa[li];
          if (dense) G[(size_t)j * nv + 3 * li + c] += g;
          else coef[12 * (size_t)j + 3 * q + c] = g;
          hj -= im.w[q] * im.n[c] * xold[3 * (size_t)nd + c];
        }
      } else {
        for (int c = 0; c < 3; ++c) hj -= im.w[q] * im.n[c] * R.obs_x[3 * (size_t)(-1 - nd) + c];
      }
    }
    h[j] = hj;
  }
  rec.status = dense ? ldp(nv, k, G.data(), h.data(), u.data(), rec.lam.data())
                     : ldp_sparse(nv, k, cols.data(), coef.data(), h.data(), u.data(), rec.lam.data());
  if (rec.status != 1 && R.xprev && R.revert_factor > 0.0) {
    bool far = false;
    for (int i = 0; i < m && !far; ++i) {
      double mv = 0.0, st = 0.0;
      for (int c = 0; c < 3; ++c) {
        const size_t g = 3 * (size_t)nodes[i] + c;
        const double d = u[3 * i + c] * isa[i];
        mv += d * d;
        st += (xold[g] - R.xprev[g]) * (xold[g] - R.xprev[g]);
      }
      far = std::sqrt(mv) > R.revert_factor * (std::sqrt(st) + R.thickness);
    }
    if (far) rec.status = 3;
  }
  rec.xout.resize(nv);
  for (int i = 0; i < m; ++i)
    for (int c = 0; c < 3; ++c) {
      const size_t g = 3 * (size_t)nodes[i] + c;
      const double xn = rec.status == 1 ? x[g] : rec.status == 3 ? R.xprev[g] : xold[g] + u[3 * i + c] * isa[i];
      x[g] = xn;
      rec.xout[3 * i + c] = xn;
    }
  for (int i = 0; i < m; ++i) local[nodes[i]] = -1;
}

// the record's outcome into R (its counters and the tape, in zone order)
inline void record_zone(ZoneResponse& R, ZoneRecord&& rec) {
  if (rec.status == 1) R.infeasible++;
  if (rec.status == 3) R.reverted++;
  R.tape.push_back(std::move(rec));
}

}  // namespace zone_detail

// The response loop. x [n][3] (in: positions after the step, out: after the
// response); detect(x, face_active or nullptr, out) fills out with the
// impacts of the current positions (only face pairs with an active face when
// face_active is given) and returns 0 on success. mass [n] may be null
// (equal masses). Returns the detector's first non-zero status, else 0.
template <class Detect>
int zone_respond(ZoneResponse& R, double* x, const double* mass, Detect&& detect, BuildPool* pool = nullptr) {
  const int n = R.n_nodes;
  R.accepted.clear();
  R.accepted_round.clear();
  R.accepted_x.clear();
  R.accepted_xp.clear();
  R.tape.clear();
  R.rounds = R.converged = R.changed = R.zones = R.infeasible = R.zone_overflow = R.reverted = 0;
  std::vector<double> xold(x, x + 3 * (size_t)n);
  // faces around each node (the verts' adj_faces of the cloth mesh)
  std::vector<int> fo(n + 1, 0), fl(3 * (size_t)R.n_faces);
  for (int f = 0; f < R.n_faces; ++f)
    for (int q = 0; q < 3; ++q) fo[R.faces[3 * f + q] + 1]++;
  for (int i = 0; i < n; ++i) fo[i + 1] += fo[i];
  {
    std::vector<int> pos(fo.begin(), fo.end() - 1);
    for (int f = 0; f < R.n_faces; ++f)
      for (int q = 0; q < 3; ++q) fl[pos[R.faces[3 * f + q]]++] = f;
  }
  struct Zone {
    std::vector<int> nodes, imps;
    bool active = false;
  };
  std::vector<Zone> zs;        // every zone ever made (merged ones emptied)
  std::vector<int> order;      // live zones in the reference's vector order
  std::vector<int> zone_of(n, -1);
  std::vector<int> local(n, -1);
  std::vector<uint8_t> face_active(R.n_faces);
  std::vector<ZImpact> found, indep;
  std::vector<char> taken(n, 0);
  std::vector<int> active;
  std::vector<ZoneRecord> recs;
  auto find_or_create = [&](int nd) {
    if (zone_of[nd] >= 0) return zone_of[nd];
    zs.push_back(Zone());
    zs.back().nodes.push_back(nd);
    zone_of[nd] = (int)zs.size() - 1;
    order.push_back(zone_of[nd]);
    return zone_of[nd];
  };
  int iter = 0;
  for (iter = 0; iter < R.max_iter; ++iter) {
    const uint8_t* mask = nullptr;
    if (!order.empty()) {
      std::fill(face_active.begin(), face_active.end(), 0);
      for (int z : order) {
        if (!zs[z].active) continue;
        for (int nd : zs[z].nodes)
          for (int e = fo[nd]; e < fo[nd + 1]; ++e) face_active[fl[e]] = 1;
      }
      mask = face_active.data();
    }
    found.clear();
    const int st = detect((const double*)x, mask, found);
    if (st) return st;
    std::sort(found.begin(), found.end(), zimpact_less);
    // greedy independent subset: an impact conflicts with a kept one when one
    // of its free nodes is among the kept one's nodes (conflict(),
    // src/Collision.cpp:276-283)
    indep.clear();
    for (const ZImpact& im : found) {
      bool conf = false;
      for (int q = 0; q < 4 && !conf; ++q) conf = im.node[q] >= 0 && taken[im.node[q]];
      if (conf) continue;
      indep.push_back(im);
      for (int q = 0; q < 4; ++q)
        if (im.node[q] >= 0) taken[im.node[q]] = 1;
    }
    for (const ZImpact& im : indep)
      for (int q = 0; q < 4; ++q)
        if (im.node[q] >= 0) taken[im.node[q]] = 0;
    if (indep.empty()) break;
    // add_impacts
    for (int z : order) zs[z].active = false;
    for (const ZImpact& im : indep) {
      const int id = (int)R.accepted.size();
      R.accepted.push_back(im);
      R.accepted_round.push_back(iter);
      for (int q = 0; q < 4; ++q)
        for (int c = 0; c < 3; ++c) {
          R.accepted_x.push_back(zone_detail::node_x(x, R.obs_x, im.node[q], c));
          R.accepted_xp.push_back(R.xprev ? zone_detail::node_x(R.xprev, R.obs_xprev, im.node[q], c) : 0.0);
        }
      const int z0 = find_or_create(im.node[0] >= 0 ? im.node[0] : im.node[3]);
      for (int q = 0; q < 4; ++q) {
        if (im.node[q] < 0) continue;
        const int z1 = find_or_create(im.node[q]);
        if (z1 == z0) continue;
        for (int nd : zs[z1].nodes) zone_of[nd] = z0;
        zs[z0].nodes.insert(zs[z0].nodes.end(), zs[z1].nodes.begin(), zs[z1].nodes.end());
        zs[z0].imps.insert(zs[z0].imps.end(), zs[z1].imps.begin(), zs[z1].imps.end());
        zs[z1].nodes.clear();
        zs[z1].imps.clear();
        order.erase(std::find(order.begin(), order.end(), z1));
      }
      zs[z0].imps.push_back(id);
      zs[z0].active = true;
    }
    for (int z : order)
      if (zs[z].active && (int)zs[z].imps.size() > R.max_zone_impacts) R.zone_overflow = 1;
    if (R.zone_overflow) break;
    // the active zones' projections: their nodes are disjoint, so on a pool
    // they run at once and are recorded in zone order afterwards
    active.clear();
    for (int z : order)
      if (zs[z].active) active.push_back(z);
    if (!active.empty()) R.changed = 1;
    recs.clear();
    recs.resize(active.size());
    auto proj = [&](int i) {
      const Zone& zn = zs[active[i]];
      zone_detail::project_zone(R, zn.nodes, zn.imps, mass, xold.data(), x, local, iter, recs[i]);
    };
    if (pool && pool->size() > 1 && active.size() > 1) pool->run((int)active.size(), proj);
    else
      for (size_t i = 0; i < active.size(); ++i) proj((int)i);
    for (ZoneRecord& rec : recs) zone_detail::record_zone(R, std::move(rec));
  }
  R.rounds = iter;
  R.converged = iter < R.max_iter && !R.zone_overflow;
  R.zones = (int)order.size();
  return 0;
}

namespace zone_detail {

// forward-mode number with the 24 directions of one impact's inputs: the
// four nodes' positions at the end (3 k + c) and start (12 + 3 k + c) of the
// step
struct D24 {
  double v;
  double d[24];
};
inline D24 dc(double v) {
  D24 r;
  r.v = v;
  for (double& x : r.d) x = 0.0;
  return r;
}
inline D24 operator+(const D24& a, const D24& b) {
  D24 r;
  r.v = a.v + b.v;
  for (int i = 0; i < 24; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
inline D24 operator-(const D24& a, const D24& b) {
  D24 r;
  r.v = a.v - b.v;
  for (int i = 0; i < 24; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
inline D24 operator-(const D24& a) {
  D24 r;
  r.v = -a.v;
  for (int i = 0; i < 24; ++i) r.d[i] = -a.d[i];
  return r;
}
inline D24 operator*(const D24& a, const D24& b) {
  D24 r;
  r.v = a.v * b.v;
  for (int i = 0; i < 24; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
inline D24 operator/(const D24& a, const D24& b) {
  D24 r;
  r.v = a.v / b.v;
  for (int i = 0; i < 24; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
  return r;
}
inline D24 dsqrt(const D24& a) {
  D24 r;
  r.v = std::sqrt(a.v);
  for (int i = 0; i < 24; ++i) r.d[i] = a.d[i] / (2.0 * r.v);
  return r;
}
inline void dcross(const D24* a, const D24* b, D24* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
inline D24 ddot(const D24* a, const D24* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline D24 dtriple(const D24* a, const D24* b, const D24* c) {
  D24 t[3];
  dcross(b, c, t);
  return ddot(a, t);
}

}  // namespace zone_detail

// d(w, n) / d(positions) of one impact of type `type` found at time t with
// node positions x [4][3] (end of step) and xp [4][3] (start): J [7][24], rows
// w0..w3, n0..n2, columns x of node k (3 k + c) then xp (12 + 3 k + c). The
// computation is collision_test's (src/Collision.cpp:376-436: the cubic's
// root t, the positions at t, sub_signed_vf / ee_distance, the orientation
// of n), differentiated forward. cubic_sign -1 takes the root's exact
// derivative dt = -(t^3 da3 + t^2 da2 + t da1 + da0) / p'(t); +1 takes the
// reference's CubicSolver backward (src/Solvers.cpp:172-178), which drops
// that minus sign. Returns false where the reference would have found no
// impact (degenerate normal).
inline bool impact_jacobian(int type, const double* x, const double* xp, double troot, int cubic_sign,
                            double J[7][24]) {
  using namespace zone_detail;
  D24 X[4][3], XP[4][3];
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 3; ++c) {
      X[k][c] = dc(x[3 * k + c]);
      X[k][c].d[3 * k + c] = 1.0;
      XP[k][c] = dc(xp[3 * k + c]);
      XP[k][c].d[12 + 3 * k + c] = 1.0;
    }
  D24 x1[3], x2[3], x3[3], v0[3], v1[3], v2[3], v3[3];
  for (int i = 0; i < 3; ++i) {
    v0[i] = X[0][i] - XP[0][i];
    x1[i] = XP[1][i] - XP[0][i];
    x2[i] = XP[2][i] - XP[0][i];
    x3[i] = XP[3][i] - XP[0][i];
    v1[i] = X[1][i] - XP[1][i] - v0[i];
    v2[i] = X[2][i] - XP[2][i] - v0[i];
    v3[i] = X[3][i] - XP[3][i] - v0[i];
  }
  const D24 a0 = dtriple(x1, x2, x3);
  const D24 a1 = dtriple(v1, x2, x3) + dtriple(x1, v2, x3) + dtriple(x1, x2, v3);
  const D24 a2 = dtriple(x1, v2, v3) + dtriple(v1, x2, v3) + dtriple(v1, v2, x3);
  const D24 a3 = dtriple(v1, v2, v3);
  const double t = troot;
  const double dp = (3.0 * a3.v * t + 2.0 * a2.v) * t + a1.v;
  D24 T = dc(t);
  for (int i = 0; i < 24; ++i)
    T.d[i] = cubic_sign * (((a3.d[i] * t + a2.d[i]) * t + a1.d[i]) * t + a0.d[i]) / dp;
  D24 b1[3], b2[3], b3[3];
  for (int i = 0; i < 3; ++i) {
    b1[i] = x1[i] + T * v1[i];
    b2[i] = x2[i] + T * v2[i];
    b3[i] = x3[i] + T * v3[i];
  }
  D24 n[3], w[4];
  if (type == 0) {  // sub_signed_vf_distance(b1, b2, b3)
    D24 a[3], b[3], tt[3];
    for (int i = 0; i < 3; ++i) {
      a[i] = b2[i] - b1[i];
      b[i] = b3[i] - b1[i];
    }
    dcross(a, b, n);
    const D24 l = dsqrt(ddot(n, n));
    if (!(l.v > 0.0)) return false;
    for (int i = 0; i < 3; ++i) n[i] = n[i] / l;
    dcross(b3, n, tt);
    const D24 c0 = ddot(b2, tt);
    dcross(b1, n, tt);
    const D24 c1 = ddot(b3, tt);
    dcross(b2, n, tt);
    const D24 c2 = ddot(b1, tt);
    const D24 sum = dc(1.0) / (c0 + c1 + c2);
    w[0] = dc(1.0);
    w[1] = -(c0 * sum);
    w[2] = -(c1 * sum);
    w[3] = -(c2 * sum);
  } else {  // sub_signed_ee_distance(b1, b2, b3, b2 - b1, b3 - b1, b3 - b2)
    D24 x1mx0[3], y0mx0[3], y1mx0[3], y0mx1[3], y1mx1[3], y1my0[3], tt[3];
    for (int i = 0; i < 3; ++i) {
      x1mx0[i] = b1[i];
      y0mx0[i] = b2[i];
      y1mx0[i] = b3[i];
      y0mx1[i] = b2[i] - b1[i];
      y1mx1[i] = b3[i] - b1[i];
      y1my0[i] = b3[i] - b2[i];
    }
    dcross(x1mx0, y1my0, n);
    const D24 l = dsqrt(ddot(n, n));
    if (!(l.v > 0.0)) return false;
    for (int i = 0; i < 3; ++i) n[i] = n[i] / l;
    dcross(y0mx1, n, tt);
    const D24 e0 = ddot(y1mx1, tt);
    dcross(y1mx0, n, tt);
    const D24 e1 = ddot(y0mx0, tt);
    dcross(y1mx0, n, tt);
    const D24 f0 = ddot(y1mx1, tt);
    dcross(y0mx1, n, tt);
    const D24 f1 = ddot(y0mx0, tt);
    const D24 suma = dc(1.0) / (e0 + e1), sumb = dc(1.0) / (f0 + f1);
    w[0] = e0 * suma;
    w[1] = e1 * suma;
    w[2] = -(f0 * sumb);
    w[3] = -(f1 * sumb);
  }
  double rv[3];
  for (int i = 0; i < 3; ++i) rv[i] = w[1].v * v1[i].v + w[2].v * v2[i].v + w[3].v * v3[i].v;
  const double flip = (n[0].v * rv[0] + n[1].v * rv[1] + n[2].v * rv[2]) > 0.0 ? -1.0 : 1.0;
  for (int i = 0; i < 24; ++i) {
    for (int q = 0; q < 4; ++q) J[q][i] = w[q].d[i];
    for (int c = 0; c < 3; ++c) J[4 + c][i] = flip * n[c].d[i];
  }
  return true;
}

// Backward of the projections: g [n][3] in: dL/dx after the response, out:
// dL/dx before it (through the projections only); gw [accepted][4] and
// gn [accepted][3] receive dL/dw and dL/dn of every accepted impact
// (accumulated; zero them first).
//
// flags & 1 also carries the impacts' weight and normal gradients into the
// positions they were computed from, as the reference's autograd does through
// collision_test: rounds are undone last to first, and an impact's gradient
// is complete once the projections of its own and later rounds are undone;
// gxp [n][3] (accumulated) receives the part for the step's start positions.
// flags & 2 takes the cubic root's exact derivative instead of the
// reference's CubicSolver backward (impact_jacobian).
inline void zone_backward(const ZoneResponse& R, double* g, double* gw, double* gn, int flags = 0,
                          double* gxp = nullptr) {
  using namespace zone_detail;
  std::vector<double> A, V, beta, lam, sm1, gz, t1, qtx, dz, dlam, r1l, lamp;
  std::vector<int> legal;
  int last_round = 0;
  for (const ZoneRecord& rec : R.tape) last_round = std::max(last_round, rec.round);
  for (int r : R.accepted_round) last_round = std::max(last_round, r);
  for (int round = last_round; round >= 0; --round) {
  for (int ri = (int)R.tape.size() - 1; ri >= 0; --ri) {
    const ZoneRecord& rec = R.tape[ri];
    if (rec.round != round) continue;
    if (rec.status == 3) {  // reverted: the zone's positions are the step's start positions
      for (int nd : rec.nodes)
        for (int c = 0; c < 3; ++c) {
          if (gxp) gxp[3 * (size_t)nd + c] += g[3 * (size_t)nd + c];
          g[3 * (size_t)nd + c] = 0.0;
        }
      continue;
    }
    const int m = (int)rec.nodes.size(), nv = 3 * m, k = (int)rec.imps.size();
    auto local = [&](int nd) {
      for (int i = 0; i < m; ++i)
        if (rec.nodes[i] == nd) return i;
      return -1;
    };
    sm1.resize(nv);
    for (int i = 0; i < m; ++i)
      for (int c = 0; c < 3; ++c) sm1[3 * i + c] = 1.0 / std::sqrt(rec.a[i]);
    // constraints within 1e-6 of active at the solution
    legal.clear();
    for (int j = 0; j < k; ++j) {
      const ZImpact& im = R.accepted[rec.imps[j]];
      double cj = R.thickness;
      for (int q = 0; q < 4; ++q) {
        const int nd = im.node[q];
        const int li = nd >= 0 ? local(nd) : -1;
        for (int c = 0; c < 3; ++c) {
          const double xc = li >= 0 ? rec.xout[3 * li + c] : nd < 0 ? node_x(nullptr, R.obs_x, nd, c) : 0.0;
          cj -= im.w[q] * im.n[c] * xc;
        }
      }
      if (cj < -1e-6) continue;
      legal.push_back(j);
    }
    const int L = (int)legal.size();
    A.assign((size_t)nv * std::max(L, 1), 0.0);
    for (int l = 0; l < L; ++l) {
      const ZImpact& im = R.accepted[rec.imps[legal[l]]];
      for (int q = 0; q < 4; ++q) {
        const int li = im.node[q] >= 0 ? local(im.node[q]) : -1;
        if (li < 0) continue;
        for (int c = 0; c < 3; ++c) A[(size_t)l * nv + 3 * li + c] -= im.w[q] * im.n[c] * sm1[3 * li + c];
      }
    }
    const int cols = std::min(L, nv);
    qr(nv, L, A.data(), V, beta);
    int nd0 = 0;
    while (nd0 < cols && std::fabs(A[(size_t)nd0 * nv + nd0]) >= 1e-6) ++nd0;
    // multipliers of the dropped constraints moved onto the kept ones
    lam = rec.lam;
    if (nd0 > 0) {
      r1l.assign(nd0, 0.0);
      for (int i = 0; i < nd0; ++i)
        for (int l = nd0; l < L; ++l) r1l[i] += A[(size_t)l * nv + i] * lam[legal[l]];
      lamp.assign(nd0, 0.0);
      back_solve(nv, nd0, A.data(), r1l.data(), lamp.data());
      for (int i = 0; i < nd0; ++i) lam[legal[i]] += lamp[i];
    }
    for (int l = nd0; l < L; ++l) lam[legal[l]] = 0.0;
    // qtx = Q0^T sqrt(1/a) g, dz = sqrt(1/a) (sqrt(1/a) g - Q0 qtx)
    gz.resize(nv);
    for (int i = 0; i < m; ++i)
      for (int c = 0; c < 3; ++c) gz[3 * i + c] = g[3 * (size_t)rec.nodes[i] + c];
    t1.resize(nv);
    for (int r = 0; r < nv; ++r) t1[r] = gz[r] * sm1[r];
    apply_qt(nv, cols, V, beta, t1.data());
    qtx.assign(t1.begin(), t1.begin() + nd0);
    std::vector<double> proj(nv, 0.0);
    for (int i = 0; i < nd0; ++i) proj[i] = qtx[i];
    apply_q(nv, cols, V, beta, proj.data());
    dz.resize(nv);
    for (int r = 0; r < nv; ++r) dz[r] = sm1[r] * (gz[r] * sm1[r] - proj[r]);
    dlam.assign(k, 0.0);
    if (nd0 > 0) {
      std::vector<double> d0(nd0);
      back_solve(nv, nd0, A.data(), qtx.data(), d0.data());
      for (int i = 0; i < nd0; ++i) dlam[legal[i]] = d0[i];
    }
    for (int j = 0; j < k; ++j) {
      const int id = rec.imps[j];
      const ZImpact& im = R.accepted[id];
      for (int q = 0; q < 4; ++q) {
        const int nd = im.node[q];
        const int li = nd >= 0 ? local(nd) : -1;
        for (int c = 0; c < 3; ++c) {
          double tv;
          if (li >= 0) {
            tv = dlam[j] * rec.xout[3 * li + c] + lam[j] * dz[3 * li + c];
          } else if (nd < 0) {
            tv = dlam[j] * node_x(nullptr, R.obs_x, nd, c);
          } else {
            tv = 0.0;  // a free node outside the zone: never, zones hold every free node of their impacts
          }
          gw[4 * (size_t)id + q] += tv * im.n[c];
          gn[3 * (size_t)id + c] += im.w[q] * tv;
        }
      }
    }
    for (int i = 0; i < m; ++i)
      for (int c = 0; c < 3; ++c) g[3 * (size_t)rec.nodes[i] + c] = dz[3 * i + c] / (sm1[3 * i + c] * sm1[3 * i + c]);
  }
  if (!(flags & 1)) continue;
  // the impacts found this round, into the positions they were found at
  for (size_t id = 0; id < R.accepted.size(); ++id) {
    if (R.accepted_round[id] != round) continue;
    const ZImpact& im = R.accepted[id];
    double J[7][24];
    if (!impact_jacobian(im.type, &R.accepted_x[12 * id], &R.accepted_xp[12 * id], im.t, (flags & 2) ? -1 : 1, J))
      continue;
    double gr[7];
    for (int q = 0; q < 4; ++q) gr[q] = gw[4 * id + q];
    for (int c = 0; c < 3; ++c) gr[4 + c] = gn[3 * id + c];
    for (int q = 0; q < 4; ++q) {
      const int nd = im.node[q];
      if (nd < 0) continue;  // obstacles are given
      for (int c = 0; c < 3; ++c) {
        double sx = 0.0, sp = 0.0;
        for (int row = 0; row < 7; ++row) {
          sx += J[row][3 * q + c] * gr[row];
          sp += J[row][12 + 3 * q + c] * gr[row];
        }
        g[3 * (size_t)nd + c] += sx;
        if (gxp) gxp[3 * (size_t)nd + c] += sp;
      }
    }
  }
  }
}

}  // namespace ys
