// ys_physics.cuh -- per-element yarn forces and Jacobians of one implicit step.
//
// Each routine handles one element (edge, bend segment, crossing, shear
// segment, face) and adds its contribution straight into the step's system
//     A = M - h^2 dF/dx - h dF/dv,   b = h (F - (dF/dv)^T v) + M v
// (src/TrainHelper.cpp:19-20) in the structured stencil layout of
// ys_common.cuh. Elements of one launch are graph-coloured so that no two
// threads touch the same node rows, which keeps the accumulation
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

namespace ys {

// ---------------------------------------------------------------- helpers
YS_HD double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
YS_HD double norm3(const double* a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
YS_HD void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
YS_HD void proj3(const double* d, double P[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P[i][j] = (i == j ? 1.0 : 0.0) - d[i] * d[j];
}
YS_HD void matvec3(const double P[3][3], const double* a, double* o) {
  for (int i = 0; i < 3; ++i) o[i] = P[i][0] * a[0] + P[i][1] * a[1] + P[i][2] * a[2];
}
YS_HD void outer3(const double* a, const double* b, double O[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) O[i][j] = a[i] * b[j];
}
YS_HD void matmul3(const double A[3][3], const double B[3][3], double O[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) O[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}
YS_HD double ld(const double* p, int comp, int ntot, int node) { return p[(int64_t)comp * ntot + node]; }
YS_HD double& st(double* p, int comp, int ntot, int node) { return p[(int64_t)comp * ntot + node]; }

// Adds val into A at (row node, row comp) x (col node, col comp); comp 0..2 =
// Lagrangian x,y,z, comp 3 = the Eulerian DOF k (0 = u, 1 = v).
YS_HD void add_A(const View& v, int rn, int rc, int cn, int cc, int k, double val, int du, int dv) {
  if (rc < 3 && cc < 3) {
    int s = stencil_index(du, dv);
    if (s < 0) return;  // not reachable for the element types above; keeps every store in bounds
    slot(v, YS_SLOT_LL + s * 9 + rc * 3 + cc, rn) += val;
  } else if (rc < 3) {
    int n = yarn_nbr(du, dv);
    if (n < 0) slot(v, YS_SLOT_LE_SELF + rc * 2 + k, rn) += val;
    else slot(v, YS_SLOT_LE_NBR + n * 3 + rc, rn) += val;
  } else if (cc < 3) {
    int n = yarn_nbr(du, dv);
    if (n < 0) slot(v, YS_SLOT_EL_SELF + k * 3 + cc, rn) += val;
    else slot(v, YS_SLOT_EL_NBR + n * 3 + cc, rn) += val;
  } else {
    int n = yarn_nbr(du, dv);
    if (n < 0) slot(v, YS_SLOT_EE_SELF + k, rn) += val;
    else slot(v, YS_SLOT_EE_NBR + n, rn) += val;
  }
}

// ------------------------------------------------------------ edge element
// Local DOFs of an edge: x0 (0..2), e0 (3), x1 (4..6), e1 (7), where e is the
// Eulerian coordinate along the edge's yarn (u for warp, v for weft).
struct EdgeAcc {
  double A[8][8];   // contribution to A in reference layout
  double b[8];      // contribution to b
  double Vloc[8];   // the step's velocity vector restricted to the edge
  double fe[2], kee[2], dee[2];
  double cl[2][3], cle[2][3];
  double h, h2;
  bool in[2];
};

enum Mat { kM = 0, kK = 1, kD = 2 };

// X_LL[find_index(f, d, "LL")] += s * blk; the dense matrix receives the
// block transposed (src/PhysicsCloth.cpp:202, src/MatrixMp.cpp:54-65).
template <class F>
YS_HD void acc_LL(EdgeAcc& a, int X, int f, int d, double s, const F& blk) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double val = s * blk(c, r);
      int row = 4 * f + r, col = 4 * d + c;
      if (X == kM) { a.A[row][col] += val; a.b[row] += val * a.Vloc[col]; }
      else if (X == kK) { a.A[row][col] += -a.h2 * val; }
      else { a.A[row][col] += -a.h * val; a.b[col] -= a.h * val * a.Vloc[row]; }
    }
}
// X_LE[find_index(l, e, "EL") + k] += s * vec  ->  A[x(l)][e(e)]
template <class F>
YS_HD void acc_LE(EdgeAcc& a, int X, int l, int e, double s, const F& vec) {
  for (int r = 0; r < 3; ++r) {
    double val = s * vec(r);
    int row = 4 * l + r, col = 4 * e + 3;
    if (X == kM) { a.A[row][col] += val; a.b[row] += val * a.Vloc[col]; }
    else if (X == kK) { a.A[row][col] += -a.h2 * val; }
    else { a.A[row][col] += -a.h * val; a.b[col] -= a.h * val * a.Vloc[row]; }
  }
}
// X_EL[find_index(l, e, "EL") + k] += s * row  ->  A[e(e)][x(l)]
template <class F>
YS_HD void acc_EL(EdgeAcc& a, int X, int l, int e, double s, const F& rowv) {
  for (int c = 0; c < 3; ++c) {
    double val = s * rowv(c);
    int row = 4 * e + 3, col = 4 * l + c;
    if (X == kM) { a.A[row][col] += val; a.b[row] += val * a.Vloc[col]; }
    else if (X == kK) { a.A[row][col] += -a.h2 * val; }
    else { a.A[row][col] += -a.h * val; a.b[col] -= a.h * val * a.Vloc[row]; }
  }
}
YS_HD void acc_EE(EdgeAcc& a, int X, int f, int d, double val) {
  int row = 4 * f + 3, col = 4 * d + 3;
  if (X == kM) { a.A[row][col] += val; a.b[row] += val * a.Vloc[col]; }
  else if (X == kK) { a.A[row][col] += -a.h2 * val; if (f == d) a.kee[f] += val; }
  else { a.A[row][col] += -a.h * val; a.b[col] -= a.h * val * a.Vloc[row]; if (f == d) a.dee[f] += val; }
}
YS_HD void acc_F(EdgeAcc& a, int dof, double f) {
  a.b[dof] += a.h * f;
  if ((dof & 3) == 3) a.fe[dof >> 2] += f;
}

// The write pattern shared by Inertia_D_Pos, Inertia_D_Vel, MDotVDot_D_Pos
// and MDotVDot_D_Vel (src/PhysicsCloth.cpp:1544-1600, 1848-1900,
// 2226-2308, 2505-2577): C(i, j) = d(force DOF i)/d(DOF j) in edge-local
// order, added with sign s.
template <class F>
YS_HD void acc_edge_jac(EdgeAcc& a, int X, double s, const F& C) {
  acc_LL(a, X, 0, 0, s, [&](int i, int j) { return C(i, j); });
  acc_LL(a, X, 0, 1, s, [&](int i, int j) { return C(i, 4 + j); });
  acc_LL(a, X, 1, 0, s, [&](int i, int j) { return C(4 + i, j); });
  acc_LL(a, X, 1, 1, s, [&](int i, int j) { return C(4 + i, 4 + j); });
  if (a.in[0]) {
    acc_EL(a, X, 0, 0, s, [&](int c) { return C(3, c); });
    acc_LE(a, X, 0, 0, s, [&](int r) { return C(r, 3); });
    acc_EE(a, X, 0, 0, s * C(3, 3));
  }
  if (a.in[1]) {
    acc_EL(a, X, 1, 1, s, [&](int c) { return C(7, 4 + c); });
    acc_LE(a, X, 1, 1, s, [&](int r) { return C(4 + r, 7); });
    acc_EE(a, X, 1, 1, s * C(7, 7));
  }
  if (a.in[0] && a.in[1]) {
    acc_LE(a, X, 1, 0, s, [&](int r) { return C(4 + r, 3); });
    acc_LE(a, X, 0, 1, s, [&](int r) { return C(r, 7); });
    acc_EL(a, X, 1, 0, s, [&](int c) { return C(3, 4 + c); });
    acc_EL(a, X, 0, 1, s, [&](int c) { return C(7, c); });
    acc_EE(a, X, 0, 1, s * C(3, 7));
    acc_EE(a, X, 1, 0, s * C(7, 3));
  }
}

// B y for B = [[z I, p], [q^T, s]] and a 4-vector y = (ya, ye)
struct Blk {
  double z, p[3], q[3], s;
};
YS_HD void blk_apply(const Blk& B, const double* ya, double ye, double* oa, double* oe) {
  for (int i = 0; i < 3; ++i) oa[i] = B.z * ya[i] + B.p[i] * ye;
  *oe = B.q[0] * ya[0] + B.q[1] * ya[1] + B.q[2] * ya[2] + B.s * ye;
}

// All terms of one edge (src/PhysicsCloth.cpp:64-80): Mass, Gravity, Stretch,
// Inertia, MDotVDot, ParaColli; forces and both Jacobians.
YS_HD void edge_terms(const View& v, int n0, int n1, int k, EdgeAcc& a) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n0]];
  const uint8_t f0 = v.flags[n0], f1 = v.flags[n1];
  a.in[0] = (f0 & YS_INTERIOR) != 0;
  a.in[1] = (f1 & YS_INTERIOR) != 0;
  const int line = (k == 0) ? P.warp_line_off + v.node_v[n0] : P.weft_line_off + v.node_u[n0];
  const double rho = v.line_rho[line], ks = v.line_ks[line];
  a.h = v.h;
  a.h2 = v.h * v.h;
  for (int i = 0; i < 8; ++i) {
    a.b[i] = 0.0;
    for (int j = 0; j < 8; ++j) a.A[i][j] = 0.0;
  }
  for (int t = 0; t < 2; ++t) {
    a.fe[t] = a.kee[t] = a.dee[t] = 0.0;
    for (int i = 0; i < 3; ++i) a.cl[t][i] = a.cle[t][i] = 0.0;
  }
  // geometry (src/ClothUnit.h:134-154)
  double x0[3], x1[3], a0[3], a1[3], dx[3], w[3], d[3], Pm[3][3];
  for (int i = 0; i < 3; ++i) {
    x0[i] = ld(v.X, i, nt, n0); x1[i] = ld(v.X, i, nt, n1);
    a0[i] = ld(v.V, i, nt, n0); a1[i] = ld(v.V, i, nt, n1);
  }
  const double du = ld(v.UV, k, nt, n1) - ld(v.UV, k, nt, n0);
  const double e0 = ld(v.UVD, k, nt, n0), e1 = ld(v.UVD, k, nt, n1);
  for (int i = 0; i < 3; ++i) { dx[i] = x1[i] - x0[i]; w[i] = dx[i] / du; }
  const double l = norm3(dx);
  for (int i = 0; i < 3; ++i) d[i] = dx[i] / l;
  proj3(d, Pm);
  for (int i = 0; i < 3; ++i) { a.Vloc[i] = a0[i]; a.Vloc[4 + i] = a1[i]; }
  a.Vloc[3] = a.in[0] ? e0 : 0.0;
  a.Vloc[7] = a.in[1] ? e1 : 0.0;
  const double wTw = dot3(w, w);
  const double nw = norm3(w);

  // ---- Mass (src/PhysicsCloth.cpp:250-338)
  {
    const double coeff = (1.0 / 6.0) * rho * du;
    auto I2 = [&](int i, int j) { return i == j ? 2.0 * coeff : 0.0; };
    auto I1 = [&](int i, int j) { return i == j ? coeff : 0.0; };
    acc_LL(a, kM, 0, 0, 1.0, I2);
    acc_LL(a, kM, 1, 0, 1.0, I1);
    acc_LL(a, kM, 0, 1, 1.0, I1);
    acc_LL(a, kM, 1, 1, 1.0, I2);
    auto LE2 = [&](int r) { return -2.0 * coeff * w[r]; };
    auto LE1 = [&](int r) { return -1.0 * coeff * w[r]; };
    const double EE2 = 2.0 * coeff * wTw, EE1 = 0.5 * EE2;
    if (a.in[0]) { acc_LE(a, kM, 0, 0, 1.0, LE2); acc_EL(a, kM, 0, 0, 1.0, LE2); acc_EE(a, kM, 0, 0, EE2); }
    if (a.in[1]) { acc_LE(a, kM, 1, 1, 1.0, LE2); acc_EL(a, kM, 1, 1, 1.0, LE2); acc_EE(a, kM, 1, 1, EE2); }
    if (a.in[0] && a.in[1]) {
      acc_LE(a, kM, 1, 0, 1.0, LE1);
      acc_LE(a, kM, 0, 1, 1.0, LE1);
      acc_EL(a, kM, 1, 0, 1.0, LE1);
      acc_EL(a, kM, 0, 1, 1.0, LE1);
      acc_EE(a, kM, 0, 1, EE1);
      acc_EE(a, kM, 1, 0, EE1);
    }
  }
  // ---- Gravity_F / Gravity_D (src/PhysicsCloth.cpp:340-425)
  {
    for (int i = 0; i < 3; ++i) {
      const double g = 0.5 * rho * P.G[i] * du;
      acc_F(a, i, -g);
      acc_F(a, 4 + i, -g);
    }
    double sx[3] = {x0[0] + x1[0], x0[1] + x1[1], x0[2] + x1[2]};
    const double gx = dot3(P.G, sx);
    if (a.in[0]) acc_F(a, 3, -((-0.5) * rho * gx));
    if (a.in[1]) acc_F(a, 7, -(0.5 * rho * gx));
    auto g0 = [&](int r) { return 0.5 * rho * P.G[r]; };
    auto g1 = [&](int r) { return -(0.5 * rho * P.G[r]); };
    if (a.in[0]) { acc_EL(a, kK, 0, 0, 1.0, g0); acc_LE(a, kK, 0, 0, 1.0, g0); }
    if (a.in[1]) { acc_EL(a, kK, 1, 1, 1.0, g1); acc_LE(a, kK, 1, 1, 1.0, g1); }
    if (a.in[0] && a.in[1]) {
      acc_LE(a, kK, 1, 0, 1.0, g0);
      acc_LE(a, kK, 0, 1, 1.0, g1);
      acc_EL(a, kK, 1, 0, 1.0, g0);
      acc_EL(a, kK, 0, 1, 1.0, g1);
    }
  }
  // ---- Stretch_F / Stretch_D (src/PhysicsCloth.cpp:427-577)
  {
    const double sgn = (k == 0) ? 1.0 : -1.0;
    for (int i = 0; i < 3; ++i) {
      const double f = ks * (nw - 1) * d[i];
      acc_F(a, i, f);
      acc_F(a, 4 + i, -f);
      a.cl[0][i] += sgn * f;
      a.cl[1][i] -= sgn * f;
    }
    const double fe = 0.5 * ks * (nw * nw - 1);
    if (a.in[0]) acc_F(a, 3, -fe);
    if (a.in[1]) acc_F(a, 7, fe);
    auto LL = [&](int i, int j) { return (ks / l) * Pm[i][j] - (ks / du) * (i == j ? 1.0 : 0.0); };
    const double EE = -ks * ((nw * nw) / du);
    auto LE = [&](int r) { return ks * (nw / du) * d[r]; };
    auto EL = [&](int c) { return ks / du * w[c]; };
    acc_LL(a, kK, 0, 0, 1.0, LL);
    acc_LL(a, kK, 1, 0, -1.0, LL);
    acc_LL(a, kK, 0, 1, -1.0, LL);
    acc_LL(a, kK, 1, 1, 1.0, LL);
    if (a.in[0]) {
      acc_LE(a, kK, 0, 0, 1.0, LE);
      acc_EL(a, kK, 0, 0, 1.0, EL);
      acc_EE(a, kK, 0, 0, EE);
      for (int i = 0; i < 3; ++i) a.cle[0][i] += sgn * LE(i);
    }
    if (a.in[1]) {
      acc_LE(a, kK, 1, 1, 1.0, LE);
      acc_EL(a, kK, 1, 1, 1.0, EL);
      acc_EE(a, kK, 1, 1, EE);
      for (int i = 0; i < 3; ++i) a.cle[1][i] += sgn * LE(i);
    }
    if (a.in[0] && a.in[1]) {
      acc_LE(a, kK, 1, 0, -1.0, LE);
      acc_LE(a, kK, 0, 1, -1.0, LE);
      acc_EL(a, kK, 1, 0, -1.0, EL);
      acc_EL(a, kK, 0, 1, -1.0, EL);
      acc_EE(a, kK, 0, 1, -EE);
      acc_EE(a, kK, 1, 0, -EE);
    }
  }
  // ---- ParaColli_F / ParaColli_D (src/PhysicsCloth.cpp:989-1069)
  {
    const double dd = (((f0 & YS_FLIP) != 0) != ((f1 & YS_FLIP) != 0)) ? 4.0 * P.R : 2.0 * P.R;
    double rl = dd - du;
    if (rl < 0) rl = 0.0;
    const double fu0 = P.kc * P.L * rl;
    if (a.in[0]) acc_F(a, 3, fu0);
    if (a.in[1]) acc_F(a, 7, -fu0);
    const double ee = -P.kc * P.L * rl;
    if (a.in[0]) acc_EE(a, kK, 0, 0, ee);
    if (a.in[1]) acc_EE(a, kK, 1, 1, ee);
    if (a.in[0] && a.in[1]) { acc_EE(a, kK, 0, 1, ee); acc_EE(a, kK, 1, 0, ee); }
  }

  // ---- kinetic-energy terms: shared sums
  double m0a[3], m1a[3];
  for (int i = 0; i < 3; ++i) { m0a[i] = 2.0 * a0[i] + a1[i]; m1a[i] = a0[i] + 2.0 * a1[i]; }
  const double m0e = 2.0 * e0 + e1, m1e = e0 + 2.0 * e1;
  const double Saa = dot3(a0, m0a) + dot3(a1, m1a);
  double Sae[3], Sea[3];
  for (int i = 0; i < 3; ++i) { Sae[i] = a0[i] * m0e + a1[i] * m1e; Sea[i] = e0 * m0a[i] + e1 * m1a[i]; }
  const double See = e0 * m0e + e1 * m1e;
  const double r6 = (1.0 / 6.0) * rho;
  const double sc = 1.0 / 6.0 * rho * du;
  const double wSae = dot3(w, Sae), wSea = dot3(w, Sea);

  // ---- Inertia_F (src/PhysicsCloth.cpp:1071-1186)
  {
    for (int j = 0; j < 3; ++j) {
      const double pj = -(-1.0 / du);
      const double sj = (-2.0 / (du * du) * dx[j]);
      const double T0 = 0.5 * (sc * (pj * Sae[j] + pj * Sea[j] + sj * See));
      acc_F(a, j, T0);
      acc_F(a, 4 + j, -T0);
    }
    const double QM = Saa - wSae - wSea + wTw * See;
    const double Quv = (-1.0 / du) * wSae + (-1.0 / du) * wSea + (2.0 / du) * wTw * See;
    const double Tuv0 = 0.5 * (-(1.0 / 6.0) * rho * QM + (1.0 / 6.0) * rho * du * Quv);
    if (a.in[0]) acc_F(a, 3, Tuv0);
    if (a.in[1]) acc_F(a, 7, -Tuv0);
  }
  // ---- Inertia_D_Pos (src/PhysicsCloth.cpp:1188-1601)
  {
    const double T00 = 0.5 * (r6 * ((2 / (du * du)) * See));
    double Tx0uv0[3], Tuv0x0[3];
    for (int j = 0; j < 3; ++j) {
      const double pj = -(-1.0 / du);
      const double Qx0 = pj * Sae[j] + pj * Sea[j] + (-2.0 / (du * du) * dx[j]) * See;
      const double c2 = 1.0 / (du * du);
      // the sign-asymmetric mixed block of src/PhysicsCloth.cpp:1357-1361
      const double Qx0uv0 = (-c2) * Sae[j] + (-(-c2)) * Sea[j] + ((-4.0 / (du * du)) * w[j]) * See;
      Tx0uv0[j] = 0.5 * ((-1.0 / 6.0) * rho * Qx0 + (1.0 / 6.0) * rho * du * Qx0uv0);
      Tuv0x0[j] = 0.5 * ((-1.0 / 6.0) * rho * Qx0 + (1.0 / 6.0) * rho * du * (-Qx0uv0));
    }
    const double Quv0 = (-1.0 / du) * wSae + (-1.0 / du) * wSea + (2.0 / du) * wTw * See;
    const double c6 = 2 / (du * du);
    const double Quvuv = (-c6) * wSae + (-c6) * wSea + (6 / (du * du)) * wTw * See;
    const double Tuu = 0.5 * ((-1.0 / 6.0) * rho * Quv0 - (1.0 / 6.0) * rho * Quv0 + (1.0 / 6.0) * rho * du * Quvuv);
    auto C = [&](int i, int j) -> double {
      const int bi = i >> 2, bj = j >> 2, ii = i & 3, jj = j & 3;
      const double sgn = (bi == bj) ? 1.0 : -1.0;
      if (ii < 3 && jj < 3) return ii == jj ? sgn * T00 : 0.0;
      if (ii < 3) return sgn * Tx0uv0[ii];
      if (jj < 3) return sgn * Tuv0x0[jj];
      return sgn * Tuu;
    };
    acc_edge_jac(a, kK, 1.0, C);
  }
  // ---- Inertia_D_Vel (src/PhysicsCloth.cpp:1602-1901): C(j, :) = M_xj qdot
  {
    double rowx[3][8], rowu[8];
    for (int j = 0; j < 3; ++j) {
      const double pj = -(-1.0 / du), sj = (-2.0 / (du * du) * dx[j]);
      for (int i = 0; i < 8; ++i) rowx[j][i] = 0.0;
      rowx[j][j] = sc * (pj * m0e);
      rowx[j][3] = sc * (pj * m0a[j] + sj * m0e);
      rowx[j][4 + j] = sc * (pj * m1e);
      rowx[j][7] = sc * (pj * m1a[j] + sj * m1e);
    }
    for (int t = 0; t < 2; ++t) {
      const double* ma = t == 0 ? m0a : m1a;
      const double me = t == 0 ? m0e : m1e;
      const double wm = dot3(w, ma);
      for (int i = 0; i < 3; ++i)
        rowu[4 * t + i] = -(1.0 / 6.0) * rho * (ma[i] - w[i] * me) + (1.0 / 6.0) * rho * du * ((-1.0 / du) * w[i] * me);
      rowu[4 * t + 3] = -(1.0 / 6.0) * rho * (-wm + wTw * me) +
                        (1.0 / 6.0) * rho * du * ((-1.0 / du) * wm + (2.0 / du) * wTw * me);
    }
    auto C = [&](int i, int j) -> double {
      const int bi = i >> 2, ii = i & 3;
      const double sgn = bi == 0 ? 1.0 : -1.0;
      return ii < 3 ? sgn * rowx[ii][j] : sgn * rowu[j];
    };
    acc_edge_jac(a, kD, 1.0, C);
  }
  // ---- MDotVDot (src/PhysicsCloth.cpp:1903-2577)
  {
    const double dud = e1 - e0;
    double wd[3];
    for (int i = 0; i < 3; ++i) wd[i] = ((a1[i] - a0[i]) * du - dx[i] * dud) / (du * du);
    const double wTwd = dot3(w, wd) + dot3(wd, w);
    // M_dot qdot = r6*dud*[[2BM,BM],[BM,2BM]] qdot + r6*du*[[2Bd,Bd],[Bd,2Bd]] qdot
    Blk BM, Bd;
    BM.z = 1.0; BM.s = wTw;
    Bd.z = 0.0; Bd.s = wTwd;
    for (int i = 0; i < 3; ++i) { BM.p[i] = BM.q[i] = -w[i]; Bd.p[i] = Bd.q[i] = -wd[i]; }
    double BMm[2][4], Bdm[2][4], r[8];
    blk_apply(BM, m0a, m0e, &BMm[0][0], &BMm[0][3]);
    blk_apply(BM, m1a, m1e, &BMm[1][0], &BMm[1][3]);
    blk_apply(Bd, m0a, m0e, &Bdm[0][0], &Bdm[0][3]);
    blk_apply(Bd, m1a, m1e, &Bdm[1][0], &Bdm[1][3]);
    for (int t = 0; t < 2; ++t)
      for (int i = 0; i < 4; ++i) r[4 * t + i] = r6 * dud * BMm[t][i] + r6 * du * Bdm[t][i];
    // MDotVDot_F: F -= M_dot qdot
    for (int i = 0; i < 3; ++i) { acc_F(a, i, -r[i]); acc_F(a, 4 + i, -r[4 + i]); }
    if (a.in[0]) acc_F(a, 3, -r[3]);
    if (a.in[1]) acc_F(a, 7, -r[7]);
    // column c of M_dot
    auto Mdot = [&](int i, int c) -> double {
      const int bi = i >> 2, bc = c >> 2, ii = i & 3, cc = c & 3;
      const double f = (bi == bc) ? 2.0 : 1.0;
      double m, dm;
      if (ii < 3 && cc < 3) { m = ii == cc ? 1.0 : 0.0; dm = 0.0; }
      else if (ii < 3) { m = -w[ii]; dm = -wd[ii]; }
      else if (cc < 3) { m = -w[cc]; dm = -wd[cc]; }
      else { m = wTw; dm = wTwd; }
      return r6 * dud * (f * m) + r6 * du * (f * dm);
    };
    // MDotVDot_D_Pos, added (src/PhysicsCloth.cpp:2154-2234)
    {
      double Cp[8][8];
      for (int t = 0; t < 2; ++t) {
        const double sw = t == 0 ? -1.0 : 1.0;
        for (int j = 0; j < 3; ++j) {
          const double wxj = sw * (1.0 / du);
          const double P1 = -wxj, S1 = (sw * 2.0 / (du * du) * dx[j]);
          const double wdxj = t == 0 ? (dud / (du * du)) : -(dud / (du * du));
          const double P2 = -wdxj, S2 = 2 * (wxj * wd[j]) + 2 * (w[j] * wdxj);
          const int col = 4 * t + j;
          for (int b2 = 0; b2 < 2; ++b2) {
            const double* ma = b2 == 0 ? m0a : m1a;
            const double me = b2 == 0 ? m0e : m1e;
            for (int i = 0; i < 3; ++i)
              Cp[4 * b2 + i][col] = (i == j) ? (r6 * dud * (P1 * me) + r6 * du * (P2 * me)) : 0.0;
            Cp[4 * b2 + 3][col] = r6 * dud * (P1 * ma[j] + S1 * me) + r6 * du * (P2 * ma[j] + S2 * me);
          }
        }
        double wuv[3], wduv[3];
        for (int i = 0; i < 3; ++i) wuv[i] = (sw * w[i]) / du;
        const double wTwuv = sw * (2 / du) * wTw;
        for (int i = 0; i < 3; ++i)
          wduv[i] = (a1[i] - a0[i]) / (du * du) - (4 * dx[i] * dud) / (du * du * du);
        if (t == 1)
          for (int i = 0; i < 3; ++i) wduv[i] = -wduv[i];
        const double wTwduv = 2 * dot3(wuv, wd) + 2 * dot3(wduv, w);
        const int col = 4 * t + 3;
        for (int b2 = 0; b2 < 2; ++b2) {
          const double* ma = b2 == 0 ? m0a : m1a;
          const double me = b2 == 0 ? m0e : m1e;
          for (int i = 0; i < 3; ++i)
            Cp[4 * b2 + i][col] = r6 * dud * (wuv[i] * me) - r6 * r[4 * b2 + i] + r6 * du * (-wduv[i] * me);
          Cp[4 * b2 + 3][col] = r6 * dud * (dot3(wuv, ma) + wTwuv * me) - r6 * r[4 * b2 + 3] +
                                r6 * du * (-dot3(wduv, ma) + wTwduv * me);
        }
      }
      acc_edge_jac(a, kK, 1.0, [&](int i, int j) { return Cp[i][j]; });
    }
    // MDotVDot_D_Vel, subtracted (src/PhysicsCloth.cpp:2342-2577)
    {
      double Cv[8][8];
      for (int t = 0; t < 2; ++t) {
        const double sw = t == 0 ? -1.0 : 1.0;
        for (int j = 0; j < 3; ++j) {
          const double wdj = sw * (1.0 / du);
          const double P1 = -wdj, S1 = 2 * (w[j] * wdj);
          const int col = 4 * t + j;
          for (int b2 = 0; b2 < 2; ++b2) {
            const double* ma = b2 == 0 ? m0a : m1a;
            const double me = b2 == 0 ? m0e : m1e;
            for (int i = 0; i < 3; ++i)
              Cv[4 * b2 + i][col] = (1.0 / 6.0) * rho * du * ((i == j) ? P1 * me : 0.0) + Mdot(4 * b2 + i, col);
            Cv[4 * b2 + 3][col] = (1.0 / 6.0) * rho * du * (P1 * ma[j] + S1 * me) + Mdot(4 * b2 + 3, col);
          }
        }
        double wdv[3];
        for (int i = 0; i < 3; ++i) wdv[i] = (t == 0 ? (1.0 / du) : (-1.0 / du)) * w[i];
        const double wtwd = 2 * dot3(w, wdv);
        const double cm = (t == 0 ? -1.0 : 1.0) * (1.0 / 6.0) * rho;
        const int col = 4 * t + 3;
        for (int b2 = 0; b2 < 2; ++b2) {
          const double* ma = b2 == 0 ? m0a : m1a;
          const double me = b2 == 0 ? m0e : m1e;
          for (int i = 0; i < 3; ++i)
            Cv[4 * b2 + i][col] = cm * BMm[b2][i] + (1.0 / 6.0) * rho * du * (-wdv[i] * me) + Mdot(4 * b2 + i, col);
          Cv[4 * b2 + 3][col] = cm * BMm[b2][3] + (1.0 / 6.0) * rho * du * (-dot3(wdv, ma) + wtwd * me) +
                                Mdot(4 * b2 + 3, col);
        }
      }
      acc_edge_jac(a, kD, -1.0, [&](int i, int j) { return Cv[i][j]; });
    }
  }
}

// Adds an edge's accumulated contributions into the node rows of n0 and n1.
YS_HD void edge_scatter(const View& v, int n0, int n1, int k, const EdgeAcc& a) {
  const int nt = v.ntot;
  const int nd[2] = {n0, n1};
  const int du_[2] = {0, k == 0 ? 1 : 0}, dv_[2] = {0, k == 1 ? 1 : 0};
  for (int fa = 0; fa < 2; ++fa) {
    const int rn = nd[fa];
    for (int fb = 0; fb < 2; ++fb) {
      const int ddu = du_[fb] - du_[fa], ddv = dv_[fb] - dv_[fa];
      for (int r = 0; r < 4; ++r) {
        if (r == 3 && !a.in[fa]) continue;
        for (int c = 0; c < 4; ++c) {
          if (c == 3 && !a.in[fb]) continue;
          const double val = a.A[4 * fa + r][4 * fb + c];
          add_A(v, rn, r, nd[fb], c, k, val, ddu, ddv);
        }
      }
    }
    for (int r = 0; r < 3; ++r) st(v.B, r, nt, rn) += a.b[4 * fa + r];
    for (int i = 0; i < 3; ++i) st(v.CL, i, nt, rn) += a.cl[fa][i];
    if (a.in[fa]) {
      st(v.B, 3 + k, nt, rn) += a.b[4 * fa + 3];
      st(v.FE, k, nt, rn) += a.fe[fa];
      st(v.KEE, k, nt, rn) += a.kee[fa];
      st(v.DEE, k, nt, rn) += a.dee[fa];
      for (int i = 0; i < 3; ++i) st(v.CLE, 3 * k + i, nt, rn) += a.cle[fa][i];
    }
  }
}

// ------------------------------------------------------------ bend element
struct BendGeom {
  double du, l1, l2, d1[3], d2[3], P1[3][3], P2[3][3], theta;
};
// src/ClothUnit.h:197-210; the theta clamp uses EPS = DBL_MIN
// (src/Constants.h:25) and so never changes a finite value.
YS_HD void bend_geom(const double* x2, const double* x0, const double* x1, double du, BendGeom& g) {
  double a1[3], a2[3];
  for (int i = 0; i < 3; ++i) { a1[i] = x1[i] - x0[i]; a2[i] = x2[i] - x0[i]; }
  g.du = du;
  g.l1 = norm3(a1);
  g.l2 = norm3(a2);
  for (int i = 0; i < 3; ++i) { g.d1[i] = a1[i] / g.l1; g.d2[i] = a2[i] / g.l2; }
  proj3(g.d1, g.P1);
  proj3(g.d2, g.P2);
  double c = -dot3(g.d1, g.d2);
  const double lo = -1.0 + 2.2250738585072014e-308, hi = 1.0 - 2.2250738585072014e-308;
  if (c < lo) c = lo;
  if (c > hi) c = hi;
  g.theta = acos(c);
}

// Bending force and Hessian blocks shared by Bending_* and Crimp_Bending_*
// (src/PhysicsCloth.cpp:579-822, 824-987).
struct BendTerms {
  double Fx1[3], Fx2[3];
  double L11[3][3], L12[3][3], L21[3][3], L22[3][3];
  double L1E1[3], L2E1[3];
  bool active;
};
YS_HD void bend_terms(const BendGeom& g, double kb, BendTerms& t) {
  for (int i = 0; i < 3; ++i) {
    t.Fx1[i] = t.Fx2[i] = t.L1E1[i] = t.L2E1[i] = 0.0;
    for (int j = 0; j < 3; ++j) t.L11[i][j] = t.L12[i][j] = t.L21[i][j] = t.L22[i][j] = 0.0;
  }
  const double th = g.theta, s = sin(th);
  t.active = (s != 0.0);
  if (!t.active) return;
  const double co = cos(th), du = g.du;
  double a[3], b[3];
  matvec3(g.P1, g.d2, a);
  matvec3(g.P2, g.d1, b);
  const double c1 = (-2 * kb * th) / (g.l1 * du * s), c2 = (-2 * kb * th) / (g.l2 * du * s);
  for (int i = 0; i < 3; ++i) { t.Fx1[i] = c1 * a[i]; t.Fx2[i] = c2 * b[i]; }
  const double k11 = (2 * kb) / ((g.l1 * g.l1) * du * s), k12 = (-2 * kb) / (g.l1 * g.l2 * du * s);
  const double k22 = (2 * kb) / ((g.l2 * g.l2) * du * s);
  const double cs2 = co / (s * s), is = 1 / s;
  double T[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double ad1 = a[i] * g.d1[j], aa = a[i] * a[j], d1a = g.d1[i] * a[j];
      const double bd2 = b[i] * g.d2[j], bb = b[i] * b[j], d2b = g.d2[i] * b[j];
      t.L11[i][j] = k11 * (th * (ad1 + cs2 * aa + co * g.P1[i][j] + d1a) - is * aa);
      t.L22[i][j] = k22 * (th * (bd2 + cs2 * bb + co * g.P2[i][j] + d2b) - is * bb);
      T[i][j] = th * (g.P1[i][j] - cs2 * ad1) + is * ad1;
    }
  matmul3(T, g.P2, t.L12);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t.L12[i][j] *= k12;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double bd2 = b[i] * g.d2[j];
      T[i][j] = th * (g.P2[i][j] - cs2 * bd2) + is * bd2;
    }
  matmul3(T, g.P1, t.L21);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t.L21[i][j] *= k12;
  const double e1 = (2 * kb * th) / (g.l1 * (du * du) * s), e2 = (2 * kb * th) / (g.l2 * (du * du) * s);
  for (int i = 0; i < 3; ++i) { t.L1E1[i] = e1 * a[i]; t.L2E1[i] = e2 * b[i]; }
}

// Adds A[x(rn)][x(cn)] += -h^2 * blk^T (a dF/dx block, transposed as in
// To_Sparse_Mat) for a node-node coupling at grid offset (du, dv).
YS_HD void add_K_LL(const View& v, int rn, int du, int dv, const double blk[3][3], double s) {
  const int sidx = stencil_index(du, dv);
  if (sidx < 0) return;  // not reachable for bend and shear offsets; keeps every store in bounds
  const double mh2 = -(v.h * v.h);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) slot(v, YS_SLOT_LL + sidx * 9 + r * 3 + c, rn) += mh2 * (s * blk[c][r]);
}

// Bending_F / Bending_D on the real nodes (n2, n0, n1) along yarn direction k
// (k = 0: warp, neighbours at u -+ 1; k = 1: weft, neighbours at v -+ 1).
YS_HD void bend_element(const View& v, int n2, int n0, int n1, int k, double kb) {
  const int nt = v.ntot;
  double x2[3], x0[3], x1[3];
  for (int i = 0; i < 3; ++i) { x2[i] = ld(v.X, i, nt, n2); x0[i] = ld(v.X, i, nt, n0); x1[i] = ld(v.X, i, nt, n1); }
  BendGeom g;
  bend_geom(x2, x0, x1, ld(v.UV, k, nt, n1) - ld(v.UV, k, nt, n2), g);
  BendTerms t;
  bend_terms(g, kb, t);
  const bool in2 = (v.flags[n2] & YS_INTERIOR) != 0, in0 = (v.flags[n0] & YS_INTERIOR) != 0,
             in1 = (v.flags[n1] & YS_INTERIOR) != 0;
  const double h = v.h, h2 = v.h * v.h, th = g.theta, du = g.du;
  // forces
  const double Fu2 = (-kb * th) / (du * du), Fu1 = -1 * Fu2;
  for (int i = 0; i < 3; ++i) {
    st(v.B, i, nt, n2) += h * t.Fx2[i];
    st(v.B, i, nt, n0) += h * (-(t.Fx1[i] + t.Fx2[i]));
    st(v.B, i, nt, n1) += h * t.Fx1[i];
  }
  if (in2) { st(v.B, 3 + k, nt, n2) += h * Fu2; st(v.FE, k, nt, n2) += Fu2; }
  if (in1) { st(v.B, 3 + k, nt, n1) += h * Fu1; st(v.FE, k, nt, n1) += Fu1; }
  // Jacobian blocks
  double L10[3][3], L20[3][3], L01[3][3], L02[3][3], L00[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      L10[i][j] = -(t.L11[i][j] + t.L12[i][j]);
      L20[i][j] = -(t.L21[i][j] + t.L22[i][j]);
      L01[i][j] = -(t.L11[i][j] + t.L21[i][j]);
      L02[i][j] = -(t.L12[i][j] + t.L22[i][j]);
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) L00[i][j] = -(L10[i][j] + L20[i][j]);
  const int su = k == 0 ? 1 : 0, sv = k == 1 ? 1 : 0;  // offset n2 -> n0 -> n1
  add_K_LL(v, n2, 0, 0, t.L22, 1.0);
  add_K_LL(v, n2, su, sv, L20, 1.0);
  add_K_LL(v, n2, 2 * su, 2 * sv, t.L21, 1.0);
  add_K_LL(v, n0, -su, -sv, L02, 1.0);
  add_K_LL(v, n0, 0, 0, L00, 1.0);
  add_K_LL(v, n0, su, sv, L01, 1.0);
  add_K_LL(v, n1, -2 * su, -2 * sv, t.L12, 1.0);
  add_K_LL(v, n1, -su, -sv, L10, 1.0);
  add_K_LL(v, n1, 0, 0, t.L11, 1.0);
  const double E1E1 = (-2 * kb * (th * th)) / (du * du * du);
  double L2E2[3], L0E1[3], L0E2[3], E2L2[3], E1L0[3], E2L0[3];
  for (int i = 0; i < 3; ++i) {
    L2E2[i] = -t.L2E1[i];
    L0E1[i] = -(t.L1E1[i] + t.L2E1[i]);
    L0E2[i] = -L0E1[i];
    E2L2[i] = -t.L2E1[i];           // E1L2 has the values of L2E1
    E1L0[i] = -(t.L1E1[i] + t.L2E1[i]);
    E2L0[i] = -E1L0[i];
  }
  if (in2) {
    for (int r = 0; r < 3; ++r) {
      slot(v, YS_SLOT_LE_SELF + r * 2 + k, n2) += -h2 * L2E2[r];
      slot(v, YS_SLOT_EL_SELF + k * 3 + r, n2) += -h2 * E2L2[r];
    }
    slot(v, YS_SLOT_EE_SELF + k, n2) += -h2 * E1E1;
    st(v.KEE, k, nt, n2) += E1E1;
  }
  if (in1) {
    for (int r = 0; r < 3; ++r) {
      slot(v, YS_SLOT_LE_SELF + r * 2 + k, n1) += -h2 * t.L1E1[r];
      slot(v, YS_SLOT_EL_SELF + k * 3 + r, n1) += -h2 * t.L1E1[r];
    }
    slot(v, YS_SLOT_EE_SELF + k, n1) += -h2 * E1E1;
    st(v.KEE, k, nt, n1) += E1E1;
  }
  // neighbour index of n2 seen from n0 is (-su,-sv), of n1 seen from n0 (su,sv)
  const int nb_prev = yarn_nbr(-su, -sv), nb_next = yarn_nbr(su, sv);
  if (in2 && in0) {
    // F_LE_Pos[find_index(n0, n2)]: A[x(n0)][e(n2)]
    for (int r = 0; r < 3; ++r) slot(v, YS_SLOT_LE_NBR + nb_prev * 3 + r, n0) += -h2 * L0E2[r];
    // F_EL_Pos[find_index(n2, n0)]: A[e(n0)][x(n2)] (src/PhysicsCloth.cpp:780-795)
    for (int c = 0; c < 3; ++c) slot(v, YS_SLOT_EL_NBR + nb_prev * 3 + c, n0) += -h2 * E2L0[c];
  }
  if (in0 && in1) {
    for (int r = 0; r < 3; ++r) slot(v, YS_SLOT_LE_NBR + nb_next * 3 + r, n0) += -h2 * L0E1[r];
    // F_EL_Pos[find_index(n0, n1)]: A[e(n1)][x(n0)]
    for (int c = 0; c < 3; ++c) slot(v, YS_SLOT_EL_NBR + nb_prev * 3 + c, n1) += -h2 * E1L0[c];
  }
}

// Crimp_Bending_F / Crimp_Bending_D (src/PhysicsCloth.cpp:824-987) on the
// crimp-offset centre lines; only the compression accumulators are touched.
YS_HD void crimp_element(const View& v, int n2, int n0, int n1, int k, double kb) {
  const int nt = v.ntot;
  const double R = v.cp[v.node_cloth[n0]].R;
  const double sg = k == 0 ? -1.0 : 1.0;  // warp: x - R n, weft: x + R n
  double x[3][3];
  const int nd[3] = {n2, n0, n1};
  for (int m = 0; m < 3; ++m) {
    const bool in = (v.flags[nd[m]] & YS_INTERIOR) != 0;
    for (int i = 0; i < 3; ++i)
      x[m][i] = in ? ld(v.X, i, nt, nd[m]) + sg * (R * ld(v.NRM, i, nt, nd[m])) : ld(v.X, i, nt, nd[m]);
  }
  // crimp segments keep the EPos of the build (src/Cloth.cpp:107)
  BendGeom g;
  bend_geom(x[0], x[1], x[2], ld(v.UV0, k, nt, n1) - ld(v.UV0, k, nt, n2), g);
  BendTerms t;
  bend_terms(g, kb, t);
  const double sgn = (k == 0) ? 1.0 : -1.0;
  for (int i = 0; i < 3; ++i) {
    st(v.CL, i, nt, n2) += sgn * t.Fx2[i];
    st(v.CL, i, nt, n0) += sgn * (-(t.Fx1[i] + t.Fx2[i]));
    st(v.CL, i, nt, n1) += sgn * t.Fx1[i];
  }
  if (v.flags[n2] & YS_INTERIOR)
    for (int i = 0; i < 3; ++i) st(v.CLE, 3 * k + i, nt, n2) += sgn * (-t.L2E1[i]);
  if (v.flags[n1] & YS_INTERIOR)
    for (int i = 0; i < 3; ++i) st(v.CLE, 3 * k + i, nt, n1) += sgn * t.L1E1[i];
}

// ------------------------------------------------------------ wind (faces)
// Wind_F (src/PhysicsCloth.cpp:3091-3107), face geometry src/ClothUnit.h:268-273.
YS_HD void wind_face(const View& v, const ClothParams& P, int n1, int n2, int n3) {
  const int nt = v.ntot;
  double e1[3], e2[3], cr[3], n[3], fv[3], rel[3];
  for (int i = 0; i < 3; ++i) {
    e1[i] = ld(v.X, i, nt, n2) - ld(v.X, i, nt, n1);
    e2[i] = ld(v.X, i, nt, n3) - ld(v.X, i, nt, n1);
  }
  cross3(e1, e2, cr);
  const double nc = norm3(cr), area = 0.5 * nc;
  for (int i = 0; i < 3; ++i) n[i] = (nc == 0.0) ? cr[i] : cr[i] / nc;
  for (int i = 0; i < 3; ++i) {
    fv[i] = (ld(v.V, i, nt, n1) + ld(v.V, i, nt, n2) + ld(v.V, i, nt, n3)) / 3.0;
    rel[i] = P.wind[i] - fv[i];
  }
  const double vn = dot3(n, rel);
  for (int i = 0; i < 3; ++i) {
    const double tang = rel[i] - vn * n[i];
    const double f = P.wind_rho * area * fabs(vn) * vn * n[i] + P.wind_drag * area * tang;
    st(v.B, i, nt, n1) += v.h * (f / 3.0);
    st(v.B, i, nt, n2) += v.h * (f / 3.0);
    st(v.B, i, nt, n3) += v.h * (f / 3.0);
  }
}

// ------------------------------------------------------------ crossing node
// Node normal (src/Cloth.cpp:440-463): smallest right singular vector of the
// centred 5-point stencil = eigenvector of the smallest eigenvalue of its 3x3
// scatter matrix (cyclic Jacobi rotations), signed by warp x weft and the
// weave's flip flag.
YS_HD void sym3_min_eigvec(const double S[3][3], double* out) {
  double a[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
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
  int m = 0;
  if (a[1][1] < a[m][m]) m = 1;
  if (a[2][2] < a[m][m]) m = 2;
  for (int k = 0; k < 3; ++k) out[k] = V[k][m];
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
  double nn[3];
  sym3_min_eigvec(S, nn);
  const double len = norm3(nn);
  for (int i = 0; i < 3; ++i) nn[i] /= len;
  double vw[3], vf[3], cr[3];
  for (int i = 0; i < 3; ++i) { vw[i] = p[2][i] - p[1][i]; vf[i] = p[4][i] - p[3][i]; }
  cross3(vw, vf, cr);
  if (dot3(cr, nn) / (norm3(cr) * norm3(nn)) < 0)
    for (int i = 0; i < 3; ++i) nn[i] = -nn[i];
  if (v.flags[n] & YS_FLIP)
    for (int i = 0; i < 3; ++i) nn[i] = -nn[i];
  for (int i = 0; i < 3; ++i) st(v.NRM, i, nt, n) = nn[i];
}

// ConSlideFriction (src/PhysicsCloth.cpp:2579-2641) for interior node n, after
// every edge and bend term has been accumulated.
YS_HD void friction_node(const View& v, int n) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  double nrm[3], cl[3], cleu[3], clev[3];
  for (int i = 0; i < 3; ++i) {
    nrm[i] = ld(v.NRM, i, nt, n);
    cl[i] = ld(v.CL, i, nt, n);
    cleu[i] = ld(v.CLE, i, nt, n);
    clev[i] = ld(v.CLE, 3 + i, nt, n);
  }
  double comp = 0.5 * dot3(nrm, cl);
  if (comp < 0) comp = 0.0;
  const double compEE[2] = {0.5 * dot3(nrm, cleu), 0.5 * dot3(nrm, clev)};
  st(v.COMP, 0, nt, n) = comp;
  const double mu = P.mu, kf = P.kf, df = P.df, h = v.h, h2 = v.h * v.h;
  const double lim = 1.0 * comp * mu;
  for (int k = 0; k < 2; ++k) {
    const double uvm = ld(v.UV, k, nt, n) - ld(v.UVB, k, nt, n);
    const double FEns = ld(v.FE, k, nt, n), EEp = ld(v.KEE, k, nt, n), EEv = ld(v.DEE, k, nt, n);
    const double slide = 1.0 / (1.0 + exp(-(1e4 * (fabs(FEns) - lim))));
    const double t = tanh(10 * uvm), tl = tanh(10 * (lim - FEns));
    const double uvdot = ld(v.UVD, k, nt, n);
    const double force = (-0.5 * (kf * uvm - t * comp * mu) * tl + 0.5 * (kf * uvm + t * comp * mu)) - df * uvdot;
    const double pos = (-0.5 * (kf - (1.0 - t * t) * mu * comp - t * mu * compEE[k])) * tl -
                       (0.5 * (kf * uvm - t * mu * comp)) * (1.0 - tl * tl) * (EEp - mu * compEE[k]) -
                       (0.5 * (kf + (1.0 - t * t) * mu * comp + t * mu * compEE[k]));
    // tanh(10 * fric_lim - F) as written at src/PhysicsCloth.cpp:2630-2631
    const double tq = tanh(10 * lim - FEns);
    const double vel = (-0.5 * (kf * uvm - t * mu * comp)) * (1.0 - tq * tq) * EEv - df;
    st(v.SLIDE, k, nt, n) = slide;
    slot(v, YS_SLOT_EE_SELF + k, n) += -h2 * pos - h * vel;
    st(v.B, 3 + k, nt, n) += h * (force - vel * uvdot);
  }
}

// ------------------------------------------------------------ shear
// Shear_F / Shear_D (src/PhysicsCloth.cpp:2643-3089) for crossing n0 with warp
// neighbour n1 (grid offset (s1u, 0)) and weft neighbour n3 (offset (0, s3v)).
YS_HD void shear_element(const View& v, const ClothParams& P, int n0, int n1, int n3, int s1u, int s3v) {
  const int nt = v.ntot;
  const double Lc = P.L, R = P.R, S = P.S;
  const double comp = ld(v.COMP, 0, nt, n0);
  double a1v[3], a3v[3], d1[3], d3[3], P1[3][3], P3[3][3];
  for (int i = 0; i < 3; ++i) {
    const double x0 = ld(v.X, i, nt, n0);
    a1v[i] = ld(v.X, i, nt, n1) - x0;
    a3v[i] = ld(v.X, i, nt, n3) - x0;
  }
  const double l1 = norm3(a1v), l3 = norm3(a3v);
  for (int i = 0; i < 3; ++i) { d1[i] = a1v[i] / l1; d3[i] = a3v[i] / l3; }
  proj3(d1, P1);
  proj3(d3, P3);
  const double phi = acos(dot3(d1, d3));
  const double s = sin(phi), co = cos(phi);
  double a3[3], a1[3];  // a3 = P1 d3, a1 = P3 d1
  matvec3(P1, d3, a3);
  matvec3(P3, d1, a1);
  const uint8_t f0 = v.flags[n0], f1 = v.flags[n1], f3 = v.flags[n3];
  const bool jam = (((f0 & YS_FLIP) != 0) != ((f1 & YS_FLIP) != 0)) && (((f0 & YS_FLIP) != 0) != ((f3 & YS_FLIP) != 0));
  double Fx1[3], Fx3[3], J11[3][3], J13[3][3], J31[3][3], J33[3][3];
  const double cs2 = co / (s * s), is = 1 / s;
  double a3d1[3][3], d1a3[3][3], a3a3[3][3], a1d3[3][3], d3a1[3][3], a1a1[3][3];
  outer3(a3, d1, a3d1); outer3(d1, a3, d1a3); outer3(a3, a3, a3a3);
  outer3(a1, d3, a1d3); outer3(d3, a1, d3a1); outer3(a1, a1, a1a1);
  if (!jam) {
    const double kx = (comp + 1.0) * S * R * R * kPi;
    const double ph = phi - kPi / 2;
    const double cf1 = (kx * Lc * ph) / (l1 * s), cf3 = (kx * Lc * ph) / (l3 * s);
    for (int i = 0; i < 3; ++i) { Fx1[i] = cf1 * a3[i]; Fx3[i] = cf3 * a1[i]; }
    const double k11 = (kx * Lc) / ((l1 * l1) * s), k33 = (kx * Lc) / ((l3 * l3) * s);
    const double k13 = (kx * Lc) / (l3 * l1 * s), k31 = (kx * Lc) / (l1 * l3 * s);
    double T[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        J11[i][j] = k11 * (ph * (-1 * a3d1[i][j] + cs2 * a3a3[i][j] - co * P1[i][j] - d1a3[i][j]) - is * a3a3[i][j]);
        J33[i][j] = k33 * (ph * (-1 * a1d3[i][j] + cs2 * a1a1[i][j] - co * P3[i][j] - d3a1[i][j]) - is * a1a1[i][j]);
        T[i][j] = ph * (cs2 * a3d1[i][j] - is * a3d1[i][j]);
      }
    matmul3(T, P3, J13);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        J13[i][j] *= k13;
        T[i][j] = ph * (cs2 * a1d3[i][j] - is * a1d3[i][j]);
      }
    matmul3(T, P1, J31);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) J31[i][j] *= k31;
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
    const double rl1s = 1.0 / (l1 * s), rl3s = 1.0 / (l3 * s);
    double px1[3], px3[3];
    for (int i = 0; i < 3; ++i) { px1[i] = -a3[i] * rl1s; px3[i] = -a1[i] * rl3s; }
    const double gamma = (Lc * sqrt(2.0) - 2 * Lc * sin(0.5 * phi)) / R;
    const double sh = sin(0.5 * phi), ch = cos(0.5 * phi);
    const double kap = -LR * ch;                       // gamma_x = kap * phi_x
    const double Aq = phi - pl, Bq = phi - pb;
    const double phs = phi * Aq * Bq;
    const double sgm = Aq * Bq + phi * Bq + phi * Aq;  // phi_s_x = sgm * phi_x
    const double omg = 2.0 * (Aq + Bq + phi);
    const double pb5 = P.pb5, pb4 = P.pb4;
    const double num = pb5 * Aq, den = phs * phs + pb4 * sig * sig;
    const double cf = tanh(num / den);
    const double den2 = den * den, rden2 = 1.0 / den2, rden22 = 1.0 / (den2 * den2);
    const double tau = pb5 * den - num * (2 * phs * sgm);  // con_func_x_x numerator / phi_x
    const double muc = tau * rden2;                         // con_func_x_x = muc * phi_x
    const double g3 = gamma * gamma * gamma, g2 = gamma * gamma;
    const double base = 0.5 * (comp + 1.0) * S * kPi * (R * R);
    const double kx = base * ((1 + g3) + (1 - g3) * cf);
    const double beta0 = base * (1 - g3);
    const double beta1 = base * (cc * g2 * kap * (1 - cf) - (1 - g3) * cf * cf * muc);
    const double Bq2 = Bq * Bq;
    const double cf1 = (kx * Lc * Bq) * rl1s, cf3 = (kx * Lc * Bq) * rl3s;
    for (int i = 0; i < 3; ++i) {
      Fx1[i] = -0.5 * (beta0 + beta1 * px1[i]) * Lc * Bq2 + cf1 * a3[i];
      Fx3[i] = -0.5 * (beta0 + beta1 * px3[i]) * Lc * Bq2 + cf3 * a1[i];
    }
    // pass-invariant coefficients
    double P1P3[3][3], P3P1[3][3], e3[3];
    matmul3(P1, P3, P1P3);
    matmul3(P3, P1, P3P1);
    matvec3(P3, d3, e3);  // P3 d3: src/PhysicsCloth.cpp:2775-2777 multiplies outer(P3 d1, d3) by P3
    const double cfq = -2 * cf * (1 - cf * cf);
    const double c1 = cc * (cc - 1) * gamma, c2 = cc * g2;
    const double base2 = 0.5 * (comp + 1.0) * S * (R * R);
    const double kO = c1 * kap * kap * (1 - cf) - 2 * c2 * kap * (1 - cf * cf) * muc;
    const double kG = c2 * (1 - cf);
    const double cfqm2 = cfq * muc * muc;
    const double X4 = 4 * tau * den * phs * sgm;
    const double two_num_sgm2 = 2 * num * sgm * sgm, two_num_phs = 2 * num * phs, pb5den = pb5 * den;
    const double cross = 2 * phs * pb5 * sgm;
    const double hLB2 = 0.5 * Lc * Bq2, LB = Lc * Bq;
    const double kL = kx * Lc;
    const double r11 = 1.0 / ((l1 * l1) * s), r33 = 1.0 / ((l3 * l3) * s), r13 = 1.0 / (l1 * l3 * s);
    const double qR11 = 0.5 * LR * sh / ((l1 * s) * (l1 * s)), qR33 = 0.5 * LR * sh / ((l3 * s) * (l3 * s));
    const double qR13 = 0.5 * LR * sh / (l1 * l3 * (s * s));
    for (int pass = 0; pass < 4; ++pass) {
      // pass 0: (x1,x1) 1: (x3,x3) 2: (x1,x3) 3: (x3,x1)
      const double* pA = (pass == 0 || pass == 2) ? px1 : px3;
      const double* pB = (pass == 0 || pass == 3) ? px1 : px3;
      double (*J)[3] = pass == 0 ? J11 : pass == 1 ? J33 : pass == 2 ? J13 : J31;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const double O = pA[i] * pB[j], Ob = pB[i] * pA[j];
          double pxx, Rg, fo;
          if (pass == 0) {
            const double aa = a3[i] * a3[j];
            pxx = (a3[i] * d1[j] + d1[i] * a3[j] - cs2 * aa + co * P1[i][j]) * r11;
            Rg = qR11 * aa;
            fo = (kL * r11) * (Bq * (-(a3[i] * d1[j]) + cs2 * aa - co * P1[i][j] - d1[i] * a3[j]) - is * aa);
          } else if (pass == 1) {
            const double aa = a1[i] * a1[j];
            pxx = (a1[i] * d3[j] + d3[i] * a1[j] - cs2 * aa + co * P3[i][j]) * r33;
            Rg = qR33 * aa;
            fo = (kL * r33) * (Bq * (-(a1[i] * d3[j]) + cs2 * aa - co * P3[i][j] - d3[i] * a1[j]) - is * aa);
          } else if (pass == 2) {
            const double aa = a3[i] * a1[j];
            pxx = -(cs2 * aa + P1P3[i][j]) * r13;
            Rg = qR13 * aa;
            fo = (kL * r13) * (Bq * (cs2 * aa + P1P3[i][j]) - is * aa);
          } else {
            const double aa = a1[i] * a3[j];
            pxx = -(cs2 * (a1[i] * e3[j]) + P3P1[i][j]) * r13;
            Rg = qR13 * aa;
            fo = (kL * r13) * (Bq * (cs2 * aa + P3P1[i][j]) - is * aa);
          }
          const double gxx = Rg + kap * pxx;
          const double psx = sgm * pxx + (pass == 2 ? 0.5 * omg * (O + Ob) : omg * O);
          double nx = pb5den * pxx - two_num_sgm2 * O - two_num_phs * psx;
          if (pass >= 2) nx += cross * (O - Ob);
          const double cfxx = (nx * den2 - X4 * O) * rden22;
          const double cfdd = pass < 2 ? cfqm2 * O + (1 - cf * cf * cfxx) : cfqm2 * Ob + (1 - cf * cf) * cfxx;
          const double kxx = base2 * (kO * O + kG * gxx + (1 - g3) * cfdd);
          double kk;
          if (pass < 2) kk = 2 * LB * (beta0 * pB[j] + beta1 * O);
          else kk = LB * (beta0 * pB[j] + beta1 * O) + LB * (beta0 * pA[i] + beta1 * O);
          J[i][j] = -kxx * hLB2 - kk + fo;
        }
    }
  }
  const double h = v.h;
  for (int i = 0; i < 3; ++i) {
    const double Fx0 = -1 * (Fx1[i] + Fx3[i]);
    st(v.B, i, nt, n0) += h * Fx0;
    st(v.B, i, nt, n1) += h * Fx1[i];
    st(v.B, i, nt, n3) += h * Fx3[i];
  }
  double J10[3][3], J30[3][3], J01[3][3], J03[3][3], J00[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      J10[i][j] = -(J11[i][j] + J13[i][j]);
      J30[i][j] = -(J31[i][j] + J33[i][j]);
      J01[i][j] = -(J11[i][j] + J31[i][j]);
      J03[i][j] = -(J13[i][j] + J33[i][j]);
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J00[i][j] = -(J10[i][j] + J30[i][j]);
  add_K_LL(v, n0, 0, 0, J00, 1.0);
  add_K_LL(v, n0, s1u, 0, J01, 1.0);
  add_K_LL(v, n0, 0, s3v, J03, 1.0);
  add_K_LL(v, n1, -s1u, 0, J10, 1.0);
  add_K_LL(v, n1, 0, 0, J11, 1.0);
  add_K_LL(v, n1, -s1u, s3v, J13, 1.0);
  add_K_LL(v, n3, 0, -s3v, J30, 1.0);
  add_K_LL(v, n3, s1u, -s3v, J31, 1.0);
  add_K_LL(v, n3, 0, 0, J33, 1.0);
}

}  // namespace ys
