// ys_items.cuh -- per-node bodies of the step kernels that are not element
// terms: clearing, finalising a row block, the stencil SpMV row, and the
// state update. Kept separate from the launch code so one node's work is a
// plain function of (View, node).
#pragma once

#include "ys_physics.cuh"

namespace ys {

YS_HD void clear_node(const View& v, int n) {
  const int nt = v.ntot;
  for (int s = 0; s < YS_NUM_SLOTS; ++s) slot(v, s, n) = 0.0;
  for (int c = 0; c < 5; ++c) st(v.B, c, nt, n) = 0.0;
  for (int c = 0; c < 3; ++c) st(v.CL, c, nt, n) = 0.0;
  for (int c = 0; c < 6; ++c) st(v.CLE, c, nt, n) = 0.0;
  for (int c = 0; c < 2; ++c) {
    st(v.FE, c, nt, n) = 0.0;
    st(v.KEE, c, nt, n) = 0.0;
    st(v.DEE, c, nt, n) = 0.0;
  }
}

// Handle springs (Constraint_F / Constraint_D, src/PhysicsCloth.cpp:232-248),
// the external force of SimStep(..., ext_force) (src/TrainHelper.cpp:63),
// identity rows for the Eulerian DOFs that boundary nodes do not have, and the
// Jacobi preconditioner (zero diagonal -> 1, as Eigen's
// DiagonalPreconditioner). Returns false if the row block holds a non-finite
// value (SimStep's DetectNaN / DetectInf, src/TrainHelper.cpp:22-37).
YS_HD bool finalize_node(const View& v, int n, double* dinv) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const uint8_t fl = v.flags[n];
  const double h = v.h;
  if (fl & YS_FIXED) {
    for (int i = 0; i < 3; ++i) {
      st(v.B, i, nt, n) += h * (-(P.kh * (ld(v.X, i, nt, n) - ld(v.XF, i, nt, n))));
      slot(v, YS_SLOT_LL + i * 3 + i, n) += -(h * h) * (-P.kh);
    }
  }
  if (v.ext) {
    for (int i = 0; i < 3; ++i) st(v.B, i, nt, n) += h * ld(v.ext, i, nt, n);
    if (fl & YS_INTERIOR)
      for (int k = 0; k < 2; ++k) st(v.B, 3 + k, nt, n) += h * ld(v.ext, 3 + k, nt, n);
  }
  if (!(fl & YS_INTERIOR)) {
    for (int k = 0; k < 2; ++k) {
      slot(v, YS_SLOT_EE_SELF + k, n) = 1.0;
      st(v.B, 3 + k, nt, n) = 0.0;
    }
  }
  bool ok = true;
  for (int s = 0; s < YS_NUM_SLOTS; ++s) ok = ok && isfinite(slot(v, s, n));
  for (int c = 0; c < 5; ++c) ok = ok && isfinite(ld(v.B, c, nt, n));
  for (int i = 0; i < 3; ++i) {
    const double dg = slot(v, YS_SLOT_LL + i * 3 + i, n);
    st(dinv, i, nt, n) = dg != 0.0 ? 1.0 / dg : 1.0;
  }
  for (int k = 0; k < 2; ++k) {
    const double dg = slot(v, YS_SLOT_EE_SELF + k, n);
    st(dinv, 3 + k, nt, n) = dg != 0.0 ? 1.0 / dg : 1.0;
  }
  return ok;
}

// y = A x for row block n (5 rows). Couplings to grid positions outside the
// cloth have zero coefficients; their column index is clamped to n so the
// load stays in bounds and adds 0 * x(n).
YS_HD void spmv_row(const View& v, const double* YS_RESTRICT x, int n, double y[5]) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  double yl0 = 0.0, yl1 = 0.0, yl2 = 0.0;
  for (int s = 0; s < kNumStencil; ++s) {
    const int uu = u + stencil_du(s), vv = w + stencil_dv(s);
    const bool ok = uu >= 0 && uu < P.W && vv >= 0 && vv < P.H;
    const int j = ok ? n + stencil_du(s) + stencil_dv(s) * P.W : n;
    const double xj0 = x[j], xj1 = x[nt + j], xj2 = x[2 * nt + j];
    const int b = YS_SLOT_LL + 9 * s;
    yl0 += slot(v, b + 0, n) * xj0 + slot(v, b + 1, n) * xj1 + slot(v, b + 2, n) * xj2;
    yl1 += slot(v, b + 3, n) * xj0 + slot(v, b + 4, n) * xj1 + slot(v, b + 5, n) * xj2;
    yl2 += slot(v, b + 6, n) * xj0 + slot(v, b + 7, n) * xj1 + slot(v, b + 8, n) * xj2;
  }
  const double xu = x[3 * nt + n], xv = x[4 * nt + n];
  yl0 += slot(v, YS_SLOT_LE_SELF + 0, n) * xu + slot(v, YS_SLOT_LE_SELF + 1, n) * xv;
  yl1 += slot(v, YS_SLOT_LE_SELF + 2, n) * xu + slot(v, YS_SLOT_LE_SELF + 3, n) * xv;
  yl2 += slot(v, YS_SLOT_LE_SELF + 4, n) * xu + slot(v, YS_SLOT_LE_SELF + 5, n) * xv;
  const double xl0 = x[n], xl1 = x[nt + n], xl2 = x[2 * nt + n];
  double ye[2];
  for (int k = 0; k < 2; ++k)
    ye[k] = slot(v, YS_SLOT_EL_SELF + 3 * k + 0, n) * xl0 + slot(v, YS_SLOT_EL_SELF + 3 * k + 1, n) * xl1 +
            slot(v, YS_SLOT_EL_SELF + 3 * k + 2, n) * xl2 + slot(v, YS_SLOT_EE_SELF + k, n) * x[(3 + k) * nt + n];
  for (int m = 0; m < 4; ++m) {
    const int du = m == 0 ? -1 : m == 1 ? 1 : 0, dv = m == 2 ? -1 : m == 3 ? 1 : 0;
    const int k = m < 2 ? 0 : 1;
    const int uu = u + du, vv = w + dv;
    const bool ok = uu >= 0 && uu < P.W && vv >= 0 && vv < P.H;
    const int j = ok ? n + du + dv * P.W : n;
    const double xe = x[(3 + k) * nt + j];
    yl0 += slot(v, YS_SLOT_LE_NBR + 3 * m + 0, n) * xe;
    yl1 += slot(v, YS_SLOT_LE_NBR + 3 * m + 1, n) * xe;
    yl2 += slot(v, YS_SLOT_LE_NBR + 3 * m + 2, n) * xe;
    ye[k] += slot(v, YS_SLOT_EL_NBR + 3 * m + 0, n) * x[j] + slot(v, YS_SLOT_EL_NBR + 3 * m + 1, n) * x[nt + j] +
             slot(v, YS_SLOT_EL_NBR + 3 * m + 2, n) * x[2 * nt + j] + slot(v, YS_SLOT_EE_NBR + m, n) * xe;
  }
  y[0] = yl0;
  y[1] = yl1;
  y[2] = yl2;
  y[3] = ye[0];
  y[4] = ye[1];
}

// Cloth::update (src/Cloth.cpp:111-148) for node n with the solved velocity.
YS_HD void update_node(const View& v, const double* YS_RESTRICT xs, int n) {
  const int nt = v.ntot;
  const uint8_t fl = v.flags[n];
  const double h = v.h;
  for (int i = 0; i < 3; ++i) {
    const double vel = xs[i * nt + n];
    st(v.V, i, nt, n) = vel;
    const double x = ld(v.X, i, nt, n) + vel * h;
    st(v.X, i, nt, n) = x;
    if (!(fl & YS_FIXED)) st(v.XF, i, nt, n) = x;
  }
  if (fl & YS_INTERIOR) {
    for (int k = 0; k < 2; ++k) {
      const double e = xs[(3 + k) * nt + n];
      st(v.UVD, k, nt, n) = e;
      st(v.UV, k, nt, n) = ld(v.UV, k, nt, n) + e * h;
      st(v.UVB, k, nt, n) = ld(v.UVB, k, nt, n) + ld(v.SLIDE, k, nt, n) * e * h;
    }
  }
}

}  // namespace ys
