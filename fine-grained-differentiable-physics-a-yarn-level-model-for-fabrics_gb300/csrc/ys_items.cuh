// ys_items.cuh -- per-node bodies of the step kernels that are not element
// terms: gathering the element records into a row block, the stencil SpMV row,
// and the state update. Kept separate from the launch code so one node's work
// is a plain function of (View, node).
#pragma once

#include <type_traits>

#include "ys_physics.cuh"

namespace ys {

// Per-element record buffers of one step (field-major, coalesced over the
// anchor node). Edges and bend segments have one slot per node and yarn
// direction (slot = k * ntot + anchor), faces one per cell (top-left node),
// shear segments four per crossing (slot = type * ntot + crossing).
struct Records {
  double* edge;   // [kEdgeFields][2][ntot]
  double* bend;   // [kBendFields][2][ntot]
  double* face;   // [6][ntot]
  double* shear;  // [kShearFields][4][ntot]
  // tangents of the same records (forward-mode runs only; layout of ys_physics.cuh lds)
  double* dedge;
  double* dbend;
  double* dface;
  double* dshear;
  // per node: 1 if a coefficient or right-hand side the gather wrote is not
  // finite (null: the finalize checks every slot itself)
  uint8_t* nonfinite;
};

YS_HD double rec(const double* buf, int field, int nslot, int slot_, int ntot, int node) {
  return buf[((int64_t)field * nslot + slot_) * ntot + node];
}
template <class T>
YS_HD T recT(const double* buf, const double* dbuf, int field, int nslot, int slot_, int ntot, int node) {
  return ldT<T>(buf, dbuf, field * nslot + slot_, ntot, node);
}

// one coefficient slot of row block n (value, and tangents when T is a Dual)
template <class T>
YS_HD void stA(const View& v, int s, int n, const T& x) { stT(v.A, v.dA, s, v.ntot, n, x); }
template <class T>
YS_HD T ldA(const View& v, int s, int n) { return ldT<T>(v.A, v.dA, s, v.ntot, n); }

// Gathers, for row block n, every contribution of the edges, bend segments
// and faces that touch it, runs ConSlideFriction on the gathered no-slide
// quantities, and writes all 159 coefficient slots and b (the diagonal
// blocks, which only shear segments fill, are set to 0 here). Node-node
// blocks of X_LL are written transposed into the dense matrix
// (src/MatrixMp.cpp:54-65), hence the blk[3 * c + r] reads.
template <class T>
YS_HD void gather_elements(const View& v, const Records& R, int n) {
  bool fin = true;  // every value written below is finite
  auto putA = [&](int s_, int n_, const T& x) {
    fin = fin && isfinite(val(x));
    stA(v, s_, n_, x);
  };
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int W = P.W, H = P.H, u = v.node_u[n], w = v.node_v[n];
  const bool in = (v.flags[n] & YS_INTERIOR) != 0;
  const double h = v.h, mh2 = -(v.h * v.h);
  // ------------------------------------------------------------ self block
  {
    T LL[9], LE[6], EL[6], EE[2], B[5], FE[2], KEE[2], DEE[2], CL[3], CLE[6];
    for (int i = 0; i < 9; ++i) LL[i] = 0.0;
    for (int i = 0; i < 6; ++i) LE[i] = EL[i] = CLE[i] = 0.0;
    for (int i = 0; i < 2; ++i) EE[i] = FE[i] = KEE[i] = DEE[i] = 0.0;
    for (int i = 0; i < 5; ++i) B[i] = 0.0;
    for (int i = 0; i < 3; ++i) CL[i] = 0.0;
    // unrolled: the accumulators are indexed by k, and a rolled loop would
    // put them in local memory
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      // edges along k: this node as n0 (anchor n) and as n1 (anchor n - step)
      const int step = k == 0 ? 1 : W;
      const bool has0 = k == 0 ? (u < W - 1) : (w < H - 1);
      const bool has1 = k == 0 ? (u > 0) : (w > 0);
      for (int a = 0; a < 2; ++a) {
        if (!(a == 0 ? has0 : has1)) continue;
        const int anc = a == 0 ? n : n - step;
        auto E = [&](int f) { return recT<T>(R.edge, R.dedge, f, 2, k, nt, anc); };
        const int p = 3 * a;  // block (a, a)
        const T cI = E(kE_llI + p), cP = E(kE_llP + p);
        const T d[3] = {E(kE_d), E(kE_d + 1), E(kE_d + 2)};
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) LL[3 * r + c] += (r == c ? cI : 0.0) + cP * ((r == c ? 1.0 : 0.0) - d[r] * d[c]);
        for (int r = 0; r < 3; ++r) {
          LE[2 * r + k] += E(kE_le + 3 * p + r);
          EL[3 * k + r] += E(kE_el + 3 * p + r);
          B[r] += E(kE_b + 4 * a + r);
          CL[r] += E(kE_cl + 3 * a + r);
          CLE[3 * k + r] += E(kE_cle + 3 * a + r);
        }
        EE[k] += E(kE_ee + p);
        B[3 + k] += E(kE_b + 4 * a + 3);
        FE[k] += E(kE_fkd + 3 * a);
        KEE[k] += E(kE_fkd + 3 * a + 1);
        DEE[k] += E(kE_fkd + 3 * a + 2);
      }
      // bend segments along k with middle m: this node is n2 (m = n + step),
      // n0 (m = n) or n1 (m = n - step)
      const int pos = k == 0 ? u : w, len = k == 0 ? W : H;
      const double sgn = (k == 0) ? 1.0 : -1.0;
      for (int role = 0; role < 3; ++role) {
        const int mid = role == 0 ? pos + 1 : role == 1 ? pos : pos - 1;
        if (mid < 1 || mid > len - 2) continue;
        const int anc = role == 0 ? n + step : role == 1 ? n : n - step;
        auto Bf = [&](int f) { return recT<T>(R.bend, R.dbend, f, 2, k, nt, anc); };
        T blk[9];
        if (role == 0) {
          for (int i = 0; i < 9; ++i) blk[i] = Bf(kB_L22 + i);
        } else if (role == 2) {
          for (int i = 0; i < 9; ++i) blk[i] = Bf(kB_L11 + i);
        } else {  // L00 = -(L10 + L20) (src/PhysicsCloth.cpp:709)
          for (int i = 0; i < 9; ++i) {
            const T L10 = -(Bf(kB_L11 + i) + Bf(kB_L12 + i)), L20 = -(Bf(kB_L21 + i) + Bf(kB_L22 + i));
            blk[i] = -(L10 + L20);
          }
        }
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) LL[3 * r + c] += mh2 * blk[3 * c + r];
        if (role == 0) {  // n2 (src/PhysicsCloth.cpp:737-753)
          for (int r = 0; r < 3; ++r) {
            B[r] += h * Bf(kB_Fx2 + r);
            CL[r] += sgn * Bf(kB_cFx2 + r);
          }
          if (in) {
            const T e11 = Bf(kB_E1E1), fu2 = Bf(kB_Fu2);
            for (int r = 0; r < 3; ++r) {
              const T l2e2 = -Bf(kB_L2E1 + r);
              LE[2 * r + k] += mh2 * l2e2;
              EL[3 * k + r] += mh2 * l2e2;  // E2L2 = -E1L2 carries the values of -L2E1
              CLE[3 * k + r] += sgn * (-Bf(kB_cL2E1 + r));
            }
            EE[k] += mh2 * e11;
            KEE[k] += e11;
            B[3 + k] += h * fu2;
            FE[k] += fu2;
          }
        } else if (role == 2) {  // n1 (src/PhysicsCloth.cpp:755-772)
          for (int r = 0; r < 3; ++r) {
            B[r] += h * Bf(kB_Fx1 + r);
            CL[r] += sgn * Bf(kB_cFx1 + r);
          }
          if (in) {
            const T e11 = Bf(kB_E1E1), fu1 = -1 * Bf(kB_Fu2);
            for (int r = 0; r < 3; ++r) {
              const T l1e1 = Bf(kB_L1E1 + r);
              LE[2 * r + k] += mh2 * l1e1;
              EL[3 * k + r] += mh2 * l1e1;
              CLE[3 * k + r] += sgn * Bf(kB_cL1E1 + r);
            }
            EE[k] += mh2 * e11;
            KEE[k] += e11;
            B[3 + k] += h * fu1;
            FE[k] += fu1;
          }
        } else {  // n0: F_x0 = -(F_x1 + F_x2), F_u0 = 0
          for (int r = 0; r < 3; ++r) {
            B[r] += h * (-(Bf(kB_Fx1 + r) + Bf(kB_Fx2 + r)));
            CL[r] += sgn * (-(Bf(kB_cFx1 + r) + Bf(kB_cFx2 + r)));
          }
        }
      }
    }
    // faces of the (up to) four cells around the node (src/Cloth.cpp:271-287)
    for (int cj = w - 1; cj <= w; ++cj)
      for (int ci = u - 1; ci <= u; ++ci) {
        if (ci < 0 || ci >= W - 1 || cj < 0 || cj >= H - 1) continue;
        const int tl = n + (ci - u) + (cj - w) * W;
        const bool right = ci != u, below = cj != w;  // node is tr / bl / br of that cell
        const bool even = ((ci + cj) & 1) == 0;
        bool inA, inB;
        if (!right && !below) { inA = true; inB = even; }       // tl
        else if (right && !below) { inA = true; inB = !even; }  // tr
        else if (!right && below) { inA = !even; inB = true; }  // bl
        else { inA = even; inB = true; }                        // br
        for (int r = 0; r < 3; ++r) {
          if (inA) B[r] += h * ldT<T>(R.face, R.dface, r, nt, tl);
          if (inB) B[r] += h * ldT<T>(R.face, R.dface, 3 + r, nt, tl);
        }
      }
    if (in) {
      T aEE[2], bE[2];
      friction_node(v, n, FE, KEE, DEE, CL, CLE, aEE, bE);
      for (int k = 0; k < 2; ++k) {
        EE[k] += aEE[k];
        B[3 + k] += bE[k];
      }
    }
    for (int i = 0; i < 9; ++i) putA(YS_SLOT_LL + i, n, LL[i]);
    for (int i = 0; i < 6; ++i) {
      putA(YS_SLOT_LE_SELF + i, n, LE[i]);
      putA(YS_SLOT_EL_SELF + i, n, EL[i]);
    }
    for (int k = 0; k < 2; ++k) putA(YS_SLOT_EE_SELF + k, n, EE[k]);
    for (int i = 0; i < 5; ++i) {
      fin = fin && isfinite(val(B[i]));
      stT(v.B, v.dB, i, nt, n, B[i]);
    }
  }
  // ------------------------------------------------ yarn neighbours (+-1)
  for (int m = 0; m < 4; ++m) {
    const int k = m < 2 ? 0 : 1;
    const int dir = (m & 1) ? 1 : -1;  // -1: previous, +1: next along the yarn
    const int step = k == 0 ? 1 : W;
    const int pos = k == 0 ? u : w, len = k == 0 ? W : H;
    const int s = stencil_index(k == 0 ? dir : 0, k == 1 ? dir : 0);
    T LL[9], LE[3], EL[3], EE = 0.0;
    for (int i = 0; i < 9; ++i) LL[i] = 0.0;
    for (int i = 0; i < 3; ++i) LE[i] = EL[i] = 0.0;
    if (pos + dir >= 0 && pos + dir < len) {
      const int nb = n + dir * step;
      const bool inb = (v.flags[nb] & YS_INTERIOR) != 0;
      // the edge between n and nb: n is its n0 when dir = +1
      const int a = dir > 0 ? 0 : 1, o = 1 - a;
      const int anc = dir > 0 ? n : nb;
      auto E = [&](int f) { return recT<T>(R.edge, R.dedge, f, 2, k, nt, anc); };
      const int p = 2 * a + o;
      const T cI = E(kE_llI + p), cP = E(kE_llP + p);
      const T d[3] = {E(kE_d), E(kE_d + 1), E(kE_d + 2)};
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) LL[3 * r + c] += (r == c ? cI : 0.0) + cP * ((r == c ? 1.0 : 0.0) - d[r] * d[c]);
      for (int r = 0; r < 3; ++r) {
        LE[r] += E(kE_le + 3 * p + r);
        EL[r] += E(kE_el + 3 * p + r);
      }
      EE += E(kE_ee + p);
      // bend segments containing both n and nb
      for (int which = 0; which < 2; ++which) {
        // which 0: middle = n (nb is n1 if dir = +1, n2 if dir = -1)
        // which 1: middle = nb (n is n2 if dir = +1, n1 if dir = -1)
        const int mid = which == 0 ? pos : pos + dir;
        if (mid < 1 || mid > len - 2) continue;
        const int ancb = which == 0 ? n : nb;
        auto Bf = [&](int f) { return recT<T>(R.bend, R.dbend, f, 2, k, nt, ancb); };
        T blk[9];
        for (int i = 0; i < 9; ++i) {
          const T L11 = Bf(kB_L11 + i), L12 = Bf(kB_L12 + i), L21 = Bf(kB_L21 + i), L22 = Bf(kB_L22 + i);
          if (which == 0) blk[i] = dir > 0 ? -(L11 + L21) : -(L12 + L22);  // L01 or L02
          else blk[i] = dir > 0 ? -(L21 + L22) : -(L11 + L12);             // L20 or L10
        }
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) LL[3 * r + c] += mh2 * blk[3 * c + r];
        // Eulerian couplings of Bending_D (src/PhysicsCloth.cpp:774-822):
        // q = L1E1 + L2E1 = L0E2 = E2L0 = -L0E1 = -E1L0
        T q[3];
        for (int r = 0; r < 3; ++r) q[r] = Bf(kB_L1E1 + r) + Bf(kB_L2E1 + r);
        if (which == 0 && in && inb) {
          if (dir < 0)  // row n0 = n, column e / x of n2 = nb
            for (int r = 0; r < 3; ++r) { LE[r] += mh2 * q[r]; EL[r] += mh2 * q[r]; }
          else  // row n0 = n, column e of n1 = nb
            for (int r = 0; r < 3; ++r) LE[r] += mh2 * (-q[r]);
        }
        if (which == 1 && dir < 0 && in && inb)  // row n1 = n, column x of n0 = nb
          for (int r = 0; r < 3; ++r) EL[r] += mh2 * (-q[r]);
      }
    }
    for (int i = 0; i < 9; ++i) putA(YS_SLOT_LL + 9 * s + i, n, LL[i]);
    for (int r = 0; r < 3; ++r) {
      putA(YS_SLOT_LE_NBR + 3 * m + r, n, LE[r]);
      putA(YS_SLOT_EL_NBR + 3 * m + r, n, EL[r]);
    }
    putA(YS_SLOT_EE_NBR + m, n, EE);
  }
  // ------------------------------------------- second neighbours (+-2)
  for (int m = 0; m < 4; ++m) {
    const int k = m < 2 ? 0 : 1;
    const int dir = (m & 1) ? 1 : -1;
    const int step = k == 0 ? 1 : W;
    const int pos = k == 0 ? u : w, len = k == 0 ? W : H;
    const int s = stencil_index(k == 0 ? 2 * dir : 0, k == 1 ? 2 * dir : 0);
    const int mid = pos + dir;
    const bool ok = mid >= 1 && mid <= len - 2;
    const int anc = n + dir * step;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c)  // n is n2 (dir +1): L21; n is n1 (dir -1): L12
        putA(YS_SLOT_LL + 9 * s + 3 * r + c, n,
            ok ? T(mh2 * recT<T>(R.bend, R.dbend, (dir > 0 ? kB_L21 : kB_L12) + 3 * c + r, 2, k, nt, anc)) : T(0.0));
  }
  // diagonal neighbours: shear only (gather_shear_finalize)
  for (int s = 9; s < 13; ++s)
    for (int i = 0; i < 9; ++i) putA(YS_SLOT_LL + 9 * s + i, n, T(0.0));
  if (R.nonfinite) R.nonfinite[n] = fin ? 0 : 1;
}

// Adds the shear segments touching row block n (as crossing n0, as warp
// neighbour n1 or as weft neighbour n3; src/PhysicsCloth.cpp:2643-3089), then
// the handle springs (Constraint_F / Constraint_D, src/PhysicsCloth.cpp:232-248),
// the external force of SimStep(..., ext_force) (src/TrainHelper.cpp:63),
// identity rows for the Eulerian DOFs boundary nodes do not have, and the
// Jacobi preconditioner (zero diagonal -> 1, as Eigen's
// DiagonalPreconditioner). Returns false if the row block holds a non-finite
// value (SimStep's DetectNaN / DetectInf, src/TrainHelper.cpp:22-37).
template <class T>
YS_HD bool gather_shear_finalize(const View& v, const Records& R, int n, double* dinv) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int W = P.W, H = P.H, u = v.node_u[n], w = v.node_v[n];
  const uint8_t fl = v.flags[n];
  const double h = v.h, mh2 = -(v.h * v.h);
  auto interior = [&](int uu, int vv) { return uu >= 1 && uu <= W - 2 && vv >= 1 && vv <= H - 2; };
  auto S = [&](int f, int seg, int anc) { return recT<T>(R.shear, R.dshear, f, 4, seg, nt, anc); };
  bool finf = true;  // every slot value this routine writes is finite
  auto addLL = [&](int du, int dv, const T* blk) {  // A[x(n)][x(n + (du, dv))] += -h^2 blk^T
    const int s = stencil_index(du, dv);
    if (s < 0) return;
    // the block's nine slots are loaded together, then updated: a load per
    // slot behind the previous slot's store would wait out one memory
    // latency per slot
    T a[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) a[i] = ldA<T>(v, YS_SLOT_LL + 9 * s + i, n);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        T& x = a[3 * r + c];
        x += mh2 * blk[3 * c + r];
        finf = finf && isfinite(val(x));
      }
#pragma unroll
    for (int i = 0; i < 9; ++i) stA(v, YS_SLOT_LL + 9 * s + i, n, a[i]);
  };
  auto addB = [&](int c, const T& x) {
    T b = ldT<T>(v.B, v.dB, c, nt, n);
    b += x;
    stT(v.B, v.dB, c, nt, n, b);
  };
  T Bx[3] = {0.0, 0.0, 0.0};
  if constexpr (std::is_same<T, double>::value) {
    // The contributions below are summed per target block in registers and
    // each slot of A is then updated once (a global read-modify-write per
    // contribution would serialise on its own stores). Same terms as the
    // tangent path in the else branch, summed in another order.
    const bool in0 = (fl & YS_INTERIOR) != 0;
    {  // the node's own block and its four yarn neighbours
      double self[9], xa[2][9], ya[2][9];  // xa: (-1, 0), (1, 0); ya: (0, -1), (0, 1)
#pragma unroll
      for (int i = 0; i < 9; ++i) self[i] = xa[0][i] = xa[1][i] = ya[0][i] = ya[1][i] = 0.0;
#pragma unroll
      for (int seg = 0; seg < 4; ++seg) {
        const int du = shear_du(seg), dv = shear_dv(seg);
        const int ix = du < 0 ? 0 : 1, iy = dv < 0 ? 0 : 1;
        if (in0) {  // as the crossing n0 (src/PhysicsCloth.cpp:3033-3047)
#pragma unroll
          for (int i = 0; i < 9; ++i) {
            const double a11 = S(kS_J11 + i, seg, n), a13 = S(kS_J13 + i, seg, n);
            const double a31 = S(kS_J31 + i, seg, n), a33 = S(kS_J33 + i, seg, n);
            self[i] += -(-(a11 + a13) + -(a31 + a33));  // -(J10 + J30)
            xa[ix][i] += -(a11 + a31);                   // J01, towards n1 = n + (du, 0)
            ya[iy][i] += -(a13 + a33);                   // J03, towards n3 = n + (0, dv)
          }
          for (int r = 0; r < 3; ++r) Bx[r] += h * (-1 * (S(kS_F1 + r, seg, n) + S(kS_F3 + r, seg, n)));
        }
        if (interior(u - du, w)) {  // as the warp neighbour n1 of the crossing n - (du, 0)
          const int anc = n - du;
#pragma unroll
          for (int i = 0; i < 9; ++i) {
            const double b11 = S(kS_J11 + i, seg, anc), b13 = S(kS_J13 + i, seg, anc);
            self[i] += b11;
            xa[1 - ix][i] += -(b11 + b13);  // J10, towards n0 = n + (-du, 0)
          }
          for (int r = 0; r < 3; ++r) Bx[r] += h * S(kS_F1 + r, seg, anc);
        }
        if (interior(u, w - dv)) {  // as the weft neighbour n3 of the crossing n - (0, dv)
          const int anc = n - dv * W;
#pragma unroll
          for (int i = 0; i < 9; ++i) {
            const double c31 = S(kS_J31 + i, seg, anc), c33 = S(kS_J33 + i, seg, anc);
            self[i] += c33;
            ya[1 - iy][i] += -(c31 + c33);  // J30, towards n0 = n + (0, -dv)
          }
          for (int r = 0; r < 3; ++r) Bx[r] += h * S(kS_F3 + r, seg, anc);
        }
      }
      addLL(0, 0, self);
      addLL(-1, 0, xa[0]);
      addLL(1, 0, xa[1]);
      addLL(0, -1, ya[0]);
      addLL(0, 1, ya[1]);
    }
    {  // the diagonal neighbours: J13 of a warp-neighbour role, J31 of a weft-neighbour role
      double dg[4][9];  // (-1, -1), (1, -1), (-1, 1), (1, 1)
#pragma unroll
      for (int i = 0; i < 9; ++i) dg[0][i] = dg[1][i] = dg[2][i] = dg[3][i] = 0.0;
#pragma unroll
      for (int seg = 0; seg < 4; ++seg) {
        const int du = shear_du(seg), dv = shear_dv(seg);
        if (interior(u - du, w)) {  // towards n3 = n + (-du, dv)
          const int t = (-du < 0 ? 0 : 1) + (dv < 0 ? 0 : 2);
#pragma unroll
          for (int i = 0; i < 9; ++i) dg[t][i] += S(kS_J13 + i, seg, n - du);
        }
        if (interior(u, w - dv)) {  // towards n1 = n + (du, -dv)
          const int t = (du < 0 ? 0 : 1) + (-dv < 0 ? 0 : 2);
#pragma unroll
          for (int i = 0; i < 9; ++i) dg[t][i] += S(kS_J31 + i, seg, n - dv * W);
        }
      }
      addLL(-1, -1, dg[0]);
      addLL(1, -1, dg[1]);
      addLL(-1, 1, dg[2]);
      addLL(1, 1, dg[3]);
    }
  } else {
    T J[9];
    // as the crossing n0 (src/PhysicsCloth.cpp:3033-3047)
    if (fl & YS_INTERIOR) {
      for (int seg = 0; seg < 4; ++seg) {
        for (int i = 0; i < 9; ++i) {
          const T J10 = -(S(kS_J11 + i, seg, n) + S(kS_J13 + i, seg, n));
          const T J30 = -(S(kS_J31 + i, seg, n) + S(kS_J33 + i, seg, n));
          J[i] = -(J10 + J30);
        }
        addLL(0, 0, J);
        for (int i = 0; i < 9; ++i) J[i] = -(S(kS_J11 + i, seg, n) + S(kS_J31 + i, seg, n));  // J01
        addLL(shear_du(seg), 0, J);
        for (int i = 0; i < 9; ++i) J[i] = -(S(kS_J13 + i, seg, n) + S(kS_J33 + i, seg, n));  // J03
        addLL(0, shear_dv(seg), J);
        for (int r = 0; r < 3; ++r) Bx[r] += h * (-1 * (S(kS_F1 + r, seg, n) + S(kS_F3 + r, seg, n)));
      }
    }
    // as the warp neighbour n1 = n0 + (du, 0)
    for (int seg = 0; seg < 4; ++seg) {
      const int du = shear_du(seg), dv = shear_dv(seg);
      if (!interior(u - du, w)) continue;
      const int anc = n - du;
      for (int i = 0; i < 9; ++i) J[i] = S(kS_J11 + i, seg, anc);
      addLL(0, 0, J);
      for (int i = 0; i < 9; ++i) J[i] = -(S(kS_J11 + i, seg, anc) + S(kS_J13 + i, seg, anc));  // J10
      addLL(-du, 0, J);
      for (int i = 0; i < 9; ++i) J[i] = S(kS_J13 + i, seg, anc);  // towards n3 = n + (-du, dv)
      addLL(-du, dv, J);
      for (int r = 0; r < 3; ++r) Bx[r] += h * S(kS_F1 + r, seg, anc);
    }
    // as the weft neighbour n3 = n0 + (0, dv)
    for (int seg = 0; seg < 4; ++seg) {
      const int du = shear_du(seg), dv = shear_dv(seg);
      if (!interior(u, w - dv)) continue;
      const int anc = n - dv * W;
      for (int i = 0; i < 9; ++i) J[i] = S(kS_J33 + i, seg, anc);
      addLL(0, 0, J);
      for (int i = 0; i < 9; ++i) J[i] = -(S(kS_J31 + i, seg, anc) + S(kS_J33 + i, seg, anc));  // J30
      addLL(0, -dv, J);
      for (int i = 0; i < 9; ++i) J[i] = S(kS_J31 + i, seg, anc);  // towards n1 = n + (du, -dv)
      addLL(du, -dv, J);
      for (int r = 0; r < 3; ++r) Bx[r] += h * S(kS_F3 + r, seg, anc);
    }
  }
  for (int r = 0; r < 3; ++r) addB(r, Bx[r]);
  // handles, external force, boundary identity rows
  if (fl & YS_FIXED) {
    for (int i = 0; i < 3; ++i) {
      addB(i, h * (-(P.kh * (ldT<T>(v.X, v.dX, i, nt, n) - ld(v.XF, i, nt, n)))));
      const int sl = YS_SLOT_LL + i * 3 + i;
      T a = ldA<T>(v, sl, n);
      a += -(h * h) * (-P.kh);
      finf = finf && isfinite(val(a));
      stA(v, sl, n, a);
    }
  }
  if (v.ext) {
    for (int i = 0; i < 3; ++i) addB(i, T(h * ld(v.ext, i, nt, n)));
    if (fl & YS_INTERIOR)
      for (int k = 0; k < 2; ++k) addB(3 + k, T(h * ld(v.ext, 3 + k, nt, n)));
  }
  if (!(fl & YS_INTERIOR)) {
    for (int k = 0; k < 2; ++k) {
      stA(v, YS_SLOT_EE_SELF + k, n, T(1.0));
      stT(v.B, v.dB, 3 + k, nt, n, T(0.0));
    }
  }
  bool ok = true;
  if (R.nonfinite) {
    // the gather checked what it wrote; the slots changed here were checked
    // as they were written
    ok = finf && !R.nonfinite[n];
  } else {
    for (int s = 0; s < YS_NUM_SLOTS; ++s) ok = ok && isfinite(slot(v, s, n));
  }
  for (int c = 0; c < 5; ++c) ok = ok && isfinite(ld(v.B, c, nt, n));
  if (dinv) {
    for (int i = 0; i < 3; ++i) {
      const double dg = slot(v, YS_SLOT_LL + i * 3 + i, n);
      st(dinv, i, nt, n) = dg != 0.0 ? 1.0 / dg : 1.0;
    }
    for (int k = 0; k < 2; ++k) {
      const double dg = slot(v, YS_SLOT_EE_SELF + k, n);
      st(dinv, 3 + k, nt, n) = dg != 0.0 ? 1.0 / dg : 1.0;
    }
  }
  return ok;
}

// The SpMV rows read their input vector through an accessor: at(j) is a
// handle of node j and get(p, c) its component c. The global form below
// reads a [5][ntot] array; the persistent PCG reads its direction from the
// shared memory of the CTAs of a cluster through another accessor. Both run
// the same arithmetic, so they give the same bits.
struct GlobalVec {
  const double* YS_RESTRICT x;
  int64_t nt;
  typedef const double* Ptr;
  YS_HD Ptr at(int j) const { return x + j; }
  YS_HD double get(Ptr p, int c) const { return p[c * nt]; }
};

// y = A x for row block n (5 rows). Couplings to grid positions outside the
// cloth have zero coefficients; their column index is clamped to n so the
// load stays in bounds and adds 0 * x(n). Every coefficient enters one fused
// multiply-add into its row's running sum, in slot order: 159 FMAs a row
// block, the FP64 pipe's floor for this product.
template <class XV>
YS_HD void spmv_row_sv(const View& v, const double* YS_RESTRICT Ab, int64_t ss, const XV& xv, int n, double y[5]) {
  auto slot = [&](const View&, int s_, int n_) { return Ab[(int64_t)s_ * ss + n_]; };
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  double yl0 = 0.0, yl1 = 0.0, yl2 = 0.0;
  for (int s = 0; s < kNumStencil; ++s) {
    const int uu = u + stencil_du(s), vv = w + stencil_dv(s);
    const bool ok = uu >= 0 && uu < P.W && vv >= 0 && vv < P.H;
    const int j = ok ? n + stencil_du(s) + stencil_dv(s) * P.W : n;
    const typename XV::Ptr xp = xv.at(j);
    const double xj0 = xv.get(xp, 0), xj1 = xv.get(xp, 1), xj2 = xv.get(xp, 2);
    const int b = YS_SLOT_LL + 9 * s;
    yl0 = fma(slot(v, b + 0, n), xj0, yl0); yl0 = fma(slot(v, b + 1, n), xj1, yl0); yl0 = fma(slot(v, b + 2, n), xj2, yl0);
    yl1 = fma(slot(v, b + 3, n), xj0, yl1); yl1 = fma(slot(v, b + 4, n), xj1, yl1); yl1 = fma(slot(v, b + 5, n), xj2, yl1);
    yl2 = fma(slot(v, b + 6, n), xj0, yl2); yl2 = fma(slot(v, b + 7, n), xj1, yl2); yl2 = fma(slot(v, b + 8, n), xj2, yl2);
  }
  const typename XV::Ptr xn = xv.at(n);
  const double xu = xv.get(xn, 3), xv_ = xv.get(xn, 4);
  yl0 = fma(slot(v, YS_SLOT_LE_SELF + 0, n), xu, yl0); yl0 = fma(slot(v, YS_SLOT_LE_SELF + 1, n), xv_, yl0);
  yl1 = fma(slot(v, YS_SLOT_LE_SELF + 2, n), xu, yl1); yl1 = fma(slot(v, YS_SLOT_LE_SELF + 3, n), xv_, yl1);
  yl2 = fma(slot(v, YS_SLOT_LE_SELF + 4, n), xu, yl2); yl2 = fma(slot(v, YS_SLOT_LE_SELF + 5, n), xv_, yl2);
  const double xl0 = xv.get(xn, 0), xl1 = xv.get(xn, 1), xl2 = xv.get(xn, 2);
  double ye[2];
  for (int k = 0; k < 2; ++k) {
    double e = slot(v, YS_SLOT_EL_SELF + 3 * k + 0, n) * xl0;
    e = fma(slot(v, YS_SLOT_EL_SELF + 3 * k + 1, n), xl1, e);
    e = fma(slot(v, YS_SLOT_EL_SELF + 3 * k + 2, n), xl2, e);
    ye[k] = fma(slot(v, YS_SLOT_EE_SELF + k, n), k ? xv_ : xu, e);
  }
  for (int m = 0; m < 4; ++m) {
    const int du = m == 0 ? -1 : m == 1 ? 1 : 0, dv = m == 2 ? -1 : m == 3 ? 1 : 0;
    const int k = m < 2 ? 0 : 1;
    const int uu = u + du, vv = w + dv;
    const bool ok = uu >= 0 && uu < P.W && vv >= 0 && vv < P.H;
    const int j = ok ? n + du + dv * P.W : n;
    const typename XV::Ptr xp = xv.at(j);
    const double xe = xv.get(xp, 3 + k);
    yl0 = fma(slot(v, YS_SLOT_LE_NBR + 3 * m + 0, n), xe, yl0);
    yl1 = fma(slot(v, YS_SLOT_LE_NBR + 3 * m + 1, n), xe, yl1);
    yl2 = fma(slot(v, YS_SLOT_LE_NBR + 3 * m + 2, n), xe, yl2);
    ye[k] = fma(slot(v, YS_SLOT_EL_NBR + 3 * m + 0, n), xv.get(xp, 0), ye[k]);
    ye[k] = fma(slot(v, YS_SLOT_EL_NBR + 3 * m + 1, n), xv.get(xp, 1), ye[k]);
    ye[k] = fma(slot(v, YS_SLOT_EL_NBR + 3 * m + 2, n), xv.get(xp, 2), ye[k]);
    ye[k] = fma(slot(v, YS_SLOT_EE_NBR + m, n), xe, ye[k]);
  }
  y[0] = yl0;
  y[1] = yl1;
  y[2] = yl2;
  y[3] = ye[0];
  y[4] = ye[1];
}

YS_HD void spmv_row_s(const View& v, const double* YS_RESTRICT Ab, int64_t ss, const double* YS_RESTRICT x, int n,
                      double y[5]) {
  spmv_row_sv(v, Ab, ss, GlobalVec{x, v.ntot}, n, y);
}

YS_HD void spmv_row(const View& v, const double* YS_RESTRICT x, int n, double y[5]) {
  spmv_row_s(v, v.A, v.ntot, x, n, y);
}

// y = A^T x for row block n: every coefficient that row block i stores for
// column block n (i = n - offset of its slot) is read from row i, transposed.
template <class XV>
YS_HD void spmv_row_tv(const View& v, const XV& xv, int n, double y[5]) {
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  double yl[3] = {0.0, 0.0, 0.0}, ye[2] = {0.0, 0.0};
  for (int s = 0; s < kNumStencil; ++s) {
    const int du = stencil_du(s), dv = stencil_dv(s);
    const int uu = u - du, vv = w - dv;  // the row that refers to n through slot s
    if (uu < 0 || uu >= P.W || vv < 0 || vv >= P.H) continue;
    const int i = n - du - dv * P.W;
    const typename XV::Ptr xp = xv.at(i);
    const double x0 = xv.get(xp, 0), x1 = xv.get(xp, 1), x2 = xv.get(xp, 2);
    const int b = YS_SLOT_LL + 9 * s;
    for (int c = 0; c < 3; ++c) {
      yl[c] = fma(slot(v, b + c, i), x0, yl[c]);
      yl[c] = fma(slot(v, b + 3 + c, i), x1, yl[c]);
      yl[c] = fma(slot(v, b + 6 + c, i), x2, yl[c]);
    }
  }
  {  // the node's own Eulerian couplings
    const typename XV::Ptr xp = xv.at(n);
    const double x0 = xv.get(xp, 0), x1 = xv.get(xp, 1), x2 = xv.get(xp, 2);
    for (int k = 0; k < 2; ++k) {
      const double xe = xv.get(xp, 3 + k);
      ye[k] = fma(slot(v, YS_SLOT_LE_SELF + 0 + k, n), x0, ye[k]);
      ye[k] = fma(slot(v, YS_SLOT_LE_SELF + 2 + k, n), x1, ye[k]);
      ye[k] = fma(slot(v, YS_SLOT_LE_SELF + 4 + k, n), x2, ye[k]);
      ye[k] = fma(slot(v, YS_SLOT_EE_SELF + k, n), xe, ye[k]);
      for (int c = 0; c < 3; ++c) yl[c] = fma(slot(v, YS_SLOT_EL_SELF + 3 * k + c, n), xe, yl[c]);
    }
  }
  for (int m = 0; m < 4; ++m) {  // yarn neighbour i = n - offset(m) refers to n through m
    const int du = m == 0 ? -1 : m == 1 ? 1 : 0, dv = m == 2 ? -1 : m == 3 ? 1 : 0;
    const int k = m < 2 ? 0 : 1;
    const int uu = u - du, vv = w - dv;
    if (uu < 0 || uu >= P.W || vv < 0 || vv >= P.H) continue;
    const int i = n - du - dv * P.W;
    const typename XV::Ptr xp = xv.at(i);
    const double xe = xv.get(xp, 3 + k);
    ye[k] = fma(slot(v, YS_SLOT_LE_NBR + 3 * m + 0, i), xv.get(xp, 0), ye[k]);
    ye[k] = fma(slot(v, YS_SLOT_LE_NBR + 3 * m + 1, i), xv.get(xp, 1), ye[k]);
    ye[k] = fma(slot(v, YS_SLOT_LE_NBR + 3 * m + 2, i), xv.get(xp, 2), ye[k]);
    ye[k] = fma(slot(v, YS_SLOT_EE_NBR + m, i), xe, ye[k]);
    for (int c = 0; c < 3; ++c) yl[c] = fma(slot(v, YS_SLOT_EL_NBR + 3 * m + c, i), xe, yl[c]);
  }
  y[0] = yl[0];
  y[1] = yl[1];
  y[2] = yl[2];
  y[3] = ye[0];
  y[4] = ye[1];
}

YS_HD void spmv_row_t(const View& v, const double* YS_RESTRICT x, int n, double y[5]) {
  spmv_row_tv(v, GlobalVec{x, v.ntot}, n, y);
}

// Right-hand side of the tangent solve of row block n for tangent k:
// A dq = db - dA q (q the step's solution; dA, db the tangents of A, b).
YS_HD void tangent_rhs_row(const View& v, const double* YS_RESTRICT q, int n, int k, double r[5]) {
  const int64_t nt = v.ntot;
  double y[5];
  spmv_row_s(v, v.dA + k * nt, (int64_t)v.K * nt, q, n, y);
  for (int c = 0; c < 5; ++c) r[c] = v.dB[((int64_t)c * v.K + k) * nt + n] - (v.trunc ? 0.0 : y[c]);
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

// update_node with tangents: xs / dxs hold the solution and its tangents
// ([5][K][ntot]); the state arrays and their tangent arrays are updated
// together (the slide indicator's value is the step's, its tangents dSLIDE).
template <int K>
YS_HD void update_node_dual(const View& v, const double* YS_RESTRICT xs, const double* YS_RESTRICT dxs, double* dX,
                            double* dV, double* dUV, double* dUVD, double* dUVB, int n) {
  typedef Dual<K> D;
  const int nt = v.ntot;
  const uint8_t fl = v.flags[n];
  const double h = v.h;
  for (int i = 0; i < 3; ++i) {
    const D vel = ldT<D>(xs, dxs, i, nt, n);
    stT(v.V, dV, i, nt, n, vel);
    const D x = ldT<D>(v.X, dX, i, nt, n) + vel * h;
    stT(v.X, dX, i, nt, n, x);
    if (!(fl & YS_FIXED)) st(v.XF, i, nt, n) = x.v;
  }
  if (fl & YS_INTERIOR) {
    for (int k = 0; k < 2; ++k) {
      const D e = ldT<D>(xs, dxs, 3 + k, nt, n);
      stT(v.UVD, dUVD, k, nt, n, e);
      stT(v.UV, dUV, k, nt, n, ldT<D>(v.UV, dUV, k, nt, n) + e * h);
      stT(v.UVB, dUVB, k, nt, n,
          ldT<D>(v.UVB, dUVB, k, nt, n) + ldT<D>(v.SLIDE, v.dSLIDE, k, nt, n) * e * h);
    }
  }
}

}  // namespace ys
