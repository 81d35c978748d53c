// ys_adjoint.cu -- kernels of the reverse-mode (adjoint) step.
//
// One step maps the state s = (LPos, LVel, EPos, EVel, EPosBar) and the
// parameters to s' through: assembly of A(s), b(s); q = A^-1 b; Cloth::update
// (src/Cloth.cpp:111-148). Given the adjoint g' = dL/ds', the adjoint step
// returns dL/ds, dL/d(parameters) and dL/d(external force):
//
//   1. the update's transpose: q_bar from g' (k_adj_update), the slide
//      indicator's adjoint, and the parts of g' that pass straight through;
//   2. lambda = A^-T q_bar (exact), or A^-1 q_bar (the reference's own
//      backward of its solve, src/Solvers.cpp:33-58), by the PCG kernels;
//   3. the residual's vector-Jacobian product: with r(s) = A(s) q - b(s),
//      dL/ds_j = -lambda . dr/ds_j + slide_bar . dslide/ds_j. Row block i of
//      r depends only on the state of nodes within L1 grid distance 4 of i
//      (bend segments reach 2 along a yarn, node normals 1 more, the
//      compression that crimp bends build at a crossing feeds the crossing's
//      shear segments, which reach 1 more), so the columns of dr/ds are
//      compressed by colouring the nodes with (u + 9 v) mod 41: nodes of one
//      colour are at L1 distance >= 9, their 41-node neighbourhoods (L1 ball
//      of radius 4) are disjoint, and one forward-mode direction per
//      (colour, state component) seeds all of them at once. The forward-mode
//      step kernels (ys_tangent.cu, the same element code over Dual<K>) give
//      the directional derivatives dr of every direction on copies of the
//      cloth; k_adj_contract folds each row's dr with lambda, and
//      k_adj_gather_state sums, for node j and component c, the folded rows
//      in j's neighbourhood from the direction of (colour(j), c). Per-line
//      material is compressed the same way (a line's material reaches the
//      rows of the line and its two neighbour lines; lines coloured mod 3),
//      S and mu are one direction each.
#include "ys_kernels.cuh"

namespace ys {

namespace {
constexpr int K = kTangents;
}

// number of forward-mode directions one adjoint step needs
//   41 colours x 12 state components, 2 orientations x 3 line colours x
//   (rho, Y, B), S, mu
constexpr int kAdjColors = 41;
constexpr int kAdjStateComps = 12;
constexpr int kAdjStateDirs = kAdjColors * kAdjStateComps;        // 492
constexpr int kAdjLineDirs = 2 * 3 * 3;                           // 18
constexpr int kAdjDirs = kAdjStateDirs + kAdjLineDirs + 2;        // 512

YS_HD int adj_color(int u, int v) { return (u + 9 * v) % kAdjColors; }

// Cloth::update transposed. gin: [5 arrays] g' of LPos [3][nt], LVel [3][nt],
// EPos [2][nt], EVel [2][nt], EPosBar [2][nt] (component-major). Writes
// qbar [5][nt], the pass-through part of g (gout, same layout) and
// slide_bar [2][nt].
__global__ void k_adj_update(View v, AdjIO io, const double* __restrict__ q, double* __restrict__ qbar,
                             double* __restrict__ slide_bar) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const int nt = v.ntot;
  const double h = v.h;
  const bool in = (v.flags[n] & YS_INTERIOR) != 0;
  for (int i = 0; i < 3; ++i) {
    const double gx = io.gin[0][i * nt + n], gv = io.gin[1][i * nt + n];
    qbar[i * nt + n] = gv + h * gx;  // V' = q, X' = X + h q
    io.gout[0][i * nt + n] = gx;
    io.gout[1][i * nt + n] = 0.0;
  }
  for (int k = 0; k < 2; ++k) {
    const double ge = io.gin[2][k * nt + n], gd = io.gin[3][k * nt + n], gb = io.gin[4][k * nt + n];
    io.gout[2][k * nt + n] = ge;
    io.gout[4][k * nt + n] = gb;
    if (in) {
      // EVel' = q_e, EPos' = EPos + h q_e, EPosBar' = EPosBar + slide q_e h
      const double s = v.SLIDE[k * nt + n], qe = q[(3 + k) * nt + n];
      qbar[(3 + k) * nt + n] = gd + h * ge + s * h * gb;
      io.gout[3][k * nt + n] = 0.0;
      slide_bar[k * nt + n] = gb * qe * h;
    } else {  // boundary crossings keep their Eulerian state
      qbar[(3 + k) * nt + n] = 0.0;
      io.gout[3][k * nt + n] = gd;
      slide_bar[k * nt + n] = 0.0;
    }
  }
}

// dst[c][copy][nt] = src[c][nt] for `copies` copies of `nt` entries
__global__ void k_adj_broadcast(const double* __restrict__ src, double* __restrict__ dst, int nt, int ncomp,
                                int copies) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t per = (int64_t)nt * copies;
  if (t >= per * ncomp) return;
  const int c = (int)(t / per);
  const int64_t r = t - (int64_t)c * per;
  dst[t] = src[(int64_t)c * nt + r % nt];
}

// forward-mode seeds of one pass: copy c of the pass carries directions
// 4 (base + c) .. 4 (base + c) + 3. State seeds in the tangent layout
// [comp][K][ntc] of the copies' batch.
__global__ void k_adj_seed_state(View vc, int nt, int base, AdjSeeds sd) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t ntc = vc.ntot;
  if (i >= ntc) return;
  const int copy = (int)(i / nt);
  const int col = adj_color(vc.node_u[i], vc.node_v[i]);
  for (int k = 0; k < K; ++k) {
    const int dir = 4 * (base + copy) + k;
    const int comp = (dir < kAdjStateDirs && dir / kAdjStateComps == col) ? dir % kAdjStateComps : -1;
    for (int c = 0; c < 3; ++c) {
      sd.dX[((int64_t)c * K + k) * ntc + i] = comp == c ? 1.0 : 0.0;
      sd.dV[((int64_t)c * K + k) * ntc + i] = comp == 3 + c ? 1.0 : 0.0;
    }
    for (int c = 0; c < 2; ++c) {
      sd.dUV[((int64_t)c * K + k) * ntc + i] = comp == 6 + c ? 1.0 : 0.0;
      sd.dUVD[((int64_t)c * K + k) * ntc + i] = comp == 8 + c ? 1.0 : 0.0;
      sd.dUVB[((int64_t)c * K + k) * ntc + i] = comp == 10 + c ? 1.0 : 0.0;
    }
  }
}

// material seeds: line l of copy c (primal line l % nl); warp lines are
// node rows v, weft lines node columns u (ClothParams line offsets)
__global__ void k_adj_seed_params(View vc, int nl, int ncl, int base, const double* __restrict__ line_a,
                                  const int* __restrict__ line_kind, AdjSeeds sd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nlc = vc.nlines, ncc = vc.ncloth;
  if (t < nlc) {
    const int copy = t / nl, l = t - copy * nl;
    const int kind = line_kind[l];  // orientation * 3 + (line position mod 3)
    for (int k = 0; k < K; ++k) {
      const int dir = 4 * (base + copy) + k - kAdjStateDirs;
      const bool mine = dir >= 0 && dir < kAdjLineDirs && dir / 3 == kind;
      const int p = dir % 3;
      sd.drho[(int64_t)k * nlc + t] = mine && p == 0 ? 1.0 : 0.0;
      sd.dks[(int64_t)k * nlc + t] = mine && p == 1 ? line_a[l] : 0.0;  // ks = Y pi R^2
      sd.dkb[(int64_t)k * nlc + t] = mine && p == 2 ? line_a[l] : 0.0;  // kb = B pi R^2
    }
  }
  if (t < ncc) {
    const int copy = t / ncl;
    for (int k = 0; k < K; ++k) {
      const int dir = 4 * (base + copy) + k - kAdjStateDirs - kAdjLineDirs;
      sd.dS[(int64_t)k * ncc + t] = dir == 0 ? 1.0 : 0.0;
      sd.dmu[(int64_t)k * ncc + t] = dir == 1 ? 1.0 : 0.0;
    }
  }
}

// T[k][i] = lambda(n) . rt_k(i) + slide_bar(n) . dslide_k(i) for row block i
// of the copies (n its primal node); rt_k = db_k - dA_k q (db_k in the
// reference mode) as k_tangent_rhs writes it: [k][5][ntc]
__global__ void k_adj_contract(View vc, int nt, const double* __restrict__ lambda,
                               const double* __restrict__ slide_bar, const double* __restrict__ rt,
                               double* __restrict__ T) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t ntc = vc.ntot;
  if (i >= ntc) return;
  const int n = (int)(i % nt);
  double lam[5], sb[2];
  for (int c = 0; c < 5; ++c) lam[c] = lambda[(int64_t)c * nt + n];
  for (int c = 0; c < 2; ++c) sb[c] = slide_bar[(int64_t)c * nt + n];
  for (int k = 0; k < K; ++k) {
    double t = 0.0;
    for (int c = 0; c < 5; ++c) t += lam[c] * rt[((int64_t)k * 5 + c) * ntc + i];
    for (int c = 0; c < 2; ++c) t += sb[c] * vc.dSLIDE[((int64_t)c * K + k) * ntc + i];
    T[(int64_t)k * ntc + i] = t;
  }
}

// gout(j, comp) += sum of T over the L1 ball of radius 4 around j, from the
// direction (colour(j), comp) when this pass holds it
__global__ void k_adj_gather_state(View v, int base, int copies, const double* __restrict__ T, int64_t ntc,
                                   AdjIO io) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = v.ntot;
  if (t >= (int64_t)nt * kAdjStateComps) return;
  const int comp = (int)(t / nt), j = (int)(t - (int64_t)comp * nt);
  const int u = v.node_u[j], w = v.node_v[j];
  const int dir = adj_color(u, w) * kAdjStateComps + comp;
  const int copy = dir / 4 - base, k = dir % 4;
  if (copy < 0 || copy >= copies) return;
  const ClothParams& P = v.cp[v.node_cloth[j]];
  const double* Tk = T + (int64_t)k * ntc + (int64_t)copy * nt;
  double s = 0.0;
  for (int dv = -4; dv <= 4; ++dv) {
    const int rem = 4 - (dv < 0 ? -dv : dv);
    for (int du = -rem; du <= rem; ++du) {
      const int uu = u + du, vv = w + dv;
      if (uu < 0 || uu >= P.W || vv < 0 || vv >= P.H) continue;
      s += Tk[j + du + dv * P.W];
    }
  }
  // components: LPos 0-2, LVel 3-5, EPos 6-7, EVel 8-9, EPosBar 10-11
  const int arr = comp < 3 ? 0 : comp < 6 ? 1 : comp < 8 ? 2 : comp < 10 ? 3 : 4;
  const int c = comp < 3 ? comp : comp < 6 ? comp - 3 : comp < 8 ? comp - 6 : comp < 10 ? comp - 8 : comp - 10;
  io.gout[arr][(int64_t)c * nt + j] += s;
}

// material adjoints: warp line v of a cloth sums rows v-1..v+1, weft line u
// columns u-1..u+1; S and mu sum the whole cloth. gp: [5][nl or ncl]
// (rho, Y, B per line; S, mu per cloth), accumulated.
__global__ void k_adj_gather_params(View v, int base, int copies, const double* __restrict__ T, int64_t ntc,
                                    const int* __restrict__ line_cloth, const int* __restrict__ line_kind,
                                    AdjParamOut gp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nl = v.nlines, ncl = v.ncloth, nt = v.ntot;
  if (t < 3 * nl) {
    const int p = t / nl, l = t - p * nl;
    const int kind = line_kind[l], orient = kind / 3;
    const int dir = kAdjStateDirs + kind * 3 + p;
    const int copy = dir / 4 - base, k = dir % 4;
    if (copy >= 0 && copy < copies) {
      const ClothParams& P = v.cp[line_cloth[l]];
      const double* Tk = T + (int64_t)k * ntc + (int64_t)copy * nt + P.node_off;
      double s = 0.0;
      if (orient == 0) {  // warp line: node row v
        const int row = l - P.warp_line_off;
        for (int vv = row - 1; vv <= row + 1; ++vv)
          if (vv >= 0 && vv < P.H)
            for (int uu = 0; uu < P.W; ++uu) s += Tk[uu + vv * P.W];
      } else {  // weft line: node column u
        const int col = l - P.weft_line_off;
        for (int vv = 0; vv < P.H; ++vv)
          for (int uu = col - 1; uu <= col + 1; ++uu)
            if (uu >= 0 && uu < P.W) s += Tk[uu + vv * P.W];
      }
      gp.line[p][l] += s;
    }
  }
  if (t < 2 * ncl) {
    const int p = t / ncl, c = t - p * ncl;
    const int dir = kAdjStateDirs + kAdjLineDirs + p;
    const int copy = dir / 4 - base, k = dir % 4;
    if (copy >= 0 && copy < copies) {
      const ClothParams& P = v.cp[c];
      const double* Tk = T + (int64_t)k * ntc + (int64_t)copy * nt + P.node_off;
      double s = 0.0;
      for (int i = 0; i < P.W * P.H; ++i) s += Tk[i];
      gp.cloth[p][c] += s;
    }
  }
}

// dL/d ext = h lambda on the components the gather adds ext to (x, y, z of
// every node, u, v of interior crossings); node layout [nt][5]
__global__ void k_adj_ext(View v, const double* __restrict__ lambda, double* __restrict__ gext) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const bool in = (v.flags[n] & YS_INTERIOR) != 0;
  for (int c = 0; c < 5; ++c) gext[(int64_t)n * 5 + c] = (c < 3 || in) ? v.h * lambda[(int64_t)c * v.ntot + n] : 0.0;
}

static inline unsigned nb256(int64_t n) { return (unsigned)((n + 255) / 256); }

int adjoint_direction_count() { return kAdjDirs; }

void launch_adj_update(const View& v, const AdjIO& io, const double* q, double* qbar, double* slide_bar,
                       cudaStream_t s) {
  k_adj_update<<<nb256(v.ntot), 256, 0, s>>>(v, io, q, qbar, slide_bar);
}
void launch_adj_broadcast(const double* src, double* dst, int nt, int ncomp, int copies, cudaStream_t s) {
  k_adj_broadcast<<<nb256((int64_t)nt * copies * ncomp), 256, 0, s>>>(src, dst, nt, ncomp, copies);
}
void launch_adj_seed(const View& vc, int nt, int nl, int ncl, int base, const double* line_a, const int* line_kind,
                     const AdjSeeds& sd, cudaStream_t s) {
  k_adj_seed_state<<<nb256(vc.ntot), 256, 0, s>>>(vc, nt, base, sd);
  k_adj_seed_params<<<nb256(vc.nlines > vc.ncloth ? vc.nlines : vc.ncloth), 256, 0, s>>>(vc, nl, ncl, base, line_a,
                                                                                          line_kind, sd);
}
void launch_adj_contract(const View& vc, int nt, const double* lambda, const double* slide_bar, const double* rt,
                         double* T, cudaStream_t s) {
  k_adj_contract<<<nb256(vc.ntot), 256, 0, s>>>(vc, nt, lambda, slide_bar, rt, T);
}
void launch_adj_gather(const View& v, int base, int copies, const double* T, int64_t ntc, const int* line_cloth,
                       const int* line_kind, const AdjIO& io, const AdjParamOut& gp, cudaStream_t s) {
  k_adj_gather_state<<<nb256((int64_t)v.ntot * kAdjStateComps), 256, 0, s>>>(v, base, copies, T, ntc, io);
  const int np = 3 * v.nlines > 2 * v.ncloth ? 3 * v.nlines : 2 * v.ncloth;
  k_adj_gather_params<<<nb256(np), 256, 0, s>>>(v, base, copies, T, ntc, line_cloth, line_kind, gp);
}
void launch_adj_ext(const View& v, const double* lambda, double* gext, cudaStream_t s) {
  k_adj_ext<<<nb256(v.ntot), 256, 0, s>>>(v, lambda, gext);
}

}  // namespace ys
