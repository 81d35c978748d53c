// ys_kernels.cu -- CUDA kernels of one implicit step of a batch of cloths.
//
// Assembly: one thread per element writes that element's record (forces and
// Jacobian blocks), then one thread per node gathers the records touching its
// row block in a fixed order, so every row is accumulated deterministically
// without atomics. The element and gather kernels are templates over the
// scalar type: double for the step, Dual<kTangents> for its forward-mode
// sensitivities.
// Solve: per-cloth Jacobi-PCG (Eigen's ConjugateGradient algorithm, as used by
// src/Solvers.cpp:3-31) on the structured stencil matrix; thread blocks never
// straddle cloths, so each cloth's dot products are a fixed-order sum of its
// blocks' partials, recomputed redundantly by every block that needs them.
#include <cfloat>

#include "ys_elem_kernels.cuh"
#include "ys_items.cuh"
#include "ys_kernels.cuh"

namespace ys {

static inline int nblocks(int n) { return (n + kBlock - 1) / kBlock; }

__global__ void k_geom(View v, const int* __restrict__ nodes, int count) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int n = nodes[t];
  node_normal(v, n, v.cp[v.node_cloth[n]].W);
}

// ----------------------------------------------------------------- solve
__device__ __forceinline__ double block_sum(double val, double* sh) {
  for (int o = 16; o > 0; o >>= 1) val += __shfl_down_sync(0xffffffffu, val, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = val;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  return s;  // valid in thread 0
}

// fixed-order sum of cloth c's block partials in row `which`
__device__ __forceinline__ double cloth_sum(const Blocks& b, const double* part, int which, int c) {
  const int b0 = b.cloth_blk0[c], nb = b.cloth_nblk[c];
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += part[which * b.nblk + b0 + i];
  return s;
}

// shear records into the row blocks, then handles, external force, boundary
// identity rows, Jacobi diagonal and the finite check of the system
__global__ void __launch_bounds__(kBlock) k_finalize(View v, Records R, Blocks b, Solver so) {
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  const int n = b.blk_node0[blk] + threadIdx.x;
  bool bad = false;
  if (threadIdx.x < b.blk_count[blk]) bad = !gather_shear_finalize<double>(v, R, n, so.dinv);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&so.pc[c].status, 1);
}

// x = 0, r = b, p = z = Dinv r; partials |b|^2 (row 0), |r|^2 (row 1) and
// r.z (row 2)
__global__ void __launch_bounds__(kBlock) k_pcg_setup(View v, Blocks b, Solver so) {
  __shared__ double sh[kBlock / 32];
  const int blk = blockIdx.x;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  double rr = 0.0, rz = 0.0;
  if (threadIdx.x < b.blk_count[blk]) {
    for (int k = 0; k < 5; ++k) {
      const double r = ld(v.B, k, nt, n);
      const double z = ld(so.dinv, k, nt, n) * r;
      st(so.x, k, nt, n) = 0.0;
      st(so.r, k, nt, n) = r;
      st(so.p, k, nt, n) = z;
      rr += r * r;
      rz += r * z;
    }
  }
  double s1 = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    so.part[0 * b.nblk + blk] = s1;  // r = b here
    so.part[1 * b.nblk + blk] = s1;
  }
  double s2 = block_sum(rz, sh);
  if (threadIdx.x == 0) so.part[2 * b.nblk + blk] = s2;
}

__global__ void k_pcg_start(Blocks b, Solver so, int ncloth) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncloth) return;
  PcgCloth& pc = so.pc[c];
  const double bb = cloth_sum(b, so.part, 0, c);
  const double rr = cloth_sum(b, so.part, 1, c);
  const double rz = cloth_sum(b, so.part, 2, c);
  pc.bb = bb;
  double thr = so.tol * so.tol * bb;
  if (thr < DBL_MIN) thr = DBL_MIN;
  pc.thr = thr;
  pc.rr = rr;
  pc.rz[0] = rz;
  pc.iters = 0;
  pc.active = (pc.status == 0 && bb != 0.0 && rr >= thr) ? 1 : 0;
}

// q = A p and partial p.q (row 0)
template <bool TRANS>
__global__ void __launch_bounds__(kBlock) k_pcg_spmv(View v, Blocks b, Solver so) {
  __shared__ double sh[kBlock / 32];
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  if (!so.pc[c].active) return;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  double pq = 0.0;
  if (threadIdx.x < b.blk_count[blk]) {
    double y[5];
    if (TRANS) spmv_row_t(v, so.p, n, y);
    else spmv_row(v, so.p, n, y);
    for (int k = 0; k < 5; ++k) {
      st(so.q, k, nt, n) = y[k];
      pq += ld(so.p, k, nt, n) * y[k];
    }
  }
  const double s = block_sum(pq, sh);
  if (threadIdx.x == 0) so.part[0 * b.nblk + blk] = s;
}

// alpha = rz / pq; x += alpha p; r -= alpha q; partials |r|^2 (row 1), r.z (row 2)
__global__ void __launch_bounds__(kBlock) k_pcg_axpy(View v, Blocks b, Solver so, int parity) {
  __shared__ double sh[kBlock / 32];
  __shared__ double alpha_sh;
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  if (!so.pc[c].active) return;
  if (threadIdx.x == 0) alpha_sh = so.pc[c].rz[parity] / cloth_sum(b, so.part, 0, c);
  __syncthreads();
  const double alpha = alpha_sh;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  double rr = 0.0, rz = 0.0;
  if (threadIdx.x < b.blk_count[blk]) {
    for (int k = 0; k < 5; ++k) {
      st(so.x, k, nt, n) += alpha * ld(so.p, k, nt, n);
      const double r = ld(so.r, k, nt, n) - alpha * ld(so.q, k, nt, n);
      st(so.r, k, nt, n) = r;
      rr += r * r;
      rz += r * (ld(so.dinv, k, nt, n) * r);
    }
  }
  double s1 = block_sum(rr, sh);
  if (threadIdx.x == 0) so.part[1 * b.nblk + blk] = s1;
  double s2 = block_sum(rz, sh);
  if (threadIdx.x == 0) so.part[2 * b.nblk + blk] = s2;
}

// stop test |r|^2 < thr, else beta = rz_new / rz and p = z + beta p. Every
// block of a cloth reaches the same decision from the same fixed-order sums;
// only the cloth's first block writes the cloth's bookkeeping.
__global__ void __launch_bounds__(kBlock) k_pcg_dir(View v, Blocks b, Solver so, int parity, int it_local) {
  __shared__ int go_sh;
  const int it = so.it_base ? *so.it_base + it_local : it_local;
  __shared__ double beta_sh;
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  PcgCloth& pc = so.pc[c];
  if (!pc.active) return;
  if (threadIdx.x == 0) {
    const double rr = cloth_sum(b, so.part, 1, c);
    const double rzn = cloth_sum(b, so.part, 2, c);
    const bool lead = blk == b.cloth_blk0[c];
    const bool conv = rr < pc.thr;
    // every active cloth has completed exactly `it` iterations before this one
    const bool cap = !conv && it + 1 >= pc.maxiter;
    go_sh = !(conv || cap);
    beta_sh = rzn / pc.rz[parity];
    if (lead) {
      pc.rr = rr;
      pc.rz[parity ^ 1] = rzn;
      pc.iters = conv ? it : it + 1;
      if (conv || cap) pc.active = 0;
      if (cap) pc.status |= 4;
    }
  }
  __syncthreads();
  if (!go_sh) return;
  const double beta = beta_sh;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  if (threadIdx.x < b.blk_count[blk])
    for (int k = 0; k < 5; ++k)
      st(so.p, k, nt, n) = ld(so.dinv, k, nt, n) * ld(so.r, k, nt, n) + beta * ld(so.p, k, nt, n);
}

__global__ void k_count_active(Solver so, int ncloth) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int mine = 0;
  for (int c = threadIdx.x; c < ncloth; c += blockDim.x) mine += so.pc[c].active;
  atomicAdd(&cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0) *so.nactive = cnt;
}

// flags a cloth whose solution holds a non-finite value (src/TrainHelper.cpp:41-48)
__global__ void __launch_bounds__(kBlock) k_check_solution(View v, Blocks b, Solver so) {
  if (so.hold && *so.hold) return;
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  const int n = b.blk_node0[blk] + threadIdx.x;
  bool ok = true;
  if (threadIdx.x < b.blk_count[blk])
    for (int k = 0; k < 5; ++k) ok = ok && isfinite(ld(so.x, k, v.ntot, n));
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(&so.pc[c].status, 2);
}

// Cloth::update for every cloth whose step succeeded
__global__ void __launch_bounds__(kBlock) k_update(View v, Blocks b, Solver so) {
  if (so.hold && *so.hold) return;
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  const int n = b.blk_node0[blk] + threadIdx.x;
  if (threadIdx.x >= b.blk_count[blk]) return;
  if (so.pc[c].status & 3) return;  // SimStep returns false and leaves the cloth as it was
  update_node(v, so.x, n);
}

__global__ void k_learned_verdict(Solver so, int ncloth, const int* err, int caller_cap, int* hold) {
  int redo = *err != 0;
  for (int c = threadIdx.x; c < ncloth; c += blockDim.x) {
    const int st = so.pc[c].status;
    if (!(st & 1) && ((st & 8) || ((st & 4) && !caller_cap))) redo = 1;
  }
  redo = __syncthreads_or(redo);
  if (threadIdx.x == 0) *hold = redo;
}

__global__ void k_spmv_plain(View v, const double* x, double* y) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  double r[5];
  spmv_row(v, x, n, r);
  for (int k = 0; k < 5; ++k) y[(int64_t)k * v.ntot + n] = r[k];
}

// ----------------------------------------------------------------- launchers
void launch_geom(const View& v, const int* nodes, int n, cudaStream_t s) {
  if (n) k_geom<<<nblocks(n), kBlock, 0, s>>>(v, nodes, n);
}
static inline unsigned pblocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }
void launch_edge_records(const View& v, const Records& R, cudaStream_t s, int t) {
  t = t < kBlock ? t : kBlock;  // k_edge_rec is compiled for at most kBlock threads
  k_edge_rec<double><<<pblocks(2LL * v.ntot, t), t, 0, s>>>(v, R);
}
void launch_bend_records(const View& v, const Records& R, cudaStream_t s, int t) {
  k_bend_rec<double><<<pblocks(2LL * v.ntot, t), t, 0, s>>>(v, R);
}
void launch_face_records(const View& v, const Records& R, cudaStream_t s, int t) {
  k_face_rec<double><<<pblocks(v.ntot, t), t, 0, s>>>(v, R);
}
void launch_gather(const View& v, const Records& R, cudaStream_t s, int t) {
  k_gather<double><<<pblocks(v.ntot, t), t, 0, s>>>(v, R);
}
void launch_shear_records(const View& v, const Records& R, cudaStream_t s, int t) {
  k_shear_rec<double><<<pblocks(4LL * v.ntot, t), t, 0, s>>>(v, R);
}
void launch_finalize(const View& v, const Records& R, const Blocks& b, const Solver& so, cudaStream_t s) {
  k_finalize<<<b.nblk, kBlock, 0, s>>>(v, R, b, so);
}
void launch_pcg_setup(const View& v, const Blocks& b, const Solver& so, cudaStream_t s) {
  k_pcg_setup<<<b.nblk, kBlock, 0, s>>>(v, b, so);
  k_pcg_start<<<(v.ncloth + 127) / 128, 128, 0, s>>>(b, so, v.ncloth);
}
void launch_pcg_spmv(const View& v, const Blocks& b, const Solver& so, cudaStream_t s) {
  if (so.trans) k_pcg_spmv<true><<<b.nblk, kBlock, 0, s>>>(v, b, so);
  else k_pcg_spmv<false><<<b.nblk, kBlock, 0, s>>>(v, b, so);
}
void launch_pcg_axpy(const View& v, const Blocks& b, const Solver& so, int it, cudaStream_t s) {
  k_pcg_axpy<<<b.nblk, kBlock, 0, s>>>(v, b, so, it & 1);
}
void launch_pcg_dir(const View& v, const Blocks& b, const Solver& so, int it, cudaStream_t s) {
  k_pcg_dir<<<b.nblk, kBlock, 0, s>>>(v, b, so, it & 1, it);
}
void launch_count_active(const View& v, const Solver& so, cudaStream_t s) {
  k_count_active<<<1, 256, 0, s>>>(so, v.ncloth);
}
__global__ void k_graph_loop_begin(Solver so) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *so.it_base = 0;
}
__global__ void k_graph_loop_tail(Solver so, int ncloth, int m, int cap, cudaGraphConditionalHandle h) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int mine = 0;
  for (int c = threadIdx.x; c < ncloth; c += blockDim.x) mine += so.pc[c].active;
  atomicAdd(&cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0) {
    *so.nactive = cnt;
    const int done = *so.it_base + m;
    *so.it_base = done;
    // the loop ends when no cloth iterates or at the iteration cap, whichever first
    cudaGraphSetConditional(h, (cnt > 0 && done < cap) ? 1u : 0u);
  }
}
void launch_graph_loop_begin(const Solver& so, cudaStream_t s) { k_graph_loop_begin<<<1, 32, 0, s>>>(so); }
void launch_graph_loop_tail(const Solver& so, int ncloth, int m, int cap, cudaGraphConditionalHandle h,
                            cudaStream_t s) {
  k_graph_loop_tail<<<1, 256, 0, s>>>(so, ncloth, m, cap, h);
}
void launch_check_solution(const View& v, const Blocks& b, const Solver& so, cudaStream_t s) {
  k_check_solution<<<b.nblk, kBlock, 0, s>>>(v, b, so);
}
void launch_update(const View& v, const Blocks& b, const Solver& so, cudaStream_t s) {
  k_check_solution<<<b.nblk, kBlock, 0, s>>>(v, b, so);
  k_update<<<b.nblk, kBlock, 0, s>>>(v, b, so);
}
void launch_learned_verdict(const Solver& so, int ncloth, const int* err, int caller_cap, int* hold,
                            cudaStream_t s) {
  k_learned_verdict<<<1, 256, 0, s>>>(so, ncloth, err, caller_cap, hold);
}
void launch_spmv(const View& v, const double* x, double* y, cudaStream_t s) {
  k_spmv_plain<<<nblocks(v.ntot), kBlock, 0, s>>>(v, x, y);
}

}  // namespace ys
