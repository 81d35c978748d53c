// ys_pcg_cluster.cu -- the persistent per-cloth Jacobi-PCG: one thread-block
// cluster runs one cloth's whole solve (set-up, every iteration, the stop
// test) in a single launch.
//
// Each thread owns one node of its cloth (cloth-local index rank * T + tid):
// its solution, residual and inverse diagonal stay in registers for the whole
// solve, and its search direction sits in the CTA's shared memory, where the
// other CTAs of the cluster read it through distributed shared memory when
// their stencil reaches it. The system matrix is the only array streamed from
// HBM per iteration. An iteration has three cluster barriers: after the p.q
// partials, after the |r|^2 and r.z partials, and after the new direction.
//
// The arithmetic is the batched PCG's (k_pcg_setup, k_pcg_spmv, k_pcg_axpy,
// k_pcg_dir in ys_kernels.cu) term for term, and the dot products are summed
// in its order: a warp shuffle tree per 32 nodes, the four warp sums of each
// 128-node block in warp order, then the cloth's blocks in node order. So the
// two schedules give the same bits, and both restate Eigen's
// ConjugateGradient with its diagonal preconditioner (src/Solvers.cpp:3-31).
#include <cooperative_groups.h>

#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "ys_items.cuh"
#include "ys_kernels.cuh"

namespace cg = cooperative_groups;

namespace ys {

namespace {

constexpr int kMaxClusterBlocks = 128;  // 128-node blocks per cloth (16 CTAs x 1024 threads)

// The cluster's direction vector: node li of the cloth at rank li / T, slot
// li % T of that CTA's [5][T] slice. Handles are 32-bit shared::cluster
// addresses (mapa), read with ld.shared::cluster; without a cluster, plain
// shared-memory pointers.
template <int T, bool CLUSTER>
struct ClusterVec {
  double* base;    // this CTA's [5][T] slice
  uint32_t base32; // its shared::cta address
  int off;         // the cloth's first node
  typedef typename std::conditional<CLUSTER, uint32_t, const double*>::type Ptr;
  __device__ __forceinline__ Ptr at(int j) const {
    const int lj = j - off;
    if constexpr (!CLUSTER) {
      return base + lj;
    } else {
      const int rk = lj / T;
      const uint32_t a = base32 + 8u * (uint32_t)(lj - rk * T);
      uint32_t r;
      asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rk));
      return r;
    }
  }
  __device__ __forceinline__ double get(Ptr p, int c) const {
    if constexpr (!CLUSTER) {
      return p[c * T];
    } else {
      double x;
      asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(x) : "r"(p + 8u * (uint32_t)(c * T)));
      return x;
    }
  }
};

// Sums NQ per-thread values over the cloth in the batched solver's order and
// returns them in every thread. wp is this CTA's [NQ][T/32] warp-partial
// buffer for this reduction (double-buffered by the caller); out is a shared
// [NQ] broadcast slot.
template <int T, bool CLUSTER, int NQ>
__device__ __forceinline__ void cloth_reduce(double (&val)[NQ], double* wp, double* out, int nblk) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    double s = val[q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) wp[q * (T / 32) + wid] = s;
  }
  if (CLUSTER) cg::this_cluster().sync();
  else __syncthreads();
  if (wid == 0) {
    // lane l forms the partials of blocks l, l + 32, ...: each the four warp
    // sums of the block added to 0 in warp order (block_sum)
    double bp[NQ][kMaxClusterBlocks / 32];
#pragma unroll
    for (int m = 0; m < kMaxClusterBlocks / 32; ++m) {
      const int blk = lane + 32 * m;
#pragma unroll
      for (int q = 0; q < NQ; ++q) bp[q][m] = 0.0;
      if (blk < nblk) {
        const int g0 = 4 * blk;  // the block's first warp in the cloth
        const int rk = g0 / (T / 32), lw = g0 - rk * (T / 32);
        const double* src = CLUSTER ? cg::this_cluster().map_shared_rank(wp, rk) : wp;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          double s = 0.0;
#pragma unroll
          for (int i = 0; i < 4; ++i) s += src[q * (T / 32) + lw + i];
          bp[q][m] = s;
        }
      }
    }
    // the cloth sum: the block partials added to 0 in block order (cloth_sum)
    double tot[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) tot[q] = 0.0;
#pragma unroll
    for (int m = 0; m < kMaxClusterBlocks / 32; ++m) {
      const int cnt = min(32, nblk - 32 * m);  // <= 0 past the last block
      for (int l = 0; l < cnt; ++l) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) tot[q] += __shfl_sync(0xffffffffu, bp[q][m], l);
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) out[q] = tot[q];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) val[q] = out[q];
}

template <int T, bool CLUSTER, bool TRANS>
__global__ void __launch_bounds__(T, 1) k_pcg_cluster(View v, Solver so, const int* __restrict__ cloths, int cap) {
  __shared__ double psm[5 * T];
  __shared__ double wp[2][3 * (T / 32)];
  __shared__ double bc[3];
  const int csize = CLUSTER ? (int)cg::this_cluster().num_blocks() : 1;
  const int rank = CLUSTER ? (int)cg::this_cluster().block_rank() : 0;
  const int c = cloths[blockIdx.x / csize];
  PcgCloth& pc = so.pc[c];
  const ClothParams& P = v.cp[c];
  const int N = P.W * P.H, off = P.node_off;
  const int nblk = (N + kBlock - 1) / kBlock;
  const int li = rank * T + threadIdx.x;
  const bool own = li < N;
  const int n = off + (own ? li : 0);
  const int nt = v.ntot;
  const ClusterVec<T, CLUSTER> pv{psm, (uint32_t)__cvta_generic_to_shared(psm), off};
  const int maxiter = pc.maxiter;
  const bool ok_sys = pc.status == 0;  // read before any CTA of the cluster can write it
  int red = 0;  // reductions so far: selects the warp-partial buffer

  // set-up (k_pcg_setup, k_pcg_start): x = 0, r = b, p = z = Dinv r. The
  // solution and residual stay in registers; p lives in shared memory and the
  // inverse diagonal is re-read (L1) where it is needed, which keeps the
  // 1024-thread form within its 64 registers.
  double x[5], r[5];
  double rr = 0.0, rz = 0.0;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    x[k] = 0.0;
    r[k] = own ? ld(v.B, k, nt, n) : 0.0;
    const double z = (own ? __ldg(so.dinv + (int64_t)k * nt + n) : 0.0) * r[k];
    psm[k * T + threadIdx.x] = z;
    rr += r[k] * r[k];
    rz += r[k] * z;
  }
  double s0[2] = {rr, rz};
  cloth_reduce<T, CLUSTER, 2>(s0, wp[red++ & 1], bc, nblk);
  const double bb = s0[0];
  double thr = so.tol * so.tol * bb;
  if (thr < DBL_MIN) thr = DBL_MIN;
  double rzc = s0[1], rrc = bb;
  bool active = ok_sys && bb != 0.0 && bb >= thr;
  int iters = 0, capped = 0;
  int it = 0;
  for (; it < cap && active; ++it) {
    // q = A p and p.q (k_pcg_spmv)
    double q[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    double pq[1] = {0.0};
    if (own) {
      if (TRANS) spmv_row_tv(v, pv, n, q);
      else spmv_row_sv(v, v.A, v.ntot, pv, n, q);
#pragma unroll
      for (int k = 0; k < 5; ++k) pq[0] += psm[k * T + threadIdx.x] * q[k];
    }
    cloth_reduce<T, CLUSTER, 1>(pq, wp[red++ & 1], bc, nblk);
    // alpha, x += alpha p, r -= alpha q, |r|^2 and r.z (k_pcg_axpy)
    const double alpha = rzc / pq[0];
    double s1[2] = {0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        x[k] += alpha * psm[k * T + threadIdx.x];
        const double rk = r[k] - alpha * q[k];
        r[k] = rk;
        s1[0] += rk * rk;
        s1[1] += rk * (__ldg(so.dinv + (int64_t)k * nt + n) * rk);
      }
    }
    cloth_reduce<T, CLUSTER, 2>(s1, wp[red++ & 1], bc, nblk);
    // the stop test, then beta and p = z + beta p (k_pcg_dir)
    const bool conv = s1[0] < thr;
    const bool cp = !conv && it + 1 >= maxiter;
    const double beta = s1[1] / rzc;
    rrc = s1[0];
    rzc = s1[1];
    iters = conv ? it : it + 1;
    if (conv || cp) {
      active = false;
      capped = cp;
      break;
    }
    if (own) {
#pragma unroll
      for (int k = 0; k < 5; ++k)
        psm[k * T + threadIdx.x] = __ldg(so.dinv + (int64_t)k * nt + n) * r[k] + beta * psm[k * T + threadIdx.x];
    }
    if (CLUSTER) cg::this_cluster().sync();
    else __syncthreads();
  }
  if (own)
#pragma unroll
    for (int k = 0; k < 5; ++k) st(so.x, k, nt, n) = x[k];
  if (rank == 0 && threadIdx.x == 0) {
    pc.bb = bb;
    pc.thr = thr;
    pc.rr = rrc;
    pc.rz[0] = rzc;
    pc.rz[1] = rzc;
    pc.iters = iters;
    pc.active = active ? 1 : 0;
    if (capped) pc.status |= 4;
  }
  // no CTA of the cluster may exit while another can still read its shared memory
  if (CLUSTER) cg::this_cluster().sync();
}

template <int T, bool CLUSTER, bool TRANS>
cudaError_t launch_t(const View& v, const Solver& so, const int* cloths, int ncl, int csize, int cap, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(ncl * csize));
  cfg.blockDim = dim3(T);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = CLUSTER ? 1 : 0;
  // clusters above 8 CTAs were enabled by occupancy_t (ys_set_pcg_schedule)
  return cudaLaunchKernelEx(&cfg, k_pcg_cluster<T, CLUSTER, TRANS>, v, so, cloths, cap);
}

template <int T, bool CLUSTER>
cudaError_t occupancy_t(int csize, int* clusters) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)csize);
  cfg.blockDim = dim3(T);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (csize > 8) {
    // both forms, before any launch (and outside any stream capture)
    cudaError_t e = cudaFuncSetAttribute(k_pcg_cluster<T, CLUSTER, false>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_pcg_cluster<T, CLUSTER, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  return cudaOccupancyMaxActiveClusters(clusters, k_pcg_cluster<T, CLUSTER, false>, &cfg);
}

}  // namespace

bool pcg_cluster_shape_ok(int threads, int csize) {
  if (threads != 128 && threads != 256 && threads != 512 && threads != 1024) return false;
  if (csize != 1 && csize != 2 && csize != 4 && csize != 8 && csize != 16) return false;
  return threads * csize <= kMaxClusterBlocks * kBlock;
}

cudaError_t pcg_cluster_occupancy(int threads, int csize, int* clusters) {
  *clusters = 0;
  if (!pcg_cluster_shape_ok(threads, csize)) return cudaErrorInvalidValue;
  if (csize == 1) {
    *clusters = 1;  // plain CTAs: one always fits
    return cudaSuccess;
  }
  switch (threads) {
    case 128: return occupancy_t<128, true>(csize, clusters);
    case 256: return occupancy_t<256, true>(csize, clusters);
    case 512: return occupancy_t<512, true>(csize, clusters);
    default: return occupancy_t<1024, true>(csize, clusters);
  }
}

cudaError_t launch_pcg_cluster(const View& v, const Solver& so, const int* cloths, int ncl, int threads, int csize,
                               int cap, cudaStream_t s) {
  if (!pcg_cluster_shape_ok(threads, csize) || ncl <= 0) return cudaErrorInvalidValue;
  const bool cl = csize > 1, tr = so.trans != 0;
#define YS_PCGC(TT)                                                                              \
  case TT:                                                                                       \
    if (cl) return tr ? launch_t<TT, true, true>(v, so, cloths, ncl, csize, cap, s)              \
                      : launch_t<TT, true, false>(v, so, cloths, ncl, csize, cap, s);            \
    return tr ? launch_t<TT, false, true>(v, so, cloths, ncl, 1, cap, s)                         \
              : launch_t<TT, false, false>(v, so, cloths, ncl, 1, cap, s);
  switch (threads) {
    YS_PCGC(128)
    YS_PCGC(256)
    YS_PCGC(512)
    YS_PCGC(1024)
  }
#undef YS_PCGC
  return cudaErrorInvalidValue;
}

}  // namespace ys
