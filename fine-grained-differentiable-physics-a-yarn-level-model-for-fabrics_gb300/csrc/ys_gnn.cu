// ys_gnn.cu -- kernels of the learned preconditioner: system features, the
// graph network's BF16 tcgen05 GEMMs (forward, data and weight gradients),
// the blocks of G, the stochastic Frobenius loss with its hand-written
// gradient, Adam, and the preconditioned conjugate-gradient iteration that
// applies M^-1 = G^T G.
#include <cfloat>
#include <cmath>

#include "ys_gnn.cuh"
#include "ys_items.cuh"
#include "ys_tc.cuh"

namespace ys {

using bf16 = __nv_bfloat16;

namespace {

constexpr int kNB = 128;  // threads per block of the node kernels
inline int nblk(int n) { return (n + kNB - 1) / kNB; }
__device__ __forceinline__ int opp(int d) { return d ^ 1; }  // left<->right, down<->up
__device__ __forceinline__ int lt(int r, int c) { return r * (r + 1) / 2 + c; }

// ------------------------------------------------------------ neighbours
// yarn neighbours (message passing) and the lower pattern of G with its transpose
__global__ void k_gnn_nbr(View v, GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  g.nbr[4 * n + 0] = u > 0 ? n - 1 : -1;
  g.nbr[4 * n + 1] = u < P.W - 1 ? n + 1 : -1;
  g.nbr[4 * n + 2] = w > 0 ? n - P.W : -1;
  g.nbr[4 * n + 3] = w < P.H - 1 ? n + P.W : -1;
  for (int b = 0; b < 8; ++b) {
    int src = -1, row = -1;
    if (b < kGBlocks) {
      const int du = gpat_du(b), dv = gpat_dv(b);
      if (u + du >= 0 && u + du < P.W && w + dv >= 0 && w + dv < P.H) src = n + du + dv * P.W;
      if (u - du >= 0 && u - du < P.W && w - dv >= 0 && w - dv < P.H) row = n - du - dv * P.W;
    }
    g.pat[8 * n + b] = src;
    g.upat[8 * n + b] = row;
  }
}

// ------------------------------------------------- block factor and features
// 5 x 5 diagonal block of row block n (DOF order x, y, z, u, v), in FP32
__device__ __forceinline__ void diag_block(const View& v, int n, float D[5][5]) {
  const int64_t nt = v.ntot;
  const double* a = v.A + n;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c) D[r][c] = (float)a[(YS_SLOT_LL + 3 * r + c) * nt];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      D[r][3 + k] = (float)a[(YS_SLOT_LE_SELF + 2 * r + k) * nt];
      D[3 + k][r] = (float)a[(YS_SLOT_EL_SELF + 3 * k + r) * nt];
    }
  }
  D[3][3] = (float)a[YS_SLOT_EE_SELF * nt];
  D[4][4] = (float)a[(YS_SLOT_EE_SELF + 1) * nt];
  D[3][4] = D[4][3] = 0.f;
}

// 5 x 5 block A(n, j) of yarn neighbour d (j = n + offset(d)); warp
// neighbours (d < 2) couple u, weft neighbours v (selects, no runtime indexing)
__device__ __forceinline__ void nbr_block(const View& v, int n, int d, float B[5][5]) {
  const int s = d + 1;  // stencil slots 1..4 are (-1,0), (1,0), (0,-1), (0,1)
  const bool ku = d < 2;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c) B[r][c] = (float)slot(v, YS_SLOT_LL + 9 * s + 3 * r + c, n);
    const float le = (float)slot(v, YS_SLOT_LE_NBR + 3 * d + r, n);
    const float el = (float)slot(v, YS_SLOT_EL_NBR + 3 * d + r, n);
    B[r][3] = ku ? le : 0.f;
    B[r][4] = ku ? 0.f : le;
    B[3][r] = ku ? el : 0.f;
    B[4][r] = ku ? 0.f : el;
  }
  const float ee = (float)slot(v, YS_SLOT_EE_NBR + d, n);
  B[3][3] = ku ? ee : 0.f;
  B[4][4] = ku ? 0.f : ee;
  B[3][4] = B[4][3] = 0.f;
}

// 5 x 5 block A(n, src) of lower-pattern block b > 0 (couplings through the
// stencil slot of its offset; Eulerian entries for the yarn neighbours)
__device__ __forceinline__ void pat_block(const View& v, int n, int b, float B[5][5]) {
  if (b == 1 || b == 2) {
    nbr_block(v, n, b == 1 ? 0 : 2, B);
    return;
  }
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) B[r][c] = 0.f;
  const int s = stencil_index(gpat_du(b), gpat_dv(b));
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) B[r][c] = (float)slot(v, YS_SLOT_LL + 9 * s + 3 * r + c, n);
}

__device__ __forceinline__ void load_linv(const float* linv, int nt, int n, float L[5][5]) {
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) L[r][c] = c <= r ? linv[(int64_t)lt(r, c) * nt + n] : 0.f;
}

// L^-1 of the Cholesky factor of the symmetric part of the diagonal block;
// a block that does not factorise falls back to the scalar Jacobi scaling
__global__ void k_gnn_linv(View v, float* linv, int* chol_ok) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  // single precision: the factor only shapes the preconditioner
  float D[5][5], L[5][5] = {};
  diag_block(v, n, D);
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    float s = D[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
    ok = ok && s > 0.f && isfinite(s);
    L[j][j] = sqrtf(fmaxf(s, FLT_MIN));
#pragma unroll
    for (int i = j + 1; i < 5; ++i) {
      float t = 0.5f * (D[i][j] + D[j][i]);
#pragma unroll
      for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
      L[i][j] = t / L[j][j];
    }
  }
  if (!ok) {
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) L[r][c] = 0.f;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const float d = fabsf(D[j][j]);
      L[j][j] = (d > 0.f && isfinite(d)) ? sqrtf(d) : 1.f;
    }
  }
  float X[5][5] = {};
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    X[c][c] = 1.f / L[c][c];
#pragma unroll
    for (int r = c + 1; r < 5; ++r) {
      float t = 0.f;
#pragma unroll
      for (int k = c; k < r; ++k) t += L[r][k] * X[k][c];
      X[r][c] = -t / L[r][r];
    }
  }
  const int nt = v.ntot;
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c <= r; ++c) linv[(int64_t)lt(r, c) * nt + n] = X[r][c];
  chol_ok[n] = ok ? 1 : 0;
}

// C = A * B^T for 5 x 5 (B given as its rows)
__device__ __forceinline__ void mul_abt(const float A[5][5], const float B[5][5], float C[5][5]) {
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) {
      float s = 0.f;
      for (int k = 0; k < 5; ++k) s += A[r][k] * B[c][k];
      C[r][c] = s;
    }
}
__device__ __forceinline__ void mul_ab(const float A[5][5], const float B[5][5], float C[5][5]) {
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) {
      float s = 0.f;
      for (int k = 0; k < 5; ++k) s += A[r][k] * B[k][c];
      C[r][c] = s;
    }
}

__device__ __forceinline__ float frob(const float M[5][5]) {
  float s = 0.f;
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) s += M[r][c] * M[r][c];
  return sqrtf(s);
}

// one thread per (coupling q, node): q < 6 the lower block b = q + 1 (its E
// kept for the prior; features: E of left and down (50), x part of E of the
// four other lower blocks (36)); q >= 6 the norm of the scaled coupling to
// the upper neighbour right, up, right-up, left-up, right-2, up-2 (6); q = 0
// also writes the flags (5) and the zero padding. A block covers kFeatNodes
// nodes x 12 couplings and assembles their feature rows in shared memory, so
// the rows leave in whole 16-byte chunks.
constexpr int kFeatNodes = 32;
constexpr int kFeatRow = kGIn + 8;  // padded shared row (BF16 elements), 16-byte multiple

__global__ void __launch_bounds__(12 * kFeatNodes) k_gnn_feat(View v, GnnBufs g) {
  __shared__ __align__(16) bf16 fs[kFeatNodes][kFeatRow];
  const int nt = v.ntot;
  const int q = threadIdx.x / kFeatNodes, ln = threadIdx.x - q * kFeatNodes;
  const int n0 = blockIdx.x * kFeatNodes;
  const int n = n0 + ln;
  const int cnt = min(kFeatNodes, nt - n0);
  bf16* f = fs[ln];
  if (ln < cnt) {
    float Li[5][5], Lj[5][5], Bk[5][5], T[5][5], E[5][5];
    const ClothParams& P = v.cp[v.node_cloth[n]];
    const int u = v.node_u[n], w = v.node_v[n];
    if (q < 6) {
      const int b = q + 1;  // lower offset (gpat_du, gpat_dv)(b), whether or not G uses it
      const int ub = u + gpat_du(b), vb = w + gpat_dv(b);
      const int j = (ub >= 0 && ub < P.W && vb >= 0 && vb < P.H) ? n + gpat_du(b) + gpat_dv(b) * P.W : -1;
      if (j >= 0) {
        load_linv(g.linv, nt, n, Li);
        pat_block(v, n, b, Bk);
        load_linv(g.linv, nt, j, Lj);
        mul_ab(Li, Bk, T);
        mul_abt(T, Lj, E);
      } else {
#pragma unroll
        for (int r = 0; r < 5; ++r)
#pragma unroll
          for (int c = 0; c < 5; ++c) E[r][c] = 0.f;
      }
#pragma unroll
      for (int r = 0; r < 5; ++r)
#pragma unroll
        for (int c = 0; c < 5; ++c) g.E[(int64_t)(25 * q + 5 * r + c) * nt + n] = E[r][c];
      if (b <= 2) {
#pragma unroll
        for (int r = 0; r < 5; ++r)
#pragma unroll
          for (int c = 0; c < 5; ++c) f[25 * q + 5 * r + c] = __float2bfloat16(E[r][c]);
      } else {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) f[50 + 9 * (b - 3) + 3 * r + c] = __float2bfloat16(E[r][c]);
      }
      if (q == 0) {
        const uint8_t fl = v.flags[n];
        f[92] = __float2bfloat16(g.chol_ok[n] ? 0.f : 1.f);
        f[93] = __float2bfloat16((fl & YS_INTERIOR) ? 1.f : 0.f);
        f[94] = __float2bfloat16((fl & YS_FIXED) ? 1.f : 0.f);
        f[95] = __float2bfloat16((u == 0 || u == P.W - 1) ? 1.f : 0.f);
        f[96] = __float2bfloat16((w == 0 || w == P.H - 1) ? 1.f : 0.f);
        for (int k = 97; k < kGIn; ++k) f[k] = __float2bfloat16(0.f);
      }
    } else {
      const int k = q - 6;
      const int du = k == 0 ? 1 : k == 1 ? 0 : k == 2 ? 1 : k == 3 ? -1 : k == 4 ? 2 : 0;
      const int dv = k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 1 : k == 3 ? 1 : k == 4 ? 0 : 2;
      float nrm = 0.f;
      if (u + du >= 0 && u + du < P.W && w + dv >= 0 && w + dv < P.H) {
        const int j = n + du + dv * P.W;
        load_linv(g.linv, nt, n, Li);
        load_linv(g.linv, nt, j, Lj);
        if (k < 2) {
          nbr_block(v, n, k == 0 ? 1 : 3, Bk);
        } else {
          const int s = stencil_index(du, dv);
#pragma unroll
          for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int c = 0; c < 5; ++c)
              Bk[r][c] = (r < 3 && c < 3) ? (float)slot(v, YS_SLOT_LL + 9 * s + 3 * r + c, n) : 0.f;
        }
        mul_ab(Li, Bk, T);
        mul_abt(T, Lj, E);
        nrm = frob(E);
      }
      f[86 + k] = __float2bfloat16(nrm);
    }
  }
  __syncthreads();
  // rows of kGIn BF16 = kGIn / 8 chunks of 16 bytes
  constexpr int kChunks = kGIn / 8;
  for (int k = threadIdx.x; k < cnt * kChunks; k += blockDim.x) {
    const int row = k / kChunks, ch = k - row * kChunks;
    *reinterpret_cast<uint4*>(g.f + (int64_t)(n0 + row) * kGIn + 8 * ch) =
        *reinterpret_cast<const uint4*>(&fs[row][8 * ch]);
  }
}

// ------------------------------------------------------------ tensor-core GEMM
// C[m][n] = sum_k A(m, k) B(n, k) over 128-row tiles (blockIdx.x), NT-column
// tiles (blockIdx.y) and K splits (blockIdx.z); the Op stages A and B chunks
// of 64 K into shared memory and consumes the FP32 accumulator rows.
// asynchronous 16-byte global -> shared copies (zero-filled when !valid)
__device__ __forceinline__ void cp_async16(uint8_t* dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc::smem_u32(dst)), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

constexpr int kGemmThreads = 128;
constexpr int kGemmSmem = 56 * 1024;  // keeps at most 4 CTAs (4 x 128 TMEM columns) per SM
constexpr uint32_t kWaitLimit = 1u << 22;

// KCH chunks are staged before one batch of MMAs (all of K when it fits),
// so a CTA pays one global-load round trip per KCH chunks
template <class Op, int KCH>
__global__ void __launch_bounds__(kGemmThreads) k_tc_gemm(Op op, int nchunk_total, int chunks_per_split, int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int kABytes = 16384, kBBytes = Op::NT * 128;
  uint8_t* sA = smem;
  uint8_t* sB = smem + KCH * kABytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + KCH * (kABytes + kBBytes));
  uint32_t* slot_ = reinterpret_cast<uint32_t*>(bar + 1);
  constexpr uint32_t kCols = Op::NT < 32 ? 32 : Op::NT;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) tc::mbar_init(bar, 1);
  if (warp == 0) tc::tmem_alloc(slot_, kCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot_;
  const int m0 = blockIdx.x * tc::kTileM, n0 = blockIdx.y * Op::NT;
  const int kc0 = blockIdx.z * chunks_per_split;
  const int kc1 = min(nchunk_total, kc0 + chunks_per_split);
  constexpr uint32_t idesc = tc::idesc_bf16(tc::kTileM, Op::NT);
  uint32_t phase = 0;
  bool ok = true;
  for (int kc = kc0; kc < kc1; kc += KCH) {
    const int nk = min(KCH, kc1 - kc);
    for (int q = 0; q < nk; ++q) {
      op.stage_a(sA + q * kABytes, m0, kc + q);
      op.stage_b(sB + q * kBBytes, n0, kc + q);
    }
    cp_async_wait_all();
    tc::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      for (int q = 0; q < nk; ++q) {
        const uint32_t a0 = tc::smem_u32(sA + q * kABytes), b0 = tc::smem_u32(sB + q * kBBytes);
#pragma unroll
        for (int k = 0; k < tc::kChunkK / 16; ++k)
          tc::mma_bf16(tmem, tc::smem_desc(a0 + k * 256), tc::smem_desc(b0 + k * 256), idesc,
                       (kc > kc0 || q > 0 || k > 0) ? 1u : 0u);
      }
      tc::mma_commit(bar);
    }
    bool done = tc::mbar_wait(bar, phase, kWaitLimit);
    ok = __syncthreads_and(done) != 0;
    if (!ok) break;
    phase ^= 1;
    tc::fence_after_sync();
  }
  if (ok && kc1 > kc0) {
    // 32-column slabs of the accumulator go through shared memory (row
    // stride 33 floats: conflict-free both ways) so that the stores of a warp
    // cover 32 consecutive columns of one row
    float* stage = reinterpret_cast<float*>(smem);
    const int row = warp * 32 + (threadIdx.x & 31);
#pragma unroll 1
    for (int c = 0; c < Op::NT; c += 32) {
      float acc[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, acc);
#pragma unroll
      for (int i = 0; i < 16; ++i) stage[row * 33 + i] = acc[i];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c + 16), acc);
#pragma unroll
      for (int i = 0; i < 16; ++i) stage[row * 33 + 16 + i] = acc[i];
      __syncthreads();
      // row-major outputs: a warp stores 32 columns of a row; column-major
      // ones (Op::kColMajor): 32 rows of a column. The operands an epilogue
      // reads (bias, residual) are all loaded before the first store, so
      // they are in flight together.
      constexpr int kPer = tc::kTileM * 32 / kGemmThreads;
      float2 pre[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k) {
        const int i = threadIdx.x + k * kGemmThreads;
        const int r = Op::kColMajor ? (i & 127) : (i >> 5), cc = Op::kColMajor ? (i >> 7) : (i & 31);
        pre[k] = op.prefetch(m0 + r, n0 + c + cc);
      }
#pragma unroll
      for (int k = 0; k < kPer; ++k) {
        const int i = threadIdx.x + k * kGemmThreads;
        const int r = Op::kColMajor ? (i & 127) : (i >> 5), cc = Op::kColMajor ? (i >> 7) : (i & 31);
        op.store(m0 + r, n0 + c + cc, stage[r * 33 + cc], pre[k]);
      }
      __syncthreads();
    }
  } else if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    tc::mbar_wait(bar, phase, kWaitLimit);  // let the MMAs in flight finish before freeing
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kCols);
  }
}

__device__ __forceinline__ void store1(uint8_t* tile, int r, int k, bf16 val) {
  *reinterpret_cast<bf16*>(tile + tc::core_off(r, k)) = val;
}

// rows of X (ld elements, 64-wide chunk kc, or the neighbour given by the chunk
// when gathering), one thread per row, as asynchronous 16-byte copies
// (missing rows are zero-filled); cp_async_wait_all completes them
__device__ __forceinline__ void stage_rows(uint8_t* sA, const bf16* X, int ld, int M, const int* nbr, bool gather,
                                           int m0, int kc) {
  const int r = threadIdx.x;
  const int node = m0 + r;
  int src = -1;
  if (node < M) src = gather ? (kc == 0 ? node : nbr[4 * node + kc - 1]) : node;
  const bf16* p = X + (int64_t)(src >= 0 ? src : 0) * ld + (gather ? 0 : kc * 64);
#pragma unroll
  for (int q = 0; q < 8; ++q) cp_async16(sA + tc::core_off(r, q * 8), p + q * 8, src >= 0);
}
// NT rows of a row-major [rows][K] weight matrix
template <int NT>
__device__ __forceinline__ void stage_weights(uint8_t* sB, const bf16* W, int K, int n0, int kc) {
  for (int i = threadIdx.x; i < NT * 8; i += kGemmThreads) {
    const int n = i >> 3, q = i & 7;
    cp_async16(sB + tc::core_off(n, q * 8), W + (int64_t)(n0 + n) * K + kc * 64 + q * 8, true);
  }
}

// forward: out = epilogue(X W^T + b)
enum { kEpiEnc = 0, kEpiLayer = 1, kEpiHead = 2 };
template <int NT_, int EPI>
struct FwdOp {
  static constexpr int NT = NT_;
  static constexpr bool kColMajor = EPI == kEpiHead;  // o is stored [kGOut][ntot]
  const bf16* X;
  int ld, M;
  const int* nbr;
  int gather;
  const bf16* W;
  int K;
  const float* bias;
  const float* h_in;
  float* h_out;
  bf16* hb_out;
  bf16* act_out;
  float* o_out;
  __device__ void stage_a(uint8_t* s, int m0, int kc) const { stage_rows(s, X, ld, M, nbr, gather != 0, m0, kc); }
  __device__ void stage_b(uint8_t* s, int n0, int kc) const { stage_weights<NT>(s, W, K, n0, kc); }
  // (bias, residual) of output (node, j)
  __device__ float2 prefetch(int node, int j) const {
    if (node >= M) return make_float2(0.f, 0.f);
    return make_float2(bias[j], EPI == kEpiLayer ? h_in[(int64_t)node * kGHid + j] : 0.f);
  }
  __device__ void store(int node, int j, float acc, float2 pre) const {
    if (node >= M) return;
    const float z = acc + pre.x;
    if (EPI == kEpiHead) {
      o_out[(int64_t)j * M + node] = z;
    } else {
      const float a = fmaxf(z, 0.f);
      const int64_t at = (int64_t)node * kGHid + j;
      float hn = a;
      if (EPI == kEpiLayer) {
        if (act_out) act_out[at] = __float2bfloat16(a);
        hn = pre.y + a;
      }
      if (h_out) h_out[at] = hn;
      hb_out[at] = __float2bfloat16(hn);
    }
  }
};

// data gradient: dX = dZ W, with B = W^T stored [K_in][Nout]
struct BwdDataOp {
  static constexpr int NT = 64;
  static constexpr bool kColMajor = false;
  const bf16* dZ;
  int nout, M;
  const bf16* WT;
  float* out;
  int kin;
  __device__ void stage_a(uint8_t* s, int m0, int kc) const { stage_rows(s, dZ, nout, M, nullptr, false, m0, kc); }
  __device__ void stage_b(uint8_t* s, int n0, int kc) const { stage_weights<NT>(s, WT, nout, n0, kc); }
  __device__ float2 prefetch(int, int) const { return make_float2(0.f, 0.f); }
  __device__ void store(int node, int col, float acc, float2) const {
    if (node < M) out[(int64_t)node * kin + col] = acc;
  }
};

// weight gradient: C[k'][j] = sum_node X(node, k') dZ[node][j], k' < kin;
// row kin is a column of ones (the bias gradient). One 64-node chunk per
// K round; partial sums per split.
template <int NT_>
struct WgradOp {
  static constexpr int NT = NT_;
  static constexpr bool kColMajor = false;
  const bf16* X;
  int ld, kin, nodes;
  const int* nbr;
  int gather;
  const bf16* dZ;
  int ldz;      // columns of dZ and of the partial sums; this CTA's are n0 .. n0 + NT
  float* part;  // [split][kWgradRows][ldz]
  __device__ void stage_a(uint8_t* s, int m0, int kc) const {
    const int r = threadIdx.x;
    const int feat = m0 + r;
    for (int kk = 0; kk < 64; ++kk) {
      const int node = kc * 64 + kk;
      float val = 0.f;
      if (node < nodes) {
        if (feat < kin) {
          int src = node, col = feat;
          if (gather) {
            const int c = feat >> 6;
            col = feat & 63;
            src = c == 0 ? node : nbr[4 * node + c - 1];
          }
          if (src >= 0) val = __bfloat162float(X[(int64_t)src * ld + col]);
        } else if (feat == kin) {
          val = 1.f;
        }
      }
      store1(s, r, kk, __float2bfloat16(val));
    }
  }
  __device__ void stage_b(uint8_t* s, int n0, int kc) const {
    for (int i = threadIdx.x; i < NT * 64; i += kGemmThreads) {
      const int n = i % NT, kk = i / NT;
      const int node = kc * 64 + kk;
      store1(s, n, kk, node < nodes ? dZ[(int64_t)node * ldz + n0 + n] : __float2bfloat16(0.f));
    }
  }
  __device__ float2 prefetch(int, int) const { return make_float2(0.f, 0.f); }
  __device__ void store(int row, int col, float acc, float2) const {
    if (row <= kin) part[((int64_t)blockIdx.z * kWgradRows + row) * ldz + col] = acc;
  }
};

// C = A B^T for row-major BF16 A [M][K] and B [N][K] (the GEMM self-test)
template <int NT_>
struct PlainOp {
  static constexpr int NT = NT_;
  static constexpr bool kColMajor = false;
  const bf16* A;
  const bf16* B;
  float* C;
  int M, N, K;
  __device__ void stage_a(uint8_t* s, int m0, int kc) const { stage_rows(s, A, K, M, nullptr, false, m0, kc); }
  __device__ void stage_b(uint8_t* s, int n0, int kc) const { stage_weights<NT>(s, B, K, n0, kc); }
  __device__ float2 prefetch(int, int) const { return make_float2(0.f, 0.f); }
  __device__ void store(int m, int col, float acc, float2) const {
    if (m < M) C[(int64_t)m * N + col] = acc;
  }
};

// dynamic shared memory of a GEMM kernel: at least 56 KB keeps at most 4
// CTAs (4 x 128 TMEM columns) on an SM
template <class Op, int KCH>
constexpr int gemm_smem() {
  return KCH * (16384 + Op::NT * 128) + 64 > kGemmSmem ? KCH * (16384 + Op::NT * 128) + 64 : kGemmSmem;
}
template <class Op, int KCH = 1>
void gemm_attr() {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_tc_gemm<Op, KCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, gemm_smem<Op, KCH>());
    attr = true;
  }
}

template <class Op, int KCH = 1>
void launch_gemm(const Op& op, int M, int ncol_tiles, int nchunk, int nsplit, int* err, cudaStream_t s) {
  constexpr int smem = gemm_smem<Op, KCH>();
  gemm_attr<Op, KCH>();
  const int per = (nchunk + nsplit - 1) / nsplit;
  const int splits = (nchunk + per - 1) / per;
  dim3 grid((M + tc::kTileM - 1) / tc::kTileM, ncol_tiles, splits);
  k_tc_gemm<Op, KCH><<<grid, kGemmThreads, smem, s>>>(op, nchunk, per, err);
}

// sums the splits in a fixed order into the gradient: weights [ncol][kin]
// and the bias row
__global__ void k_wgrad_reduce(const float* part, int splits, int kin, int ncol, float* gW, float* gb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // (row, j)
  if (i >= (kin + 1) * ncol) return;
  const int row = i / ncol, j = i % ncol;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[((int64_t)z * kWgradRows + row) * ncol + j];
  if (row < kin) gW[(int64_t)j * kin + row] = s;
  else gb[j] = s;
}

// ------------------------------------------------------------------ G blocks
// one thread per (block b, node); the blocks of N are kept only for training
__global__ void __launch_bounds__(kNB, 8) k_gnn_g(GnnBufs g, int keep_n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (t >= (int64_t)kGBlocks * nt) return;
  const int b = (int)(t / nt), n = (int)(t - (int64_t)b * nt);
  const int j = g.pat[8 * n + b];
  if (j < 0) {
    for (int q = 0; q < 13; ++q) g.Gh[(int64_t)(13 * b + q) * nt + n] = __floats2bfloat162_rn(0.f, 0.f);
    for (int k = 0; k < 25; ++k) {
      if (keep_n) g.G[(int64_t)(25 * b + k) * nt + n] = 0.f;
      if (keep_n) g.Gn[(int64_t)(25 * b + k) * nt + n] = 0.f;
    }
    return;
  }
  const float* o = g.o + (int64_t)(25 * b) * nt + n;  // component-major
  const float* E = b > 0 ? g.E + (int64_t)(25 * (b - 1)) * nt + n : nullptr;
  float L[5][5], N[5][5], Gb[5][5];
  load_linv(g.linv, nt, j, L);
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const int k = 5 * r + c;
      float val = kGOutScale * o[(int64_t)k * nt];
      if (b > 0) val -= E[(int64_t)k * nt];
      N[r][c] = val;
      if (keep_n) g.Gn[(int64_t)(25 * b + k) * nt + n] = val;
    }
  if (b == 0)
#pragma unroll
    for (int r = 0; r < 5; ++r) N[r][r] += 1.f;
  mul_ab(N, L, Gb);
#pragma unroll
  for (int q = 0; q < 13; ++q)
    g.Gh[(int64_t)(13 * b + q) * nt + n] =
        __floats2bfloat162_rn(Gb[(2 * q) / 5][(2 * q) % 5], 2 * q + 1 < 25 ? Gb[(2 * q + 1) / 5][(2 * q + 1) % 5] : 0.f);
  if (keep_n)
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) g.G[(int64_t)(25 * b + 5 * r + c) * nt + n] = Gb[r][c];
}

// ------------------------------------------------- blocked applications
// a G coefficient of the FP32 copy (training)
__device__ __forceinline__ float coef(const float* g, int64_t i) { return g[i]; }

// z_n = sum over the rows i = upat(n, b) of G_i,b^T x_i
template <class TG, class TX>
__device__ __forceinline__ void apply_cols(const TG* Gk, const int* upat, int nt, const TX* x, int n, float z[5]) {
  int row[kGBlocks];
#pragma unroll
  for (int b = 0; b < kGBlocks; ++b) row[b] = upat[8 * n + b];
  float xs[kGBlocks][5];
#pragma unroll
  for (int b = 0; b < kGBlocks; ++b) {
    const int i = row[b] >= 0 ? row[b] : n;
    const float m = row[b] >= 0 ? 1.f : 0.f;
#pragma unroll
    for (int r = 0; r < 5; ++r) xs[b][r] = m * (float)x[(int64_t)r * nt + i];
  }
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    float s = 0.f;
#pragma unroll
    for (int b = 0; b < kGBlocks; ++b) {
      const int i = row[b] >= 0 ? row[b] : n;
#pragma unroll
      for (int r = 0; r < 5; ++r) s += coef(Gk, (int64_t)(25 * b + 5 * r + c) * nt + i) * xs[b][r];
    }
    z[c] = s;
  }
}

// ------------------------------------------------- learned-preconditioner PCG
__device__ __forceinline__ double blk_sum(double val, double* sh) {
  for (int o = 16; o > 0; o >>= 1) val += __shfl_down_sync(0xffffffffu, val, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = val;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  return s;
}
__device__ __forceinline__ double cl_sum(const Blocks& b, const double* part, int which, int c) {
  const int b0 = b.cloth_blk0[c], nb = b.cloth_nblk[c];
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += part[which * b.nblk + b0 + i];
  return s;
}

// alpha = r.z / p.q; x += alpha p; r -= alpha q (setup: x = 0, r = b); the
// FP32 copy of r the preconditioner reads; partial |r|^2 (row 1; setup also
// |b|^2, row 0)
__global__ void __launch_bounds__(kBlock) k_lp_axpy(View v, Blocks b, Solver so, LpcgExtra lx, int parity,
                                                     int setup) {
  __shared__ double sh[kBlock / 32];
  __shared__ double alpha_sh;
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  if (!setup && !so.pc[c].active) return;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  const bool own = threadIdx.x < b.blk_count[blk];
  // the loads that do not need alpha go out before the cloth sum
  double r[5], q[5], p[5];
  if (own)
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      r[k] = setup ? ld(v.B, k, nt, n) : ld(so.r, k, nt, n);
      q[k] = setup ? 0.0 : ld(so.q, k, nt, n);
      p[k] = setup ? 0.0 : ld(so.p, k, nt, n);
    }
  if (threadIdx.x == 0) alpha_sh = setup ? 0.0 : so.pc[c].rz[parity] / cl_sum(b, so.part, 0, c);
  __syncthreads();
  const double alpha = alpha_sh;
  double rr = 0.0;
  if (own)
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      if (setup) st(so.x, k, nt, n) = 0.0;
      else st(so.x, k, nt, n) += alpha * p[k];
      const double rn = setup ? r[k] : fma(-alpha, q[k], r[k]);
      st(so.r, k, nt, n) = rn;
      lx.rf[(int64_t)k * nt + n] = (float)rn;
      rr += rn * rn;
    }
  const double s1 = blk_sum(rr, sh);
  if (threadIdx.x == 0) {
    so.part[1 * b.nblk + blk] = s1;
    if (setup) so.part[0 * b.nblk + blk] = s1;
  }
}

// z = G^T G r (FP32 r, BF16 G, FP32 sums). Block b of row i couples node
// i + (du_b, dv_b) (the lower offsets gpat_du / gpat_dv, dv_b in {0, -1, -2}),
// so node n's z sums G_i,b^T y_i over the rows i = n - (du_b, dv_b), with
// y_i = sum_b G_i,b r(i + (du_b, dv_b)). A block of nodes [n0, n0 + cnt)
// computes y of the rows it needs into shared memory -- by -dv_b the windows
// [n0, n0 + cnt + 2), [n0 + W - 1, n0 + W + cnt + 1) and [n0 + 2W, n0 + 2W +
// cnt), one range when they touch -- then z of its own nodes: no grid-wide
// barrier between G and G^T. Partials r.z (row 2) and z.q (row 3); setup:
// p = z and r.z only.
constexpr int kLpY = 3 * kBlock + 4;  // staged rows of a block
static_assert(kGBlocks <= 7, "the staged rows cover lower offsets with dv in {0, -1, -2}, du in [-2, 1]");

__global__ void __launch_bounds__(kBlock, 6) k_lp_prec(View v, Blocks b, Solver so, LpcgExtra lx, int setup) {
  __shared__ double sh[kBlock / 32];
  __shared__ float ys_[5][kLpY];
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  if (!setup && !so.pc[c].active) return;
  const int nt = v.ntot;
  const ClothParams& P = v.cp[c];
  const int W = P.W, H = P.H, cs = P.node_off, ce = P.node_off + P.W * P.H;
  const int n0 = b.blk_node0[blk], cnt = b.blk_count[blk];
  // entry of row i in window w is i - yoff[w]
  const bool yone = W <= cnt + 1;
  const int ytotal = yone ? cnt + 2 * W : 3 * cnt + 4;
  const int yoff0 = n0, yoff1 = yone ? n0 : n0 + W - 1 - (cnt + 2), yoff2 = yone ? n0 : n0 + 2 * W - (2 * cnt + 4);
  for (int e = threadIdx.x; e < ytotal; e += kBlock) {
    const int i = e + (yone || e < cnt + 2 ? yoff0 : e < 2 * cnt + 4 ? yoff1 : yoff2);
    float y[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (i < ce) {
      const int u = (i - cs) % W, w = (i - cs) / W;
      float xs[kGBlocks][5];
#pragma unroll
      for (int bb = 0; bb < kGBlocks; ++bb) {
        const int du = gpat_du(bb), dv = gpat_dv(bb);
        const bool in = u + du >= 0 && u + du < W && w + dv >= 0;
        const int j = in ? i + du + dv * W : i;
        const float m = in ? 1.f : 0.f;
#pragma unroll
        for (int cc = 0; cc < 5; ++cc) xs[bb][cc] = m * lx.rf[(int64_t)cc * nt + j];
      }
      // coefficient k = 5 r + c of block bb comes with its pair; each y[r]
      // sums in block, then column order
#pragma unroll
      for (int bb = 0; bb < kGBlocks; ++bb)
#pragma unroll
        for (int q = 0; q < 13; ++q) {
          const float2 g2 = __bfloat1622float2(lx.G[(int64_t)(13 * bb + q) * nt + i]);
          y[(2 * q) / 5] += g2.x * xs[bb][(2 * q) % 5];
          if (2 * q + 1 < 25) y[(2 * q + 1) / 5] += g2.y * xs[bb][(2 * q + 1) % 5];
        }
    }
#pragma unroll
    for (int cc = 0; cc < 5; ++cc) ys_[cc][e] = y[cc];
  }
  __syncthreads();
  const int n = n0 + threadIdx.x;
  double rz = 0.0, zq = 0.0;
  if (threadIdx.x < cnt) {
    const int u = (n - cs) % W, w = (n - cs) / W;
    float z[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int bb = 0; bb < kGBlocks; ++bb) {
      const int du = gpat_du(bb), dv = gpat_dv(bb);
      if (u - du < 0 || u - du >= W || w - dv >= H) continue;
      const int i = n - du - dv * W;
      const int ei = i - (dv == 0 ? yoff0 : dv == -1 ? yoff1 : yoff2);
#pragma unroll
      for (int q = 0; q < 13; ++q) {
        const float2 g2 = __bfloat1622float2(lx.G[(int64_t)(13 * bb + q) * nt + i]);
        z[(2 * q) % 5] += g2.x * ys_[(2 * q) / 5][ei];
        if (2 * q + 1 < 25) z[(2 * q + 1) % 5] += g2.y * ys_[(2 * q + 1) / 5][ei];
      }
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const double zk = (double)z[k];
      lx.z[(int64_t)k * nt + n] = zk;
      rz += ld(so.r, k, nt, n) * zk;
      if (setup) st(so.p, k, nt, n) = zk;
      else zq += zk * ld(so.q, k, nt, n);
    }
  }
  const double s2 = blk_sum(rz, sh);
  if (threadIdx.x == 0) so.part[2 * b.nblk + blk] = s2;
  if (!setup) {
    const double s3 = blk_sum(zq, sh);
    if (threadIdx.x == 0) so.part[3 * b.nblk + blk] = s3;
  }
}

__global__ void k_lp_start(Blocks b, Solver so, int ncloth) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncloth) return;
  PcgCloth& pc = so.pc[c];
  const double bb = cl_sum(b, so.part, 0, c);
  const double rr = cl_sum(b, so.part, 1, c);
  const double rz = cl_sum(b, so.part, 2, c);
  pc.bb = bb;
  double thr = so.tol * so.tol * bb;
  if (thr < DBL_MIN) thr = DBL_MIN;
  pc.thr = thr;
  pc.rr = rr;
  pc.rz[0] = rz;
  pc.iters = 0;
  pc.active = (pc.status == 0 && bb != 0.0 && rr >= thr) ? 1 : 0;
}

// stop test |r|^2 < thr, else the flexible (Polak-Ribiere) direction update
// beta = z_new . (r_new - r_old) / (z_old . r_old) = -alpha z_new . q / rz,
// which stays a conjugate-gradient method when M^-1 is applied in FP32
// (it: the iteration, counted from *so.it_base in a graph body)
__global__ void __launch_bounds__(kBlock) k_lp_dir(View v, Blocks b, Solver so, LpcgExtra lx, int parity,
                                                    int it_local) {
  __shared__ int go_sh;
  __shared__ double beta_sh;
  __shared__ double sums_sh[4];
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  PcgCloth& pc = so.pc[c];
  if (!pc.active) return;
  // the four cloth sums (p.q, |r|^2, r.z, z.q), each in block order, in four
  // lanes at once; the direction's operands load meanwhile
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  const bool own = threadIdx.x < b.blk_count[blk];
  double zk[5], pk[5];
  if (own)
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      zk[k] = lx.z[(int64_t)k * nt + n];
      pk[k] = ld(so.p, k, nt, n);
    }
  if (threadIdx.x < 4) sums_sh[threadIdx.x] = cl_sum(b, so.part, threadIdx.x, c);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int it = so.it_base ? *so.it_base + it_local : it_local;
    const double rr = sums_sh[1];
    const double rzn = sums_sh[2];
    const double zq = sums_sh[3];
    const double alpha = pc.rz[parity] / sums_sh[0];
    const bool lead = blk == b.cloth_blk0[c];
    const bool conv = rr < pc.thr;
    const bool cap = !conv && it + 1 >= pc.maxiter;
    go_sh = !(conv || cap);
    beta_sh = -alpha * zq / pc.rz[parity];
    if (lead) {
      pc.rr = rr;
      pc.rz[parity ^ 1] = rzn;
      pc.iters = conv ? it : it + 1;
      if (conv || cap) pc.active = 0;
      if (cap) pc.status |= 4;
      if (!isfinite(rzn) || !isfinite(beta_sh)) {  // breakdown: bit 3
        pc.active = 0;
        pc.status |= 8;
      }
    }
  }
  __syncthreads();
  if (!go_sh || !isfinite(beta_sh)) return;
  const double beta = beta_sh;
  if (own)
#pragma unroll
    for (int k = 0; k < 5; ++k) st(so.p, k, nt, n) = zk[k] + beta * pk[k];
}

// ------------------------------------------------------------- training
// FP32 y = A x and y = A^T x of row block n (the FP64 step's spmv_row and
// spmv_row_t in single precision)
__device__ __forceinline__ void spmv_f(const View& v, const float* x, int n, float y[5]) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  float yl[3] = {0.f, 0.f, 0.f}, ye[2];
  for (int s = 0; s < kNumStencil; ++s) {
    const int uu = u + stencil_du(s), vv = w + stencil_dv(s);
    if (uu < 0 || uu >= P.W || vv < 0 || vv >= P.H) continue;
    const int j = n + stencil_du(s) + stencil_dv(s) * P.W;
    const int b = YS_SLOT_LL + 9 * s;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) yl[r] += (float)slot(v, b + 3 * r + c, n) * x[c * nt + j];
  }
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 2; ++k) yl[r] += (float)slot(v, YS_SLOT_LE_SELF + 2 * r + k, n) * x[(3 + k) * nt + n];
  for (int k = 0; k < 2; ++k) {
    ye[k] = (float)slot(v, YS_SLOT_EE_SELF + k, n) * x[(3 + k) * nt + n];
    for (int c = 0; c < 3; ++c) ye[k] += (float)slot(v, YS_SLOT_EL_SELF + 3 * k + c, n) * x[c * nt + n];
  }
  for (int m = 0; m < 4; ++m) {
    const int du = m == 0 ? -1 : m == 1 ? 1 : 0, dv = m == 2 ? -1 : m == 3 ? 1 : 0;
    const int k = m < 2 ? 0 : 1;
    const int uu = u + du, vv = w + dv;
    if (uu < 0 || uu >= P.W || vv < 0 || vv >= P.H) continue;
    const int j = n + du + dv * P.W;
    const float xe = x[(3 + k) * nt + j];
    for (int r = 0; r < 3; ++r) yl[r] += (float)slot(v, YS_SLOT_LE_NBR + 3 * m + r, n) * xe;
    ye[k] += (float)slot(v, YS_SLOT_EE_NBR + m, n) * xe;
    for (int c = 0; c < 3; ++c) ye[k] += (float)slot(v, YS_SLOT_EL_NBR + 3 * m + c, n) * x[c * nt + j];
  }
  y[0] = yl[0];
  y[1] = yl[1];
  y[2] = yl[2];
  y[3] = ye[0];
  y[4] = ye[1];
}
__device__ __forceinline__ void spmv_tf(const View& v, const float* x, int n, float y[5]) {
  const int nt = v.ntot;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  float yl[3] = {0.f, 0.f, 0.f}, ye[2] = {0.f, 0.f};
  for (int s = 0; s < kNumStencil; ++s) {
    const int du = stencil_du(s), dv = stencil_dv(s);
    const int uu = u - du, vv = w - dv;
    if (uu < 0 || uu >= P.W || vv < 0 || vv >= P.H) continue;
    const int i = n - du - dv * P.W;
    const int b = YS_SLOT_LL + 9 * s;
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) yl[c] += (float)slot(v, b + 3 * r + c, i) * x[r * nt + i];
  }
  for (int k = 0; k < 2; ++k) {
    const float xe = x[(3 + k) * nt + n];
    ye[k] += (float)slot(v, YS_SLOT_EE_SELF + k, n) * xe;
    for (int r = 0; r < 3; ++r) ye[k] += (float)slot(v, YS_SLOT_LE_SELF + 2 * r + k, n) * x[r * nt + n];
    for (int c = 0; c < 3; ++c) yl[c] += (float)slot(v, YS_SLOT_EL_SELF + 3 * k + c, n) * xe;
  }
  for (int m = 0; m < 4; ++m) {
    const int du = m == 0 ? -1 : m == 1 ? 1 : 0, dv = m == 2 ? -1 : m == 3 ? 1 : 0;
    const int k = m < 2 ? 0 : 1;
    const int uu = u - du, vv = w - dv;
    if (uu < 0 || uu >= P.W || vv < 0 || vv >= P.H) continue;
    const int i = n - du - dv * P.W;
    const float xe = x[(3 + k) * nt + i];
    for (int r = 0; r < 3; ++r) ye[k] += (float)slot(v, YS_SLOT_LE_NBR + 3 * m + r, i) * x[r * nt + i];
    ye[k] += (float)slot(v, YS_SLOT_EE_NBR + m, i) * xe;
    for (int c = 0; c < 3; ++c) yl[c] += (float)slot(v, YS_SLOT_EL_NBR + 3 * m + c, i) * xe;
  }
  y[0] = yl[0];
  y[1] = yl[1];
  y[2] = yl[2];
  y[3] = ye[0];
  y[4] = ye[1];
}

enum { kVw = 0, kVu, kVs, kVcount };
__device__ __forceinline__ float* vslot(const GnnBufs& g, int k) { return g.vec + (int64_t)k * 5 * g.ntot; }

// Rademacher probe from a counter hash (splitmix64 finaliser)
__device__ __forceinline__ float rademacher(uint64_t seed, uint64_t idx) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (idx + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (z & 1) ? 1.f : -1.f;
}

__global__ void k_tr_probe(GnnBufs g, uint64_t seed) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.ntot) return;
  float* w = vslot(g, kVw);
  for (int c = 0; c < 5; ++c) w[(int64_t)c * g.ntot + n] = rademacher(seed, (uint64_t)c * g.ntot + n);
}

// inverse and log |det| of a 5 x 5 matrix (Gauss-Jordan with partial pivoting)
__device__ __forceinline__ float inv5(const float M[5][5], float X[5][5]) {
  float a[5][10];
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 10; ++c) a[r][c] = c < 5 ? M[r][c] : (c - 5 == r ? 1.f : 0.f);
  float logdet = 0.f;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    int p = k;
    float best = fabsf(a[k][k]);
#pragma unroll
    for (int r = k + 1; r < 5; ++r)
      if (fabsf(a[r][k]) > best) {
        best = fabsf(a[r][k]);
        p = r;
      }
#pragma unroll
    for (int r = k + 1; r < 5; ++r)
      if (r == p)
#pragma unroll
        for (int c = 0; c < 10; ++c) {
          const float t = a[k][c];
          a[k][c] = a[r][c];
          a[r][c] = t;
        }
    const float piv = a[k][k];
    logdet += logf(fabsf(piv));
    const float ip = 1.f / piv;
#pragma unroll
    for (int c = 0; c < 10; ++c) a[k][c] *= ip;
#pragma unroll
    for (int r = 0; r < 5; ++r)
      if (r != k) {
        const float f = a[r][k];
#pragma unroll
        for (int c = 0; c < 10; ++c) a[r][c] -= f * a[k][c];
      }
  }
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) X[r][c] = a[r][5 + c];
  return logdet;
}

// u = G^T w
__global__ void k_tr_u(GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  float u[5];
  apply_cols(g.G, g.upat, nt, vslot(g, kVw), n, u);
  for (int c = 0; c < 5; ++c) vslot(g, kVu)[(int64_t)c * nt + n] = u[c];
}

// t = (A + A^T) u / 2, s = L^-1 t; per-block partials of u.t (= w^T G A G^T w,
// lpart row 0) and of log |det G_n,0| = log |det(I + N_n,0)| + log det L_n^-1 (row 1)
__global__ void __launch_bounds__(kNB) k_tr_t(View v, GnnBufs g) {
  __shared__ double sh[kNB / 32];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  double ut = 0.0, ld = 0.0;
  if (n < nt) {
    float t1[5], t2[5], L[5][5];
    const float* u = vslot(g, kVu);
    spmv_f(v, u, n, t1);
    spmv_tf(v, u, n, t2);
    load_linv(g.linv, nt, n, L);
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      const float t = 0.5f * (t1[r] + t2[r]);
      ut += (double)u[(int64_t)r * nt + n] * t;
      t1[r] = t;
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      float a = 0.f;
#pragma unroll
      for (int c = 0; c <= r; ++c) a += L[r][c] * t1[c];
      vslot(g, kVs)[(int64_t)r * nt + n] = a;
      ld += log((double)L[r][r]);
    }
    float N0[5][5], X[5][5];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) N0[r][c] = g.Gn[(int64_t)(5 * r + c) * nt + n] + (r == c ? 1.f : 0.f);
    ld += (double)inv5(N0, X);
  }
  const double s1 = blk_sum(ut, sh);
  if (threadIdx.x == 0) g.lpart[blockIdx.x] = s1;
  const double s2 = blk_sum(ld, sh);
  if (threadIdx.x == 0) g.lpart[g.nlblk + blockIdx.x] = s2;
}

// loss = log(tr / n) - 2 logdet / n (n = DOFs; fixed-order sums) into
// lpart[2 nlblk], its scales 2 / tr and 2 / n into the next two entries
__global__ void k_tr_loss(GnnBufs g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double tr = 0.0, ld = 0.0;
  for (int i = 0; i < g.nlblk; ++i) {
    tr += g.lpart[i];
    ld += g.lpart[g.nlblk + i];
  }
  const double nd = 5.0 * g.ntot;
  g.lpart[2 * g.nlblk] = tr > 0.0 ? log(tr / nd) - 2.0 * ld / nd : 0.0;
  g.lpart[2 * g.nlblk + 1] = tr > 0.0 ? 2.0 / tr : 0.0;
  g.lpart[2 * g.nlblk + 2] = 2.0 / nd;
}

// d loss / d N_n,b = (2 / tr) w_n s_src^T - [b = 0] (2 / n) (I + N_n,0)^-T;
// d o = 0.1 d N (BF16: the head's GEMM operand)
__global__ void k_tr_do(GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  const float c1 = (float)g.lpart[2 * g.nlblk + 1], c2 = (float)g.lpart[2 * g.nlblk + 2];
  float w[5];
  for (int r = 0; r < 5; ++r) w[r] = vslot(g, kVw)[(int64_t)r * nt + n];
  float N0[5][5], X[5][5];
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) N0[r][c] = g.Gn[(int64_t)(5 * r + c) * nt + n] + (r == c ? 1.f : 0.f);
  inv5(N0, X);
  bf16* d = g.dob + (int64_t)n * kGOut;
  for (int b = 0; b < kGBlocks; ++b) {
    const int j = g.pat[8 * n + b];
    float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (j >= 0)
      for (int c = 0; c < 5; ++c) s[c] = vslot(g, kVs)[(int64_t)c * nt + j];
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) {
        float dn = j >= 0 ? c1 * w[r] * s[c] : 0.f;
        if (b == 0) dn -= c2 * X[c][r];
        d[25 * b + 5 * r + c] = __float2bfloat16(kGOutScale * dn);
      }
  }
  for (int k = kGUsed; k < kGOut; ++k) d[k] = __float2bfloat16(0.f);
}

// ---- the FSAI objective. The factorised sparse approximate inverse of a
// pattern (Kolotilina and Yeremin) minimises the Kaporin number of G A G^T
// over the G with that pattern: per row block i, with P_i its present
// sources (i first), S = sym(A)[P_i, P_i], X = S^-1 E_i (E_i the identity at
// i's block), G*_i = chol(X_ii)^-1 X^T, so that (G* S G*^T)_ii = I. The
// objective is the mean over nodes of |N - N*|_F^2, N* = (G*_i,0 L_i - I,
// G*_i,b L_src), the network's own parametrisation of G*.
constexpr int kFsaiMax = 5 * kGBlocks;

// A(n, n + (du, dv)) in FP32: the diagonal block, a yarn neighbour's block
// with its Eulerian couplings, the x part of the other stencil offsets, zero
// outside the stencil
__device__ void a_block(const View& v, int n, int du, int dv, float B[5][5]) {
  if (du == 0 && dv == 0) {
    diag_block(v, n, B);
    return;
  }
  const int d = yarn_nbr(du, dv);
  if (d >= 0) {
    nbr_block(v, n, d, B);
    return;
  }
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) B[r][c] = 0.f;
  const int s = stencil_index(du, dv);
  if (s < 0) return;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) B[r][c] = (float)slot(v, YS_SLOT_LL + 9 * s + 3 * r + c, n);
}

// N* of node n (one thread; the 35 x 35 local system lives in local memory);
// a local system that does not factorise keeps N* = N (no gradient)
__global__ void __launch_bounds__(kNB) k_fsai_target(View v, GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  int src[kGBlocks], pos[kGBlocks];
  int m = 0;
  for (int b = 0; b < kGBlocks; ++b) {
    const int du = gpat_du(b), dv = gpat_dv(b);
    const bool in = u + du >= 0 && u + du < P.W && w + dv >= 0 && w + dv < P.H;
    src[b] = in ? n + du + dv * P.W : -1;
    pos[b] = in ? m++ : -1;
  }
  const int dm = 5 * m;
  float S[kFsaiMax][kFsaiMax];
  for (int i = 0; i < dm; ++i)
    for (int k = 0; k < dm; ++k) S[i][k] = 0.f;
  for (int b1 = 0; b1 < kGBlocks; ++b1) {
    if (src[b1] < 0) continue;
    for (int b2 = 0; b2 < kGBlocks; ++b2) {
      if (src[b2] < 0) continue;
      float B[5][5];  // A(src1, src2)
      a_block(v, src[b1], gpat_du(b2) - gpat_du(b1), gpat_dv(b2) - gpat_dv(b1), B);
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) {
          S[5 * pos[b1] + r][5 * pos[b2] + c] += 0.5f * B[r][c];
          S[5 * pos[b2] + c][5 * pos[b1] + r] += 0.5f * B[r][c];
        }
    }
  }
  bool ok = true;
  for (int k = 0; k < dm && ok; ++k) {  // S = C C^T, C in the lower triangle
    float d = S[k][k];
    for (int q = 0; q < k; ++q) d -= S[k][q] * S[k][q];
    ok = d > 0.f && isfinite(d);
    const float ck = sqrtf(fmaxf(d, FLT_MIN));
    S[k][k] = ck;
    for (int i = k + 1; i < dm; ++i) {
      float t = S[i][k];
      for (int q = 0; q < k; ++q) t -= S[i][q] * S[k][q];
      S[i][k] = t / ck;
    }
  }
  float X[kFsaiMax][5];
  for (int c = 0; c < 5; ++c) {
    for (int i = 0; i < dm; ++i) {
      float t = i == c ? 1.f : 0.f;
      for (int q = 0; q < i; ++q) t -= S[i][q] * X[q][c];
      X[i][c] = t / S[i][i];
    }
    for (int i = dm - 1; i >= 0; --i) {
      float t = X[i][c];
      for (int q = i + 1; q < dm; ++q) t -= S[q][i] * X[q][c];
      X[i][c] = t / S[i][i];
    }
  }
  // chol(X_ii) (symmetrised), then G*^T rows: Z = Lx^-1 X^T
  float Lx[5][5] = {};
  for (int k = 0; k < 5 && ok; ++k) {
    float d = 0.5f * (X[k][k] + X[k][k]);
    for (int q = 0; q < k; ++q) d -= Lx[k][q] * Lx[k][q];
    ok = d > 0.f && isfinite(d);
    Lx[k][k] = sqrtf(fmaxf(d, FLT_MIN));
    for (int i = k + 1; i < 5; ++i) {
      float t = 0.5f * (X[i][k] + X[k][i]);
      for (int q = 0; q < k; ++q) t -= Lx[i][q] * Lx[k][q];
      Lx[i][k] = t / Lx[k][k];
    }
  }
  for (int b = 0; b < kGBlocks; ++b) {
    float Nb[5][5] = {};
    if (src[b] >= 0) {
      float Gs[5][5];  // G*_n,b
      for (int c = 0; c < 5; ++c)
        for (int r = 0; r < 5; ++r) {
          float t = X[5 * pos[b] + c][r];
          for (int q = 0; q < r; ++q) t -= Lx[r][q] * Gs[q][c];
          Gs[r][c] = t / Lx[r][r];
        }
      // L_src = (L_src^-1)^-1, lower triangular
      float Li[5][5], L[5][5] = {};
      load_linv(g.linv, nt, src[b], Li);
      for (int c = 0; c < 5; ++c) {
        L[c][c] = 1.f / Li[c][c];
        for (int r = c + 1; r < 5; ++r) {
          float t = 0.f;
          for (int q = c; q < r; ++q) t += Li[r][q] * L[q][c];
          L[r][c] = -t / Li[r][r];
        }
      }
      mul_ab(Gs, L, Nb);
      if (b == 0)
        for (int r = 0; r < 5; ++r) Nb[r][r] -= 1.f;
    }
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) {
        const int64_t at = (int64_t)(25 * b + 5 * r + c) * nt + n;
        g.Nt[at] = (ok && isfinite(Nb[r][c])) ? Nb[r][c] : g.Gn[at];
      }
  }
}

// d loss / d N = (2 / nodes) (N - N*), d o = 0.1 d N (BF16); per-block
// partials of |N - N*|^2 into lpart row 0
__global__ void __launch_bounds__(kNB) k_fsai_do(GnnBufs g) {
  __shared__ double sh[kNB / 32];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  double l = 0.0;
  if (n < nt) {
    const float sc = 2.f / (float)nt;
    bf16* d = g.dob + (int64_t)n * kGOut;
    for (int k = 0; k < kGUsed; ++k) {
      const int64_t at = (int64_t)k * nt + n;
      const float e = g.Gn[at] - g.Nt[at];
      l += (double)e * e;
      d[k] = __float2bfloat16(kGOutScale * sc * e);
    }
    for (int k = kGUsed; k < kGOut; ++k) d[k] = __float2bfloat16(0.f);
  }
  const double s1 = blk_sum(l, sh);
  if (threadIdx.x == 0) g.lpart[blockIdx.x] = s1;
}

__global__ void k_fsai_loss(GnnBufs g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double l = 0.0;
  for (int i = 0; i < g.nlblk; ++i) l += g.lpart[i];
  g.lpart[2 * g.nlblk] = l / g.ntot;
}

// dz = dh * (a > 0) in BF16
__global__ void k_relu_bwd(const float* dh, const bf16* act, const float* hpos, bf16* dzb, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const bool on = act ? __bfloat162float(act[i]) > 0.f : hpos[i] > 0.f;
  dzb[i] = __float2bfloat16(on ? dh[i] : 0.f);
}
// dh_i = dm_i[0:64] (set) or dh_i + dm_i[0:64] + sum_d dm_j[64 (d + 1) ...] over
// the nodes j whose message chunk d + 1 is node i
__global__ void k_msg_bwd(const float* dm, const int* nbr, float* dh, int ntot, int accumulate_self) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntot * kGHid) return;
  const int n = i / kGHid, k = i % kGHid;
  float s = dm[(int64_t)n * kGMsg + k];
  if (accumulate_self) s += dh[i];
  for (int d = 0; d < 4; ++d) {
    const int j = nbr[4 * n + opp(d)];
    if (j >= 0) s += dm[(int64_t)j * kGMsg + 64 * (d + 1) + k];
  }
  dh[i] = s;
}
// Adam on the FP32 master parameters
__global__ void k_adam(float* w, const float* grad, float* m, float* v, int count, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gr = grad[i];
  if (!isfinite(gr)) return;
  const float mi = b1 * m[i] + (1.f - b1) * gr;
  const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}
// BF16 operand copies (and transposes) of the FP32 parameters
__global__ void k_refresh(GnnNet net) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kGHid * kGIn) net.W0[i] = __float2bfloat16(net.w[kPW0 + i]);
  if (i < kGLayers * kGHid * kGMsg) {
    const int l = i / (kGHid * kGMsg), k = i % (kGHid * kGMsg);
    const int j = k / kGMsg, c = k % kGMsg;
    const float val = net.w[kPW(l) + k];
    net.Wl[i] = __float2bfloat16(val);
    net.WlT[(int64_t)l * kGMsg * kGHid + (int64_t)c * kGHid + j] = __float2bfloat16(val);
  }
  if (i < kGOut * kGHid) {
    const int j = i / kGHid, c = i % kGHid;
    const float val = net.w[kPWh + i];
    net.Wh[i] = __float2bfloat16(val);
    net.WhT[(int64_t)c * kGOut + j] = __float2bfloat16(val);
  }
}

}  // namespace

// ------------------------------------------------------------------ launchers
void gnn_neighbours(const View& v, const GnnBufs& g, cudaStream_t s) { k_gnn_nbr<<<nblk(v.ntot), kNB, 0, s>>>(v, g); }

void gnn_prepare(const View& v, const GnnBufs& g, cudaStream_t s) {
  k_gnn_linv<<<nblk(v.ntot), kNB, 0, s>>>(v, g.linv, g.chol_ok);
  k_gnn_feat<<<(v.ntot + kFeatNodes - 1) / kFeatNodes, 12 * kFeatNodes, 0, s>>>(v, g);
}

void gnn_forward(const GnnNet& net, const GnnBufs& g, bool training, cudaStream_t s) {
  const int M = g.ntot;
  const int64_t hs = (int64_t)M * kGHid;
  {
    FwdOp<64, kEpiEnc> op{g.f, kGIn, M, nullptr, 0, net.W0, kGIn, net.w + kPb0, nullptr, g.h, g.hb, nullptr, nullptr};
    launch_gemm<decltype(op), kGIn / 64>(op, M, 1, kGIn / 64, 1, g.err, s);
  }
  for (int l = 0; l < kGLayers; ++l) {
    // the last layer's FP32 output is read by nothing (the head reads its BF16
    // copy); the ReLU outputs only by the training's backward pass
    FwdOp<64, kEpiLayer> op{g.hb + l * hs, kGHid, M, g.nbr, 1, net.Wl + (int64_t)l * kGHid * kGMsg, kGMsg,
                            net.w + kPb(l), g.h + l * hs, l + 1 < kGLayers ? g.h + (l + 1) * hs : nullptr,
                            g.hb + (l + 1) * hs, training ? g.act + l * hs : nullptr, nullptr};
    launch_gemm<decltype(op), 2>(op, M, 1, kGMsg / 64, 1, g.err, s);
  }
  {
    FwdOp<64, kEpiHead> op{g.hb + 3 * hs, kGHid, M, nullptr, 0, net.Wh, kGHid, net.w + kPbh, nullptr, nullptr,
                           nullptr, nullptr, g.o};
    launch_gemm(op, M, kGOut / 64, 1, 1, g.err, s);
  }
}

void gnn_forward_attrs() {
  gemm_attr<FwdOp<64, kEpiEnc>, kGIn / 64>();
  gemm_attr<FwdOp<64, kEpiLayer>, 2>();
  gemm_attr<FwdOp<64, kEpiHead>, 1>();
}

void gnn_make_g(const GnnBufs& g, bool keep_n, cudaStream_t s) {
  k_gnn_g<<<(int)(((int64_t)kGBlocks * g.ntot + kNB - 1) / kNB), kNB, 0, s>>>(g, keep_n ? 1 : 0);
}

void gnn_refresh_bf16(const GnnNet& net, cudaStream_t s) {
  k_refresh<<<(kGLayers * kGHid * kGMsg + 255) / 256, 256, 0, s>>>(net);
}

void gnn_loss_grad(const View& v, const GnnNet& net, const GnnBufs& g, uint64_t seed, bool probes_given,
                   int objective, cudaStream_t s) {
  const int M = g.ntot;
  const int64_t hs = (int64_t)M * kGHid;
  if (objective == 1) {
    k_fsai_target<<<nblk(M), kNB, 0, s>>>(v, g);
    k_fsai_do<<<g.nlblk, kNB, 0, s>>>(g);
    k_fsai_loss<<<1, 32, 0, s>>>(g);
  } else {
    if (!probes_given) k_tr_probe<<<nblk(M), kNB, 0, s>>>(g, seed);
    k_tr_u<<<nblk(M), kNB, 0, s>>>(g);
    k_tr_t<<<g.nlblk, kNB, 0, s>>>(v, g);
    k_tr_loss<<<1, 32, 0, s>>>(g);
    k_tr_do<<<nblk(M), kNB, 0, s>>>(g);
  }
  const int nchunk = (M + 63) / 64;
  const int per = (nchunk + g.nsplit - 1) / g.nsplit;
  const int splits = (nchunk + per - 1) / per;
  // head
  {
    WgradOp<64> op{g.hb + 3 * hs, kGHid, kGHid, M, nullptr, 0, g.dob, kGOut, g.wpart};
    launch_gemm(op, kGHid + 1, kGOut / 64, nchunk, g.nsplit, g.err, s);
    k_wgrad_reduce<<<((kGHid + 1) * kGOut + 255) / 256, 256, 0, s>>>(g.wpart, splits, kGHid, kGOut, g.grad + kPWh,
                                                                      g.grad + kPbh);
    BwdDataOp dop{g.dob, kGOut, M, net.WhT, g.dh, kGHid};
    launch_gemm(dop, M, kGHid / 64, kGOut / 64, 1, g.err, s);
  }
  for (int l = kGLayers - 1; l >= 0; --l) {
    k_relu_bwd<<<(int)((hs + 255) / 256), 256, 0, s>>>(g.dh, g.act + l * hs, nullptr, g.dzb, (int)hs);
    WgradOp<64> op{g.hb + l * hs, kGHid, kGMsg, M, g.nbr, 1, g.dzb, kGHid, g.wpart};
    launch_gemm(op, kGMsg + 1, 1, nchunk, g.nsplit, g.err, s);
    k_wgrad_reduce<<<((kGMsg + 1) * kGHid + 255) / 256, 256, 0, s>>>(g.wpart, splits, kGMsg, kGHid, g.grad + kPW(l),
                                                                      g.grad + kPb(l));
    BwdDataOp dop{g.dzb, kGHid, M, net.WlT + (int64_t)l * kGMsg * kGHid, g.dm, kGMsg};
    launch_gemm(dop, M, kGMsg / 64, 1, 1, g.err, s);
    k_msg_bwd<<<(int)((hs + 255) / 256), 256, 0, s>>>(g.dm, g.nbr, g.dh, M, 1);
  }
  k_relu_bwd<<<(int)((hs + 255) / 256), 256, 0, s>>>(g.dh, nullptr, g.h, g.dzb, (int)hs);
  WgradOp<64> op{g.f, kGIn, kGIn, M, nullptr, 0, g.dzb, kGHid, g.wpart};
  launch_gemm(op, kGIn + 1, 1, nchunk, g.nsplit, g.err, s);
  k_wgrad_reduce<<<((kGIn + 1) * kGHid + 255) / 256, 256, 0, s>>>(g.wpart, splits, kGIn, kGHid, g.grad + kPW0,
                                                                   g.grad + kPb0);
}

void gnn_adam(const GnnNet& net, const GnnBufs& g, float* m, float* vv, float lr, int step, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<(kGParams + 255) / 256, 256, 0, s>>>(net.w, g.grad, m, vv, kGParams, lr, b1, b2, 1e-8f, c1, c2);
  gnn_refresh_bf16(net, s);
}

void lpcg_setup(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s) {
  k_lp_axpy<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, 0, 1);
  k_lp_prec<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, 1);
  k_lp_start<<<(v.ncloth + 127) / 128, 128, 0, s>>>(b, so, v.ncloth);
}

void lpcg_axpy(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, int parity, cudaStream_t s) {
  k_lp_axpy<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, parity, 0);
}

void lpcg_precondition(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s) {
  k_lp_prec<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, 0);
}

void lpcg_dir(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, int parity, int it,
              cudaStream_t s) {
  k_lp_dir<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, parity, it);
}

void tc_gemm_bf16(const bf16* A, const bf16* B, float* C, int M, int N, int K, int* err, cudaStream_t s) {
  if (N == 128) {
    PlainOp<128> op{A, B, C, M, N, K};
    launch_gemm(op, M, 1, K / 64, 1, err, s);
  } else {
    PlainOp<64> op{A, B, C, M, N, K};
    launch_gemm(op, M, N / 64, K / 64, 1, err, s);
  }
}

}  // namespace ys
