// ys_gnn.cu -- kernels of the learned preconditioner: system features, the
// graph network's BF16 tcgen05 GEMMs (forward, data and weight gradients),
// the blocks of G, the stochastic Frobenius loss with its hand-written
// gradient, Adam, and the preconditioned conjugate-gradient iteration that
// applies M^-1 = G^T G.
#include <cfloat>

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
__global__ void k_gnn_nbr(View v, int* nbr) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  nbr[4 * n + 0] = u > 0 ? n - 1 : -1;
  nbr[4 * n + 1] = u < P.W - 1 ? n + 1 : -1;
  nbr[4 * n + 2] = w > 0 ? n - P.W : -1;
  nbr[4 * n + 3] = w < P.H - 1 ? n + P.W : -1;
}

// ------------------------------------------------- block factor and features
// 5 x 5 diagonal block of row block n (DOF order x, y, z, u, v)
__device__ void diag_block(const View& v, int n, double D[5][5]) {
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) D[r][c] = 0.0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) D[r][c] = slot(v, YS_SLOT_LL + 3 * r + c, n);
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 2; ++k) {
      D[r][3 + k] = slot(v, YS_SLOT_LE_SELF + 2 * r + k, n);
      D[3 + k][r] = slot(v, YS_SLOT_EL_SELF + 3 * k + r, n);
    }
  D[3][3] = slot(v, YS_SLOT_EE_SELF + 0, n);
  D[4][4] = slot(v, YS_SLOT_EE_SELF + 1, n);
}

// 5 x 5 block A(n, j) of yarn neighbour d (j = n + offset(d))
__device__ void nbr_block(const View& v, int n, int d, float B[5][5]) {
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) B[r][c] = 0.f;
  const int s = d + 1;  // stencil slots 1..4 are (-1,0), (1,0), (0,-1), (0,1)
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) B[r][c] = (float)slot(v, YS_SLOT_LL + 9 * s + 3 * r + c, n);
  const int k = d < 2 ? 0 : 1;
  for (int r = 0; r < 3; ++r) {
    B[r][3 + k] = (float)slot(v, YS_SLOT_LE_NBR + 3 * d + r, n);
    B[3 + k][r] = (float)slot(v, YS_SLOT_EL_NBR + 3 * d + r, n);
  }
  B[3 + k][3 + k] = (float)slot(v, YS_SLOT_EE_NBR + d, n);
}

__device__ void load_linv(const float* linv, int nt, int n, float L[5][5]) {
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) L[r][c] = c <= r ? linv[(int64_t)lt(r, c) * nt + n] : 0.f;
}

// L^-1 of the Cholesky factor of the symmetric part of the diagonal block;
// a block that does not factorise falls back to the scalar Jacobi scaling
__global__ void k_gnn_linv(View v, float* linv, int* chol_ok) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  double D[5][5], L[5][5] = {};
  diag_block(v, n, D);
  bool ok = true;
  for (int j = 0; j < 5 && ok; ++j) {
    double s = 0.5 * (D[j][j] + D[j][j]);
    for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
    if (!(s > 0.0) || !isfinite(s)) {
      ok = false;
      break;
    }
    L[j][j] = sqrt(s);
    for (int i = j + 1; i < 5; ++i) {
      double t = 0.5 * (D[i][j] + D[j][i]);
      for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
      L[i][j] = t / L[j][j];
    }
  }
  if (!ok) {
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) L[r][c] = 0.0;
    for (int j = 0; j < 5; ++j) {
      const double d = fabs(D[j][j]);
      L[j][j] = (d > 0.0 && isfinite(d)) ? sqrt(d) : 1.0;
    }
  }
  double X[5][5] = {};
  for (int c = 0; c < 5; ++c) {
    X[c][c] = 1.0 / L[c][c];
    for (int r = c + 1; r < 5; ++r) {
      double t = 0.0;
      for (int k = c; k < r; ++k) t += L[r][k] * X[k][c];
      X[r][c] = -t / L[r][r];
    }
  }
  const int nt = v.ntot;
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c <= r; ++c) linv[(int64_t)lt(r, c) * nt + n] = (float)X[r][c];
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

__global__ void k_gnn_feat(View v, GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const int nt = v.ntot;
  float Li[5][5], Lj[5][5], Bk[5][5], T[5][5], E[5][5];
  load_linv(g.linv, nt, n, Li);
  bf16* f = g.f + (int64_t)n * kGIn;
  float* Eo = g.E + (int64_t)n * 100;
  for (int d = 0; d < 4; ++d) {
    const int j = g.nbr[4 * n + d];
    if (j >= 0) {
      nbr_block(v, n, d, Bk);
      load_linv(g.linv, nt, j, Lj);
      mul_ab(Li, Bk, T);
      mul_abt(T, Lj, E);
    } else {
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) E[r][c] = 0.f;
    }
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) {
        Eo[25 * d + 5 * r + c] = E[r][c];
        f[25 * d + 5 * r + c] = __float2bfloat16(E[r][c]);
      }
  }
  // norms of the 8 other node-node couplings, scaled the same way (x part)
  const ClothParams& P = v.cp[v.node_cloth[n]];
  const int u = v.node_u[n], w = v.node_v[n];
  for (int s = 5; s < kNumStencil; ++s) {
    const int uu = u + stencil_du(s), vv = w + stencil_dv(s);
    float nrm = 0.f;
    if (uu >= 0 && uu < P.W && vv >= 0 && vv < P.H) {
      const int j = n + stencil_du(s) + stencil_dv(s) * P.W;
      load_linv(g.linv, nt, j, Lj);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          float t = 0.f;
          for (int a = 0; a <= r; ++a)
            for (int b = 0; b <= c; ++b) t += Li[r][a] * (float)slot(v, YS_SLOT_LL + 9 * s + 3 * a + b, n) * Lj[c][b];
          nrm += t * t;
        }
    }
    f[100 + s - 5] = __float2bfloat16(sqrtf(nrm));
  }
  const uint8_t fl = v.flags[n];
  f[108] = __float2bfloat16(g.chol_ok[n] ? 0.f : 1.f);
  f[109] = __float2bfloat16((fl & YS_INTERIOR) ? 1.f : 0.f);
  f[110] = __float2bfloat16((fl & YS_FIXED) ? 1.f : 0.f);
  f[111] = __float2bfloat16((u == 0 || u == P.W - 1) ? 1.f : 0.f);
  f[112] = __float2bfloat16((w == 0 || w == P.H - 1) ? 1.f : 0.f);
  for (int k = 113; k < kGIn; ++k) f[k] = __float2bfloat16(0.f);
}

// ------------------------------------------------------------ tensor-core GEMM
// C[m][n] = sum_k A(m, k) B(n, k) over 128-row tiles (blockIdx.x), NT-column
// tiles (blockIdx.y) and K splits (blockIdx.z); the Op stages A and B chunks
// of 64 K into shared memory and consumes the FP32 accumulator rows.
constexpr int kGemmThreads = 128;
constexpr int kGemmSmem = 56 * 1024;  // keeps at most 4 CTAs (4 x 128 TMEM columns) per SM
constexpr uint32_t kWaitLimit = 1u << 22;

template <class Op>
__global__ void __launch_bounds__(kGemmThreads) k_tc_gemm(Op op, int nchunk_total, int chunks_per_split, int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;
  uint8_t* sB = smem + 16384;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 16384 + Op::NT * 128);
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
  for (int kc = kc0; kc < kc1; ++kc) {
    op.stage_a(sA, m0, kc);
    op.stage_b(sB, n0, kc);
    tc::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
#pragma unroll
      for (int k = 0; k < tc::kChunkK / 16; ++k)
        tc::mma_bf16(tmem, tc::smem_desc(a0 + k * 256), tc::smem_desc(b0 + k * 256), idesc,
                     (kc > kc0 || k > 0) ? 1u : 0u);
      tc::mma_commit(bar);
    }
    bool done = tc::mbar_wait(bar, phase, kWaitLimit);
    ok = __syncthreads_and(done) != 0;
    if (!ok) break;
    phase ^= 1;
    tc::fence_after_sync();
  }
  if (ok && kc1 > kc0) {
    const int row = warp * 32 + (threadIdx.x & 31);
#pragma unroll 1
    for (int c = 0; c < Op::NT; c += 16) {
      float acc[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, acc);
      op.epilogue(m0 + row, n0 + c, acc);
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

__device__ __forceinline__ void store16(uint8_t* tile, int r, int k8, uint4 val) {
  *reinterpret_cast<uint4*>(tile + tc::core_off(r, k8)) = val;
}
__device__ __forceinline__ void store1(uint8_t* tile, int r, int k, bf16 val) {
  *reinterpret_cast<bf16*>(tile + tc::core_off(r, k)) = val;
}

// rows of X (ld elements, 64-wide chunk kc, or the neighbour given by the chunk
// when gathering), one thread per row
__device__ __forceinline__ void stage_rows(uint8_t* sA, const bf16* X, int ld, int M, const int* nbr, bool gather,
                                           int m0, int kc) {
  const int r = threadIdx.x;
  const int node = m0 + r;
  int src = -1;
  if (node < M) src = gather ? (kc == 0 ? node : nbr[4 * node + kc - 1]) : node;
  const uint4* p = src >= 0 ? reinterpret_cast<const uint4*>(X + (int64_t)src * ld + (gather ? 0 : kc * 64)) : nullptr;
#pragma unroll
  for (int q = 0; q < 8; ++q) store16(sA, r, q * 8, p ? p[q] : make_uint4(0, 0, 0, 0));
}
// NT rows of a row-major [rows][K] weight matrix
template <int NT>
__device__ __forceinline__ void stage_weights(uint8_t* sB, const bf16* W, int K, int n0, int kc) {
  for (int i = threadIdx.x; i < NT * 8; i += kGemmThreads) {
    const int n = i >> 3, q = i & 7;
    store16(sB, n, q * 8, *reinterpret_cast<const uint4*>(W + (int64_t)(n0 + n) * K + kc * 64 + q * 8));
  }
}

// forward: out = epilogue(X W^T + b)
enum { kEpiEnc = 0, kEpiLayer = 1, kEpiHead = 2 };
template <int NT_, int EPI>
struct FwdOp {
  static constexpr int NT = NT_;
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
  __device__ void epilogue(int node, int c0, const float* acc) const {
    if (node >= M) return;
    for (int i = 0; i < 16; ++i) {
      const int j = c0 + i;
      const float z = acc[i] + bias[j];
      if (EPI == kEpiHead) {
        o_out[(int64_t)node * kGOut + j] = z;
      } else {
        const float a = fmaxf(z, 0.f);
        const int64_t at = (int64_t)node * kGHid + j;
        float hn = a;
        if (EPI == kEpiLayer) {
          act_out[at] = __float2bfloat16(a);
          hn = h_in[at] + a;
        }
        h_out[at] = hn;
        hb_out[at] = __float2bfloat16(hn);
      }
    }
  }
};

// data gradient: dX = dZ W, with B = W^T stored [K_in][Nout]
struct BwdDataOp {
  static constexpr int NT = 64;
  const bf16* dZ;
  int nout, M;
  const bf16* WT;
  float* out;
  int kin;
  __device__ void stage_a(uint8_t* s, int m0, int kc) const { stage_rows(s, dZ, nout, M, nullptr, false, m0, kc); }
  __device__ void stage_b(uint8_t* s, int n0, int kc) const { stage_weights<NT>(s, WT, nout, n0, kc); }
  __device__ void epilogue(int node, int c0, const float* acc) const {
    if (node >= M) return;
    for (int i = 0; i < 16; ++i) out[(int64_t)node * kin + c0 + i] = acc[i];
  }
};

// weight gradient: C[k'][j] = sum_node X(node, k') dZ[node][j], k' < kin;
// row kin is a column of ones (the bias gradient). One 64-node chunk per
// K round; partial sums per split.
template <int NT_>
struct WgradOp {
  static constexpr int NT = NT_;
  const bf16* X;
  int ld, kin, nodes;
  const int* nbr;
  int gather;
  const bf16* dZ;
  float* part;  // [split][kWgradRows][NT]
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
  __device__ void stage_b(uint8_t* s, int, int kc) const {
    for (int i = threadIdx.x; i < NT * 64; i += kGemmThreads) {
      const int n = i % NT, kk = i / NT;
      const int node = kc * 64 + kk;
      store1(s, n, kk, node < nodes ? dZ[(int64_t)node * NT + n] : __float2bfloat16(0.f));
    }
  }
  __device__ void epilogue(int row, int c0, const float* acc) const {
    if (row > kin) return;
    float* p = part + ((int64_t)blockIdx.z * kWgradRows + row) * NT + c0;
    for (int i = 0; i < 16; ++i) p[i] = acc[i];
  }
};

// C = A B^T for row-major BF16 A [M][K] and B [N][K] (the GEMM self-test)
template <int NT_>
struct PlainOp {
  static constexpr int NT = NT_;
  const bf16* A;
  const bf16* B;
  float* C;
  int M, N, K;
  __device__ void stage_a(uint8_t* s, int m0, int kc) const {
    const int r = threadIdx.x, m = m0 + r;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      store16(s, r, q * 8,
              m < M ? *reinterpret_cast<const uint4*>(A + (int64_t)m * K + kc * 64 + q * 8) : make_uint4(0, 0, 0, 0));
  }
  __device__ void stage_b(uint8_t* s, int n0, int kc) const { stage_weights<NT>(s, B, K, n0, kc); }
  __device__ void epilogue(int m, int c0, const float* acc) const {
    if (m >= M) return;
    for (int i = 0; i < 16; ++i) C[(int64_t)m * N + c0 + i] = acc[i];
  }
};

template <class Op>
void launch_gemm(const Op& op, int M, int ncol_tiles, int nchunk, int nsplit, int* err, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_tc_gemm<Op>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    attr = true;
  }
  const int per = (nchunk + nsplit - 1) / nsplit;
  const int splits = (nchunk + per - 1) / per;
  dim3 grid((M + tc::kTileM - 1) / tc::kTileM, ncol_tiles, splits);
  k_tc_gemm<Op><<<grid, kGemmThreads, kGemmSmem, s>>>(op, nchunk, per, err);
}

// sums the splits in a fixed order into the gradient: weights [nout][kin]
// and the bias row
template <int NT>
__global__ void k_wgrad_reduce(const float* part, int splits, int kin, float* gW, float* gb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // (row, j)
  if (i >= (kin + 1) * NT) return;
  const int row = i / NT, j = i % NT;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[((int64_t)z * kWgradRows + row) * NT + j];
  if (row < kin) gW[(int64_t)j * kin + row] = s;
  else gb[j] = s;
}

// ------------------------------------------------------------------ G blocks
__global__ void k_gnn_g(GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  const float* o = g.o + (int64_t)n * kGOut;
  const float* E = g.E + (int64_t)n * 100;
  float L[5][5], N[5][5], Gb[5][5];
  for (int b = 0; b < 5; ++b) {
    const int j = b == 0 ? n : g.nbr[4 * n + b - 1];
    if (j < 0) {
      for (int k = 0; k < 25; ++k) {
        g.G[(int64_t)(25 * b + k) * nt + n] = 0.f;
        g.Gn[(int64_t)(25 * b + k) * nt + n] = 0.f;
      }
      continue;
    }
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) {
        const int k = 5 * r + c;
        float val = kGOutScale * o[25 * b + k];
        if (b > 0) val -= 0.5f * E[25 * (b - 1) + k];
        N[r][c] = val;
        g.Gn[(int64_t)(25 * b + k) * nt + n] = val;
      }
    if (b == 0)
      for (int r = 0; r < 5; ++r) N[r][r] += 1.f;
    load_linv(g.linv, nt, j, L);
    mul_ab(N, L, Gb);
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c) g.G[(int64_t)(25 * b + 5 * r + c) * nt + n] = Gb[r][c];
  }
}

// ------------------------------------------------- blocked applications
// y_i = sum_b B_ib x_src(b)  (B = blocks [125][nt] of G or of N (+ I on the
// self block when add_identity)); x in [5][nt]
template <class TX>
__device__ __forceinline__ void apply_rows(const float* Bk, const int* nbr, int nt, const TX* x, int n,
                                           bool add_identity, float y[5]) {
  for (int r = 0; r < 5; ++r) y[r] = add_identity ? (float)x[(int64_t)r * nt + n] : 0.f;
  for (int b = 0; b < 5; ++b) {
    const int j = b == 0 ? n : nbr[4 * n + b - 1];
    if (j < 0) continue;
    float xj[5];
    for (int c = 0; c < 5; ++c) xj[c] = (float)x[(int64_t)c * nt + j];
    for (int r = 0; r < 5; ++r) {
      float s = 0.f;
      for (int c = 0; c < 5; ++c) s += Bk[(int64_t)(25 * b + 5 * r + c) * nt + n] * xj[c];
      y[r] += s;
    }
  }
}
// z_j = sum over the blocks B_ib with src(b) = j of B_ib^T x_i
template <class TX>
__device__ __forceinline__ void apply_cols(const float* Bk, const int* nbr, int nt, const TX* x, int n,
                                           bool add_identity, float z[5]) {
  for (int c = 0; c < 5; ++c) z[c] = add_identity ? (float)x[(int64_t)c * nt + n] : 0.f;
  for (int b = 0; b < 5; ++b) {
    const int i = b == 0 ? n : nbr[4 * n + opp(b - 1)];  // row i refers to n through block b
    if (i < 0) continue;
    float xi[5];
    for (int r = 0; r < 5; ++r) xi[r] = (float)x[(int64_t)r * nt + i];
    for (int c = 0; c < 5; ++c) {
      float s = 0.f;
      for (int r = 0; r < 5; ++r) s += Bk[(int64_t)(25 * b + 5 * r + c) * nt + i] * xi[r];
      z[c] += s;
    }
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

// x = 0, r = b; partials |b|^2 (row 0) and |r|^2 (row 1)
__global__ void __launch_bounds__(kBlock) k_lp_setup(View v, Blocks b, Solver so) {
  __shared__ double sh[kBlock / 32];
  const int blk = blockIdx.x;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  double rr = 0.0;
  if (threadIdx.x < b.blk_count[blk])
    for (int k = 0; k < 5; ++k) {
      const double r = ld(v.B, k, nt, n);
      st(so.x, k, nt, n) = 0.0;
      st(so.r, k, nt, n) = r;
      rr += r * r;
    }
  const double s = blk_sum(rr, sh);
  if (threadIdx.x == 0) {
    so.part[0 * b.nblk + blk] = s;
    so.part[1 * b.nblk + blk] = s;
  }
}

// y = G r for the nodes of active cloths
__global__ void __launch_bounds__(kBlock) k_lp_g(View v, Blocks b, Solver so, LpcgExtra lx, int setup) {
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  if (!setup && !so.pc[c].active) return;
  if (threadIdx.x >= b.blk_count[blk]) return;
  const int n = b.blk_node0[blk] + threadIdx.x;
  float y[5];
  apply_rows(lx.G, lx.nbr, v.ntot, so.r, n, false, y);
  for (int k = 0; k < 5; ++k) lx.y[(int64_t)k * v.ntot + n] = y[k];
}

// z = G^T y; partials r.z (row 2) and z.q (row 3); at setup also p = z
__global__ void __launch_bounds__(kBlock) k_lp_gt(View v, Blocks b, Solver so, LpcgExtra lx, int setup) {
  __shared__ double sh[kBlock / 32];
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  if (!setup && !so.pc[c].active) return;
  const int nt = v.ntot;
  const int n = b.blk_node0[blk] + threadIdx.x;
  double rz = 0.0, zq = 0.0;
  if (threadIdx.x < b.blk_count[blk]) {
    float z[5];
    apply_cols(lx.G, lx.nbr, nt, lx.y, n, false, z);
    for (int k = 0; k < 5; ++k) {
      const double zk = (double)z[k];
      lx.z[(int64_t)k * nt + n] = zk;
      rz += ld(so.r, k, nt, n) * zk;
      if (setup) st(so.p, k, nt, n) = zk;
      else zq += zk * ld(so.q, k, nt, n);
    }
  }
  const double s1 = blk_sum(rz, sh);
  if (threadIdx.x == 0) so.part[2 * b.nblk + blk] = s1;
  const double s2 = blk_sum(zq, sh);
  if (threadIdx.x == 0) so.part[3 * b.nblk + blk] = s2;
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

// alpha = r.z / p.q; x += alpha p; r -= alpha q; partial |r|^2 (row 1)
__global__ void __launch_bounds__(kBlock) k_lp_axpy(View v, Blocks b, Solver so, int parity) {
  __shared__ double sh[kBlock / 32];
  __shared__ double alpha_sh;
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  if (!so.pc[c].active) return;
  if (threadIdx.x == 0) alpha_sh = so.pc[c].rz[parity] / cl_sum(b, so.part, 0, c);
  __syncthreads();
  const double alpha = alpha_sh;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  double rr = 0.0;
  if (threadIdx.x < b.blk_count[blk])
    for (int k = 0; k < 5; ++k) {
      st(so.x, k, nt, n) += alpha * ld(so.p, k, nt, n);
      const double r = ld(so.r, k, nt, n) - alpha * ld(so.q, k, nt, n);
      st(so.r, k, nt, n) = r;
      rr += r * r;
    }
  const double s = blk_sum(rr, sh);
  if (threadIdx.x == 0) so.part[1 * b.nblk + blk] = s;
}

// stop test |r|^2 < thr, else the flexible (Polak-Ribiere) direction update
// beta = z_new . (r_new - r_old) / (z_old . r_old) = -alpha z_new . q / rz,
// which stays a conjugate-gradient method when M^-1 is applied in FP32
__global__ void __launch_bounds__(kBlock) k_lp_dir(View v, Blocks b, Solver so, LpcgExtra lx, int parity, int it) {
  __shared__ int go_sh;
  __shared__ double beta_sh;
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  PcgCloth& pc = so.pc[c];
  if (!pc.active) return;
  if (threadIdx.x == 0) {
    const double rr = cl_sum(b, so.part, 1, c);
    const double rzn = cl_sum(b, so.part, 2, c);
    const double zq = cl_sum(b, so.part, 3, c);
    const double alpha = pc.rz[parity] / cl_sum(b, so.part, 0, c);
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
      if (!isfinite(rzn) || !isfinite(beta_sh)) {
        pc.active = 0;
        pc.status |= 4;
      }
    }
  }
  __syncthreads();
  if (!go_sh || !isfinite(beta_sh)) return;
  const double beta = beta_sh;
  const int n = b.blk_node0[blk] + threadIdx.x;
  const int nt = v.ntot;
  if (threadIdx.x < b.blk_count[blk])
    for (int k = 0; k < 5; ++k)
      st(so.p, k, nt, n) = lx.z[(int64_t)k * nt + n] + beta * ld(so.p, k, nt, n);
}

// ------------------------------------------------------------- training
// FP32 y = A x and y = A^T x of row block n (the FP64 step's spmv_row and
// spmv_row_t in single precision)
__device__ void spmv_f(const View& v, const float* x, int n, float y[5]) {
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
__device__ void spmv_tf(const View& v, const float* x, int n, float y[5]) {
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

enum { kVw = 0, kVv, kVu, kVt, kVs, kVe, kVgs, kVgt, kVgu, kVgv, kVcount };
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

// v = (I + N)^T w, u = L^-T v; per-block partial of |w|^2 (lpart row 1)
__global__ void __launch_bounds__(kNB) k_tr_vu(GnnBufs g) {
  __shared__ double sh[kNB / 32];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  double ww = 0.0;
  if (n < nt) {
    float vv[5], L[5][5];
    apply_cols(g.Gn, g.nbr, nt, vslot(g, kVw), n, true, vv);
    load_linv(g.linv, nt, n, L);
    float* u = vslot(g, kVu);
    for (int c = 0; c < 5; ++c) {
      float s = 0.f;
      for (int r = c; r < 5; ++r) s += L[r][c] * vv[r];
      u[(int64_t)c * nt + n] = s;
      const float w = vslot(g, kVw)[(int64_t)c * nt + n];
      ww += (double)w * w;
    }
  }
  const double s = blk_sum(ww, sh);
  if (threadIdx.x == 0) g.lpart[g.nlblk + blockIdx.x] = s;
}

// s = L^-1 (A u)
__global__ void k_tr_ts(View v, GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  float t[5], L[5][5];
  spmv_f(v, vslot(g, kVu), n, t);
  load_linv(g.linv, nt, n, L);
  float* s = vslot(g, kVs);
  for (int r = 0; r < 5; ++r) {
    float a = 0.f;
    for (int c = 0; c <= r; ++c) a += L[r][c] * t[c];
    s[(int64_t)r * nt + n] = a;
  }
}

// e = (I + N) s - w; per-block partial of |e|^2 (lpart row 0)
__global__ void __launch_bounds__(kNB) k_tr_e(GnnBufs g) {
  __shared__ double sh[kNB / 32];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  double ee = 0.0;
  if (n < nt) {
    float y[5];
    apply_rows(g.Gn, g.nbr, nt, vslot(g, kVs), n, true, y);
    for (int r = 0; r < 5; ++r) {
      const float e = y[r] - vslot(g, kVw)[(int64_t)r * nt + n];
      vslot(g, kVe)[(int64_t)r * nt + n] = e;
      ee += (double)e * e;
    }
  }
  const double s = blk_sum(ee, sh);
  if (threadIdx.x == 0) g.lpart[blockIdx.x] = s;
}

// loss = |e|^2 / |w|^2 (fixed-order sums) into lpart[2 nlblk], its scale
// 2 / |w|^2 into lpart[2 nlblk + 1]
__global__ void k_tr_loss(GnnBufs g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double ee = 0.0, ww = 0.0;
  for (int i = 0; i < g.nlblk; ++i) {
    ee += g.lpart[i];
    ww += g.lpart[g.nlblk + i];
  }
  g.lpart[2 * g.nlblk] = ww > 0.0 ? ee / ww : 0.0;
  g.lpart[2 * g.nlblk + 1] = ww > 0.0 ? 2.0 / ww : 0.0;
}

// ge = (2 / |w|^2) e (in place); gs = (I + N)^T ge; gt = L^-T gs
__global__ void k_tr_ge(GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  const float sc = (float)g.lpart[2 * g.nlblk + 1];
  for (int r = 0; r < 5; ++r) vslot(g, kVgs)[(int64_t)r * nt + n] = sc * vslot(g, kVe)[(int64_t)r * nt + n];
}
__global__ void k_tr_gt(GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  float gs[5], L[5][5];
  apply_cols(g.Gn, g.nbr, nt, vslot(g, kVgs), n, true, gs);
  load_linv(g.linv, nt, n, L);
  for (int c = 0; c < 5; ++c) {
    float s = 0.f;
    for (int r = c; r < 5; ++r) s += L[r][c] * gs[r];
    vslot(g, kVgt)[(int64_t)c * nt + n] = s;
  }
}
// gv = L^-1 (A^T gt)
__global__ void k_tr_gv(View v, GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  float gu[5], L[5][5];
  spmv_tf(v, vslot(g, kVgt), n, gu);
  load_linv(g.linv, nt, n, L);
  for (int r = 0; r < 5; ++r) {
    float a = 0.f;
    for (int c = 0; c <= r; ++c) a += L[r][c] * gu[c];
    vslot(g, kVgv)[(int64_t)r * nt + n] = a;
  }
}
// dN_ib = ge_i s_src(b)^T + w_i gv_src(b)^T  ->  d o = 0.1 dN (BF16, GEMM operand)
__global__ void k_tr_do(GnnBufs g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = g.ntot;
  if (n >= nt) return;
  float ge[5], w[5];
  for (int r = 0; r < 5; ++r) {
    ge[r] = vslot(g, kVgs)[(int64_t)r * nt + n];
    w[r] = vslot(g, kVw)[(int64_t)r * nt + n];
  }
  bf16* d = g.dob + (int64_t)n * kGOut;
  for (int b = 0; b < 5; ++b) {
    const int j = b == 0 ? n : g.nbr[4 * n + b - 1];
    float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, gv[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (j >= 0)
      for (int c = 0; c < 5; ++c) {
        s[c] = vslot(g, kVs)[(int64_t)c * nt + j];
        gv[c] = vslot(g, kVgv)[(int64_t)c * nt + j];
      }
    for (int r = 0; r < 5; ++r)
      for (int c = 0; c < 5; ++c)
        d[25 * b + 5 * r + c] = __float2bfloat16(j >= 0 ? kGOutScale * (ge[r] * s[c] + w[r] * gv[c]) : 0.f);
  }
  for (int k = kGUsed; k < kGOut; ++k) d[k] = __float2bfloat16(0.f);
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
__global__ void k_copy_f(const float* a, float* b, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) b[i] = a[i];
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
void gnn_neighbours(const View& v, int* nbr, cudaStream_t s) { k_gnn_nbr<<<nblk(v.ntot), kNB, 0, s>>>(v, nbr); }

void gnn_prepare(const View& v, const GnnBufs& g, cudaStream_t s) {
  k_gnn_linv<<<nblk(v.ntot), kNB, 0, s>>>(v, g.linv, g.chol_ok);
  k_gnn_feat<<<nblk(v.ntot), kNB, 0, s>>>(v, g);
}

void gnn_forward(const GnnNet& net, const GnnBufs& g, cudaStream_t s) {
  const int M = g.ntot;
  const int64_t hs = (int64_t)M * kGHid;
  {
    FwdOp<64, kEpiEnc> op{g.f, kGIn, M, nullptr, 0, net.W0, kGIn, net.w + kPb0, nullptr, g.h, g.hb, nullptr, nullptr};
    launch_gemm(op, M, 1, kGIn / 64, 1, g.err, s);
  }
  for (int l = 0; l < kGLayers; ++l) {
    FwdOp<64, kEpiLayer> op{g.hb + l * hs, kGHid, M, g.nbr, 1, net.Wl + (int64_t)l * kGHid * kGMsg, kGMsg,
                            net.w + kPb(l), g.h + l * hs, g.h + (l + 1) * hs, g.hb + (l + 1) * hs,
                            g.act + l * hs, nullptr};
    launch_gemm(op, M, 1, kGMsg / 64, 1, g.err, s);
  }
  {
    FwdOp<128, kEpiHead> op{g.hb + 3 * hs, kGHid, M, nullptr, 0, net.Wh, kGHid, net.w + kPbh, nullptr, nullptr,
                            nullptr, nullptr, g.o};
    launch_gemm(op, M, 1, 1, 1, g.err, s);
  }
}

void gnn_make_g(const GnnBufs& g, cudaStream_t s) { k_gnn_g<<<nblk(g.ntot), kNB, 0, s>>>(g); }

void gnn_refresh_bf16(const GnnNet& net, cudaStream_t s) {
  k_refresh<<<(kGLayers * kGHid * kGMsg + 255) / 256, 256, 0, s>>>(net);
}

void gnn_loss_grad(const View& v, const GnnNet& net, const GnnBufs& g, uint64_t seed, bool probes_given,
                   cudaStream_t s) {
  const int M = g.ntot;
  const int64_t hs = (int64_t)M * kGHid;
  if (!probes_given) k_tr_probe<<<nblk(M), kNB, 0, s>>>(g, seed);
  k_tr_vu<<<g.nlblk, kNB, 0, s>>>(g);
  k_tr_ts<<<nblk(M), kNB, 0, s>>>(v, g);
  k_tr_e<<<g.nlblk, kNB, 0, s>>>(g);
  k_tr_loss<<<1, 32, 0, s>>>(g);
  k_tr_ge<<<nblk(M), kNB, 0, s>>>(g);
  k_tr_gt<<<nblk(M), kNB, 0, s>>>(g);
  k_tr_gv<<<nblk(M), kNB, 0, s>>>(v, g);
  k_tr_do<<<nblk(M), kNB, 0, s>>>(g);
  const int nchunk = (M + 63) / 64;
  const int per = (nchunk + g.nsplit - 1) / g.nsplit;
  const int splits = (nchunk + per - 1) / per;
  // head
  {
    WgradOp<128> op{g.hb + 3 * hs, kGHid, kGHid, M, nullptr, 0, g.dob, g.wpart};
    launch_gemm(op, kGHid + 1, 1, nchunk, g.nsplit, g.err, s);
    k_wgrad_reduce<128><<<((kGHid + 1) * 128 + 255) / 256, 256, 0, s>>>(g.wpart, splits, kGHid, g.grad + kPWh,
                                                                         g.grad + kPbh);
    BwdDataOp dop{g.dob, kGOut, M, net.WhT, g.dh, kGHid};
    launch_gemm(dop, M, kGHid / 64, kGOut / 64, 1, g.err, s);
  }
  for (int l = kGLayers - 1; l >= 0; --l) {
    k_relu_bwd<<<(int)((hs + 255) / 256), 256, 0, s>>>(g.dh, g.act + l * hs, nullptr, g.dzb, (int)hs);
    WgradOp<64> op{g.hb + l * hs, kGHid, kGMsg, M, g.nbr, 1, g.dzb, g.wpart};
    launch_gemm(op, kGMsg + 1, 1, nchunk, g.nsplit, g.err, s);
    k_wgrad_reduce<64><<<((kGMsg + 1) * 64 + 255) / 256, 256, 0, s>>>(g.wpart, splits, kGMsg, g.grad + kPW(l),
                                                                       g.grad + kPb(l));
    BwdDataOp dop{g.dzb, kGHid, M, net.WlT + (int64_t)l * kGMsg * kGHid, g.dm, kGMsg};
    launch_gemm(dop, M, kGMsg / 64, 1, 1, g.err, s);
    k_msg_bwd<<<(int)((hs + 255) / 256), 256, 0, s>>>(g.dm, g.nbr, g.dh, M, 1);
  }
  k_relu_bwd<<<(int)((hs + 255) / 256), 256, 0, s>>>(g.dh, nullptr, g.h, g.dzb, (int)hs);
  WgradOp<64> op{g.f, kGIn, kGIn, M, nullptr, 0, g.dzb, g.wpart};
  launch_gemm(op, kGIn + 1, 1, nchunk, g.nsplit, g.err, s);
  k_wgrad_reduce<64><<<((kGIn + 1) * 64 + 255) / 256, 256, 0, s>>>(g.wpart, splits, kGIn, g.grad + kPW0,
                                                                    g.grad + kPb0);
}

void gnn_adam(const GnnNet& net, const GnnBufs& g, float* m, float* vv, float lr, int step, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<(kGParams + 255) / 256, 256, 0, s>>>(net.w, g.grad, m, vv, kGParams, lr, b1, b2, 1e-8f, c1, c2);
  gnn_refresh_bf16(net, s);
}

void lpcg_setup(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s) {
  k_lp_setup<<<b.nblk, kBlock, 0, s>>>(v, b, so);
  k_lp_g<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, 1);
  k_lp_gt<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, 1);
  k_lp_start<<<(v.ncloth + 127) / 128, 128, 0, s>>>(b, so, v.ncloth);
}

void lpcg_axpy(const View& v, const Blocks& b, const Solver& so, int parity, cudaStream_t s) {
  k_lp_axpy<<<b.nblk, kBlock, 0, s>>>(v, b, so, parity);
}
void lpcg_precondition(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s) {
  k_lp_g<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, 0);
  k_lp_gt<<<b.nblk, kBlock, 0, s>>>(v, b, so, lx, 0);
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
