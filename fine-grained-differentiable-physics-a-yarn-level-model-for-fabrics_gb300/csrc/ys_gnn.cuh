// ys_gnn.cuh -- the learned preconditioner (no counterpart in the reference):
// a graph network over the crossing graph of a batch (each node linked to its
// four yarn neighbours) that reads the assembled system and emits, per node,
// a correction N of a factorised sparse approximate inverse
//
//   M^-1 = G^T G,   G = (I + N) L^-1,
//
// where L_i L_i^T is the Cholesky factorisation of the symmetric part of the
// node's 5 x 5 diagonal block (block Jacobi when N = 0) and N has a 5 x 5
// block on the node itself and one per yarn neighbour. M^-1 is symmetric
// positive semi-definite for every N, so the conjugate-gradient recurrences
// stay valid whatever the network emits.
//
// Network (BF16 operands, FP32 accumulation on the tensor cores):
//   f_i   = 128 features of node i (the scaled neighbour blocks L_i^-1 A_ij L_j^-T
//           of its 4 yarn neighbours, norms of its 8 other couplings, flags)
//   h1    = relu(W0 f + b0)                                   (64)
//   h_l+1 = h_l + relu(W_l [h_i, h_left, h_right, h_down, h_up] + b_l)   l = 1..3
//   o     = Wh h4 + bh                                        (128, 125 used)
//   N_ii  = 0.1 o[0:25],  N_i,d = -E_i,d / 2 + 0.1 o[25 + 25 d : 50 + 25 d]
// where E_i,d is the scaled neighbour block; -E/2 is the first-order term of
// (I + E)^-1 = (I + N)^T (I + N), so an untrained network (head weights zero)
// starts from that analytic approximate inverse.
//
// Training minimises the stochastic Frobenius norm
//   loss = sum |(G A G^T - I) w|^2 / sum |w|^2   over Rademacher probes w,
// with gradients through G A G^T written out by hand (ys_gnn.cu).
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "ys_common.cuh"
#include "ys_kernels.cuh"

namespace ys {

constexpr int kGIn = 128, kGHid = 64, kGMsg = 320, kGOut = 128, kGLayers = 3, kGUsed = 125;
constexpr float kGOutScale = 0.1f;
// packed FP32 parameter vector: W0 [64][128], b0, then per layer W [64][320], b,
// then Wh [128][64], bh
constexpr int kPW0 = 0;
constexpr int kPb0 = kPW0 + kGHid * kGIn;
constexpr int kPL0 = kPb0 + kGHid;
constexpr int kPLStride = kGHid * kGMsg + kGHid;
YS_HD constexpr int kPW(int l) { return kPL0 + l * kPLStride; }
YS_HD constexpr int kPb(int l) { return kPW(l) + kGHid * kGMsg; }
constexpr int kPWh = kPL0 + kGLayers * kPLStride;
constexpr int kPbh = kPWh + kGOut * kGHid;
constexpr int kGParams = kPbh + kGOut;
constexpr int kWgradRows = 384;  // largest K_in + 1 (bias row), rounded to the 128-row tile

struct GnnNet {  // device arrays
  float* w;             // [kGParams] FP32 master parameters
  __nv_bfloat16* W0;    // [64][128]
  __nv_bfloat16* Wl;    // [3][64][320]
  __nv_bfloat16* Wh;    // [128][64]
  __nv_bfloat16* WlT;   // [3][320][64]
  __nv_bfloat16* WhT;   // [64][128]
};

struct GnnBufs {  // device arrays sized for ntot nodes
  int ntot;
  int nsplit;           // weight-gradient node splits
  int* nbr;             // [ntot][4] yarn neighbours (left, right, down, up) or -1
  float* linv;          // [15][ntot] L^-1, packed lower triangle (r (r + 1) / 2 + c)
  int* chol_ok;         // [ntot] 1 if the diagonal block factorised
  float* E;             // [ntot][100] scaled neighbour blocks
  __nv_bfloat16* f;     // [ntot][128]
  float* h;             // [4][ntot][64] h1..h4
  __nv_bfloat16* hb;    // [4][ntot][64]
  __nv_bfloat16* act;   // [3][ntot][64] relu outputs of the message layers
  float* o;             // [ntot][128]
  float* G;             // [125][ntot] blocks of G (self, left, right, down, up), row-major 5 x 5
  float* Gn;            // [125][ntot] blocks of N (training)
  float* vec;           // [12][5][ntot] training vectors
  __nv_bfloat16* dob;   // [ntot][128]
  float* dh;            // [ntot][64]
  __nv_bfloat16* dzb;   // [ntot][64]
  float* dm;            // [ntot][320]
  float* wpart;         // [nsplit][kWgradRows][128]
  float* grad;          // [kGParams]
  double* lpart;        // [2][nlblk] loss partials
  int nlblk;
  int* err;             // device error word (non-zero: a tensor-core wait ran out)
};

// learned-preconditioner PCG state lives in Solver; these hold its extras
struct LpcgExtra {
  const float* G;   // [125][ntot]
  const int* nbr;   // [ntot][4]
  float* y;         // [5][ntot] G r
  double* z;        // [5][ntot] G^T G r
};

// ---- launchers (ys_gnn.cu)
void gnn_neighbours(const View& v, int* nbr, cudaStream_t s);
void gnn_prepare(const View& v, const GnnBufs& g, cudaStream_t s);
void gnn_forward(const GnnNet& net, const GnnBufs& g, cudaStream_t s);
void gnn_make_g(const GnnBufs& g, cudaStream_t s);
void gnn_refresh_bf16(const GnnNet& net, cudaStream_t s);
// one training pass: probes from seed (or host-given vec slot 0 when seed == 0
// and probes_given), loss partials, parameter gradient into g.grad
void gnn_loss_grad(const View& v, const GnnNet& net, const GnnBufs& g, uint64_t seed, bool probes_given,
                   cudaStream_t s);
double gnn_loss_value_host(const GnnBufs& g, cudaStream_t s, cudaError_t* e);
void gnn_adam(const GnnNet& net, const GnnBufs& g, float* m, float* vv, float lr, int step, cudaStream_t s);

void lpcg_setup(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s);
void lpcg_axpy(const View& v, const Blocks& b, const Solver& so, int parity, cudaStream_t s);
void lpcg_precondition(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s);
void lpcg_dir(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, int parity, int it,
              cudaStream_t s);
// C [M][N] = A [M][K] B [N][K]^T (BF16 in, FP32 out; N = 64 k or 128, K = 64 k)
void tc_gemm_bf16(const __nv_bfloat16* A, const __nv_bfloat16* B, float* C, int M, int N, int K, int* err,
                  cudaStream_t s);

}  // namespace ys
