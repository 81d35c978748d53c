// ys_gnn.cuh -- the learned preconditioner (no counterpart in the reference):
// a graph network over the crossing graph of a batch (each node linked to its
// four yarn neighbours) that reads the assembled system and emits a factorised
// sparse approximate inverse
//
//   M^-1 = G^T G,  G block lower triangular in node order,
//   G_i,b = N_i,b L_src(b)^-1 (b > 0),  G_i,0 = (I + N_i,0) L_i^-1,
//
// over the lower pattern b = self, left, down (the node's predecessors along
// its two yarns in the node order u + v W), where
// L_i L_i^T is the Cholesky factorisation of the symmetric part of node i's
// 5 x 5 diagonal block. M^-1 is symmetric positive definite whenever every
// I + N_i,0 is non-singular, so the conjugate-gradient recurrences stay valid.
//
// Network (BF16 operands, FP32 accumulation on the tensor cores):
//   f_i   = 128 features of node i (its scaled couplings E_i,b = L_i^-1 A_i,src L_src^-T
//           to the left, down, left-down, right-down, left-2 and down-2 nodes,
//           norms of its upper couplings, flags)
//   h1    = relu(W0 f + b0)                                   (64)
//   h_l+1 = h_l + relu(W_l [h_i, h_left, h_right, h_down, h_up] + b_l)   l = 1..3
//   o     = Wh h4 + bh                                        (192, 175 used)
//   N_i,0 = 0.1 o[0:25],   N_i,b = -E_i,b + 0.1 o[25 b : 25 b + 25]
// The untrained network (head weights zero) is the first-order factorised
// approximate inverse G = (I - E_lower) L^-1.
//
// Training minimises the Kaporin condition number of G A G^T, the quantity
// the factorised sparse approximate inverse (FSAI) minimises over a pattern:
//   loss = log(tr(G A G^T) / n) - (2 / n) sum_i log |det G_i,0|   (n = DOFs)
// with the trace from Rademacher probes (w^T G A G^T w) and the determinant
// exact (G is block triangular); gradients are written out by hand (ys_gnn.cu).
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "ys_common.cuh"
#include "ys_kernels.cuh"

namespace ys {

constexpr int kGIn = 128, kGHid = 64, kGMsg = 320, kGOut = 192, kGLayers = 3, kGBlocks = 7, kGUsed = 25 * kGBlocks;
constexpr float kGOutScale = 0.1f;
// the solve's BF16 copy of G holds each block's 25 coefficients in 13 pairs
// (the last padded with zero): pair q of block b of node n at [13 b + q][n]
constexpr int kGPairs = 13 * kGBlocks;
// packed FP32 parameter vector: W0 [64][128], b0, then per layer W [64][320], b,
// then Wh [192][64], bh
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
// lower offsets (du, dv) b = 0..6: self, left, down, left-down, right-down,
// left-2, down-2; G uses the first kGBlocks, the features all six couplings
YS_HD constexpr int gpat_du(int b) { return b == 1 ? -1 : b == 3 ? -1 : b == 4 ? 1 : b == 5 ? -2 : 0; }
YS_HD constexpr int gpat_dv(int b) { return b == 2 ? -1 : b == 3 ? -1 : b == 4 ? -1 : b == 6 ? -2 : 0; }

struct GnnNet {  // device arrays
  float* w;             // [kGParams] FP32 master parameters
  __nv_bfloat16* W0;    // [64][128]
  __nv_bfloat16* Wl;    // [3][64][320]
  __nv_bfloat16* Wh;    // [192][64]
  __nv_bfloat16* WlT;   // [3][320][64]
  __nv_bfloat16* WhT;   // [64][192]
};

struct GnnBufs {  // device arrays sized for ntot nodes
  int ntot;
  int nsplit;           // weight-gradient node splits
  int* nbr;             // [ntot][4] yarn neighbours (left, right, down, up) or -1
  int* pat;             // [ntot][8] source node of block b of G (b < kGBlocks) or -1
  int* upat;            // [ntot][8] the row i whose block b has this node as source, or -1
  float* linv;          // [15][ntot] L^-1, packed lower triangle (r (r + 1) / 2 + c)
  int* chol_ok;         // [ntot] 1 if the diagonal block factorised
  float* E;             // [150][ntot] scaled couplings E_i,b, b = 1..6
  __nv_bfloat16* f;     // [ntot][128]
  float* h;             // [4][ntot][64] h1..h4
  __nv_bfloat16* hb;    // [4][ntot][64]
  __nv_bfloat16* act;   // [3][ntot][64] relu outputs of the message layers
  float* o;             // [192][ntot] network outputs (component-major)
  float* G;             // [175][ntot] blocks of G, row-major 5 x 5 (training, export)
  __nv_bfloat162* Gh;   // [kGPairs][ntot] the same in BF16 pairs (the solve's preconditioner)
  float* Gn;            // [175][ntot] blocks of N (training)
  float* Nt;            // [175][ntot] the exact FSAI's blocks of N (the FSAI objective's target)
  float* vec;           // [4][5][ntot] training vectors (w, u, t, s)
  __nv_bfloat16* dob;   // [ntot][192]
  float* dh;            // [ntot][64]
  __nv_bfloat16* dzb;   // [ntot][64]
  float* dm;            // [ntot][320]
  float* wpart;         // [nsplit][kWgradRows][192]
  float* grad;          // [kGParams]
  double* lpart;        // [2][nlblk] loss partials, then loss and its two scales
  int nlblk;
  int* err;             // device error word (non-zero: a tensor-core wait ran out)
};

// learned-preconditioner PCG state lives in Solver; these hold its extras
struct LpcgExtra {
  const __nv_bfloat162* G;  // [kGPairs][ntot]
  float* rf;        // [5][ntot] the residual in FP32, as the preconditioner reads it
  double* z;        // [5][ntot] G^T G r
};

// ---- launchers (ys_gnn.cu)
void gnn_neighbours(const View& v, const GnnBufs& g, cudaStream_t s);
void gnn_prepare(const View& v, const GnnBufs& g, cudaStream_t s);
// (training: keep the ReLU outputs the backward pass reads)
void gnn_forward(const GnnNet& net, const GnnBufs& g, bool training, cudaStream_t s);
// sets the forward GEMMs' function attributes (done by gnn_forward's first
// call; call it before capturing gnn_forward into a graph)
void gnn_forward_attrs();
// G (and, for training, the blocks of N) from the network outputs
void gnn_make_g(const GnnBufs& g, bool keep_n, cudaStream_t s);
void gnn_refresh_bf16(const GnnNet& net, cudaStream_t s);
// one training pass, the loss and the parameter gradient into g.grad:
// objective 0 (Kaporin number; probes from seed, or host-given in vec slot 0
// when probes_given) or 1 (distance of N to the exact FSAI's blocks)
void gnn_loss_grad(const View& v, const GnnNet& net, const GnnBufs& g, uint64_t seed, bool probes_given,
                   int objective, cudaStream_t s);
void gnn_adam(const GnnNet& net, const GnnBufs& g, float* m, float* vv, float lr, int step, cudaStream_t s);

// x = 0, r = b, z = G^T G r, p = z and the per-cloth start of the iteration
void lpcg_setup(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s);
// after the SpMV q = A p of iteration `parity`: x, r (and its FP32 copy)
void lpcg_axpy(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, int parity, cudaStream_t s);
// z = G^T G r with the partial dot products the direction update needs
void lpcg_precondition(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, cudaStream_t s);
// the stop test and p = z + beta p (it: the iteration, from *so.it_base in a graph body)
void lpcg_dir(const View& v, const Blocks& b, const Solver& so, const LpcgExtra& lx, int parity, int it,
              cudaStream_t s);
// C [M][N] = A [M][K] B [N][K]^T (BF16 in, FP32 out; N = 64 k or 128, K = 64 k)
void tc_gemm_bf16(const __nv_bfloat16* A, const __nv_bfloat16* B, float* C, int M, int N, int K, int* err,
                  cudaStream_t s);

}  // namespace ys
