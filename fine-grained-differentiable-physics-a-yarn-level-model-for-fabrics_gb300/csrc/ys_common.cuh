// ys_common.cuh -- device-side data layout of a batch of yarn-level cloths.
//
// Every array is structure-of-arrays over the concatenated nodes of all
// cloths in the batch (node i of cloth c lives at cloth_off[c] + u + v*W).
// A per-node quantity with k components is stored component-major:
// comp j of node i at ptr[j * ntot + i], so one warp reading component j of
// 32 consecutive nodes issues one coalesced 256-byte transaction.
//
// The implicit system A x = b of one step is stored as a structured stencil:
// row block i (5 DOFs: x, y, z, u, v) couples only to the 13 grid
// neighbours reachable by an edge, a bend segment (two crossings along a
// yarn) or a shear segment (diagonal). The coefficient slots of one row
// block are listed in YS_SLOT_* below; slot j of node i is A[j * ntot + i].
// No column indices are stored: the neighbour is implied by the slot.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define YS_HD __host__ __device__ __forceinline__
#define YS_RESTRICT __restrict__
#else
#define YS_HD inline
#define YS_RESTRICT
#endif

namespace ys {

constexpr double kPi = 3.1415926535897;  // the reference's PI (src/Constants.h:24)

// stencil offsets (du, dv) of the 13 node-node couplings
constexpr int kNumStencil = 13;
YS_HD int stencil_du(int s) {
  const int t[13] = {0, -1, 1, 0, 0, -2, 2, 0, 0, -1, 1, -1, 1};
  return t[s];
}
YS_HD int stencil_dv(int s) {
  const int t[13] = {0, 0, 0, -1, 1, 0, 0, -2, 2, -1, -1, 1, 1};
  return t[s];
}
YS_HD int stencil_index(int du, int dv) {
  // inverse of the tables above; -1 when outside the stencil
  if (dv == 0) {
    switch (du) { case 0: return 0; case -1: return 1; case 1: return 2; case -2: return 5; case 2: return 6; }
    return -1;
  }
  if (du == 0) {
    switch (dv) { case -1: return 3; case 1: return 4; case -2: return 7; case 2: return 8; }
    return -1;
  }
  if (du == -1 && dv == -1) return 9;
  if (du == 1 && dv == -1) return 10;
  if (du == -1 && dv == 1) return 11;
  if (du == 1 && dv == 1) return 12;
  return -1;
}
// the four yarn neighbours that carry Eulerian couplings: 0:(-1,0) 1:(1,0)
// 2:(0,-1) 3:(0,1); warp neighbours couple the u DOF, weft neighbours v.
YS_HD int yarn_nbr(int du, int dv) {
  if (dv == 0 && du == -1) return 0;
  if (dv == 0 && du == 1) return 1;
  if (du == 0 && dv == -1) return 2;
  if (du == 0 && dv == 1) return 3;
  return -1;
}

// coefficient slots of one row block
constexpr int YS_SLOT_LL = 0;        // 13 x 3 x 3: [s][r][c] = A[x_r(i)][x_c(j_s)]
constexpr int YS_SLOT_LE_SELF = 117; // 3 x 2:      [r][k]    = A[x_r(i)][e_k(i)]
constexpr int YS_SLOT_EL_SELF = 123; // 2 x 3:      [k][c]    = A[e_k(i)][x_c(i)]
constexpr int YS_SLOT_EE_SELF = 129; // 2:          [k]       = A[e_k(i)][e_k(i)]
constexpr int YS_SLOT_LE_NBR = 131;  // 4 x 3:      [n][r]    = A[x_r(i)][e_k(n)(j_n)]
constexpr int YS_SLOT_EL_NBR = 143;  // 4 x 3:      [n][c]    = A[e_k(n)(i)][x_c(j_n)]
constexpr int YS_SLOT_EE_NBR = 155;  // 4:          [n]       = A[e_k(n)(i)][e_k(n)(j_n)]
constexpr int YS_NUM_SLOTS = 159;

// node flags
constexpr uint8_t YS_INTERIOR = 1;
constexpr uint8_t YS_FIXED = 2;
constexpr uint8_t YS_FLIP = 4;

struct ClothParams {
  int W, H, node_off, warp_line_off, weft_line_off;
  int pad_;
  double L, R, kc, kf, df, mu, S, kh, jam;
  double G[3];
  double wind[3];
  double wind_rho, wind_drag;
  double pb4, pb5;  // (PI/2)^4 and (PI/2)^5 as std::pow gives them (src/PhysicsCloth.cpp:2680-2681)
};

// Device view of a batch (trivially copyable; passed by value to kernels).
struct View {
  int ntot;
  int ncloth;
  const int* YS_RESTRICT node_cloth;  // [ntot]
  const int* YS_RESTRICT node_u;      // [ntot]
  const int* YS_RESTRICT node_v;      // [ntot]
  const uint8_t* YS_RESTRICT flags;   // [ntot]
  const ClothParams* YS_RESTRICT cp;  // [ncloth]
  const double* YS_RESTRICT line_rho; // per yarn line
  const double* YS_RESTRICT line_ks;
  const double* YS_RESTRICT line_kb;
  // state
  double* X;     // [3][ntot] LPos
  double* V;     // [3][ntot] LVel
  double* XF;    // [3][ntot] LPosFix
  double* UV;    // [2][ntot] EPos
  double* UVD;   // [2][ntot] EVel
  double* UVB;   // [2][ntot] EPosBar
  double* UV0;   // [2][ntot] EPos at construction (crimp segments keep it)
  double* NRM;   // [3][ntot] node normal (interior nodes)
  double* COMP;  // [ntot] crossing compression
  double* SLIDE; // [2][ntot] soft slide indicator
  // one step's system and accumulators
  double* A;     // [YS_NUM_SLOTS][ntot]
  double* B;     // [5][ntot]
  double* CL;    // [3][ntot]  StrhBend_C_L
  double* CLE;   // [6][ntot]  StrhBend_C_LE self entries (u: 0..2, v: 3..5)
  double* FE;    // [2][ntot]  Eulerian force before friction
  double* KEE;   // [2][ntot]  dF_E/dE diagonal before friction (position)
  double* DEE;   // [2][ntot]  same, velocity
  const double* ext;  // [5][ntot] external force or null
  double h;
  // Forward-mode tangents (null in the plain step). Per-node arrays hold
  // tangent k of comp c of node i at [(c * K + k) * ntot + i]; parameter
  // tables hold tangent k of entry i at [k * n + i].
  int K;
  int trunc;  // 1: tangents of b through F and v only (M, D, A held constant)
  int nlines;
  const double* dX;
  const double* dV;
  const double* dUV;
  const double* dUVD;
  const double* dUVB;
  double* dNRM;
  double* dCOMP;
  double* dSLIDE;
  const double* dline_rho;  // [K][nlines]
  const double* dline_ks;
  const double* dline_kb;
  const double* dS;   // [K][ncloth]
  const double* dmu;
  double* dA;  // [YS_NUM_SLOTS][K][ntot]
  double* dB;  // [5][K][ntot]
};

YS_HD double& slot(const View& v, int s, int node) { return v.A[(int64_t)s * v.ntot + node]; }

}  // namespace ys
