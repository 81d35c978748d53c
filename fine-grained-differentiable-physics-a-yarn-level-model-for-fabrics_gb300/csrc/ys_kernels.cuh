// ys_kernels.cuh -- launch wrappers of the per-step kernels (ys_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "ys_items.cuh"

namespace ys {

// per-cloth Jacobi-PCG bookkeeping (one entry per cloth)
struct PcgCloth {
  double bb;        // |b|^2
  double thr;       // stop when |r|^2 < thr
  double rz[2];     // r.z of the current iterate, double-buffered by parity
  double rr;        // |r|^2 after the last update
  int active;       // 1 while iterating
  int iters;        // completed iterations
  int maxiter;
  int status;       // bit 0: non-finite system, bit 1: non-finite solution, bit 2: iteration cap
};

// thread-block partition of the nodes: blocks never straddle two cloths, so
// per-cloth reductions are a fixed-order sum over a contiguous block range
struct Blocks {
  int nblk;
  const int* blk_cloth;   // [nblk]
  const int* blk_node0;   // [nblk] first node
  const int* blk_count;   // [nblk] nodes in the block
  const int* cloth_blk0;  // [ncloth] first block
  const int* cloth_nblk;  // [ncloth]
};

struct Solver {
  double* x;      // [5][ntot]
  double* r;      // [5][ntot]
  double* p;      // [5][ntot]
  double* q;      // [5][ntot]
  double* dinv;   // [5][ntot]
  double* part;   // [3][nblk] block partial sums
  PcgCloth* pc;   // [ncloth]
  int* nactive;   // device counter
  double tol;
  int trans;      // 1: solve A^T x = b (the reference-mode tangent solves)
  int* it_base;   // graph mode: iterations completed before this graph body (device), else null
  const int* hold;  // graph mode: when *hold != 0 the solution check and the update leave every cloth
                    // as it was (the learned solve handed the step to Jacobi-PCG), else null
};

constexpr int kBlock = 128;
constexpr int kMaxProducerBlock = 256;  // block size limit of the record producers and the gather

// the producers' `threads` (per block, 32..kMaxProducerBlock) does not change results
void launch_geom(const View& v, const int* nodes, int n, cudaStream_t s);
void launch_edge_records(const View& v, const Records& R, cudaStream_t s, int threads = kBlock);
void launch_bend_records(const View& v, const Records& R, cudaStream_t s, int threads = kBlock);
void launch_face_records(const View& v, const Records& R, cudaStream_t s, int threads = kBlock);
void launch_gather(const View& v, const Records& R, cudaStream_t s, int threads = kBlock);
void launch_shear_records(const View& v, const Records& R, cudaStream_t s, int threads = kBlock);
void launch_finalize(const View& v, const Records& R, const Blocks& b, const Solver& so, cudaStream_t s);
void launch_pcg_setup(const View& v, const Blocks& b, const Solver& so, cudaStream_t s);
void launch_pcg_spmv(const View& v, const Blocks& b, const Solver& so, cudaStream_t s);
void launch_pcg_axpy(const View& v, const Blocks& b, const Solver& so, int it, cudaStream_t s);
void launch_pcg_dir(const View& v, const Blocks& b, const Solver& so, int it, cudaStream_t s);
void launch_count_active(const View& v, const Solver& so, cudaStream_t s);
void launch_check_solution(const View& v, const Blocks& b, const Solver& so, cudaStream_t s);
// graph mode: *it_base = 0 before the loop; after each body of m iterations
// count the active cloths, advance *it_base by m and set the while node's
// condition to (some cloth active and *it_base < cap)
void launch_graph_loop_begin(const Solver& so, cudaStream_t s);
void launch_graph_loop_tail(const Solver& so, int ncloth, int m, int cap, cudaGraphConditionalHandle h,
                            cudaStream_t s);
void launch_update(const View& v, const Blocks& b, const Solver& so, cudaStream_t s);
// graph mode of the learned solve: *so.hold = 1 if the solve must be redone by
// Jacobi-PCG (an expired tensor-core wait in *err, a breakdown, or the default
// iteration cap when the caller set none; cloths with a non-finite system excepted)
void launch_learned_verdict(const Solver& so, int ncloth, const int* err, int caller_cap, int* hold,
                            cudaStream_t s);
void launch_spmv(const View& v, const double* x, double* y, cudaStream_t s);

// ---- persistent per-cloth PCG (ys_pcg_cluster.cu): one cluster of csize
// CTAs of `threads` threads per listed cloth runs that cloth's whole solve
// (set-up included) with at most `cap` iterations; a cloth needs
// width * length <= threads * csize. Same results as the phase kernels above.
bool pcg_cluster_shape_ok(int threads, int csize);
// clusters of this shape that fit on the GPU at once (0: the shape cannot run)
cudaError_t pcg_cluster_occupancy(int threads, int csize, int* clusters);
cudaError_t launch_pcg_cluster(const View& v, const Solver& so, const int* cloths, int ncl, int threads, int csize,
                               int cap, cudaStream_t s);

// state tangents updated by the tangent step (layout [c][kTangents][ntot])
struct TangentState {
  double* dX;
  double* dV;
  double* dUV;
  double* dUVD;
  double* dUVB;
};
// the element / gather / finalize kernels over Dual<kTangents>
void launch_assembly_dual(const View& v, const Records& R, const int* geom_nodes, int geom_n, cudaStream_t s);
// rt[k][c][ntot] = db_k - dA_k q (or db_k when v.trunc) for k < kact
void launch_tangent_rhs(const View& v, const double* q, double* rt, int kact, cudaStream_t s);
// rt_k += h dext_k for the external force's tangents dext [kact][ntot][5]
void launch_tangent_ext(const View& v, const double* dext, double* rt, double h, int kact, cudaStream_t s);
// solution check, then Cloth::update of the state (solution so.x) and its
// tangents (dq, [5][kTangents][ntot])
void launch_update_dual(const View& v, const Blocks& b, const Solver& so, const double* dq, const TangentState& ts,
                        cudaStream_t s);

// ---- reverse-mode step (ys_adjoint.cu)
// state adjoints, component-major: [0] LPos [3][nt], [1] LVel [3][nt],
// [2] EPos [2][nt], [3] EVel [2][nt], [4] EPosBar [2][nt]
struct AdjIO {
  const double* gin[5];  // dL/d(state after the step)
  double* gout[5];       // dL/d(state before the step)
};
// the forward-mode seeds of the copies' batch (its tangent arrays)
struct AdjSeeds {
  double *dX, *dV, *dUV, *dUVD, *dUVB;
  double *drho, *dks, *dkb, *dS, *dmu;
};
// material adjoints, accumulated: line[p][l] for p = rho, Y, B of primal
// line l; cloth[p][c] for p = S, mu
struct AdjParamOut {
  double* line[3];
  double* cloth[2];
};
int adjoint_direction_count();
void launch_adj_update(const View& v, const AdjIO& io, const double* q, double* qbar, double* slide_bar,
                       cudaStream_t s);
void launch_adj_broadcast(const double* src, double* dst, int nt, int ncomp, int copies, cudaStream_t s);
void launch_adj_seed(const View& vc, int nt, int nl, int ncl, int base, const double* line_a, const int* line_kind,
                     const AdjSeeds& sd, cudaStream_t s);
void launch_adj_contract(const View& vc, int nt, const double* lambda, const double* slide_bar, const double* rt,
                         double* T, cudaStream_t s);
void launch_adj_gather(const View& v, int base, int copies, const double* T, int64_t ntc, const int* line_cloth,
                       const int* line_kind, const AdjIO& io, const AdjParamOut& gp, cudaStream_t s);
void launch_adj_ext(const View& v, const double* lambda, double* gext, cudaStream_t s);

}  // namespace ys
