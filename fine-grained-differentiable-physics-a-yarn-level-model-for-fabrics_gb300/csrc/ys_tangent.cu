// ys_tangent.cu -- forward-mode sensitivity kernels of one step: the
// element and gather kernels over Dual<kTangents>, the right-hand sides of
// the tangent solves and the update of state tangents.
#include "ys_elem_kernels.cuh"
#include "ys_items.cuh"
#include "ys_kernels.cuh"

namespace ys {

static inline int nblocks_t(int n) { return (n + kBlock - 1) / kBlock; }

// ------------------------------------------------------------- tangents
// The same element and gather kernels over Dual<kTangents>: each value they
// compute carries its derivatives along the seeded directions. The view
// passed here writes the values of A and b to shadow arrays (the step's own
// A and b stay for the tangent solves) and every tangent to its d* array.
typedef Dual<kTangents> TD;

__global__ void k_geom_dual(View v, const int* __restrict__ nodes, int count) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int n = nodes[t];
  node_normal_dual<kTangents>(v, n, v.cp[v.node_cloth[n]].W);
}

__global__ void __launch_bounds__(kBlock) k_finalize_dual(View v, Records R) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < v.ntot) gather_shear_finalize<TD>(v, R, n, nullptr);
}

// right-hand sides of the tangent solves, rt[k][c][ntot] for k < kact
__global__ void k_tangent_rhs(View v, const double* __restrict__ q, double* __restrict__ rt, int kact) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const int64_t nt = v.ntot;
  for (int k = 0; k < kact; ++k) {
    double r[5];
    tangent_rhs_row(v, q, n, k, r);
    for (int c = 0; c < 5; ++c) rt[((int64_t)k * 5 + c) * nt + n] = r[c];
  }
}

// the external force's tangents in the right-hand sides: the gather adds
// h ext to b (x, y, z of every node, u, v of interior nodes), so direction k
// gains h dext_k; dext [kact][ntot][5]
__global__ void k_tangent_ext(View v, const double* __restrict__ dext, double* __restrict__ rt, double h, int kact) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const int64_t nt = v.ntot;
  const int nc = (v.flags[n] & YS_INTERIOR) ? 5 : 3;
  for (int k = 0; k < kact; ++k)
    for (int c = 0; c < nc; ++c) rt[((int64_t)k * 5 + c) * nt + n] += h * dext[((int64_t)k * nt + n) * 5 + c];
}

// Cloth::update of state and tangents for every cloth whose step succeeded
__global__ void __launch_bounds__(kBlock) k_update_dual(View v, Blocks b, Solver so, const double* __restrict__ dq,
                                                        TangentState ts) {
  const int blk = blockIdx.x;
  const int c = b.blk_cloth[blk];
  const int n = b.blk_node0[blk] + threadIdx.x;
  if (threadIdx.x >= b.blk_count[blk]) return;
  if (so.pc[c].status & 3) return;
  update_node_dual<kTangents>(v, so.x, dq, ts.dX, ts.dV, ts.dUV, ts.dUVD, ts.dUVB, n);
}

void launch_assembly_dual(const View& v, const Records& R, const int* geom_nodes, int geom_n, cudaStream_t s) {
  if (geom_n) k_geom_dual<<<nblocks_t(geom_n), kBlock, 0, s>>>(v, geom_nodes, geom_n);
  k_edge_rec<TD><<<nblocks_t(2 * v.ntot), kBlock, 0, s>>>(v, R);
  k_bend_rec<TD><<<nblocks_t(2 * v.ntot), kBlock, 0, s>>>(v, R);
  k_face_rec<TD><<<nblocks_t(v.ntot), kBlock, 0, s>>>(v, R);
  k_gather<TD><<<nblocks_t(v.ntot), kBlock, 0, s>>>(v, R);
  k_shear_rec<TD><<<nblocks_t(4 * v.ntot), kBlock, 0, s>>>(v, R);
  k_finalize_dual<<<nblocks_t(v.ntot), kBlock, 0, s>>>(v, R);
}
void launch_tangent_rhs(const View& v, const double* q, double* rt, int kact, cudaStream_t s) {
  k_tangent_rhs<<<nblocks_t(v.ntot), kBlock, 0, s>>>(v, q, rt, kact);
}
void launch_tangent_ext(const View& v, const double* dext, double* rt, double h, int kact, cudaStream_t s) {
  k_tangent_ext<<<nblocks_t(v.ntot), kBlock, 0, s>>>(v, dext, rt, h, kact);
}
void launch_update_dual(const View& v, const Blocks& b, const Solver& so, const double* dq, const TangentState& ts,
                        cudaStream_t s) {
  launch_check_solution(v, b, so, s);
  k_update_dual<<<b.nblk, kBlock, 0, s>>>(v, b, so, dq, ts);
}

}  // namespace ys
