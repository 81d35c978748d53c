// ys_elem_kernels.cuh -- the element-record and gather kernels of one step,
// templates over the scalar type (double for the step, Dual<kTangents> for
// its forward-mode sensitivities); instantiated in ys_kernels.cu and
// ys_tangent.cu.
#pragma once

#include "ys_items.cuh"
#include "ys_kernels.cuh"

namespace ys {

// The record producers and the gather: one thread per element (or node),
// nothing shared between threads, so any block size gives the same bits; the
// block size is a schedule choice (up to kMaxProducerBlock threads; up to
// kBlock for the edges, whose 254 registers spill when compiled for 256-thread
// blocks).

// one thread per (yarn direction, node): the edge starting at that node
template <class T>
__global__ void __launch_bounds__(kBlock) k_edge_rec(View v, Records R) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2LL * v.ntot) return;
  const int k = t >= v.ntot ? 1 : 0;
  const int n0 = (int)(t - (int64_t)k * v.ntot);
  const ClothParams& P = v.cp[v.node_cloth[n0]];
  if (k == 0 ? v.node_u[n0] >= P.W - 1 : v.node_v[n0] >= P.H - 1) return;
  EdgeOut<T> o;
  edge_element(v, n0, n0 + (k == 0 ? 1 : P.W), k, o, R.edge, R.dedge);
  edge_store_groups(v, R.edge, R.dedge, n0, k, o, false, true);
}

// one thread per (yarn direction, middle node) of a bend segment
template <class T>
__global__ void __launch_bounds__(kMaxProducerBlock) k_bend_rec(View v, Records R) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2LL * v.ntot) return;
  const int k = t >= v.ntot ? 1 : 0;
  const int n0 = (int)(t - (int64_t)k * v.ntot);
  const ClothParams& P = v.cp[v.node_cloth[n0]];
  const int pos = k == 0 ? v.node_u[n0] : v.node_v[n0], len = k == 0 ? P.W : P.H;
  if (pos < 1 || pos > len - 2) return;
  const int step = k == 0 ? 1 : P.W;
  const int line = k == 0 ? P.warp_line_off + v.node_v[n0] : P.weft_line_off + v.node_u[n0];
  bend_element<T>(v, R.bend, R.dbend, n0 - step, n0, n0 + step, k, line);
}

// one thread per grid cell (top-left node): its two faces
template <class T>
__global__ void __launch_bounds__(kMaxProducerBlock) k_face_rec(View v, Records R) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  const ClothParams& P = v.cp[v.node_cloth[n]];
  if (v.node_u[n] >= P.W - 1 || v.node_v[n] >= P.H - 1) return;
  cell_faces<T>(v, R.face, R.dface, n);
}

// row blocks from edge / bend / face records, plus sliding friction
template <class T>
__global__ void __launch_bounds__(kMaxProducerBlock) k_gather(View v, Records R) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < v.ntot) gather_elements<T>(v, R, n);
}

// one thread per (segment type, crossing)
template <class T>
__global__ void __launch_bounds__(kMaxProducerBlock) k_shear_rec(View v, Records R) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4LL * v.ntot) return;
  const int seg = (int)(t / v.ntot);
  const int n0 = (int)(t - (int64_t)seg * v.ntot);
  if (!(v.flags[n0] & YS_INTERIOR)) return;
  shear_element<T>(v, R.shear, R.dshear, n0, seg);
}

}  // namespace ys
