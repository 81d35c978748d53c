// ys_collide.cu -- continuous collision detection of a cloth mesh against
// itself and an obstacle mesh (the reference's Collision::find_impacts,
// src/Collision.cpp:184-208): host tree construction (ys_bvh.h), device
// refit, broad phase (one thread per cloth face traversing the cloth tree
// and the obstacle tree) and narrow phase (one thread per face pair), with
// deterministic output order (face-major, tree order within a face; impacts
// in pair order, then the reference's test order).
#include <cuda_runtime.h>

#include <cuda/atomic>

#include <algorithm>
#include <chrono>
#include <memory>
#include <thread>
#include <cmath>
#include <cstring>
#include <future>
#include <string>
#include <vector>

#include "../../include/yarnsim.h"
#include "ys_bvh.h"
#include "ys_collide.cuh"
#include "ys_zones.h"

extern "C" ys_status ys_internal_fail(ys_status s, const char* msg);

namespace {

using ys::CFace;
using ys::CMesh;
using ys::Impact;
using ys::Kdop;

constexpr int kStack = 64;  // traversal stack; deeper trees report an error
constexpr int kBroadBlock = 64;
constexpr int kSliceDepth = 4;  // broad-phase slices: up to 16 subtrees per tree

#define YC_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return ys_internal_fail(YS_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

struct DevTree {
  const int* left;
  const int* right;
  const int* face;
  Kdop* box;
  int nnodes;
  float* fbox;  // [nnodes][18] the boxes widened to float (lower bounds down, upper up)
};

// inner-node prune in FP32 on the widened boxes: wider again by a relative
// 1e-6 of the magnitudes, far above float rounding, it keeps every subtree
// holding a pair the exact FP64 leaf test accepts
__device__ __forceinline__ bool kdop_overlap_f(const float* a, const float* b, float d1, float d2) {
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const float dd = i < 3 ? d1 : d2;
    const float slack = 1e-6f * (fabsf(a[i]) + fabsf(a[i + 9]) + fabsf(b[i]) + fabsf(b[i + 9])) + 1e-30f;
    if (a[i] > b[i + 9] + dd + slack) return false;
    if (a[i + 9] < b[i] - dd - slack) return false;
  }
  return true;
}

// Boxes of every tree node (BVHNode::refit, src/BVH.cpp:150-160) in one
// launch, bottom-up: thread i computes leaf i's box from its face's nodes,
// then climbs while it is the second of its parent's two children to arrive
// (an atomic count per inner node; the first arrival stops), forming the
// parent's box as the union of its children's. Unions of min / max bounds do
// not depend on the order, so the boxes are those of a refit level by level,
// bit for bit. No thread waits for another: every climb ends at the root or
// at a first arrival.
__device__ __forceinline__ void kdop_load_l2(Kdop& b, const Kdop* src) {
  const double* p = reinterpret_cast<const double*>(src);
#pragma unroll
  for (int k = 0; k < 18; ++k) b.d[k] = __ldcg(p + k);
}
__device__ __forceinline__ void refit_store(const DevTree& t, int n, const Kdop& b) {
  t.box[n] = b;
  for (int k = 0; k < 9; ++k) {
    t.fbox[18 * (int64_t)n + k] = __double2float_rd(b.d[k]);
    t.fbox[18 * (int64_t)n + 9 + k] = __double2float_ru(b.d[k + 9]);
  }
}
__global__ void k_refit_up(DevTree t, const int* __restrict__ leaves, int nleaves, const int* __restrict__ parent,
                           int* arrive, const CFace* __restrict__ faces, CMesh m, int ccd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nleaves) return;
  int n = leaves[i];
  {
    const CFace& fc = faces[t.face[n]];
    Kdop b;
    ys::kdop_node(b, ys::cc_pos(m, fc.v[0], false), ys::cc_pos(m, fc.v[0], true), ccd != 0);
    for (int k = 1; k < 3; ++k) {
      Kdop nb;
      ys::kdop_node(nb, ys::cc_pos(m, fc.v[k], false), ys::cc_pos(m, fc.v[k], true), ccd != 0);
      ys::kdop_add(b, nb);
    }
    refit_store(t, n, b);
  }
  for (;;) {
    const int p = parent[n];
    if (p < 0) return;
    // release: this node's box is visible before the count says so; acquire:
    // the second arrival sees its sibling's box
    cuda::atomic_ref<int, cuda::thread_scope_device> cnt(arrive[p]);
    if (cnt.fetch_add(1, cuda::memory_order_acq_rel) == 0) return;  // the sibling's thread goes on
    Kdop b, rb;
    kdop_load_l2(b, t.box + t.left[p]);
    kdop_load_l2(rb, t.box + t.right[p]);
    ys::kdop_add(b, rb);
    refit_store(t, p, b);
    n = p;
  }
}

struct BroadArgs {
  DevTree cloth, obs;
  const int* leaf_of_face;
  const int* rank;
  const int* upper;
  int nfaces;
  double thickness;
  const int64_t* offset;  // write pass: first slot of each face
  int* out;               // write pass: [P][3]
  int64_t* count;         // count pass: pairs of each face
  int* overflow;
  // active faces (null: all): a pair is reported only if one of its faces is
  // active, obstacle faces never are (update_active and the traversal's
  // active test, src/Collision.cpp:158-182, 289-310)
  const uint8_t* face_active;
  const uint8_t* node_active;  // cloth-tree nodes with an active leaf below
  float thick1, thick2;        // the thickness and sqrt(2) times it, widened, for the FP32 prune
  const int* cslice;           // slice roots of the cloth tree, depth-first order
  const int* oslice;           // and of the obstacle tree
  int ncs, nos;
  // the count pass keeps each (face, slice)'s first kBroadKeep partner faces
  // here ([work][kBroadKeep]); the write pass copies them instead of
  // traversing again when that is all of them
  int* keep;
  // write pass: pair slots available (a pair at or past it is not written
  // and sets bit 1 of *overflow)
  int64_t cap;
};
constexpr int kBroadKeep = 16;

// one thread per (cloth face f, slice): the slices are the subtrees rooted at
// depth kSliceDepth of the cloth tree, then of the obstacle tree, in
// depth-first order, so a face's pairs come out in the order of one
// depth-first traversal of both trees: cloth faces g the reference reports
// with f first, then obstacle faces
template <bool WRITE>
__global__ void k_broad(BroadArgs a) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int S = a.ncs + a.nos;
  if (idx >= (int64_t)a.nfaces * S) return;
  const int f = (int)(idx / S), sl = (int)(idx % S);
  const int pass = sl < a.ncs ? 0 : 1;
  const bool fa = a.face_active == nullptr || a.face_active[f] != 0;
  int64_t c = 0;
  if (WRITE && a.count[idx] <= kBroadKeep) {
    // every partner was kept by the count pass, in traversal order
    const int64_t o = a.offset[idx], nk = a.count[idx];
    for (int64_t j = 0; j < nk; ++j) {
      if (o + j >= a.cap) {
        atomicOr(a.overflow, 2);
        break;
      }
      a.out[3 * (o + j)] = f;
      a.out[3 * (o + j) + 1] = a.keep[idx * kBroadKeep + j];
      a.out[3 * (o + j) + 2] = pass;
    }
    return;
  }
  if (pass == 0 || fa) {
    const DevTree& t = pass == 0 ? a.cloth : a.obs;
    const int root = pass == 0 ? a.cslice[sl] : a.oslice[sl - a.ncs];
    const int leaf = a.leaf_of_face[f];
    const Kdop bf = a.cloth.box[leaf];
    float bfl[18];  // the face's widened box, as refit left it for its leaf
    for (int k = 0; k < 18; ++k) bfl[k] = a.cloth.fbox[18 * (int64_t)leaf + k];
    const int uf = a.upper[f], rf = a.rank[f];
    const int64_t o = WRITE ? a.offset[idx] : 0;
    int stack[kStack];
    int sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
      const int n = stack[--sp];
      if (!fa && a.node_active[n] == 0) continue;  // pass 0 only: no active face below
      const int g = t.face[n];
      if (g >= 0) {
        if (pass == 0) {
          if (g == f || !ys::bvh_first(uf, rf, a.upper[g], a.rank[g])) continue;
        }
        // the FP32 test first: it rejects only boxes the exact test rejects
        if (!kdop_overlap_f(bfl, t.fbox + 18 * (int64_t)n, a.thick1, a.thick2)) continue;
        if (!ys::kdop_overlap(bf, t.box[n], a.thickness)) continue;
        if (WRITE) {
          if (o + c < a.cap) {
            a.out[3 * (o + c)] = f;
            a.out[3 * (o + c) + 1] = g;
            a.out[3 * (o + c) + 2] = pass;
          } else {
            atomicOr(a.overflow, 2);
          }
        } else if (c < kBroadKeep) {
          a.keep[idx * kBroadKeep + c] = g;
        }
        ++c;
      } else {
        if (!kdop_overlap_f(bfl, t.fbox + 18 * (int64_t)n, a.thick1, a.thick2)) continue;
        if (sp + 2 > kStack) {
          atomicOr(a.overflow, 1);
          continue;
        }
        stack[sp++] = t.right[n];
        stack[sp++] = t.left[n];
      }
    }
  }
  if (!WRITE) a.count[idx] = c;
}

// Narrow phase in two kernels. k_narrow_mask: one thread per pair forms the
// k-DOPs of its six nodes and decides which of the 15 tests run (cc_face_pair's
// overlap and shared-node rules). k_narrow_test: one thread per (test, pair),
// test-major, so a warp runs one kind of test on 32 pairs; test t of pair p
// writes slot 15 p + t (type -1: no impact) and counts its impact for the
// pair. The compaction then takes each pair's slots in test order: the
// impacts, and their order, are cc_face_pair's.
// k-DOP of every node's motion (kdop_node of its two positions): cloth node
// i at [i], obstacle node j at [n_nodes + j]
__global__ void k_node_kdop(CMesh m, int n_nodes, int n_obs, int ccd, Kdop* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes + n_obs) return;
  const int id = i < n_nodes ? i : -1 - (i - n_nodes);  // obstacle ids as -1 - id
  Kdop b;
  ys::kdop_node(b, ys::cc_pos(m, id, false), ys::cc_pos(m, id, true), ccd != 0);
  out[i] = b;
}
struct NodeKdops {
  const Kdop* k;
  int n_nodes;
  __device__ __forceinline__ Kdop operator()(int id) const { return k[id >= 0 ? id : n_nodes + (-1 - id)]; }
};
// (np_dev: the pair count on the device, the launch covering npairs >= it
// entries, or null: npairs pairs)
__global__ void k_narrow_mask(const int* __restrict__ pairs, int64_t npairs, const CFace* __restrict__ faces,
                              const CFace* __restrict__ ofaces, NodeKdops nk, double thickness,
                              int* __restrict__ mask, int64_t* __restrict__ count, const int64_t* np_dev) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  if (np_dev && p >= *np_dev) {
    count[p] = 0;  // the scan of the impact counts covers the launch's npairs entries
    mask[p] = 0;
    return;
  }
  const CFace& f0 = faces[pairs[3 * p]];
  const CFace& f1 = pairs[3 * p + 2] ? ofaces[pairs[3 * p + 1]] : faces[pairs[3 * p + 1]];
  mask[p] = ys::cc_face_pair_mask(nk, f0, f1, thickness);
  count[p] = 0;
}
__global__ void k_narrow_test(const int* __restrict__ pairs, int64_t npairs, const CFace* __restrict__ faces,
                              const CFace* __restrict__ ofaces, CMesh m, const int* __restrict__ mask, Impact* slots,
                              unsigned long long* count) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 15 * npairs) return;
  const int t = (int)(idx / npairs);
  const int64_t p = idx - (int64_t)t * npairs;
  // (pairs past a device count have mask 0: k_narrow_mask)
  Impact& out = slots[15 * p + t];
  out.type = -1;
  if (!((mask[p] >> t) & 1)) return;
  const CFace& f0 = faces[pairs[3 * p]];
  const CFace& f1 = pairs[3 * p + 2] ? ofaces[pairs[3 * p + 1]] : faces[pairs[3 * p + 1]];
  int type, ids[4];
  ys::cc_pair_test_nodes(f0, f1, t, type, ids);
  const double* xs[4];
  const double* xps[4];
  for (int k = 0; k < 4; ++k) {
    xs[k] = ys::cc_pos(m, ids[k], false);
    xps[k] = ys::cc_pos(m, ids[k], true);
  }
  Impact im;
  if (ys::cc_test(type, xs, xps, im)) {
    for (int k = 0; k < 4; ++k) im.node[k] = ids[k];
    out = im;
    atomicAdd(count + p, 1ull);
  }
}

// (np_dev as for k_narrow_mask; impacts at or past cap are not written and
// set bit 2 of *overflow)
__global__ void k_compact(const Impact* __restrict__ slots, const int64_t* __restrict__ count,
                          const int64_t* __restrict__ offset, int64_t npairs, ys_impact* out,
                          const int64_t* np_dev, int64_t cap, int* overflow) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  if (np_dev && p >= *np_dev) return;
  int64_t k = 0;
  for (int t = 0; t < 15 && k < count[p]; ++t) {
    const Impact& s = slots[15 * p + t];
    if (s.type < 0) continue;
    if (offset[p] + k >= cap) {
      atomicOr(overflow, 4);
      return;
    }
    ys_impact& r = out[offset[p] + k++];
    r.type = s.type;
    for (int q = 0; q < 4; ++q) r.nodes[q] = s.node[q];
    r.t = s.t;
    for (int q = 0; q < 4; ++q) r.w[q] = s.w[q];
    for (int q = 0; q < 3; ++q) r.n[q] = s.n[q];
    r.pair = p;
  }
}

// exclusive scan of counts[n] into offset[n] (+ total): tiles of kScanTile
// entries scanned by one block each (8 per thread, then a warp-shuffle scan
// of the thread sums), the tile sums scanned by one block, then added back;
// integer sums, so any grouping gives the same offsets
constexpr int kScanThreads = 256, kScanPer = 8, kScanTile = kScanThreads * kScanPer;
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* warp_sums, int64_t* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t incl = v;
  for (int d = 1; d < 32; d <<= 1) {
    const int64_t o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  if (lane == 31) warp_sums[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    int64_t w = lane < nw ? warp_sums[lane] : 0;
    int64_t wi = w;
    for (int d = 1; d < 32; d <<= 1) {
      const int64_t o = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += o;
    }
    if (lane < nw) warp_sums[lane] = wi - w;  // exclusive prefix of the warps
    if (lane == nw - 1) *total = wi;
  }
  __syncthreads();
  return warp_sums[wid] + incl - v;
}
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int64_t* __restrict__ c, int64_t n,
                                                             int64_t* __restrict__ off, int64_t* __restrict__ sums) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t total;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  int64_t v[kScanPer], s = 0;
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = base + k < n ? c[base + k] : 0;
    s += v[k];
  }
  int64_t run = block_exclusive_scan(s, warp_sums, &total);
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < n) off[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}
// one block: exclusive scan of the nb tile sums in place (nb up to
// kScanTile per pass, looped), the grand total in *total
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int64_t* sums, int64_t nb, int64_t* total) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t part;
  int64_t carry = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += kScanTile) {
    const int64_t base = b0 + (int64_t)threadIdx.x * kScanPer;
    int64_t v[kScanPer], s = 0;
    for (int k = 0; k < kScanPer; ++k) {
      v[k] = base + k < nb ? sums[base + k] : 0;
      s += v[k];
    }
    int64_t run = carry + block_exclusive_scan(s, warp_sums, &part);
    for (int k = 0; k < kScanPer; ++k) {
      if (base + k < nb) sums[base + k] = run;
      run += v[k];
    }
    carry += part;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}
__global__ void k_scan_add(int64_t* off, int64_t n, const int64_t* __restrict__ sums) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) off[i] += sums[i / kScanTile];
}

template <class T>
struct DVec {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t cnt) {
    if (cnt <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(cnt, 1) * sizeof(T));
    if (e == cudaSuccess) n = std::max<size_t>(cnt, 1);
    return e;
  }
  ~DVec() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct ys_collider {
  int device = 0;
  cudaStream_t stream = nullptr;
  int n_nodes = 0, n_faces = 0, n_obs_nodes = 0, n_obs_faces = 0;
  double thickness = 5e-4;
  int ccd = 1;
  std::vector<int> fv, ofv;  // face node ids (host, obstacle ids local)
  DVec<CFace> faces, ofaces;
  DVec<double> x, xp, ox, oxp;
  std::vector<double> hx, hxp, hox, hoxp;  // host copies for the tree builds
  // trees
  ys::BvhTree ct, ot;
  DVec<int> c_left, c_right, c_face, c_lof, c_rank, c_upper, o_left, o_right, o_face;
  // bottom-up refit: parent of each node (-1 at the root), the leaves, and
  // the arrival counters of the inner nodes
  DVec<int> c_parent, c_leaves, c_arrive, o_parent, o_leaves, o_arrive;
  DVec<Kdop> c_box, o_box;
  DVec<float> c_fbox, o_fbox;
  // outputs
  DVec<int64_t> counts, offsets, sums, total;
  DVec<int> keep;  // the broad phase's kept partners ([work][kBroadKeep])
  DVec<int> pairs;
  int64_t npairs = 0;
  DVec<Impact> slots;
  DVec<int64_t> icount, ioffset;
  DVec<int> tmask;  // narrow phase: the tests each pair runs (bit t)
  DVec<Kdop> nkdop;  // narrow phase: every node's motion k-DOP (cloth, then obstacle)
  DVec<ys_impact> impacts;
  int64_t nimpacts = 0;
  DVec<int> overflow;
  int64_t* pin = nullptr;  // pinned host words: [0] a scan's total, [1] the broad phase's overflow flag
  // one-wait detection rounds: capacities of the pair and impact buffers
  // (by round kind: [0] every face, [1] the active faces of later rounds,
  // which find far fewer pairs), and the pinned copy of the impacts
  int64_t cap_pairs[2] = {4096, 1024}, cap_imp[2] = {1024, 256};
  ys_impact* pin_imp = nullptr;
  int64_t pin_imp_cap = 0;
  bool have_pairs = false, have_impacts = false;
  // impact-zone response
  DVec<uint8_t> face_active, node_active;
  std::vector<uint8_t> h_node_active;
  ys::ZoneResponse resp;
  std::vector<double> resp_x0;  // positions before the response
  bool have_response = false;
  double resp_h = 0.0, resp_damp = 0.0;
  bool obs_tree_valid = false;  // the obstacle tree and device copies match hox / hoxp
  int max_zone_impacts = 65536;
  std::vector<int> h_cslice, h_oslice;  // broad-phase slice roots
  DVec<int> cslice, oslice;
  // host threads for the cloth tree's build (the obstacle's, when it is
  // rebuilt, runs beside it on a thread of its own)
  std::unique_ptr<ys::BuildPool> pool;
  ~ys_collider() {
    if (pin) cudaFreeHost(pin);
    if (pin_imp) cudaFreeHost(pin_imp);
  }
};

namespace {

ys_status upload_tree(ys_collider* c, const ys::BvhTree& t, DVec<int>& l, DVec<int>& r, DVec<int>& f,
                      DVec<Kdop>& box, DVec<int>& parent, DVec<int>& leaves, DVec<int>& arrive) {
  const size_t nn = t.face.size();
  YC_CUDA(l.reserve(nn));
  YC_CUDA(r.reserve(nn));
  YC_CUDA(f.reserve(nn));
  YC_CUDA(box.reserve(nn));
  YC_CUDA(parent.reserve(std::max<size_t>(nn, 1)));
  YC_CUDA(leaves.reserve(std::max<size_t>(nn, 1)));
  YC_CUDA(arrive.reserve(std::max<size_t>(nn, 1)));
  std::vector<int> par(nn, -1), lf;
  for (size_t n = 0; n < nn; ++n) {
    if (t.face[n] >= 0) {
      lf.push_back((int)n);
    } else {
      par[t.left[n]] = (int)n;
      par[t.right[n]] = (int)n;
    }
  }
  if (nn) {
    YC_CUDA(cudaMemcpyAsync(l.p, t.left.data(), nn * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    YC_CUDA(cudaMemcpyAsync(r.p, t.right.data(), nn * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    YC_CUDA(cudaMemcpyAsync(f.p, t.face.data(), nn * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    YC_CUDA(cudaMemcpyAsync(parent.p, par.data(), nn * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    YC_CUDA(cudaMemcpyAsync(leaves.p, lf.data(), lf.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    YC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return YS_OK;
}

ys_status refit(ys_collider* c, bool obstacle) {
  const ys::BvhTree& t = obstacle ? c->ot : c->ct;
  if (t.face.empty()) return YS_OK;
  DVec<float>& fb = obstacle ? c->o_fbox : c->c_fbox;
  YC_CUDA(fb.reserve(18 * t.face.size()));
  DevTree dt{obstacle ? c->o_left.p : c->c_left.p, obstacle ? c->o_right.p : c->c_right.p,
             obstacle ? c->o_face.p : c->c_face.p, obstacle ? c->o_box.p : c->c_box.p, (int)t.face.size(), fb.p};
  CMesh m{c->x.p, c->xp.p, c->ox.p, c->oxp.p};
  // one launch: every leaf's thread computes its box and carries the unions
  // up as far as it is the second child to arrive
  const int nleaves = obstacle ? c->n_obs_faces : c->n_faces;
  int* arrive = obstacle ? c->o_arrive.p : c->c_arrive.p;
  YC_CUDA(cudaMemsetAsync(arrive, 0, sizeof(int) * t.face.size(), c->stream));
  k_refit_up<<<(nleaves + 127) / 128, 128, 0, c->stream>>>(dt, obstacle ? c->o_leaves.p : c->c_leaves.p, nleaves,
                                                          obstacle ? c->o_parent.p : c->c_parent.p, arrive,
                                                          obstacle ? c->ofaces.p : c->faces.p, m, c->ccd);
  YC_CUDA(cudaGetLastError());
  return YS_OK;
}

// Exclusive scan of counts into off; *total_host receives the sum. With
// flag, the device word is read back in the same wait (into *flag_host).
// One host wait per scan.
// the scan's kernels alone: exclusive scan of counts[n] into off, the total
// into *total_dev (the tile sums in c->sums, reserved by the caller)
void scan_kernels(ys_collider* c, const int64_t* counts, int64_t n, int64_t* off, int64_t* total_dev) {
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (n > 0) {
    k_scan_tiles<<<(unsigned)nb, kScanThreads, 0, c->stream>>>(counts, n, off, c->sums.p);
    k_scan_sums<<<1, kScanThreads, 0, c->stream>>>(c->sums.p, nb, total_dev);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(off, n, c->sums.p);
  } else {
    cudaMemsetAsync(total_dev, 0, sizeof(int64_t), c->stream);
  }
}

ys_status scan(ys_collider* c, const int64_t* counts, int64_t n, int64_t* off, int64_t* total_host,
               const int* flag = nullptr, int* flag_host = nullptr) {
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  YC_CUDA(c->sums.reserve(std::max<int64_t>(nb, 1)));
  YC_CUDA(c->total.reserve(1));
  c->pin[0] = 0;
  c->pin[1] = 0;
  if (n > 0) {
    k_scan_tiles<<<(unsigned)nb, kScanThreads, 0, c->stream>>>(counts, n, off, c->sums.p);
    k_scan_sums<<<1, kScanThreads, 0, c->stream>>>(c->sums.p, nb, c->total.p);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(off, n, c->sums.p);
    YC_CUDA(cudaGetLastError());
    YC_CUDA(cudaMemcpyAsync(c->pin, c->total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  }
  if (flag) YC_CUDA(cudaMemcpyAsync(c->pin + 1, flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  *total_host = c->pin[0];
  if (flag_host) *flag_host = (int)(reinterpret_cast<const int*>(c->pin + 1)[0]);
  return YS_OK;
}

void edges_of(const int* fv, int f, int e[3][2], bool obstacle, const std::vector<int>* ofv) {
  (void)ofv;
  for (int a = 0; a < 3; ++a) {
    const int b = a != 2 ? a + 1 : 0;
    e[a][0] = fv[3 * f + a];
    e[a][1] = fv[3 * f + b];
    if (obstacle && e[a][0] > e[a][1]) std::swap(e[a][0], e[a][1]);
  }
}

// roots of the subtrees at depth `depth` (and leaves above it), in
// depth-first order: the broad phase's slices
std::vector<int> tree_slices(const ys::BvhTree& t, int depth) {
  std::vector<int> out;
  if (t.face.empty()) return out;
  std::vector<int> st{0};
  while (!st.empty()) {
    const int n = st.back();
    st.pop_back();
    if (t.face[n] >= 0 || t.depth[n] >= depth) {
      out.push_back(n);
    } else {
      st.push_back(t.right[n]);
      st.push_back(t.left[n]);
    }
  }
  return out;
}

ys_status upload_slices(ys_collider* c, bool obstacle) {
  const std::vector<int>& h = obstacle ? c->h_oslice : c->h_cslice;
  DVec<int>& d = obstacle ? c->oslice : c->cslice;
  YC_CUDA(d.reserve(std::max<size_t>(h.size(), 1)));
  if (!h.empty()) YC_CUDA(cudaMemcpyAsync(d.p, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, c->stream));
  return YS_OK;
}

// the broad phase's arguments (the write pass's offsets, output and capacity
// are filled in by the caller); reserves the per-(face, slice) buffers
ys_status broad_args(ys_collider* c, bool masked, BroadArgs& a, int64_t& work) {
  const int ncs = (int)c->h_cslice.size(), nos = (int)c->h_oslice.size();
  work = (int64_t)c->n_faces * (ncs + nos);
  // the per-(face, slice) counts and offsets: sized before any pointer to
  // them is taken (a reserve may move them)
  YC_CUDA(c->counts.reserve(std::max<int64_t>(work, 1)));
  YC_CUDA(c->offsets.reserve(std::max<int64_t>(work, 1)));
  YC_CUDA(c->keep.reserve(std::max<int64_t>(work * kBroadKeep, 1)));
  a = BroadArgs{};
  a.cloth = DevTree{c->c_left.p, c->c_right.p, c->c_face.p, c->c_box.p, (int)c->ct.face.size(), c->c_fbox.p};
  a.obs = DevTree{c->o_left.p, c->o_right.p, c->o_face.p, c->o_box.p, (int)c->ot.face.size(), c->o_fbox.p};
  a.thick1 = (float)(c->thickness * (1.0 + 1e-6));
  a.thick2 = (float)(std::sqrt(2.0) * c->thickness * (1.0 + 1e-6));
  a.leaf_of_face = c->c_lof.p;
  a.rank = c->c_rank.p;
  a.upper = c->c_upper.p;
  a.nfaces = c->n_faces;
  a.thickness = c->thickness;
  a.count = c->counts.p;
  a.overflow = c->overflow.p;
  a.face_active = masked ? c->face_active.p : nullptr;
  a.node_active = masked ? c->node_active.p : nullptr;
  a.cslice = c->cslice.p;
  a.oslice = c->oslice.p;
  a.ncs = ncs;
  a.nos = nos;
  a.keep = c->keep.p;
  return YS_OK;
}

ys_status broad_phase(ys_collider* c, bool masked) {
  BroadArgs a;
  int64_t work = 0;
  ys_status s = broad_args(c, masked, a, work);
  if (s != YS_OK) return s;
  YC_CUDA(cudaMemsetAsync(c->overflow.p, 0, sizeof(int), c->stream));
  const unsigned g = (unsigned)((work + kBroadBlock - 1) / kBroadBlock);
  if (work) k_broad<false><<<g, kBroadBlock, 0, c->stream>>>(a);
  YC_CUDA(cudaGetLastError());
  int ovf = 0;
  s = scan(c, c->counts.p, work, c->offsets.p, &c->npairs, c->overflow.p, &ovf);
  if (s != YS_OK) return s;
  if (ovf) return ys_internal_fail(YS_ERR_ARG, "BVH deeper than the traversal stack");
  // a face pairs at most once with every other face
  if (c->npairs < 0 || c->npairs > (int64_t)c->n_faces * ((int64_t)c->n_faces + c->n_obs_faces))
    return ys_internal_fail(YS_ERR_CUDA, "broad phase produced an impossible pair count");
  YC_CUDA(c->pairs.reserve(3 * (size_t)std::max<int64_t>(c->npairs, 1)));
  a.offset = c->offsets.p;
  a.out = c->pairs.p;
  a.cap = c->npairs;
  if (work) k_broad<true><<<g, kBroadBlock, 0, c->stream>>>(a);
  YC_CUDA(cudaGetLastError());
  // no wait: the pairs are read on the stream (narrow phase) or by a
  // synchronous copy (ys_collider_get_pairs)
  c->have_pairs = true;
  c->have_impacts = false;
  return YS_OK;
}

ys_status narrow_phase(ys_collider* c) {
  const int64_t P = c->npairs;
  YC_CUDA(c->slots.reserve(15 * (size_t)std::max<int64_t>(P, 1)));
  YC_CUDA(c->icount.reserve(std::max<int64_t>(P, 1)));
  YC_CUDA(c->ioffset.reserve(std::max<int64_t>(P, 1)));
  YC_CUDA(c->tmask.reserve(std::max<int64_t>(P, 1)));
  YC_CUDA(c->nkdop.reserve(std::max(c->n_nodes + c->n_obs_nodes, 1)));
  CMesh m{c->x.p, c->xp.p, c->ox.p, c->oxp.p};
  if (P) {
    const int nn = c->n_nodes + c->n_obs_nodes;
    k_node_kdop<<<(nn + 127) / 128, 128, 0, c->stream>>>(m, c->n_nodes, c->n_obs_nodes, c->ccd, c->nkdop.p);
    k_narrow_mask<<<(unsigned)((P + 127) / 128), 128, 0, c->stream>>>(c->pairs.p, P, c->faces.p, c->ofaces.p,
                                                                       NodeKdops{c->nkdop.p, c->n_nodes},
                                                                       c->thickness, c->tmask.p, c->icount.p, nullptr);
    k_narrow_test<<<(unsigned)((15 * P + 127) / 128), 128, 0, c->stream>>>(
        c->pairs.p, P, c->faces.p, c->ofaces.p, m, c->tmask.p, c->slots.p,
        reinterpret_cast<unsigned long long*>(c->icount.p));
    YC_CUDA(cudaGetLastError());
  }
  ys_status s = scan(c, c->icount.p, P, c->ioffset.p, &c->nimpacts);
  if (s != YS_OK) return s;
  YC_CUDA(c->impacts.reserve(std::max<int64_t>(c->nimpacts, 1)));
  if (P) {
    k_compact<<<(unsigned)((P + 127) / 128), 128, 0, c->stream>>>(c->slots.p, c->icount.p, c->ioffset.p, P,
                                                                   c->impacts.p, nullptr, c->nimpacts,
                                                                   c->overflow.p);
    YC_CUDA(cudaGetLastError());
  }
  // no wait: the impacts are read by a synchronous copy on this stream
  c->have_impacts = true;
  return YS_OK;
}

// One detection round of the impact-zone response with a single wait: the
// pair and impact counts stay on the device, and the narrow phase, the scans
// and the compaction run over buffers sized by capacities the collider
// keeps (grown from the counts a round finds). The counts, the overflow
// flags and up to cap_imp impacts come back in one copy. A round whose pairs
// or impacts outgrew the capacities (flag bits 1, 2) is run again with
// capacities that hold them; its pair list, impacts and their order are the
// two-wait path's (the same kernels over the same counts).
ys_status detect_one_wait(ys_collider* c, bool masked, std::vector<ys_impact>& got) {
  for (int attempt = 0; attempt < 3; ++attempt) {
    BroadArgs a;
    int64_t work = 0;
    ys_status s = broad_args(c, masked, a, work);
    if (s != YS_OK) return s;
    const int kind = masked ? 1 : 0;
    const int64_t cp = c->cap_pairs[kind], ci = c->cap_imp[kind];
    const int64_t nb = (std::max<int64_t>(work, cp) + kScanTile - 1) / kScanTile;
    YC_CUDA(c->sums.reserve(std::max<int64_t>(nb, 1)));
    YC_CUDA(c->total.reserve(2));
    YC_CUDA(c->pairs.reserve(3 * (size_t)cp));
    YC_CUDA(c->slots.reserve(15 * (size_t)cp));
    YC_CUDA(c->icount.reserve(cp));
    YC_CUDA(c->ioffset.reserve(cp));
    YC_CUDA(c->tmask.reserve(cp));
    YC_CUDA(c->nkdop.reserve(std::max(c->n_nodes + c->n_obs_nodes, 1)));
    YC_CUDA(c->impacts.reserve(ci));
    if (c->pin_imp_cap < ci) {
      if (c->pin_imp) cudaFreeHost(c->pin_imp);
      c->pin_imp = nullptr;
      c->pin_imp_cap = 0;
      YC_CUDA(cudaMallocHost(reinterpret_cast<void**>(&c->pin_imp), sizeof(ys_impact) * (size_t)ci));
      c->pin_imp_cap = ci;
    }
    int64_t* np_dev = c->total.p;      // pairs
    int64_t* ni_dev = c->total.p + 1;  // impacts
    YC_CUDA(cudaMemsetAsync(c->overflow.p, 0, sizeof(int), c->stream));
    const unsigned g = (unsigned)((work + kBroadBlock - 1) / kBroadBlock);
    if (work) k_broad<false><<<g, kBroadBlock, 0, c->stream>>>(a);
    scan_kernels(c, c->counts.p, work, c->offsets.p, np_dev);
    a.offset = c->offsets.p;
    a.out = c->pairs.p;
    a.cap = cp;
    if (work) k_broad<true><<<g, kBroadBlock, 0, c->stream>>>(a);
    CMesh m{c->x.p, c->xp.p, c->ox.p, c->oxp.p};
    const int nn = c->n_nodes + c->n_obs_nodes;
    k_node_kdop<<<(nn + 127) / 128, 128, 0, c->stream>>>(m, c->n_nodes, c->n_obs_nodes, c->ccd, c->nkdop.p);
    k_narrow_mask<<<(unsigned)((cp + 127) / 128), 128, 0, c->stream>>>(c->pairs.p, cp, c->faces.p, c->ofaces.p,
                                                                        NodeKdops{c->nkdop.p, c->n_nodes},
                                                                        c->thickness, c->tmask.p, c->icount.p,
                                                                        np_dev);
    k_narrow_test<<<(unsigned)((15 * cp + 127) / 128), 128, 0, c->stream>>>(
        c->pairs.p, cp, c->faces.p, c->ofaces.p, m, c->tmask.p, c->slots.p,
        reinterpret_cast<unsigned long long*>(c->icount.p));
    scan_kernels(c, c->icount.p, cp, c->ioffset.p, ni_dev);
    k_compact<<<(unsigned)((cp + 127) / 128), 128, 0, c->stream>>>(c->slots.p, c->icount.p, c->ioffset.p, cp,
                                                                    c->impacts.p, np_dev, ci, c->overflow.p);
    YC_CUDA(cudaGetLastError());
    YC_CUDA(cudaMemcpyAsync(c->pin, c->total.p, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    YC_CUDA(cudaMemcpyAsync(c->pin + 2, c->overflow.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    YC_CUDA(cudaMemcpyAsync(c->pin_imp, c->impacts.p, sizeof(ys_impact) * (size_t)ci, cudaMemcpyDeviceToHost,
                            c->stream));
    YC_CUDA(cudaStreamSynchronize(c->stream));
    const int64_t np = c->pin[0], ni = c->pin[1];
    const int ovf = (int)(reinterpret_cast<const int*>(c->pin + 2)[0]);
    if (ovf & 1) return ys_internal_fail(YS_ERR_ARG, "BVH deeper than the traversal stack");
    if (np < 0 || np > (int64_t)c->n_faces * ((int64_t)c->n_faces + c->n_obs_faces))
      return ys_internal_fail(YS_ERR_CUDA, "broad phase produced an impossible pair count");
    c->npairs = np;
    c->nimpacts = ni;
    if (ovf & 6) {  // grow and run the round again
      c->cap_pairs[kind] = std::max(c->cap_pairs[kind], np + np / 2 + 1024);
      c->cap_imp[kind] = std::max(c->cap_imp[kind], ni + ni / 2 + 256);
      continue;
    }
    c->have_pairs = c->have_impacts = true;
    got.assign(c->pin_imp, c->pin_imp + ni);
    return YS_OK;
  }
  return ys_internal_fail(YS_ERR_CUDA, "detection round: capacities did not settle");
}

// marks the cloth-tree nodes with an active leaf below (host tree)
// (preorder numbering puts both children after their parent, so one pass
// from the last node to the root sees every child before its parent)
void mark_nodes(const ys::BvhTree& t, const uint8_t* fa, std::vector<uint8_t>& out) {
  for (int n = (int)t.face.size() - 1; n >= 0; --n) {
    const int f = t.face[n];
    out[n] = f >= 0 ? (fa[f] != 0 ? 1 : 0) : (out[t.left[n]] | out[t.right[n]]);
  }
}

}  // namespace

extern "C" {

ys_status ys_cloth_mesh_topology(int32_t width, int32_t length, int32_t* faces, int32_t* face_edges) {
  if (width < 2 || length < 2 || !faces) return ys_internal_fail(YS_ERR_ARG, "bad cloth mesh size");
  // mesh faces of Cloth::build (src/Cloth.cpp:271-294): cell (i, j), i outer,
  // faces (tl, tr, br) and (tl, br, bl); mesh edges along warp and weft point
  // to the higher u / v, the cell diagonal from tl to br
  int f = 0;
  for (int i = 0; i < width - 1; ++i)
    for (int j = 0; j < length - 1; ++j) {
      const int tl = i + j * width, tr = tl + 1, bl = tl + width, br = bl + 1;
      const int tri[2][3] = {{tl, tr, br}, {tl, br, bl}};
      for (int q = 0; q < 2; ++q, ++f) {
        for (int k = 0; k < 3; ++k) faces[3 * f + k] = tri[q][k];
        if (!face_edges) continue;
        for (int a = 0; a < 3; ++a) {
          const int b = a != 2 ? a + 1 : 0;
          int u0 = tri[q][a], u1 = tri[q][b];
          if (u0 > u1) std::swap(u0, u1);  // every cloth mesh edge runs from its lower node
          face_edges[6 * f + 2 * a] = u0;
          face_edges[6 * f + 2 * a + 1] = u1;
        }
      }
    }
  return YS_OK;
}

ys_status ys_collider_create(int32_t n_nodes, int32_t n_faces, const int32_t* faces, const int32_t* face_edges,
                             int32_t n_obs_nodes, int32_t n_obs_faces, const int32_t* obs_faces, double thickness,
                             int32_t ccd, int32_t device, void* cuda_stream, ys_collider** out) {
  if (!out || n_nodes <= 0 || n_faces <= 0 || !faces || !face_edges || n_obs_nodes < 0 || n_obs_faces < 0 ||
      (n_obs_faces > 0 && !obs_faces))
    return ys_internal_fail(YS_ERR_ARG, "bad collider arguments");
  for (int i = 0; i < 3 * n_faces; ++i)
    if (faces[i] < 0 || faces[i] >= n_nodes) return ys_internal_fail(YS_ERR_ARG, "cloth face node out of range");
  for (int i = 0; i < 3 * n_obs_faces; ++i)
    if (obs_faces[i] < 0 || obs_faces[i] >= n_obs_nodes)
      return ys_internal_fail(YS_ERR_ARG, "obstacle face node out of range");
  YC_CUDA(cudaSetDevice(device));
  ys_collider* c = new ys_collider();
  c->device = device;
  c->stream = static_cast<cudaStream_t>(cuda_stream);
  c->n_nodes = n_nodes;
  c->n_faces = n_faces;
  c->n_obs_nodes = n_obs_nodes;
  c->n_obs_faces = n_obs_faces;
  c->thickness = thickness;
  c->ccd = ccd ? 1 : 0;
  c->fv.assign(faces, faces + 3 * n_faces);
  c->ofv.assign(obs_faces, obs_faces + 3 * (size_t)n_obs_faces);
  std::vector<CFace> hf(n_faces), ho(n_obs_faces);
  for (int f = 0; f < n_faces; ++f)
    for (int k = 0; k < 3; ++k) {
      hf[f].v[k] = faces[3 * f + k];
      hf[f].e[k][0] = face_edges[6 * f + 2 * k];
      hf[f].e[k][1] = face_edges[6 * f + 2 * k + 1];
    }
  // obstacle meshes as load_obj builds them (src/Loader.cpp:317-340): edges
  // run from the lower node id; node ids are stored as -1 - id
  for (int f = 0; f < n_obs_faces; ++f) {
    int e[3][2];
    edges_of(obs_faces, f, e, true, nullptr);
    for (int k = 0; k < 3; ++k) {
      ho[f].v[k] = -1 - obs_faces[3 * f + k];
      ho[f].e[k][0] = -1 - e[k][0];
      ho[f].e[k][1] = -1 - e[k][1];
    }
  }
  auto cleanup = [&](ys_status s) {
    delete c;
    return s;
  };
  if (c->faces.reserve(n_faces) != cudaSuccess || c->ofaces.reserve(n_obs_faces) != cudaSuccess ||
      c->x.reserve(3 * (size_t)n_nodes) != cudaSuccess || c->xp.reserve(3 * (size_t)n_nodes) != cudaSuccess ||
      c->ox.reserve(3 * (size_t)n_obs_nodes) != cudaSuccess || c->oxp.reserve(3 * (size_t)n_obs_nodes) != cudaSuccess ||
      c->overflow.reserve(1) != cudaSuccess || c->counts.reserve(n_faces) != cudaSuccess ||
      c->offsets.reserve(n_faces) != cudaSuccess || c->c_lof.reserve(n_faces) != cudaSuccess ||
      c->c_rank.reserve(n_faces) != cudaSuccess || c->c_upper.reserve(n_faces) != cudaSuccess ||
      cudaMallocHost(reinterpret_cast<void**>(&c->pin), 4 * sizeof(int64_t)) != cudaSuccess)
    return cleanup(ys_internal_fail(YS_ERR_CUDA, "cudaMalloc failed"));
  if (cudaMemcpy(c->faces.p, hf.data(), sizeof(CFace) * n_faces, cudaMemcpyHostToDevice) != cudaSuccess ||
      (n_obs_faces && cudaMemcpy(c->ofaces.p, ho.data(), sizeof(CFace) * n_obs_faces, cudaMemcpyHostToDevice) !=
                          cudaSuccess))
    return cleanup(ys_internal_fail(YS_ERR_CUDA, "cudaMemcpy failed"));
  {
    const unsigned hc = std::thread::hardware_concurrency();
    const int nthreads = (int)std::min(4u, std::max(1u, hc));
    if (nthreads > 1) c->pool.reset(new ys::BuildPool(nthreads));
  }
  *out = c;
  return YS_OK;
}

void ys_collider_destroy(ys_collider* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  delete c;
}

ys_status ys_collider_set_positions(ys_collider* c, const double* x, const double* x_prev, const double* obs_x,
                                    const double* obs_x_prev, int32_t flags) {
  if (!c || !x || !x_prev || (c->n_obs_nodes > 0 && (!obs_x || !obs_x_prev)))
    return ys_internal_fail(YS_ERR_ARG, "bad collider positions");
  YC_CUDA(cudaSetDevice(c->device));
  const size_t n3 = 3 * (size_t)c->n_nodes, o3 = 3 * (size_t)c->n_obs_nodes;
  c->hx.resize(n3);
  c->hxp.resize(n3);
  const cudaMemcpyKind kind = (flags & YS_ON_DEVICE) ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
  YC_CUDA(cudaMemcpy(c->hx.data(), x, n3 * sizeof(double), kind));
  YC_CUDA(cudaMemcpy(c->hxp.data(), x_prev, n3 * sizeof(double), kind));
  // an obstacle whose positions are bit-identical to the last call's keeps its
  // tree: the build is a function of the positions alone, so the rebuild the
  // reference does every call would give the same tree and boxes
  bool same_obstacle = false;
  if (o3) {
    std::vector<double> ox(o3), oxp(o3);
    YC_CUDA(cudaMemcpy(ox.data(), obs_x, o3 * sizeof(double), kind));
    YC_CUDA(cudaMemcpy(oxp.data(), obs_x_prev, o3 * sizeof(double), kind));
    same_obstacle = c->obs_tree_valid && c->hox.size() == o3 &&
                    std::memcmp(ox.data(), c->hox.data(), o3 * sizeof(double)) == 0 &&
                    std::memcmp(oxp.data(), c->hoxp.data(), o3 * sizeof(double)) == 0;
    c->hox.swap(ox);
    c->hoxp.swap(oxp);
  } else {
    c->hox.clear();
    c->hoxp.clear();
  }
  YC_CUDA(cudaMemcpyAsync(c->x.p, c->hx.data(), n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaMemcpyAsync(c->xp.p, c->hxp.data(), n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (o3 && !same_obstacle) {
    YC_CUDA(cudaMemcpyAsync(c->ox.p, c->hox.data(), o3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    YC_CUDA(cudaMemcpyAsync(c->oxp.p, c->hoxp.data(), o3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  // the trees of a fresh AccelStruct (src/CollisionUtil.cpp:3-9): rebuilt
  // from these positions, as Collision::collision_response does every call;
  // the obstacle's on a second host thread
  std::future<ys::BvhTree> obs_tree;
  if (!same_obstacle)
    obs_tree = std::async(std::launch::async, [c] {
      std::vector<int> overts(c->n_obs_nodes);
      for (int i = 0; i < c->n_obs_nodes; ++i) overts[i] = i;
      return ys::bvh_build(c->n_obs_faces, c->ofv.data(), c->n_obs_nodes, overts.data(), c->hox.data(),
                           c->hoxp.data(), c->ccd != 0);
    });
  std::vector<int> verts(c->n_nodes);
  for (int i = 0; i < c->n_nodes; ++i) verts[i] = i;
  c->ct = ys::bvh_build(c->n_faces, c->fv.data(), c->n_nodes, verts.data(), c->hx.data(), c->hxp.data(), c->ccd != 0,
                        c->pool.get());
  if (!same_obstacle) c->ot = obs_tree.get();
  ys_status s;
  if ((s = upload_tree(c, c->ct, c->c_left, c->c_right, c->c_face, c->c_box, c->c_parent, c->c_leaves,
                       c->c_arrive)) != YS_OK)
    return s;
  if (!same_obstacle &&
      (s = upload_tree(c, c->ot, c->o_left, c->o_right, c->o_face, c->o_box, c->o_parent, c->o_leaves,
                       c->o_arrive)) != YS_OK)
    return s;
  c->h_cslice = tree_slices(c->ct, kSliceDepth);
  if ((s = upload_slices(c, false)) != YS_OK) return s;
  if (!same_obstacle) {
    c->h_oslice = tree_slices(c->ot, kSliceDepth);
    if ((s = upload_slices(c, true)) != YS_OK) return s;
  }
  YC_CUDA(cudaMemcpyAsync(c->c_lof.p, c->ct.leaf_of_face.data(), sizeof(int) * c->n_faces, cudaMemcpyHostToDevice,
                          c->stream));
  YC_CUDA(cudaMemcpyAsync(c->c_rank.p, c->ct.rank.data(), sizeof(int) * c->n_faces, cudaMemcpyHostToDevice, c->stream));
  YC_CUDA(cudaMemcpyAsync(c->c_upper.p, c->ct.upper.data(), sizeof(int) * c->n_faces, cudaMemcpyHostToDevice,
                          c->stream));
  if ((s = refit(c, false)) != YS_OK) return s;
  if (!same_obstacle && (s = refit(c, true)) != YS_OK) return s;
  YC_CUDA(cudaStreamSynchronize(c->stream));
  c->obs_tree_valid = true;
  c->have_pairs = c->have_impacts = false;
  return YS_OK;
}

ys_status ys_collider_find_pairs(ys_collider* c, int64_t* n_pairs) {
  if (!c || c->ct.face.empty()) return ys_internal_fail(YS_ERR_ARG, "ys_collider_find_pairs before set_positions");
  YC_CUDA(cudaSetDevice(c->device));
  ys_status s = broad_phase(c, false);
  if (s != YS_OK) return s;
  if (n_pairs) *n_pairs = c->npairs;
  return YS_OK;
}

ys_status ys_collider_get_pairs(ys_collider* c, int32_t* pairs, int64_t cap) {
  if (!c || !c->have_pairs) return ys_internal_fail(YS_ERR_ARG, "no pairs found yet");
  if (cap < c->npairs) return ys_internal_fail(YS_ERR_ARG, "pair buffer too small");
  YC_CUDA(cudaSetDevice(c->device));
  if (c->npairs)
    YC_CUDA(cudaMemcpyAsync(pairs, c->pairs.p, sizeof(int) * 3 * c->npairs, cudaMemcpyDeviceToHost, c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YS_OK;
}

ys_status ys_collider_find_impacts(ys_collider* c, int64_t* n_impacts) {
  if (!c || !c->have_pairs) return ys_internal_fail(YS_ERR_ARG, "ys_collider_find_impacts before find_pairs");
  YC_CUDA(cudaSetDevice(c->device));
  ys_status s = narrow_phase(c);
  if (s != YS_OK) return s;
  if (n_impacts) *n_impacts = c->nimpacts;
  return YS_OK;
}

ys_status ys_collider_get_impacts(ys_collider* c, ys_impact* impacts, int64_t cap) {
  if (!c || !c->have_impacts) return ys_internal_fail(YS_ERR_ARG, "no impacts found yet");
  if (cap < c->nimpacts) return ys_internal_fail(YS_ERR_ARG, "impact buffer too small");
  YC_CUDA(cudaSetDevice(c->device));
  if (c->nimpacts)
    YC_CUDA(cudaMemcpyAsync(impacts, c->impacts.p, sizeof(ys_impact) * c->nimpacts, cudaMemcpyDeviceToHost,
                            c->stream));
  YC_CUDA(cudaStreamSynchronize(c->stream));
  return YS_OK;
}

ys_status ys_collider_respond(ys_collider* c, const double* node_mass, double h, double damp, int32_t max_iter,
                              double* x_out, double* v, ys_response_info* info) {
  if (!c || c->ct.face.empty()) return ys_internal_fail(YS_ERR_ARG, "ys_collider_respond before set_positions");
  if (!x_out || !(h > 0.0) || !std::isfinite(damp) || max_iter <= 0)
    return ys_internal_fail(YS_ERR_ARG, "bad response arguments");
  if (node_mass)
    for (int i = 0; i < c->n_nodes; ++i)
      if (!(node_mass[i] > 0.0) || !std::isfinite(node_mass[i]))
        return ys_internal_fail(YS_ERR_ARG, "node masses must be positive and finite");
  YC_CUDA(cudaSetDevice(c->device));
  ys::ZoneResponse& R = c->resp;
  c->have_response = false;
  R.n_nodes = c->n_nodes;
  R.n_faces = c->n_faces;
  R.faces = c->fv.data();
  R.obs_x = c->hox.data();
  R.xprev = c->hxp.data();
  R.obs_xprev = c->hoxp.data();
  R.thickness = c->thickness;
  R.max_iter = max_iter;
  R.max_zone_impacts = c->max_zone_impacts;
  c->resp_x0 = c->hx;
  std::vector<double> x(c->hx);
  const size_t n3 = 3 * (size_t)c->n_nodes;
  bool first = true;
  ys_status err = YS_OK;
  std::vector<ys_impact> got;
  // one detection round on the GPU: the trees keep the topology built by
  // set_positions and are refit to the current positions (AccelStruct::update)
  double detect_ms = 0.0;
  auto detect = [&](const double* xc, const uint8_t* mask, std::vector<ys::ZImpact>& out) -> int {
    const auto t0 = std::chrono::steady_clock::now();
    struct Tick {
      std::chrono::steady_clock::time_point t0;
      double* acc;
      ~Tick() { *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
    } tick{t0, &detect_ms};
    auto fail = [&](ys_status s) {
      err = s;
      return 1;
    };
    if (!first) {
      if (cudaMemcpyAsync(c->x.p, xc, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
        return fail(ys_internal_fail(YS_ERR_CUDA, "cudaMemcpyAsync failed"));
      ys_status s = refit(c, false);
      if (s != YS_OK) return fail(s);
    }
    first = false;
    if (mask) {
      const size_t nn = c->ct.face.size();
      if (c->face_active.reserve(c->n_faces) != cudaSuccess || c->node_active.reserve(nn) != cudaSuccess)
        return fail(ys_internal_fail(YS_ERR_CUDA, "cudaMalloc failed"));
      c->h_node_active.assign(nn, 0);
      mark_nodes(c->ct, mask, c->h_node_active);
      if (cudaMemcpyAsync(c->face_active.p, mask, c->n_faces, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
          cudaMemcpyAsync(c->node_active.p, c->h_node_active.data(), nn, cudaMemcpyHostToDevice, c->stream) !=
              cudaSuccess)
        return fail(ys_internal_fail(YS_ERR_CUDA, "cudaMemcpyAsync failed"));
    }
    ys_status s = detect_one_wait(c, mask != nullptr, got);
    if (s != YS_OK) return fail(s);
    out.resize(got.size());
    for (size_t i = 0; i < got.size(); ++i) {
      ys::ZImpact& z = out[i];
      z.type = got[i].type;
      z.t = got[i].t;
      for (int q = 0; q < 4; ++q) {
        z.node[q] = got[i].nodes[q];
        z.w[q] = got[i].w[q];
      }
      for (int q = 0; q < 3; ++q) z.n[q] = got[i].n[q];
    }
    return 0;
  };
  const auto t_resp = std::chrono::steady_clock::now();
  if (ys::zone_respond(R, x.data(), node_mass, detect, c->pool.get())) return err;
  const double resp_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_resp).count();
  // the collider keeps the responded positions (the cloth mesh's x)
  c->hx = x;
  YC_CUDA(cudaMemcpyAsync(c->x.p, c->hx.data(), n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  ys_status s = refit(c, false);
  if (s != YS_OK) return s;
  YC_CUDA(cudaStreamSynchronize(c->stream));
  c->have_pairs = c->have_impacts = false;
  std::memcpy(x_out, x.data(), n3 * sizeof(double));
  // velocity update of collision_response (src/Collision.cpp:130-137)
  if (v && R.changed)
    for (size_t i = 0; i < n3; ++i) v[i] = v[i] + (damp * (x[i] - c->resp_x0[i])) / h;
  c->resp_h = h;
  c->resp_damp = damp;
  c->have_response = true;
  if (info) {
    info->rounds = R.rounds;
    info->converged = R.converged;
    info->changed = R.changed;
    info->zones = R.zones;
    info->infeasible = R.infeasible;
    info->zone_overflow = R.zone_overflow;
    info->impacts = (int64_t)R.accepted.size();
    info->projections = (int64_t)R.tape.size();
    info->reverted = R.reverted;
    info->detect_ms = detect_ms;
    info->zones_ms = resp_ms - detect_ms;
  }
  if (R.zone_overflow)
    return ys_internal_fail(YS_ERR_MAXITER, "collision response stopped: an impact zone outgrew the zone limit "
                                            "(layers tangled beyond what the response resolves)");
  if (!R.converged) return ys_internal_fail(YS_ERR_MAXITER, "collision response did not converge");
  return YS_OK;
}

ys_status ys_collider_response_impacts(ys_collider* c, ys_impact* impacts, int64_t cap) {
  if (!c || !c->have_response) return ys_internal_fail(YS_ERR_ARG, "no collision response yet");
  const ys::ZoneResponse& R = c->resp;
  if (cap < (int64_t)R.accepted.size()) return ys_internal_fail(YS_ERR_ARG, "impact buffer too small");
  for (size_t i = 0; i < R.accepted.size(); ++i) {
    const ys::ZImpact& z = R.accepted[i];
    ys_impact& o = impacts[i];
    o.type = z.type;
    o.t = z.t;
    for (int q = 0; q < 4; ++q) {
      o.nodes[q] = z.node[q];
      o.w[q] = z.w[q];
    }
    for (int q = 0; q < 3; ++q) o.n[q] = z.n[q];
    o.pair = R.accepted_round[i];
  }
  return YS_OK;
}

ys_status ys_collider_respond_backward(ys_collider* c, const double* dl_dx, const double* dl_dv, int32_t flags,
                                       double* dl_dx_in, double* dl_dv_in, double* dl_dx_prev, double* dl_dw,
                                       double* dl_dn) {
  if (!c || !c->have_response) return ys_internal_fail(YS_ERR_ARG, "no collision response yet");
  if (!dl_dx_in) return ys_internal_fail(YS_ERR_ARG, "dl_dx_in is required");
  if (flags & ~3) return ys_internal_fail(YS_ERR_ARG, "unknown response gradient flags");
  const ys::ZoneResponse& R = c->resp;
  const size_t n3 = 3 * (size_t)c->n_nodes, na = R.accepted.size();
  std::vector<double> g(n3, 0.0), gp(n3, 0.0), gw(4 * std::max<size_t>(na, 1), 0.0),
      gn(3 * std::max<size_t>(na, 1), 0.0);
  if (dl_dx) std::memcpy(g.data(), dl_dx, n3 * sizeof(double));
  const double k = c->resp_damp / c->resp_h;
  if (dl_dv && R.changed)
    for (size_t i = 0; i < n3; ++i) g[i] += k * dl_dv[i];
  ys::zone_backward(R, g.data(), gw.data(), gn.data(), flags, gp.data());
  if (dl_dv && R.changed)
    for (size_t i = 0; i < n3; ++i) g[i] -= k * dl_dv[i];
  std::memcpy(dl_dx_in, g.data(), n3 * sizeof(double));
  if (dl_dv_in) {
    if (dl_dv) std::memcpy(dl_dv_in, dl_dv, n3 * sizeof(double));
    else std::memset(dl_dv_in, 0, n3 * sizeof(double));
  }
  if (dl_dx_prev) std::memcpy(dl_dx_prev, gp.data(), n3 * sizeof(double));
  if (dl_dw && na) std::memcpy(dl_dw, gw.data(), 4 * na * sizeof(double));
  if (dl_dn && na) std::memcpy(dl_dn, gn.data(), 3 * na * sizeof(double));
  return YS_OK;
}

ys_status ys_collider_set_max_zone_impacts(ys_collider* c, int32_t n) {
  if (!c || n < 1) return ys_internal_fail(YS_ERR_ARG, "the zone limit must be at least 1");
  c->max_zone_impacts = n;
  return YS_OK;
}

}  // extern "C"
