// ys_api.cu -- host runtime and C ABI (include/yarnsim.h) of the batched
// yarn-level cloth step on one GPU.
//
// The handle builds the batch topology once: per-node cloth id / grid
// coordinates / flags, per-yarn-line material, the colour classes of every
// element pass, and the thread-block partition used by the per-cloth solver.
// All device memory is allocated here and nowhere else.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/yarnsim.h"
#include "ys_gnn.cuh"
#include "ys_kernels.cuh"

namespace {

thread_local std::string g_err;

ys_status fail(ys_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

#define YS_CUDA(call)                                                                              \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return fail(YS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));               \
  } while (0)

// node-major [n][c] <-> component-major [c][n]
// AoS [n][c] <-> SoA [c][n] (c <= kMaxComps), kTrBlock nodes per block: the
// AoS side is moved as one contiguous run of kTrBlock * c doubles (each warp
// touches consecutive addresses, which matters when that side is host memory
// read or written over the C2C link), transposed in shared memory
constexpr int kTrBlock = 256, kMaxComps = 5;
__device__ __forceinline__ void to_soa_block(const double* __restrict__ in, double* __restrict__ out, int64_t n,
                                             int c) {
  __shared__ double sh[kTrBlock * kMaxComps];
  const int64_t n0 = (int64_t)blockIdx.x * kTrBlock;
  const int cnt = (int)(n - n0 < kTrBlock ? n - n0 : kTrBlock);
  for (int j = threadIdx.x; j < cnt * c; j += kTrBlock) sh[j] = in[n0 * c + j];
  __syncthreads();
  if (threadIdx.x < cnt)
    for (int k = 0; k < c; ++k) out[k * n + n0 + threadIdx.x] = sh[threadIdx.x * c + k];
}
__device__ __forceinline__ void to_aos_block(const double* __restrict__ in, double* __restrict__ out, int64_t n,
                                             int c) {
  __shared__ double sh[kTrBlock * kMaxComps];
  const int64_t n0 = (int64_t)blockIdx.x * kTrBlock;
  const int cnt = (int)(n - n0 < kTrBlock ? n - n0 : kTrBlock);
  if (threadIdx.x < cnt)
    for (int k = 0; k < c; ++k) sh[threadIdx.x * c + k] = in[k * n + n0 + threadIdx.x];
  __syncthreads();
  for (int j = threadIdx.x; j < cnt * c; j += kTrBlock) out[n0 * c + j] = sh[j];
}
__global__ void __launch_bounds__(kTrBlock) k_to_soa(const double* __restrict__ in, double* __restrict__ out,
                                                      int64_t n, int c) {
  to_soa_block(in, out, n, c);
}
__global__ void __launch_bounds__(kTrBlock) k_to_aos(const double* __restrict__ in, double* __restrict__ out,
                                                      int64_t n, int c) {
  to_aos_block(in, out, n, c);
}
// up to six arrays of one state transfer in one launch: blockIdx.y picks the array
struct TrSet {
  const double* in[6];
  double* out[6];
  int c[6];
};
__global__ void __launch_bounds__(kTrBlock) k_to_soa_set(TrSet t, int64_t n) {
  to_soa_block(t.in[blockIdx.y], t.out[blockIdx.y], n, t.c[blockIdx.y]);
}
__global__ void __launch_bounds__(kTrBlock) k_to_aos_set(TrSet t, int64_t n) {
  to_aos_block(t.in[blockIdx.y], t.out[blockIdx.y], n, t.c[blockIdx.y]);
}
// iteration bookkeeping only; the status bits set by the assembly are kept
__global__ void k_reset_pc(ys::PcgCloth* pc, const int* maxiter, int ncloth, int maxiter_override) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncloth) return;
  pc[c].status &= 1;
  pc[c].active = 0;
  pc[c].iters = 0;
  pc[c].maxiter = maxiter_override >= 0 ? maxiter_override : maxiter[c];
}
__global__ void k_reset_status(ys::PcgCloth* pc, int ncloth) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncloth) pc[c].status = 0;
}

}  // namespace

struct ys_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  int ncloth = 0;
  int ntot = 0;
  std::vector<ys::ClothParams> cp;
  std::vector<int64_t> dims;
  std::vector<int> anchors_host;
  int geom_off = 0, geom_n = 0;  // interior-node list (normals)
  // device memory
  std::vector<void*> allocs;
  int64_t bytes = 0;
  ys::View v{};
  ys::Records rec{};
  ys::Blocks blk{};
  ys::Solver so{};
  int* anchors = nullptr;
  int* maxiter_dev = nullptr;
  double* stage = nullptr;  // [15][ntot] staging for layout changes (the six state arrays side by side)
  double* ext = nullptr;    // [5][ntot]
  int* h_nactive = nullptr; // pinned
  double* vecs = nullptr;    // the PCG vectors x, r, p, q, dinv in one allocation
  size_t l2_window = 0;      // bytes of it kept in L2 by the graph's capture streams
  float l2_hit = 0.0f;
  double* h_wind = nullptr;  // pinned [ncloth][3]: ys_set_winds' copy of the caller's array
  cudaEvent_t wind_ev = nullptr;  // recorded after the copy out of h_wind
  bool assembled = false;
  int max_maxiter = 0;
  // launch accounting and optional per-kernel-class event timing
  int64_t launches = 0;
  bool profiling = false;
  // forward-mode sensitivities (allocated by ys_tangent_enable)
  struct Tan {
    bool on = false;
    int mode = 0;
    double *dX = nullptr, *dV = nullptr, *dUV = nullptr, *dUVD = nullptr, *dUVB = nullptr;
    double *dNRM = nullptr, *dCOMP = nullptr, *dSLIDE = nullptr;
    double *drho = nullptr, *dks = nullptr, *dkb = nullptr, *dS = nullptr, *dmu = nullptr;
    double *dA = nullptr, *dB = nullptr, *As = nullptr, *Bs = nullptr, *qsave = nullptr, *rt = nullptr, *dq = nullptr;
    double *dedge = nullptr, *dbend = nullptr, *dface = nullptr, *dshear = nullptr;
    double* io = nullptr;  // [kTangents][ntot][3] staging of host tangents
    double* dext = nullptr;  // [kTangents][ntot][5] external-force tangents
  } tan;
  int nlines = 0;
  std::vector<double> line_R;  // yarn radius of each line's cloth
  // construction parameters of every cloth, kept so that an adjoint can
  // build copies of the batch (ys_adjoint_create); pointers of `d` are
  // re-aimed at the vectors where a desc is rebuilt
  struct DescStore {
    ys_cloth_desc d;
    std::vector<double> wr, wY, wB, fr, fY, fB;
    std::vector<int32_t> handles;
  };
  std::vector<DescStore> descs;
  // whole-step CUDA graph (ys_use_graphs): assembly, a conditional while node
  // over the PCG iterations, update; rebuilt when its parameters change
  // `built`: the parameters below are current; each graph is captured on its
  // first use after they change
  struct Graph {
    bool enabled = false;
    bool built = false;
    cudaStream_t capture = nullptr;  // capture needs a stream of its own
    // two more capture streams and their fork / join events: the record
    // producers that read none of each other's output are graph branches
    cudaStream_t side[2] = {nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    cudaGraph_t main = nullptr;      // Jacobi-PCG step
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t lmain[2] = {nullptr, nullptr};  // learned-preconditioner step [with the network]
    cudaGraphExec_t lexec[2] = {nullptr, nullptr};
    const void* lnet = nullptr;  // the network the learned graphs were captured with
    double h = 0.0, tol = 0.0;
    bool has_ext = false;
    int override_max = -1, m = 0, cap = 0;
    int* it_base = nullptr;  // device
    int* hold = nullptr;     // device: the learned solve handed the step to Jacobi-PCG
    int h_it = 0;
    int h_hold = 0;
    void drop() {
      if (exec) cudaGraphExecDestroy(exec);
      if (main) cudaGraphDestroy(main);
      exec = nullptr;
      main = nullptr;
      for (int k = 0; k < 2; ++k) {
        if (lexec[k]) cudaGraphExecDestroy(lexec[k]);
        if (lmain[k]) cudaGraphDestroy(lmain[k]);
        lexec[k] = nullptr;
        lmain[k] = nullptr;
      }
    }
  } graph;
  int check_every = 16;  // PCG iterations between convergence checks when the call gives none
  // PCG schedule (ys_set_pcg_schedule): phases, or the persistent per-cloth
  // kernel with `threads` x `csize` nodes per cloth; `order` lists the cloths
  // largest first, so the biggest clusters start first
  struct PcgPlan {
    int kind = YS_PCG_PHASES;
    int threads = 0, csize = 0;
    int* order = nullptr;  // device [ncloth]
    int max_nodes = 0;
  } plan;
  std::vector<ys_schedule> tuned;  // every schedule the last ys_autotune timed
  int producer_threads = ys::kBlock;  // block size of the record producers and the gather
  bool has_system = false;  // v.A / v.B hold an assembled system (kept after the update)
  // learned preconditioner (ys_set_preconditioner); buffers allocated on first use
  struct Learn {
    int kind = YS_PREC_JACOBI;
    ys_gnn* net = nullptr;
    bool ready = false;
    ys::GnnBufs g{};
    float* rf = nullptr;  // the residual in FP32 (the preconditioner's input)
    double* z = nullptr;
    int64_t fallbacks = 0;
    int64_t solves = 0;
    int refresh_every = 1;  // solves per network evaluation (G reused in between)
    int since = 0;
    bool have_g = false;
  } learn;
  struct Rec { int kind; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  double prof_ms[YS_PROF_KINDS] = {0};
  int64_t prof_n[YS_PROF_KINDS] = {0};

  cudaEvent_t ev() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  // runs one launcher; `kernels` = kernels it launches
  template <class F>
  void run(int kind, int kernels, F&& f) {
    launches += kernels;
    if (!profiling) { f(); return; }
    Rec r{kind, ev(), ev()};
    cudaEventRecord(r.a, stream);
    f();
    cudaEventRecord(r.b, stream);
    recs.push_back(r);
  }
  void drain() {
    if (recs.empty()) return;
    cudaStreamSynchronize(stream);
    for (Rec& r : recs) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.a, r.b);
      prof_ms[r.kind] += ms;
      prof_n[r.kind] += 1;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    recs.clear();
  }

  template <class T>
  ys_status alloc(T** p, size_t count) {
    void* q = nullptr;
    size_t nb = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, nb);
    if (e != cudaSuccess) return fail(YS_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    allocs.push_back(q);
    bytes += (int64_t)nb;
    *p = static_cast<T*>(q);
    return YS_OK;
  }
  ~ys_batch() {
    drain();
    graph.drop();
    if (graph.capture) cudaStreamDestroy(graph.capture);
    for (int k = 0; k < 2; ++k) {
      if (graph.side[k]) cudaStreamDestroy(graph.side[k]);
      if (graph.join[k]) cudaEventDestroy(graph.join[k]);
    }
    if (graph.fork) cudaEventDestroy(graph.fork);
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
    for (void* p : allocs) cudaFree(p);
    if (h_nactive) cudaFreeHost(h_nactive);
    if (h_wind) cudaFreeHost(h_wind);
    if (wind_ev) cudaEventDestroy(wind_ev);
  }
};

namespace {

// host (or device, YS_ON_DEVICE) AoS [ntot][c] -> device SoA [c][ntot]; a
// host array goes through the stage at `slot` (in units of ntot doubles), and
// with sync the call returns once the host array has been read
// the device's address of a page-locked host array (cudaMallocHost,
// cudaHostAlloc, cudaHostRegister: what a pinned tensor's storage is), or
// null for pageable or device memory
double* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? static_cast<double*>(a.devicePointer) : nullptr;
}

// a page-locked host array is read (written) by the transposition kernel
// itself, with no stage copy
ys_status upload_soa(ys_batch* b, const double* src, double* dst, int c, int32_t flags, int64_t slot = 0,
                     bool sync = true) {
  const int64_t n = b->ntot;
  if (!src) return YS_OK;
  if (c > kMaxComps) return fail(YS_ERR_ARG, "upload_soa: too many components");
  const double* d_src = src;
  if (!(flags & YS_ON_DEVICE)) {
    if (const double* m = mapped_host(src)) {
      d_src = m;
    } else {
      YS_CUDA(cudaMemcpyAsync(b->stage + slot * n, src, sizeof(double) * n * c, cudaMemcpyHostToDevice, b->stream));
      d_src = b->stage + slot * n;
    }
  }
  b->launches += 1;
  k_to_soa<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(d_src, dst, n, c);
  YS_CUDA(cudaGetLastError());
  if (sync && !(flags & YS_ON_DEVICE)) YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

// device SoA [c][ntot] -> AoS [ntot][c] on the host (through the stage at
// `slot`; with sync the call returns once the host array is filled) or on the
// device
ys_status download_aos(ys_batch* b, const double* src, double* dst, int c, int32_t flags, int64_t slot = 0,
                       bool sync = true) {
  const int64_t n = b->ntot;
  if (!dst) return YS_OK;
  if (c > kMaxComps) return fail(YS_ERR_ARG, "download_aos: too many components");
  double* m = (flags & YS_ON_DEVICE) ? nullptr : mapped_host(dst);
  double* d_dst = (flags & YS_ON_DEVICE) ? dst : m ? m : b->stage + slot * n;
  b->launches += 1;
  k_to_aos<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(src, d_dst, n, c);
  YS_CUDA(cudaGetLastError());
  if (!(flags & YS_ON_DEVICE)) {
    if (!m) YS_CUDA(cudaMemcpyAsync(dst, d_dst, sizeof(double) * n * c, cudaMemcpyDeviceToHost, b->stream));
    if (sync) YS_CUDA(cudaStreamSynchronize(b->stream));
  }
  return YS_OK;
}

int weave_flip(int weave, int i, int j) {
  // src/Cloth.cpp:69-92 (interior nodes only)
  if (weave == 0) return (i + j) % 2 != 0;
  if (weave == 1) {
    int rv = j % 4, ru = (i + rv) % 4;
    return ru < 2;
  }
  int rv = (j - 1) % 4, q = rv / 2, r = rv % 2, idx = q * 3 + r * 2, ru = (i - 1 + idx) % 4;
  return ru == 0;
}

}  // namespace

// error reporting for the other translation units of the library (not exported)
extern "C" __attribute__((visibility("hidden"))) ys_status ys_internal_fail(ys_status s, const char* msg) {
  return fail(s, msg);
}

extern "C" {

const char* ys_last_error(void) { return g_err.c_str(); }

ys_status ys_batch_create(int32_t n_cloths, const ys_cloth_desc* descs, int32_t device, void* cuda_stream,
                          ys_batch** out) {
  if (!out || n_cloths <= 0 || !descs) return fail(YS_ERR_ARG, "n_cloths must be > 0 and descs non-null");
  *out = nullptr;
  for (int c = 0; c < n_cloths; ++c) {
    const ys_cloth_desc& d = descs[c];
    if (d.width < 3 || d.length < 3) return fail(YS_ERR_ARG, "cloth sides must be >= 3 crossings");
    if (!d.warp_rho || !d.warp_Y || !d.warp_B || !d.weft_rho || !d.weft_Y || !d.weft_B)
      return fail(YS_ERR_ARG, "yarn line material arrays must be non-null");
    if (d.pose < 0 || d.pose > 1 || d.weave < 0 || d.weave > 2) return fail(YS_ERR_ARG, "bad pose or weave");
    if (!(d.L > 0) || !(d.R > 0) || d.R >= d.L) return fail(YS_ERR_ARG, "need 0 < R < L");
    if (d.n_handles < 0 || (d.n_handles > 0 && !d.handles)) return fail(YS_ERR_ARG, "bad handle list");
    for (int hnd = 0; hnd < d.n_handles; ++hnd) {
      // the reference's set_handles looks each up with nodes.at() and throws
      // for a node outside the cloth (src/Cloth.cpp:386-394)
      const int u = d.handles[2 * hnd], vv = d.handles[2 * hnd + 1];
      if (u < 0 || u >= d.width || vv < 0 || vv >= d.length) return fail(YS_ERR_ARG, "handle outside the cloth");
    }
  }
  YS_CUDA(cudaSetDevice(device));
  ys_batch* b = new ys_batch();
  b->device = device;
  b->stream = static_cast<cudaStream_t>(cuda_stream);
  b->ncloth = n_cloths;
  for (int c = 0; c < n_cloths; ++c) {
    const ys_cloth_desc& d = descs[c];
    ys_batch::DescStore ds;
    ds.d = d;
    ds.wr.assign(d.warp_rho, d.warp_rho + d.length); ds.wY.assign(d.warp_Y, d.warp_Y + d.length);
    ds.wB.assign(d.warp_B, d.warp_B + d.length); ds.fr.assign(d.weft_rho, d.weft_rho + d.width);
    ds.fY.assign(d.weft_Y, d.weft_Y + d.width); ds.fB.assign(d.weft_B, d.weft_B + d.width);
    if (d.n_handles > 0) ds.handles.assign(d.handles, d.handles + 2 * d.n_handles);
    b->descs.push_back(std::move(ds));
  }
  // ------------------------------------------------------------ topology
  std::vector<int> node_cloth, node_u, node_v;
  std::vector<uint8_t> flags;
  std::vector<double> X, XF, UV, rho, ks, kb;
  std::vector<int> blk_cloth, blk_node0, blk_count, cloth_blk0, cloth_nblk, maxiter;
  int off = 0, line_off = 0;
  for (int c = 0; c < n_cloths; ++c) {
    const ys_cloth_desc& d = descs[c];
    ys::ClothParams P{};
    P.W = d.width; P.H = d.length; P.node_off = off;
    P.warp_line_off = line_off;
    P.weft_line_off = line_off + d.length;
    P.L = d.L; P.R = d.R; P.kc = d.kc; P.kf = d.kf; P.df = d.df; P.mu = d.mu; P.S = d.S;
    P.kh = d.handle_stiffness;
    P.jam = 2.0 * std::asin(d.R / d.L);  // src/Cloth.cpp:29
    for (int k = 0; k < 3; ++k) { P.G[k] = d.G[k]; P.wind[k] = d.wind_vel[k]; }
    P.wind_rho = d.wind_density; P.wind_drag = d.wind_drag;
    P.pb4 = std::pow(ys::kPi / 2, 4);
    P.pb5 = std::pow(ys::kPi / 2, 5);
    b->cp.push_back(P);
    for (int i = 0; i < d.length; ++i) {
      rho.push_back(d.warp_rho[i]);
      ks.push_back(d.warp_Y[i] * ys::kPi * std::pow(d.R, 2));  // src/Yarn.h:14-15
      kb.push_back(d.warp_B[i] * ys::kPi * std::pow(d.R, 2));
    }
    for (int i = 0; i < d.width; ++i) {
      rho.push_back(d.weft_rho[i]);
      ks.push_back(d.weft_Y[i] * ys::kPi * std::pow(d.R, 2));
      kb.push_back(d.weft_B[i] * ys::kPi * std::pow(d.R, 2));
    }
    line_off += d.length + d.width;
    for (int i = 0; i < d.length + d.width; ++i) b->line_R.push_back(d.R);
    const int W = d.width, H = d.length;
    std::vector<uint8_t> fixed(W * H, 0);
    for (int hnd = 0; hnd < d.n_handles; ++hnd) {
      const int u = d.handles[2 * hnd], vv = d.handles[2 * hnd + 1];
      if (u >= 0 && u < W && vv >= 0 && vv < H) fixed[u + vv * W] = 1;
    }
    for (int j = 0; j < H; ++j)
      for (int i = 0; i < W; ++i) {
        const int n = off + i + j * W;
        node_cloth.push_back(c);
        node_u.push_back(i);
        node_v.push_back(j);
        const bool interior = !(i == 0 || i == W - 1 || j == 0 || j == H - 1);
        uint8_t f = interior ? ys::YS_INTERIOR : 0;
        if (interior && weave_flip(d.weave, i, j)) f |= ys::YS_FLIP;
        if (fixed[i + j * W]) f |= ys::YS_FIXED;
        flags.push_back(f);
        // Cloth::build (src/Cloth.cpp:52-99)
        if (d.pose == 0) { X.push_back(i * d.L); X.push_back(0.0); X.push_back(d.height - j * d.L); }
        else { X.push_back(i * d.L); X.push_back(j * d.L); X.push_back(d.height); }
        UV.push_back(i * d.L);
        UV.push_back(j * d.L);
      }
    const int nb = (W * H + ys::kBlock - 1) / ys::kBlock;
    cloth_blk0.push_back((int)blk_cloth.size());
    cloth_nblk.push_back(nb);
    for (int q = 0; q < nb; ++q) {
      blk_cloth.push_back(c);
      blk_node0.push_back(off + q * ys::kBlock);
      blk_count.push_back(std::min(ys::kBlock, W * H - q * ys::kBlock));
    }
    const int64_t dim = 3LL * W * H + 2LL * (W - 2) * (H - 2);
    b->dims.push_back(dim);
    maxiter.push_back((int)std::min<int64_t>(2 * dim, 1 << 30));
    off += W * H;
  }
  b->ntot = off;
  b->max_maxiter = *std::max_element(maxiter.begin(), maxiter.end());
  // interior nodes (normals)
  std::vector<int> interior_nodes;
  for (int n = 0; n < off; ++n)
    if (flags[n] & ys::YS_INTERIOR) interior_nodes.push_back(n);
  b->geom_off = 0;
  b->geom_n = (int)interior_nodes.size();
  b->anchors_host = interior_nodes;

  // ------------------------------------------------------------ device memory
  const int64_t nt = off;
  ys_status st = YS_OK;
  auto A = [&](auto** p, size_t cnt) {
    if (st == YS_OK) st = b->alloc(p, cnt);
  };
  int *d_nc, *d_nu, *d_nv, *d_bc, *d_bn, *d_bk, *d_cb, *d_cn;
  uint8_t* d_fl;
  ys::ClothParams* d_cp;
  double *d_rho, *d_ks, *d_kb;
  A(&d_nc, nt); A(&d_nu, nt); A(&d_nv, nt); A(&d_fl, nt); A(&d_cp, n_cloths);
  A(&d_rho, rho.size()); A(&d_ks, ks.size()); A(&d_kb, kb.size());
  A(&d_bc, blk_cloth.size()); A(&d_bn, blk_cloth.size()); A(&d_bk, blk_cloth.size());
  A(&d_cb, n_cloths); A(&d_cn, n_cloths);
  A(&b->anchors, b->anchors_host.size());
  A(&b->maxiter_dev, n_cloths);
  ys::View& v = b->v;
  A(&v.X, 3 * nt); A(&v.V, 3 * nt); A(&v.XF, 3 * nt); A(&v.UV, 2 * nt); A(&v.UVD, 2 * nt); A(&v.UVB, 2 * nt);
  A(&v.UV0, 2 * nt); A(&v.NRM, 3 * nt); A(&v.COMP, nt); A(&v.SLIDE, 2 * nt);
  A(&v.A, (size_t)ys::YS_NUM_SLOTS * nt); A(&v.B, 5 * nt);
  A(&b->rec.edge, (size_t)ys::kEdgeFields * 2 * nt); A(&b->rec.bend, (size_t)ys::kBendFields * 2 * nt);
  A(&b->rec.face, 6 * nt); A(&b->rec.shear, (size_t)ys::kShearFields * 4 * nt);
  A(&b->rec.nonfinite, nt);
  A(&b->vecs, 25 * nt);
  if (b->vecs) {
    b->so.x = b->vecs; b->so.r = b->vecs + 5 * nt; b->so.p = b->vecs + 10 * nt;
    b->so.q = b->vecs + 15 * nt; b->so.dinv = b->vecs + 20 * nt;
  }
  A(&b->so.part, 4 * blk_cloth.size()); A(&b->so.pc, n_cloths); A(&b->so.nactive, 1);
  A(&b->stage, 15 * nt); A(&b->ext, 5 * nt);
  if (st != YS_OK) { delete b; return st; }
  if (cudaMallocHost(&b->h_nactive, sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&b->h_wind, sizeof(double) * 3 * n_cloths) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->wind_ev, cudaEventDisableTiming) != cudaSuccess) {
    delete b;
    return fail(YS_ERR_CUDA, "cudaMallocHost / cudaEventCreate failed");
  }
  auto up = [&](void* dst, const void* src, size_t nbytes) -> ys_status {
    YS_CUDA(cudaMemcpy(dst, src, nbytes, cudaMemcpyHostToDevice));
    return YS_OK;
  };
  ys_status s2 = YS_OK;
  auto U = [&](void* dst, const void* src, size_t nbytes) { if (s2 == YS_OK && nbytes) s2 = up(dst, src, nbytes); };
  U(d_nc, node_cloth.data(), sizeof(int) * nt); U(d_nu, node_u.data(), sizeof(int) * nt);
  U(d_nv, node_v.data(), sizeof(int) * nt); U(d_fl, flags.data(), nt);
  U(d_cp, b->cp.data(), sizeof(ys::ClothParams) * n_cloths);
  U(d_rho, rho.data(), sizeof(double) * rho.size()); U(d_ks, ks.data(), sizeof(double) * ks.size());
  U(d_kb, kb.data(), sizeof(double) * kb.size());
  U(d_bc, blk_cloth.data(), sizeof(int) * blk_cloth.size()); U(d_bn, blk_node0.data(), sizeof(int) * blk_cloth.size());
  U(d_bk, blk_count.data(), sizeof(int) * blk_cloth.size());
  U(d_cb, cloth_blk0.data(), sizeof(int) * n_cloths); U(d_cn, cloth_nblk.data(), sizeof(int) * n_cloths);
  U(b->anchors, b->anchors_host.data(), sizeof(int) * b->anchors_host.size());
  U(b->maxiter_dev, maxiter.data(), sizeof(int) * n_cloths);
  // initial state: positions, EPos, EPosBar = EPos, LPosFix = LPos, zero velocities
  {
    std::vector<double> soa(5 * nt, 0.0);
    for (int k = 0; k < 3; ++k)
      for (int64_t i = 0; i < nt; ++i) soa[k * nt + i] = X[3 * i + k];
    U(v.X, soa.data(), sizeof(double) * 3 * nt);
    U(v.XF, soa.data(), sizeof(double) * 3 * nt);
    for (int k = 0; k < 2; ++k)
      for (int64_t i = 0; i < nt; ++i) soa[k * nt + i] = UV[2 * i + k];
    U(v.UV, soa.data(), sizeof(double) * 2 * nt);
    U(v.UVB, soa.data(), sizeof(double) * 2 * nt);
    U(v.UV0, soa.data(), sizeof(double) * 2 * nt);
  }
  if (s2 != YS_OK) { delete b; return s2; }
  if (cudaMemset(v.V, 0, sizeof(double) * 3 * nt) != cudaSuccess ||
      cudaMemset(v.UVD, 0, sizeof(double) * 2 * nt) != cudaSuccess ||
      cudaMemset(v.NRM, 0, sizeof(double) * 3 * nt) != cudaSuccess ||
      cudaMemset(v.COMP, 0, sizeof(double) * nt) != cudaSuccess ||
      cudaMemset(v.SLIDE, 0, sizeof(double) * 2 * nt) != cudaSuccess ||
      cudaMemset(b->so.pc, 0, sizeof(ys::PcgCloth) * n_cloths) != cudaSuccess) {
    delete b;
    return fail(YS_ERR_CUDA, "cudaMemset failed");
  }
  v.ntot = (int)nt;
  v.ncloth = n_cloths;
  v.node_cloth = d_nc; v.node_u = d_nu; v.node_v = d_nv; v.flags = d_fl; v.cp = d_cp;
  v.line_rho = d_rho; v.line_ks = d_ks; v.line_kb = d_kb;
  v.nlines = line_off;
  b->nlines = line_off;
  v.ext = nullptr;
  v.h = 1e-3;
  b->blk.nblk = (int)blk_cloth.size();
  b->blk.blk_cloth = d_bc; b->blk.blk_node0 = d_bn; b->blk.blk_count = d_bk;
  b->blk.cloth_blk0 = d_cb; b->blk.cloth_nblk = d_cn;
  b->so.tol = DBL_EPSILON;
  *out = b;
  return YS_OK;
}

void ys_batch_destroy(ys_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  delete b;
}

ys_status ys_batch_get_info(const ys_batch* b, ys_batch_info* info) {
  if (!b || !info) return fail(YS_ERR_ARG, "null argument");
  info->n_cloths = b->ncloth;
  info->total_nodes = b->ntot;
  info->device_bytes = b->bytes;
  return YS_OK;
}

int64_t ys_cloth_node_offset(const ys_batch* b, int32_t c) {
  if (!b || c < 0 || c >= b->ncloth) return -1;
  return b->cp[c].node_off;
}

int64_t ys_cloth_dim(const ys_batch* b, int32_t c) {
  if (!b || c < 0 || c >= b->ncloth) return -1;
  return b->dims[c];
}

ys_status ys_set_state(ys_batch* b, const double* lpos, const double* lposfix, const double* lvel,
                       const double* epos, const double* eposbar, const double* evel, int32_t flags) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  YS_CUDA(cudaSetDevice(b->device));
  // the six arrays (page-locked: read in place; pageable: through their own
  // stage slots) transposed in one launch, one wait at the end
  const double* src[6] = {lpos, lposfix, lvel, epos, eposbar, evel};
  double* dst[6] = {b->v.X, b->v.XF, b->v.V, b->v.UV, b->v.UVB, b->v.UVD};
  const int comps[6] = {3, 3, 3, 2, 2, 2};
  const int64_t n = b->ntot;
  TrSet t{};
  int cnt = 0;
  int64_t slot = 0;
  for (int k = 0; k < 6; ++k) {
    if (src[k]) {
      const double* d = src[k];
      if (!(flags & YS_ON_DEVICE)) {
        if (const double* m = mapped_host(src[k])) {
          d = m;
        } else {
          YS_CUDA(cudaMemcpyAsync(b->stage + slot * n, src[k], sizeof(double) * n * comps[k],
                                  cudaMemcpyHostToDevice, b->stream));
          d = b->stage + slot * n;
        }
      }
      t.in[cnt] = d;
      t.out[cnt] = dst[k];
      t.c[cnt] = comps[k];
      ++cnt;
    }
    slot += comps[k];
  }
  if (cnt) {
    b->launches += 1;
    k_to_soa_set<<<dim3((unsigned)((n + kTrBlock - 1) / kTrBlock), cnt), kTrBlock, 0, b->stream>>>(t, n);
    YS_CUDA(cudaGetLastError());
    if (!(flags & YS_ON_DEVICE)) YS_CUDA(cudaStreamSynchronize(b->stream));
  }
  b->assembled = false;
  return YS_OK;
}

ys_status ys_get_state(ys_batch* b, double* lpos, double* lposfix, double* lvel, double* epos, double* eposbar,
                       double* evel, int32_t flags) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  YS_CUDA(cudaSetDevice(b->device));
  // the six arrays transposed in one launch (into page-locked host arrays in
  // place, else into their own stage slots, copied out after), one wait
  double* dst[6] = {lpos, lposfix, lvel, epos, eposbar, evel};
  const double* src[6] = {b->v.X, b->v.XF, b->v.V, b->v.UV, b->v.UVB, b->v.UVD};
  const int comps[6] = {3, 3, 3, 2, 2, 2};
  const int64_t n = b->ntot;
  TrSet t{};
  double* staged[6] = {};
  int cnt = 0;
  int64_t slot = 0;
  for (int k = 0; k < 6; ++k) {
    if (dst[k]) {
      double* d = dst[k];
      if (!(flags & YS_ON_DEVICE)) {
        if (double* m = mapped_host(dst[k])) {
          d = m;
        } else {
          d = b->stage + slot * n;
          staged[k] = d;
        }
      }
      t.in[cnt] = src[k];
      t.out[cnt] = d;
      t.c[cnt] = comps[k];
      ++cnt;
    }
    slot += comps[k];
  }
  if (!cnt) return YS_OK;
  b->launches += 1;
  k_to_aos_set<<<dim3((unsigned)((n + kTrBlock - 1) / kTrBlock), cnt), kTrBlock, 0, b->stream>>>(t, n);
  YS_CUDA(cudaGetLastError());
  if (!(flags & YS_ON_DEVICE)) {
    for (int k = 0; k < 6; ++k)
      if (staged[k])
        YS_CUDA(cudaMemcpyAsync(dst[k], staged[k], sizeof(double) * n * comps[k], cudaMemcpyDeviceToHost,
                                b->stream));
    YS_CUDA(cudaStreamSynchronize(b->stream));
  }
  return YS_OK;
}

ys_status ys_get_normals(ys_batch* b, double* normals, int32_t flags) {
  if (!b || !normals) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(b->device));
  // NodeNorm of the current positions (src/Cloth.cpp:440-463), as
  // Cloth::UpdateClothUnits leaves them after every update; the step itself
  // recomputes them when it assembles
  if (b->geom_n) {
    b->launches += 1;
    ys::launch_geom(b->v, b->anchors + b->geom_off, b->geom_n, b->stream);
    YS_CUDA(cudaGetLastError());
  }
  return download_aos(b, b->v.NRM, normals, 3, flags);
}

ys_status ys_set_wind(ys_batch* b, int32_t cloth, const double wind_vel[3]) {
  if (!b || !wind_vel || cloth < -1 || cloth >= b->ncloth) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(b->device));
  const int c0 = cloth < 0 ? 0 : cloth, c1 = cloth < 0 ? b->ncloth : cloth + 1;
  for (int c = c0; c < c1; ++c) {
    for (int k = 0; k < 3; ++k) b->cp[c].wind[k] = wind_vel[k];
    ys::ClothParams* dst = const_cast<ys::ClothParams*>(b->v.cp) + c;
    YS_CUDA(cudaMemcpyAsync(&dst->wind[0], b->cp[c].wind, sizeof(double) * 3, cudaMemcpyHostToDevice, b->stream));
  }
  YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

namespace {
__global__ void k_set_winds(ys::ClothParams* cp, const double* __restrict__ w, int ncloth) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncloth)
    for (int k = 0; k < 3; ++k) cp[c].wind[k] = w[3 * c + k];
}
}  // namespace

ys_status ys_set_winds(ys_batch* b, const double* wind_vel, int32_t flags) {
  if (!b || !wind_vel) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(b->device));
  const double* src = wind_vel;
  if (!(flags & YS_ON_DEVICE)) {
    // the caller's array is copied into pinned memory here, so the call
    // returns once it is read without waiting for the stream; the previous
    // call's copy out of that memory has finished first
    const size_t nb = sizeof(double) * 3 * b->ncloth;
    YS_CUDA(cudaEventSynchronize(b->wind_ev));
    std::memcpy(b->h_wind, wind_vel, nb);
    YS_CUDA(cudaMemcpyAsync(b->stage, b->h_wind, nb, cudaMemcpyHostToDevice, b->stream));
    YS_CUDA(cudaEventRecord(b->wind_ev, b->stream));
    src = b->stage;
  }
  b->launches += 1;
  k_set_winds<<<(b->ncloth + 127) / 128, 128, 0, b->stream>>>(const_cast<ys::ClothParams*>(b->v.cp), src,
                                                                 b->ncloth);
  YS_CUDA(cudaGetLastError());
  for (int c = 0; c < b->ncloth; ++c)
    for (int k = 0; k < 3; ++k) b->cp[c].wind[k] = wind_vel == src ? b->cp[c].wind[k] : wind_vel[3 * c + k];
  return YS_OK;
}

ys_status ys_assemble(ys_batch* b, double h, const double* ext_force, int32_t flags) {
  if (!b || !(h > 0)) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(b->device));
  b->v.h = h;
  b->v.ext = nullptr;
  if (ext_force) {
    ys_status s = upload_soa(b, ext_force, b->ext, 5, flags);
    if (s != YS_OK) return s;
    b->v.ext = b->ext;
  }
  cudaStream_t s = b->stream;
  const ys::View& v = b->v;
  b->run(YS_PROF_MISC, 1, [&] { k_reset_status<<<(b->ncloth + 127) / 128, 128, 0, s>>>(b->so.pc, b->ncloth); });
  // UpdateClothUnits normals for the current positions (src/Cloth.cpp:307-327)
  if (b->geom_n) b->run(YS_PROF_GEOM, 1, [&] { ys::launch_geom(v, b->anchors + b->geom_off, b->geom_n, s); });
  // element records (FillMV's element loops, src/PhysicsCloth.cpp:64-95)
  const ys::Records& R = b->rec;
  const int pt = b->producer_threads;
  b->run(YS_PROF_EDGES, 1, [&] { ys::launch_edge_records(v, R, s, pt); });
  b->run(YS_PROF_BENDS, 1, [&] { ys::launch_bend_records(v, R, s, pt); });
  b->run(YS_PROF_FACES, 1, [&] { ys::launch_face_records(v, R, s, pt); });
  // row blocks + ConSlideFriction (needs every edge and bend term; shear
  // needs its compression, src/PhysicsCloth.cpp:97-131)
  b->run(YS_PROF_GATHER, 1, [&] { ys::launch_gather(v, R, s, pt); });
  b->run(YS_PROF_SHEAR, 1, [&] { ys::launch_shear_records(v, R, s, pt); });
  b->run(YS_PROF_FINALIZE, 1, [&] { ys::launch_finalize(v, R, b->blk, b->so, s); });
  YS_CUDA(cudaGetLastError());
  b->assembled = true;
  b->has_system = true;
  return YS_OK;
}

}  // extern "C"

namespace {
// Jacobi-PCG on the assembled A with the right-hand side v.B (the step's b,
// or the right-hand side of a tangent solve); the solution lands in so.x.
ys_status solve_impl(ys_batch* b, const ys::View& v, const ys_solve_opts* opts, ys_cloth_stats* stats) {
  cudaStream_t s = b->stream;
  b->so.tol = (opts && opts->tol > 0) ? opts->tol : DBL_EPSILON;
  const int override_max = (opts && opts->maxiter >= 0) ? opts->maxiter : -1;
  const int every = (opts && opts->check_every > 0) ? opts->check_every : b->check_every;
  const int cap = override_max >= 0 ? override_max : b->max_maxiter;
  b->run(YS_PROF_MISC, 1, [&] {
    k_reset_pc<<<(b->ncloth + 127) / 128, 128, 0, s>>>(b->so.pc, b->maxiter_dev, b->ncloth, override_max);
  });
  YS_CUDA(cudaGetLastError());
  if (b->plan.kind == YS_PCG_PERSISTENT) {
    cudaError_t e = cudaSuccess;
    b->run(YS_PROF_PCG_PERSIST, 1, [&] {
      e = ys::launch_pcg_cluster(v, b->so, b->plan.order, b->ncloth, b->plan.threads, b->plan.csize, cap, s);
    });
    if (e != cudaSuccess) return fail(YS_ERR_CUDA, std::string("persistent PCG: ") + cudaGetErrorString(e));
  }
  else {
    b->run(YS_PROF_PCG_SETUP, 2, [&] { ys::launch_pcg_setup(v, b->blk, b->so, s); });
  }
  int it = b->plan.kind == YS_PCG_PHASES ? 0 : cap;
  while (it < cap) {
    const int n = std::min(every, cap - it);
    for (int q = 0; q < n; ++q, ++it) {
      b->run(YS_PROF_SPMV, 1, [&] { ys::launch_pcg_spmv(v, b->blk, b->so, s); });
      b->run(YS_PROF_AXPY, 1, [&] { ys::launch_pcg_axpy(v, b->blk, b->so, it, s); });
      b->run(YS_PROF_DIR, 1, [&] { ys::launch_pcg_dir(v, b->blk, b->so, it, s); });
    }
    b->run(YS_PROF_MISC, 1, [&] { ys::launch_count_active(v, b->so, s); });
    YS_CUDA(cudaMemcpyAsync(b->h_nactive, b->so.nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
    YS_CUDA(cudaStreamSynchronize(s));
    if (*b->h_nactive == 0) break;
  }
  YS_CUDA(cudaGetLastError());
  std::vector<ys::PcgCloth> pc(b->ncloth);
  YS_CUDA(cudaMemcpyAsync(pc.data(), b->so.pc, sizeof(ys::PcgCloth) * b->ncloth, cudaMemcpyDeviceToHost, s));
  YS_CUDA(cudaStreamSynchronize(s));
  ys_status ret = YS_OK;
  for (int c = 0; c < b->ncloth; ++c) {
    if (pc[c].status & 1) ret = YS_ERR_NONFINITE;
    else if ((pc[c].status & 4) && ret == YS_OK) ret = YS_ERR_MAXITER;
    if (stats) {
      stats[c].ok = (pc[c].status & 3) == 0;
      stats[c].cg_iterations = pc[c].iters;
      stats[c].cg_error = pc[c].bb > 0 ? std::sqrt(pc[c].rr / pc[c].bb) : 0.0;
      stats[c].hit_maxiter = (pc[c].status & 4) ? 1 : 0;
    }
  }
  return ret;
}

ys_status solve_learned(ys_batch* b, const ys_solve_opts* opts, ys_cloth_stats* stats);
// the learned solve converges in about five iterations: it checks for
// convergence every 6 unless told otherwise (even, as the graph body needs)
constexpr int kLearnedCheckEvery = 6;

}  // namespace

extern "C" {

ys_status ys_solve(ys_batch* b, const ys_solve_opts* opts, ys_cloth_stats* stats) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (!b->assembled) return fail(YS_ERR_ARG, "ys_solve before ys_assemble");
  YS_CUDA(cudaSetDevice(b->device));
  if (b->learn.kind == YS_PREC_LEARNED) return solve_learned(b, opts, stats);
  return solve_impl(b, b->v, opts, stats);
}

ys_status ys_get_solution(ys_batch* b, double* x, int32_t flags) {
  if (!b || !x) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(b->device));
  return download_aos(b, b->so.x, x, 5, flags);
}

ys_status ys_step(ys_batch* b, double h, const double* ext_force, int32_t flags, const ys_solve_opts* opts,
                  ys_cloth_stats* stats) {
  if (b && b->graph.enabled && !b->profiling) return ys_step_graphed(b, h, ext_force, flags, opts, stats);
  ys_status s = ys_assemble(b, h, ext_force, flags);
  if (s != YS_OK) return s;
  std::vector<ys_cloth_stats> local;
  ys_cloth_stats* st = stats;
  if (!st) {
    local.resize(b->ncloth);
    st = local.data();
  }
  ys_status sol = ys_solve(b, opts, st);
  if (sol == YS_ERR_ARG || sol == YS_ERR_CUDA) return sol;
  b->run(YS_PROF_UPDATE, 2, [&] { ys::launch_update(b->v, b->blk, b->so, b->stream); });
  YS_CUDA(cudaGetLastError());
  // the solution check may have flagged more cloths
  std::vector<ys::PcgCloth> pc(b->ncloth);
  YS_CUDA(cudaMemcpyAsync(pc.data(), b->so.pc, sizeof(ys::PcgCloth) * b->ncloth, cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  ys_status ret = sol;
  for (int c = 0; c < b->ncloth; ++c) {
    st[c].ok = (pc[c].status & 3) == 0;
    if (!st[c].ok) ret = YS_ERR_NONFINITE;
  }
  b->assembled = false;
  return ret;
}

ys_status ys_apply_system(ys_batch* b, const double* x, double* y, int32_t flags) {
  if (!b || !x || !y) return fail(YS_ERR_ARG, "bad argument");
  if (!b->assembled) return fail(YS_ERR_ARG, "no assembled system");
  YS_CUDA(cudaSetDevice(b->device));
  ys_status s = upload_soa(b, x, b->so.q, 5, flags);
  if (s != YS_OK) return s;
  b->run(YS_PROF_SPMV, 1, [&] { ys::launch_spmv(b->v, b->so.q, b->so.r, b->stream); });
  YS_CUDA(cudaGetLastError());
  return download_aos(b, b->so.r, y, 5, flags);
}

ys_status ys_export_system(ys_batch* b, int32_t cloth, double* Aout, double* rhs) {
  if (!b || cloth < 0 || cloth >= b->ncloth) return fail(YS_ERR_ARG, "bad argument");
  if (!b->assembled) return fail(YS_ERR_ARG, "no assembled system");
  YS_CUDA(cudaSetDevice(b->device));
  const ys::ClothParams& P = b->cp[cloth];
  const int W = P.W, H = P.H, N = W * H, off = P.node_off;
  const int64_t nt = b->ntot, dim = b->dims[cloth];
  std::vector<double> slots((size_t)ys::YS_NUM_SLOTS * N), bv(5 * (size_t)N);
  YS_CUDA(cudaMemcpy2DAsync(slots.data(), sizeof(double) * N, b->v.A + off, sizeof(double) * nt, sizeof(double) * N,
                            ys::YS_NUM_SLOTS, cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaMemcpy2DAsync(bv.data(), sizeof(double) * N, b->v.B + off, sizeof(double) * nt, sizeof(double) * N, 5,
                            cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  auto interior = [&](int u, int v) { return !(u == 0 || u == W - 1 || v == 0 || v == H - 1); };
  auto erow = [&](int u, int v) { return 3LL * N + 2LL * ((u - 1) + (v - 1) * (W - 2)); };
  auto S = [&](int sl, int n) { return slots[(size_t)sl * N + n]; };
  if (Aout) std::memset(Aout, 0, sizeof(double) * dim * dim);
  for (int vv = 0; vv < H; ++vv)
    for (int u = 0; u < W; ++u) {
      const int n = u + vv * W;
      const bool in = interior(u, vv);
      if (rhs) {
        for (int r = 0; r < 3; ++r) rhs[3 * n + r] = bv[(size_t)r * N + n];
        if (in)
          for (int k = 0; k < 2; ++k) rhs[erow(u, vv) + k] = bv[(size_t)(3 + k) * N + n];
      }
      if (!Aout) continue;
      for (int s = 0; s < ys::kNumStencil; ++s) {
        const int uu = u + ys::stencil_du(s), w2 = vv + ys::stencil_dv(s);
        if (uu < 0 || uu >= W || w2 < 0 || w2 >= H) continue;
        const int j = uu + w2 * W;
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) Aout[(3LL * n + r) * dim + 3LL * j + c] = S(ys::YS_SLOT_LL + 9 * s + 3 * r + c, n);
      }
      if (!in) continue;
      const int64_t er = erow(u, vv);
      for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 2; ++k) Aout[(3LL * n + r) * dim + er + k] = S(ys::YS_SLOT_LE_SELF + 2 * r + k, n);
      for (int k = 0; k < 2; ++k) {
        for (int c = 0; c < 3; ++c) Aout[(er + k) * dim + 3LL * n + c] = S(ys::YS_SLOT_EL_SELF + 3 * k + c, n);
        Aout[(er + k) * dim + er + k] = S(ys::YS_SLOT_EE_SELF + k, n);
      }
      for (int m = 0; m < 4; ++m) {
        const int du = m == 0 ? -1 : m == 1 ? 1 : 0, dv = m == 2 ? -1 : m == 3 ? 1 : 0, k = m < 2 ? 0 : 1;
        const int uu = u + du, w2 = vv + dv;
        if (!interior(uu, w2)) continue;
        const int j = uu + w2 * W;
        const int64_t ej = erow(uu, w2);
        for (int r = 0; r < 3; ++r) Aout[(3LL * n + r) * dim + ej + k] = S(ys::YS_SLOT_LE_NBR + 3 * m + r, n);
        for (int c = 0; c < 3; ++c) Aout[(er + k) * dim + 3LL * j + c] = S(ys::YS_SLOT_EL_NBR + 3 * m + c, n);
        Aout[(er + k) * dim + ej + k] = S(ys::YS_SLOT_EE_NBR + m, n);
      }
    }
  return YS_OK;
}

ys_status ys_profile(ys_batch* b, int32_t enable) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  YS_CUDA(cudaSetDevice(b->device));
  b->drain();
  b->profiling = enable != 0;
  return YS_OK;
}

ys_status ys_profile_read(ys_batch* b, double* ms, int64_t* launches_per_kind, int64_t* total_launches,
                          int32_t reset) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  YS_CUDA(cudaSetDevice(b->device));
  b->drain();
  for (int k = 0; k < YS_PROF_KINDS; ++k) {
    if (ms) ms[k] = b->prof_ms[k];
    if (launches_per_kind) launches_per_kind[k] = b->prof_n[k];
  }
  if (total_launches) *total_launches = b->launches;
  if (reset) {
    for (int k = 0; k < YS_PROF_KINDS; ++k) { b->prof_ms[k] = 0; b->prof_n[k] = 0; }
    b->launches = 0;
  }
  return YS_OK;
}

ys_status ys_synchronize(ys_batch* b) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  YS_CUDA(cudaSetDevice(b->device));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

}  // extern "C"

// ------------------------------------------------- y = A x without allocation
//
// ys_apply_system_noalloc is a variant of ys_apply_system for callers that
// must not allocate at call time: a host program whose device memory is
// entirely owned by another allocator (a framework's caching pool sized to
// the device, so a cudaMalloc here could fail or fragment it), and a control
// loop that cannot afford the device-wide synchronisation cudaMalloc and
// cudaFree may imply. It launches two kernels and allocates nothing: no
// cudaMalloc / cudaFree, no pinned memory, no events, no library routine that
// allocates. Its only working memory is the file-scope array below, and it
// writes no buffer of the batch (ys_apply_system writes two PCG work vectors).
//
// Nothing in the scratch needs to start at zero: the first kernel writes all
// 5 * total_nodes entries that the second kernel reads, in the same call.
//
// The scratch is one array per device shared by every batch and thread, so
// calls that overlap in time on one device race on it: two calls on
// different streams, or from different host threads without ordering, give
// wrong results. Issue them on one stream, or order them by the caller.
namespace {

constexpr int64_t kNoAllocMaxNodes = 65536;  // 5 * 65,536 doubles = 2.5 MiB per device
static __device__ __align__(256) double g_noalloc_scratch[5 * kNoAllocMaxNodes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {nullptr};

// y[n][k] = (A x)[n][k] with x read from the component-major scratch copy;
// same row arithmetic as k_spmv_plain, written node-major.
__global__ void k_spmv_scratch_to_aos(ys::View v, const double* __restrict__ xs, double* __restrict__ y) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.ntot) return;
  double r[5];
  ys::spmv_row(v, xs, n, r);
  for (int k = 0; k < 5; ++k) y[(int64_t)n * 5 + k] = r[k];
}

// The address of this device's copy of the scratch array, looked up with
// that device current. The first lookup on a device may make the runtime load
// this module there; make that first call before any stream capture begins.
// Outside stream capture the address is looked up again on every call (the
// lookup allocates nothing), so a context that was reset and reloaded the
// module elsewhere is followed; inside a capture the last address is reused.
ys_status noalloc_scratch(int device, cudaStream_t stream, double** out) {
  if (device < 0 || device >= kNoAllocMaxDevices) return fail(YS_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess) cs = cudaStreamCaptureStatusNone;
  if (!g_noalloc_ptr[device] || cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(YS_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[device] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[device];
  return YS_OK;
}

// x and y must be memory of the batch's device (or managed memory): a host
// array handed to the kernels would fault the device instead of returning an
// error. cudaPointerGetAttributes allocates nothing.
ys_status noalloc_check_device_ptr(const void* p, int device, const char* name) {
  cudaPointerAttributes a{};
  const cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(YS_ERR_ARG, std::string("ys_apply_system_noalloc: ") + name + " is not a device pointer");
  }
  if (a.type == cudaMemoryTypeManaged) return YS_OK;
  if (a.type != cudaMemoryTypeDevice)
    return fail(YS_ERR_ARG, std::string("ys_apply_system_noalloc: ") + name + " is not device memory");
  if (a.device != device)
    return fail(YS_ERR_ARG, std::string("ys_apply_system_noalloc: ") + name + " is memory of another device");
  return YS_OK;
}

}  // namespace

extern "C" ys_status ys_apply_system_noalloc(ys_batch* b, const double* x, double* y) {
  if (!b || !x || !y) return fail(YS_ERR_ARG, "bad argument");
  if (!b->assembled) return fail(YS_ERR_ARG, "no assembled system");
  if (b->ntot > kNoAllocMaxNodes)
    return fail(YS_ERR_ARG, "ys_apply_system_noalloc: batch has " + std::to_string(b->ntot) +
                                " nodes, more than its scratch limit of " + std::to_string(kNoAllocMaxNodes));
  YS_CUDA(cudaSetDevice(b->device));
  ys_status s = noalloc_check_device_ptr(x, b->device, "x");
  if (s != YS_OK) return s;
  s = noalloc_check_device_ptr(y, b->device, "y");
  if (s != YS_OK) return s;
  double* xs = nullptr;
  s = noalloc_scratch(b->device, b->stream, &xs);
  if (s != YS_OK) return s;
  const int64_t n = b->ntot;
  const unsigned grid = (unsigned)((n + 255) / 256);
  // Not timed by the handle's per-phase profile, whose records need CUDA
  // events: the two launches are counted, their time is in no phase.
  k_to_soa<<<grid, 256, 0, b->stream>>>(x, xs, n, 5);
  k_spmv_scratch_to_aos<<<grid, 256, 0, b->stream>>>(b->v, xs, y);
  b->launches += 2;
  YS_CUDA(cudaGetLastError());
  return YS_OK;
}

// ------------------------------------------------ forward-mode sensitivities
namespace {

constexpr int KT = ys::kTangents;

// [K][ntot][c] (node layout) <-> [c][K][ntot] (device tangent layout)
__global__ void k_tan_in(const double* __restrict__ src, double* __restrict__ dst, int64_t nt, int c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt * KT) return;
  const int64_t k = t / nt, i = t - k * nt;
  for (int j = 0; j < c; ++j) dst[((int64_t)j * KT + k) * nt + i] = src ? src[(k * nt + i) * c + j] : 0.0;
}
__global__ void k_tan_out(const double* __restrict__ src, double* __restrict__ dst, int64_t nt, int c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt * KT) return;
  const int64_t k = t / nt, i = t - k * nt;
  for (int j = 0; j < c; ++j) dst[(k * nt + i) * c + j] = src[((int64_t)j * KT + k) * nt + i];
}

ys_status tan_upload(ys_batch* b, const double* src, double* dst, int c, int32_t flags) {
  const int64_t nt = b->ntot, cnt = nt * KT;
  const double* d_src = nullptr;
  if (src) {
    d_src = src;
    if (!(flags & YS_ON_DEVICE)) {
      YS_CUDA(cudaMemcpyAsync(b->tan.io, src, sizeof(double) * cnt * c, cudaMemcpyHostToDevice, b->stream));
      d_src = b->tan.io;
    }
  }
  b->launches += 1;
  k_tan_in<<<(unsigned)((cnt + 255) / 256), 256, 0, b->stream>>>(d_src, dst, nt, c);
  YS_CUDA(cudaGetLastError());
  if (src && !(flags & YS_ON_DEVICE)) YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}
ys_status tan_download(ys_batch* b, const double* src, double* dst, int c, int32_t flags) {
  if (!dst) return YS_OK;
  const int64_t nt = b->ntot, cnt = nt * KT;
  double* d_dst = (flags & YS_ON_DEVICE) ? dst : b->tan.io;
  b->launches += 1;
  k_tan_out<<<(unsigned)((cnt + 255) / 256), 256, 0, b->stream>>>(src, d_dst, nt, c);
  YS_CUDA(cudaGetLastError());
  if (!(flags & YS_ON_DEVICE)) {
    YS_CUDA(cudaMemcpyAsync(dst, b->tan.io, sizeof(double) * cnt * c, cudaMemcpyDeviceToHost, b->stream));
    YS_CUDA(cudaStreamSynchronize(b->stream));
  }
  return YS_OK;
}

// the view of the dual assembly: values of A and b into shadows, tangents alongside
ys::View dual_view(ys_batch* b) {
  ys::View dv = b->v;
  const ys_batch::Tan& t = b->tan;
  dv.A = t.As;
  dv.B = t.Bs;
  dv.K = KT;
  dv.trunc = t.mode == YS_TANGENT_REFERENCE ? 1 : 0;
  dv.dX = t.dX; dv.dV = t.dV; dv.dUV = t.dUV; dv.dUVD = t.dUVD; dv.dUVB = t.dUVB;
  dv.dNRM = t.dNRM; dv.dCOMP = t.dCOMP; dv.dSLIDE = t.dSLIDE;
  dv.dline_rho = t.drho; dv.dline_ks = t.dks; dv.dline_kb = t.dkb; dv.dS = t.dS; dv.dmu = t.dmu;
  dv.dA = t.dA; dv.dB = t.dB;
  return dv;
}

}  // namespace

extern "C" {

int32_t ys_tangent_count(void) { return KT; }

ys_status ys_tangent_enable(ys_batch* b, int32_t mode) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (mode != YS_TANGENT_EXACT && mode != YS_TANGENT_REFERENCE)
    return fail(YS_ERR_ARG, "tangent mode must be YS_TANGENT_EXACT or YS_TANGENT_REFERENCE");
  YS_CUDA(cudaSetDevice(b->device));
  ys_batch::Tan& t = b->tan;
  const size_t nt = b->ntot, nl = b->nlines, nc = b->ncloth;
  if (!t.on) {
    ys_status st = YS_OK;
    auto A = [&](double** p, size_t cnt) { if (st == YS_OK) st = b->alloc(p, cnt); };
    A(&t.dX, 3 * KT * nt); A(&t.dV, 3 * KT * nt); A(&t.dUV, 2 * KT * nt); A(&t.dUVD, 2 * KT * nt);
    A(&t.dUVB, 2 * KT * nt); A(&t.dNRM, 3 * KT * nt); A(&t.dCOMP, KT * nt); A(&t.dSLIDE, 2 * KT * nt);
    A(&t.drho, KT * nl); A(&t.dks, KT * nl); A(&t.dkb, KT * nl); A(&t.dS, KT * nc); A(&t.dmu, KT * nc);
    A(&t.dA, (size_t)ys::YS_NUM_SLOTS * KT * nt); A(&t.dB, 5 * KT * nt);
    A(&t.As, (size_t)ys::YS_NUM_SLOTS * nt); A(&t.Bs, 5 * nt); A(&t.qsave, 5 * nt); A(&t.rt, 5 * KT * nt);
    A(&t.dq, 5 * KT * nt);
    A(&t.dedge, (size_t)ys::kEdgeFields * 2 * KT * nt); A(&t.dbend, (size_t)ys::kBendFields * 2 * KT * nt);
    A(&t.dface, 6 * KT * nt); A(&t.dshear, (size_t)ys::kShearFields * 4 * KT * nt);
    A(&t.io, 3 * KT * nt);
    if (st != YS_OK) return st;
    t.on = true;
  }
  t.mode = mode;
  auto Z = [&](double* p, size_t cnt) { return cudaMemsetAsync(p, 0, sizeof(double) * cnt, b->stream); };
  if (Z(t.dX, 3 * KT * nt) || Z(t.dV, 3 * KT * nt) || Z(t.dUV, 2 * KT * nt) || Z(t.dUVD, 2 * KT * nt) ||
      Z(t.dUVB, 2 * KT * nt) || Z(t.drho, KT * nl) || Z(t.dks, KT * nl) || Z(t.dkb, KT * nl) || Z(t.dS, KT * nc) ||
      Z(t.dmu, KT * nc) || Z(t.dq, 5 * KT * nt))
    return fail(YS_ERR_CUDA, "cudaMemsetAsync failed");
  YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

ys_status ys_tangent_seed(ys_batch* b, const double* drho, const double* dY, const double* dB, const double* dS,
                          const double* dmu) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (!b->tan.on) return fail(YS_ERR_ARG, "ys_tangent_seed before ys_tangent_enable");
  YS_CUDA(cudaSetDevice(b->device));
  const size_t nl = b->nlines, nc = b->ncloth;
  std::vector<double> r(KT * nl, 0.0), ks(KT * nl, 0.0), kb(KT * nl, 0.0), S(KT * nc, 0.0), mu(KT * nc, 0.0);
  for (int k = 0; k < KT; ++k)
    for (size_t l = 0; l < nl; ++l) {
      const size_t i = k * nl + l;
      const double a = ys::kPi * std::pow(b->line_R[l], 2);  // ks, kb = (Y, B) pi R^2 (src/Yarn.h:14-15)
      if (drho) r[i] = drho[i];
      if (dY) ks[i] = dY[i] * a;
      if (dB) kb[i] = dB[i] * a;
    }
  for (size_t i = 0; i < KT * nc; ++i) {
    if (dS) S[i] = dS[i];
    if (dmu) mu[i] = dmu[i];
  }
  const ys_batch::Tan& t = b->tan;
  YS_CUDA(cudaMemcpyAsync(t.drho, r.data(), sizeof(double) * r.size(), cudaMemcpyHostToDevice, b->stream));
  YS_CUDA(cudaMemcpyAsync(t.dks, ks.data(), sizeof(double) * ks.size(), cudaMemcpyHostToDevice, b->stream));
  YS_CUDA(cudaMemcpyAsync(t.dkb, kb.data(), sizeof(double) * kb.size(), cudaMemcpyHostToDevice, b->stream));
  YS_CUDA(cudaMemcpyAsync(t.dS, S.data(), sizeof(double) * S.size(), cudaMemcpyHostToDevice, b->stream));
  YS_CUDA(cudaMemcpyAsync(t.dmu, mu.data(), sizeof(double) * mu.size(), cudaMemcpyHostToDevice, b->stream));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

ys_status ys_tangent_set_state(ys_batch* b, const double* dlpos, const double* dlvel, const double* depos,
                               const double* deposbar, const double* devel, int32_t flags) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (!b->tan.on) return fail(YS_ERR_ARG, "ys_tangent_set_state before ys_tangent_enable");
  YS_CUDA(cudaSetDevice(b->device));
  const ys_batch::Tan& t = b->tan;
  ys_status s;
  if ((s = tan_upload(b, dlpos, t.dX, 3, flags)) != YS_OK) return s;
  if ((s = tan_upload(b, dlvel, t.dV, 3, flags)) != YS_OK) return s;
  if ((s = tan_upload(b, depos, t.dUV, 2, flags)) != YS_OK) return s;
  if ((s = tan_upload(b, deposbar, t.dUVB, 2, flags)) != YS_OK) return s;
  if ((s = tan_upload(b, devel, t.dUVD, 2, flags)) != YS_OK) return s;
  YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

ys_status ys_tangent_get_state(ys_batch* b, double* dlpos, double* dlvel, double* depos, double* deposbar,
                               double* devel, int32_t flags) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (!b->tan.on) return fail(YS_ERR_ARG, "ys_tangent_get_state before ys_tangent_enable");
  YS_CUDA(cudaSetDevice(b->device));
  const ys_batch::Tan& t = b->tan;
  ys_status s;
  if ((s = tan_download(b, t.dX, dlpos, 3, flags)) != YS_OK) return s;
  if ((s = tan_download(b, t.dV, dlvel, 3, flags)) != YS_OK) return s;
  if ((s = tan_download(b, t.dUV, depos, 2, flags)) != YS_OK) return s;
  if ((s = tan_download(b, t.dUVB, deposbar, 2, flags)) != YS_OK) return s;
  if ((s = tan_download(b, t.dUVD, devel, 2, flags)) != YS_OK) return s;
  YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

ys_status ys_step_tangent(ys_batch* b, double h, const double* ext_force, int32_t flags, const ys_solve_opts* opts,
                          int32_t kact, ys_cloth_stats* stats) {
  return ys_step_tangent_ext(b, h, ext_force, nullptr, flags, opts, kact, stats);
}

ys_status ys_step_tangent_ext(ys_batch* b, double h, const double* ext_force, const double* dext_force, int32_t flags,
                              const ys_solve_opts* opts, int32_t kact, ys_cloth_stats* stats) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (!b->tan.on) return fail(YS_ERR_ARG, "ys_step_tangent before ys_tangent_enable");
  if (kact < 0 || kact > KT) return fail(YS_ERR_ARG, "kact must be in [0, ys_tangent_count()]");
  const double* d_dext = nullptr;
  if (dext_force && kact > 0) {
    if (!b->tan.dext) {
      const ys_status sa = b->alloc(&b->tan.dext, (size_t)KT * 5 * b->ntot);
      if (sa != YS_OK) return sa;
    }
    YS_CUDA(cudaMemcpyAsync(b->tan.dext, dext_force, sizeof(double) * 5 * b->ntot * kact,
                            (flags & YS_ON_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream));
    d_dext = b->tan.dext;
  }
  ys_status s = ys_assemble(b, h, ext_force, flags);
  if (s != YS_OK) return s;
  std::vector<ys_cloth_stats> local;
  ys_cloth_stats* st = stats;
  if (!st) {
    local.resize(b->ncloth);
    st = local.data();
  }
  const ys_status sol = solve_impl(b, b->v, opts, st);
  if (sol == YS_ERR_ARG || sol == YS_ERR_CUDA) return sol;
  cudaStream_t cs = b->stream;
  const int64_t nt = b->ntot;
  ys_batch::Tan& t = b->tan;
  YS_CUDA(cudaMemcpyAsync(t.qsave, b->so.x, sizeof(double) * 5 * nt, cudaMemcpyDeviceToDevice, cs));
  // dual assembly: tangents of A and b
  ys::View dv = dual_view(b);
  ys::Records dr = b->rec;
  dr.dedge = t.dedge; dr.dbend = t.dbend; dr.dface = t.dface; dr.dshear = t.dshear;
  b->run(YS_PROF_MISC, 7, [&] { ys::launch_assembly_dual(dv, dr, b->anchors, b->geom_n, cs); });
  YS_CUDA(cudaGetLastError());
  b->run(YS_PROF_MISC, 1, [&] { ys::launch_tangent_rhs(dv, t.qsave, t.rt, kact, cs); });
  YS_CUDA(cudaGetLastError());
  if (d_dext) {
    b->run(YS_PROF_MISC, 1, [&] { ys::launch_tangent_ext(dv, d_dext, t.rt, h, kact, cs); });
    YS_CUDA(cudaGetLastError());
  }
  // tangent solves with the step's A and Jacobi diagonal: A dq_k = db_k - dA_k q
  // (exact), or A^T dq_k = db_k with M, D held constant -- the transpose of
  // the reference's backward b_bar = A^-1 q_bar (src/Solvers.cpp:33-58)
  for (int k = 0; k < kact; ++k) {
    ys::View vk = b->v;
    vk.B = t.rt + (int64_t)k * 5 * nt;
    b->so.trans = t.mode == YS_TANGENT_REFERENCE ? 1 : 0;
    const ys_status sk = solve_impl(b, vk, opts, nullptr);
    b->so.trans = 0;
    if (sk == YS_ERR_ARG || sk == YS_ERR_CUDA) return sk;
    YS_CUDA(cudaMemcpy2DAsync(t.dq + (int64_t)k * nt, sizeof(double) * KT * nt, b->so.x, sizeof(double) * nt,
                              sizeof(double) * nt, 5, cudaMemcpyDeviceToDevice, cs));
  }
  YS_CUDA(cudaMemcpyAsync(b->so.x, t.qsave, sizeof(double) * 5 * nt, cudaMemcpyDeviceToDevice, cs));
  ys::TangentState ts{t.dX, t.dV, t.dUV, t.dUVD, t.dUVB};
  b->run(YS_PROF_UPDATE, 2, [&] { ys::launch_update_dual(dv, b->blk, b->so, t.dq, ts, cs); });
  YS_CUDA(cudaGetLastError());
  std::vector<ys::PcgCloth> pc(b->ncloth);
  YS_CUDA(cudaMemcpyAsync(pc.data(), b->so.pc, sizeof(ys::PcgCloth) * b->ncloth, cudaMemcpyDeviceToHost, cs));
  YS_CUDA(cudaStreamSynchronize(cs));
  ys_status ret = sol;
  for (int c = 0; c < b->ncloth; ++c) {
    st[c].ok = (pc[c].status & 3) == 0;
    if (!st[c].ok) ret = YS_ERR_NONFINITE;
  }
  b->assembled = false;
  return ret;
}

}  // extern "C"


// ------------------------------------------------------------ reverse mode
struct ys_adjoint {
  ys_batch* prim = nullptr;  // the caller's batch (not owned)
  ys_batch* cp = nullptr;    // `copies` copies of prim's cloths, copy-major (owned)
  int mode = YS_TANGENT_EXACT;
  int copies = 0, passes = 0;
  std::vector<void*> allocs;
  double *q = nullptr, *qbar = nullptr, *lambda = nullptr, *slide_bar = nullptr, *T = nullptr;
  double* gin[5] = {nullptr};
  double* gout[5] = {nullptr};
  double* gline[3] = {nullptr};
  double* gcloth[2] = {nullptr};
  double* gext = nullptr;      // [nt][5]
  double* line_a = nullptr;    // pi R^2 per primal line
  int* line_kind = nullptr;    // orientation * 3 + position mod 3
  int* line_cloth = nullptr;
  template <class T_>
  ys_status alloc(T_** p, size_t count) {
    void* m = nullptr;
    const cudaError_t e = cudaMalloc(&m, std::max<size_t>(count, 1) * sizeof(T_));
    if (e != cudaSuccess) return fail(YS_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    allocs.push_back(m);
    *p = static_cast<T_*>(m);
    return YS_OK;
  }
  ~ys_adjoint() {
    if (prim) cudaSetDevice(prim->device);
    for (void* m : allocs) cudaFree(m);
    if (cp) ys_batch_destroy(cp);
  }
};

namespace {

constexpr int kStateComps[5] = {3, 3, 2, 2, 2};

__global__ void k_adj_copy_wind(const ys::ClothParams* __restrict__ src, ys::ClothParams* dst, int ncl, int copies) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncl * copies) return;
  const ys::ClothParams& a = src[t % ncl];
  ys::ClothParams& d = dst[t];
  for (int k = 0; k < 3; ++k) d.wind[k] = a.wind[k];
}

}  // namespace

extern "C" {

ys_status ys_adjoint_create(ys_batch* b, int32_t mode, int32_t copies, ys_adjoint** out) {
  if (!b || !out) return fail(YS_ERR_ARG, "null argument");
  *out = nullptr;
  if (mode != YS_TANGENT_EXACT && mode != YS_TANGENT_REFERENCE)
    return fail(YS_ERR_ARG, "adjoint mode must be YS_TANGENT_EXACT or YS_TANGENT_REFERENCE");
  const int ndir = ys::adjoint_direction_count();
  const int maxc = (ndir + KT - 1) / KT;
  if (copies < 1 || copies > maxc) return fail(YS_ERR_ARG, "copies must be in [1, 128]");
  YS_CUDA(cudaSetDevice(b->device));
  ys_adjoint* a = new ys_adjoint();
  a->prim = b;
  a->mode = mode;
  a->copies = copies;
  a->passes = (maxc + copies - 1) / copies;
  // the copies' batch: the same cloths, `copies` times, on b's stream
  std::vector<ys_cloth_desc> d;
  d.reserve((size_t)copies * b->ncloth);
  for (int c = 0; c < copies; ++c)
    for (const ys_batch::DescStore& ds : b->descs) {
      ys_cloth_desc e = ds.d;
      e.warp_rho = ds.wr.data(); e.warp_Y = ds.wY.data(); e.warp_B = ds.wB.data();
      e.weft_rho = ds.fr.data(); e.weft_Y = ds.fY.data(); e.weft_B = ds.fB.data();
      e.handles = ds.handles.empty() ? nullptr : ds.handles.data();
      d.push_back(e);
    }
  ys_status st = ys_batch_create((int32_t)d.size(), d.data(), b->device, b->stream, &a->cp);
  if (st == YS_OK) st = ys_tangent_enable(a->cp, mode);
  const int64_t nt = b->ntot, ntc = a->cp ? a->cp->ntot : 0;
  auto A = [&](auto** p, size_t cnt) { if (st == YS_OK) st = a->alloc(p, cnt); };
  A(&a->q, 5 * nt); A(&a->qbar, 5 * nt); A(&a->lambda, 5 * nt); A(&a->slide_bar, 2 * nt);
  A(&a->T, (size_t)KT * ntc);
  for (int i = 0; i < 5; ++i) { A(&a->gin[i], kStateComps[i] * nt); A(&a->gout[i], kStateComps[i] * nt); }
  for (int i = 0; i < 3; ++i) A(&a->gline[i], b->nlines);
  for (int i = 0; i < 2; ++i) A(&a->gcloth[i], b->ncloth);
  A(&a->gext, 5 * nt);
  A(&a->line_a, b->nlines); A(&a->line_kind, b->nlines); A(&a->line_cloth, b->nlines);
  if (st != YS_OK) { delete a; return st; }
  std::vector<double> la;
  std::vector<int> lk, lc;
  for (int c = 0; c < b->ncloth; ++c) {
    const ys::ClothParams& P = b->cp[c];
    for (int v = 0; v < P.H; ++v) { lk.push_back(0 * 3 + v % 3); lc.push_back(c); la.push_back(ys::kPi * P.R * P.R); }
    for (int u = 0; u < P.W; ++u) { lk.push_back(1 * 3 + u % 3); lc.push_back(c); la.push_back(ys::kPi * P.R * P.R); }
  }
  if (cudaMemcpy(a->line_a, la.data(), sizeof(double) * la.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(a->line_kind, lk.data(), sizeof(int) * lk.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(a->line_cloth, lc.data(), sizeof(int) * lc.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    delete a;
    return fail(YS_ERR_CUDA, "cudaMemcpy of the adjoint's line tables failed");
  }
  *out = a;
  return YS_OK;
}

void ys_adjoint_destroy(ys_adjoint* a) { delete a; }

ys_status ys_adjoint_step(ys_adjoint* a, double h, const double* ext_force, const double* const* gin,
                          double* const* gout, double* const* gparams, double* gext, int32_t flags,
                          const ys_solve_opts* opts, ys_cloth_stats* stats) {
  if (!a || !(h > 0)) return fail(YS_ERR_ARG, "bad argument");
  ys_batch* b = a->prim;
  ys_batch* c = a->cp;
  YS_CUDA(cudaSetDevice(b->device));
  cudaStream_t s = b->stream;
  const int64_t nt = b->ntot, ntc = c->ntot;
  // 1. the forward step's system and solution at the current state
  ys_status st = ys_assemble(b, h, ext_force, flags);
  if (st != YS_OK) return st;
  st = solve_impl(b, b->v, opts, stats);
  if (st == YS_ERR_ARG || st == YS_ERR_CUDA) return st;
  if (st == YS_ERR_NONFINITE) return fail(YS_ERR_NONFINITE, "ys_adjoint_step: the forward step is not finite");
  YS_CUDA(cudaMemcpyAsync(a->q, b->so.x, sizeof(double) * 5 * nt, cudaMemcpyDeviceToDevice, s));
  // 2. the update's transpose
  for (int i = 0; i < 5; ++i) {
    if (gin && gin[i]) {
      st = upload_soa(b, gin[i], a->gin[i], kStateComps[i], flags);
      if (st != YS_OK) return st;
    } else {
      YS_CUDA(cudaMemsetAsync(a->gin[i], 0, sizeof(double) * kStateComps[i] * nt, s));
    }
  }
  ys::AdjIO io{};
  for (int i = 0; i < 5; ++i) { io.gin[i] = a->gin[i]; io.gout[i] = a->gout[i]; }
  b->v.h = h;
  b->run(YS_PROF_MISC, 1, [&] { ys::launch_adj_update(b->v, io, a->q, a->qbar, a->slide_bar, s); });
  YS_CUDA(cudaGetLastError());
  // 3. lambda = A^-T q_bar (exact) or A^-1 q_bar (the reference's backward)
  {
    ys::View vl = b->v;
    vl.B = a->qbar;
    b->so.trans = a->mode == YS_TANGENT_EXACT ? 1 : 0;
    st = solve_impl(b, vl, opts, nullptr);
    b->so.trans = 0;
    if (st == YS_ERR_ARG || st == YS_ERR_CUDA) return st;
    if (st == YS_ERR_NONFINITE) return fail(YS_ERR_NONFINITE, "ys_adjoint_step: the adjoint solve is not finite");
    YS_CUDA(cudaMemcpyAsync(a->lambda, b->so.x, sizeof(double) * 5 * nt, cudaMemcpyDeviceToDevice, s));
    YS_CUDA(cudaMemcpyAsync(b->so.x, a->q, sizeof(double) * 5 * nt, cudaMemcpyDeviceToDevice, s));
  }
  // 4. the copies take the state, wind, step size and external force
  {
    ys::View& vc = c->v;
    const ys::View& vb = b->v;
    const int cps = a->copies;
    b->run(YS_PROF_MISC, 7, [&] {
      ys::launch_adj_broadcast(vb.X, vc.X, (int)nt, 3, cps, s);
      ys::launch_adj_broadcast(vb.V, vc.V, (int)nt, 3, cps, s);
      ys::launch_adj_broadcast(vb.XF, vc.XF, (int)nt, 3, cps, s);
      ys::launch_adj_broadcast(vb.UV, vc.UV, (int)nt, 2, cps, s);
      ys::launch_adj_broadcast(vb.UVD, vc.UVD, (int)nt, 2, cps, s);
      ys::launch_adj_broadcast(vb.UVB, vc.UVB, (int)nt, 2, cps, s);
      k_adj_copy_wind<<<(b->ncloth * cps + 127) / 128, 128, 0, s>>>(vb.cp, const_cast<ys::ClothParams*>(vc.cp),
                                                                     b->ncloth, cps);
    });
    vc.h = h;
    vc.ext = nullptr;
    if (ext_force) {
      b->run(YS_PROF_MISC, 1, [&] { ys::launch_adj_broadcast(b->ext, c->ext, (int)nt, 5, cps, s); });
      vc.ext = c->ext;
    }
    YS_CUDA(cudaGetLastError());
  }
  // 5. the residual's vector-Jacobian product, pass by pass
  for (int i = 0; i < 3; ++i) YS_CUDA(cudaMemsetAsync(a->gline[i], 0, sizeof(double) * b->nlines, s));
  for (int i = 0; i < 2; ++i) YS_CUDA(cudaMemsetAsync(a->gcloth[i], 0, sizeof(double) * b->ncloth, s));
  ys::AdjParamOut gp{{a->gline[0], a->gline[1], a->gline[2]}, {a->gcloth[0], a->gcloth[1]}};
  ys_batch::Tan& t = c->tan;
  ys::AdjSeeds sd{t.dX, t.dV, t.dUV, t.dUVD, t.dUVB, t.drho, t.dks, t.dkb, t.dS, t.dmu};
  ys::View dv = dual_view(c);
  ys::Records dr = c->rec;
  dr.dedge = t.dedge; dr.dbend = t.dbend; dr.dface = t.dface; dr.dshear = t.dshear;
  for (int p = 0; p < a->passes; ++p) {
    const int base = p * a->copies;
    b->run(YS_PROF_MISC, 2, [&] {
      ys::launch_adj_seed(c->v, (int)nt, b->nlines, b->ncloth, base, a->line_a, a->line_kind, sd, s);
    });
    b->run(YS_PROF_MISC, 7, [&] { ys::launch_assembly_dual(dv, dr, c->anchors, c->geom_n, s); });
    b->run(YS_PROF_MISC, 2, [&] {
      ys::launch_adj_broadcast(a->q, t.qsave, (int)nt, 5, a->copies, s);
      ys::launch_tangent_rhs(dv, t.qsave, t.rt, KT, s);
    });
    b->run(YS_PROF_MISC, 3, [&] {
      ys::launch_adj_contract(dv, (int)nt, a->lambda, a->slide_bar, t.rt, a->T, s);
      ys::launch_adj_gather(b->v, base, a->copies, a->T, ntc, a->line_cloth, a->line_kind, io, gp, s);
    });
    YS_CUDA(cudaGetLastError());
  }
  // 6. outputs
  for (int i = 0; i < 5; ++i)
    if (gout && gout[i]) {
      st = download_aos(b, a->gout[i], gout[i], kStateComps[i], flags);
      if (st != YS_OK) return st;
    }
  const cudaMemcpyKind dk = (flags & YS_ON_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (gparams) {
    for (int i = 0; i < 3; ++i)
      if (gparams[i]) YS_CUDA(cudaMemcpyAsync(gparams[i], a->gline[i], sizeof(double) * b->nlines, dk, s));
    for (int i = 0; i < 2; ++i)
      if (gparams[3 + i]) YS_CUDA(cudaMemcpyAsync(gparams[3 + i], a->gcloth[i], sizeof(double) * b->ncloth, dk, s));
  }
  if (gext) {
    b->run(YS_PROF_MISC, 1, [&] { ys::launch_adj_ext(b->v, a->lambda, a->gext, s); });
    YS_CUDA(cudaMemcpyAsync(gext, a->gext, sizeof(double) * 5 * nt, dk, s));
  }
  YS_CUDA(cudaStreamSynchronize(s));
  YS_CUDA(cudaGetLastError());
  b->assembled = false;
  return YS_OK;
}

}  // extern "C"


// ----------------------------------------------------------- graphed step
namespace {

// The PCG's vectors (x, r, p, q, dinv: 200 B a node) as an L2 access-policy
// window on the capture stream, so the kernels captured from it keep them in
// L2 while the SpMV streams the matrix (1,272 B a node) through it: a
// persisting set-aside of up to the device's maximum for this context, the
// window's hit ratio scaled down when the vectors outgrow it.
void l2_window_setup(ys_batch* b, cudaStream_t s) {
  if (!b->vecs) return;
  if (!b->l2_window) {
    int max_persist = 0, max_window = 0;
    if (cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, b->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, b->device) != cudaSuccess ||
        max_persist <= 0 || max_window <= 0) {
      cudaGetLastError();
      return;
    }
    const size_t bytes = sizeof(double) * 25 * (size_t)b->ntot;
    const size_t window = std::min(bytes, (size_t)max_window);
    const size_t persist = std::min(window, (size_t)max_persist);
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, persist) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    b->l2_window = window;
    b->l2_hit = (float)((double)persist / (double)window);
  }
  cudaStreamAttrValue a = {};
  a.accessPolicyWindow.base_ptr = b->vecs;
  a.accessPolicyWindow.num_bytes = b->l2_window;
  a.accessPolicyWindow.hitRatio = b->l2_hit;
  a.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
  a.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  if (cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &a) != cudaSuccess) cudaGetLastError();
}

ys_status graph_prepare(ys_batch* b) {
  ys_batch::Graph& G = b->graph;
  if (!G.capture) {
    YS_CUDA(cudaStreamCreateWithFlags(&G.capture, cudaStreamNonBlocking));
    l2_window_setup(b, G.capture);
  }
  for (int k = 0; k < 2; ++k) {
    if (!G.side[k]) YS_CUDA(cudaStreamCreateWithFlags(&G.side[k], cudaStreamNonBlocking));
    if (!G.join[k]) YS_CUDA(cudaEventCreateWithFlags(&G.join[k], cudaEventDisableTiming));
  }
  if (!G.fork) YS_CUDA(cudaEventCreateWithFlags(&G.fork, cudaEventDisableTiming));
  ys_status s = YS_OK;
  if (!G.it_base && (s = b->alloc(&G.it_base, 1)) != YS_OK) return s;
  if (!G.hold && (s = b->alloc(&G.hold, 1)) != YS_OK) return s;
  return YS_OK;
}

// the kernels of ys_assemble and the PCG counters' reset, onto a capturing
// stream. The producers form three branches of the graph, each writing its
// own record buffer from the state: normals then bends (bends read the
// normals), edges, faces; the gather joins them.
void capture_assembly(ys_batch* b, cudaStream_t cs, int override_max) {
  const ys::View& v = b->v;
  const ys::Records& R = b->rec;
  ys_batch::Graph& G = b->graph;
  k_reset_status<<<(b->ncloth + 127) / 128, 128, 0, cs>>>(b->so.pc, b->ncloth);
  cudaEventRecord(G.fork, cs);
  for (int k = 0; k < 2; ++k) cudaStreamWaitEvent(G.side[k], G.fork, 0);
  ys::launch_edge_records(v, R, G.side[0], b->producer_threads);
  ys::launch_face_records(v, R, G.side[1], b->producer_threads);
  if (b->geom_n) ys::launch_geom(v, b->anchors + b->geom_off, b->geom_n, cs);
  ys::launch_bend_records(v, R, cs, b->producer_threads);
  for (int k = 0; k < 2; ++k) {
    cudaEventRecord(G.join[k], G.side[k]);
    cudaStreamWaitEvent(cs, G.join[k], 0);
  }
  ys::launch_gather(v, R, cs, b->producer_threads);
  ys::launch_shear_records(v, R, cs, b->producer_threads);
  ys::launch_finalize(v, R, b->blk, b->so, cs);
  k_reset_pc<<<(b->ncloth + 127) / 128, 128, 0, cs>>>(b->so.pc, b->maxiter_dev, b->ncloth, override_max);
}

// main = pre -> while (condition) { body } -> post, each part captured from
// the launches its function makes on the capture stream; body ends with the
// kernel that sets the condition (handed to it)
template <class Pre, class Body, class Post>
ys_status build_loop_graph(ys_batch* b, Pre pre_fn, Body body_fn, Post post_fn, cudaGraph_t* main,
                           cudaGraphExec_t* exec) {
  cudaStream_t cs = b->graph.capture;
  cudaGraph_t pre = nullptr, post = nullptr;
  YS_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  pre_fn(cs);
  YS_CUDA(cudaStreamEndCapture(cs, &pre));
  YS_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  post_fn(cs);
  YS_CUDA(cudaStreamEndCapture(cs, &post));
  YS_CUDA(cudaGraphCreate(main, 0));
  cudaGraphNode_t n_pre, n_loop, n_post;
  YS_CUDA(cudaGraphAddChildGraphNode(&n_pre, *main, nullptr, 0, pre));
  cudaGraphConditionalHandle hcond;
  YS_CUDA(cudaGraphConditionalHandleCreate(&hcond, *main, 1, cudaGraphCondAssignDefault));
  // cudaGraphNodeParams has no default constructor: zeroed storage instead
  alignas(cudaGraphNodeParams) unsigned char cp_raw[sizeof(cudaGraphNodeParams)] = {};
  cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cp_raw);
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hcond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  YS_CUDA(cudaGraphAddNode(&n_loop, *main, &n_pre, nullptr, 1, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  YS_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  body_fn(cs, hcond);
  YS_CUDA(cudaStreamEndCapture(cs, &body));
  YS_CUDA(cudaGraphAddChildGraphNode(&n_post, *main, &n_loop, 1, post));
  cudaGraphDestroy(pre);
  cudaGraphDestroy(post);
  YS_CUDA(cudaGraphInstantiate(exec, *main, 0));
  return YS_OK;
}

// the Jacobi-PCG step: assembly and PCG set-up, a conditional while node whose
// body is m PCG iterations (m even keeps the r.z parity of each iteration
// equal to its local index's) and the condition, then the solution check and
// Cloth::update. With the persistent PCG the solve is one kernel: one graph.
ys_status graph_build(ys_batch* b, int m, int cap, int override_max) {
  ys_batch::Graph& G = b->graph;
  if (G.exec) { cudaGraphExecDestroy(G.exec); G.exec = nullptr; }
  if (G.main) { cudaGraphDestroy(G.main); G.main = nullptr; }
  ys_status st = graph_prepare(b);
  if (st != YS_OK) return st;
  ys::Solver so = b->so;
  so.it_base = G.it_base;
  const ys::View& v = b->v;
  cudaStream_t cs = G.capture;
  if (b->plan.kind == YS_PCG_PERSISTENT) {
    YS_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    capture_assembly(b, cs, override_max);
    const cudaError_t e =
        ys::launch_pcg_cluster(v, so, b->plan.order, b->ncloth, b->plan.threads, b->plan.csize, cap, cs);
    ys::launch_update(v, b->blk, b->so, cs);
    cudaGraph_t one = nullptr;
    YS_CUDA(cudaStreamEndCapture(cs, &one));
    if (e != cudaSuccess) {
      cudaGraphDestroy(one);
      return fail(YS_ERR_CUDA, std::string("persistent PCG: ") + cudaGetErrorString(e));
    }
    G.main = one;
    YS_CUDA(cudaGraphInstantiate(&G.exec, G.main, 0));
    return YS_OK;
  }
  return build_loop_graph(
      b,
      [&](cudaStream_t c) {
        capture_assembly(b, c, override_max);
        ys::launch_pcg_setup(v, b->blk, so, c);
        ys::launch_graph_loop_begin(so, c);
      },
      [&](cudaStream_t c, cudaGraphConditionalHandle h) {
        for (int j = 0; j < m; ++j) {
          ys::launch_pcg_spmv(v, b->blk, so, c);
          ys::launch_pcg_axpy(v, b->blk, so, j, c);
          ys::launch_pcg_dir(v, b->blk, so, j, c);
        }
        ys::launch_graph_loop_tail(so, b->ncloth, m, cap, h, c);
      },
      [&](cudaStream_t c) { ys::launch_update(v, b->blk, b->so, c); }, &G.main, &G.exec);
}

ys_status graph_build_learned(ys_batch* b, int m, int cap, int override_max, int with_net);
ys_status learn_ensure(ys_batch* b);

// a step's result from the cloths' PCG records (read after the update)
ys_status step_result(ys_batch* b, const std::vector<ys::PcgCloth>& pc, ys_cloth_stats* stats) {
  ys_status ret = YS_OK;
  for (int c = 0; c < b->ncloth; ++c) {
    if (pc[c].status & 3) ret = YS_ERR_NONFINITE;
    else if ((pc[c].status & 4) && ret == YS_OK) ret = YS_ERR_MAXITER;
    if (stats) {
      stats[c].ok = (pc[c].status & 3) == 0;
      stats[c].cg_iterations = pc[c].iters;
      stats[c].cg_error = pc[c].bb > 0 ? std::sqrt(pc[c].rr / pc[c].bb) : 0.0;
      stats[c].hit_maxiter = (pc[c].status & 4) ? 1 : 0;
    }
  }
  b->assembled = false;
  return ret;
}

// the graphed step with the learned preconditioner: one graph with the
// network evaluated after the assembly, one without (G reused), chosen as
// the launch-by-launch solve chooses; when the graph's verdict kernel held
// the update back, the assembled system is solved again by Jacobi-PCG and
// updated launch by launch
ys_status step_graphed_learned(ys_batch* b, const ys_solve_opts* opts, ys_cloth_stats* stats, int m, int cap,
                               int override_max) {
  ys_batch::Graph& G = b->graph;
  ys_batch::Learn& L = b->learn;
  if (!L.net) return fail(YS_ERR_ARG, "learned preconditioner without a network");
  ys_status st = learn_ensure(b);
  if (st != YS_OK) return st;
  const int with_net = (!L.have_g || ++L.since >= L.refresh_every) ? 1 : 0;
  if (!G.lexec[with_net]) {
    st = graph_build_learned(b, m, cap, override_max, with_net);
    if (st != YS_OK) {
      G.drop();
      return st;
    }
  }
  YS_CUDA(cudaGraphLaunch(G.lexec[with_net], b->stream));
  if (with_net) {
    L.have_g = true;
    L.since = 0;
  }
  L.solves += 1;
  std::vector<ys::PcgCloth> pc(b->ncloth);
  YS_CUDA(cudaMemcpyAsync(pc.data(), b->so.pc, sizeof(ys::PcgCloth) * b->ncloth, cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaMemcpyAsync(&G.h_it, G.it_base, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaMemcpyAsync(&G.h_hold, G.hold, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  // kernels the graph ran: 11 (+ geometry) before the network, 8 for the
  // network, 4 before the loop, 4 per iteration + 1 per trip, 3 after
  b->launches += 18 + (b->geom_n ? 1 : 0) + 8 * with_net + 4LL * G.h_it + G.h_it / m;
  if (!G.h_hold) return step_result(b, pc, stats);
  L.fallbacks += 1;
  YS_CUDA(cudaMemsetAsync(L.g.err, 0, sizeof(int), b->stream));
  b->launches += 1;
  std::vector<ys_cloth_stats> local;
  ys_cloth_stats* sts = stats;
  if (!sts) {
    local.resize(b->ncloth);
    sts = local.data();
  }
  const ys_status sol = solve_impl(b, b->v, opts, sts);
  if (sol == YS_ERR_ARG || sol == YS_ERR_CUDA) return sol;
  b->run(YS_PROF_UPDATE, 2, [&] { ys::launch_update(b->v, b->blk, b->so, b->stream); });
  YS_CUDA(cudaGetLastError());
  YS_CUDA(cudaMemcpyAsync(pc.data(), b->so.pc, sizeof(ys::PcgCloth) * b->ncloth, cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  ys_status ret = sol;
  for (int c = 0; c < b->ncloth; ++c) {
    sts[c].ok = (pc[c].status & 3) == 0;
    if (!sts[c].ok) ret = YS_ERR_NONFINITE;
  }
  b->assembled = false;
  return ret;
}

}  // namespace

extern "C" {

ys_status ys_use_graphs(ys_batch* b, int32_t enable) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  b->graph.enabled = enable != 0;
  return YS_OK;
}

ys_status ys_set_producer_threads(ys_batch* b, int32_t threads) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (threads < 32 || threads > ys::kMaxProducerBlock || threads % 32)
    return fail(YS_ERR_ARG, "ys_set_producer_threads: a multiple of 32 up to 256");
  b->producer_threads = threads;
  b->graph.built = false;
  return YS_OK;
}

int32_t ys_autotune_results(const ys_batch* b, ys_schedule* out, int32_t cap) {
  if (!b) return -1;
  const int32_t n = (int32_t)b->tuned.size();
  for (int32_t i = 0; out && i < n && i < cap; ++i) out[i] = b->tuned[i];
  return n;
}

ys_status ys_set_pcg_schedule(ys_batch* b, int32_t pcg, int32_t threads, int32_t cluster) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  YS_CUDA(cudaSetDevice(b->device));
  ys_batch::PcgPlan& P = b->plan;
  if (pcg == YS_PCG_PHASES) {
    P.kind = YS_PCG_PHASES;
    b->graph.built = false;
    return YS_OK;
  }
  if (pcg != YS_PCG_PERSISTENT) return fail(YS_ERR_ARG, "ys_set_pcg_schedule: unknown schedule");
  if (!ys::pcg_cluster_shape_ok(threads, cluster))
    return fail(YS_ERR_ARG, "ys_set_pcg_schedule: threads must be 128, 256, 512 or 1024 and cluster 1, 2, 4, 8 "
                            "or 16, at most 16384 nodes");
  if (!P.order) {
    // cloths largest first
    std::vector<int> ord(b->ncloth);
    for (int c = 0; c < b->ncloth; ++c) ord[c] = c;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int x, int y) { return b->cp[x].W * b->cp[x].H > b->cp[y].W * b->cp[y].H; });
    const ys_status s = b->alloc(&P.order, b->ncloth);
    if (s != YS_OK) return s;
    YS_CUDA(cudaMemcpy(P.order, ord.data(), sizeof(int) * b->ncloth, cudaMemcpyHostToDevice));
    P.max_nodes = b->cp[ord[0]].W * b->cp[ord[0]].H;
  }
  if (P.max_nodes > threads * cluster)
    return fail(YS_ERR_ARG, "ys_set_pcg_schedule: the largest cloth has " + std::to_string(P.max_nodes) +
                                " nodes, more than threads x cluster");
  int fit = 0;
  const cudaError_t e = ys::pcg_cluster_occupancy(threads, cluster, &fit);
  if (e != cudaSuccess || fit < 1) {
    cudaGetLastError();
    return fail(YS_ERR_ARG, "ys_set_pcg_schedule: this GPU cannot run a cluster of that shape");
  }
  P.kind = YS_PCG_PERSISTENT;
  P.threads = threads;
  P.csize = cluster;
  b->graph.built = false;
  return YS_OK;
}

ys_status ys_step_graphed(ys_batch* b, double h, const double* ext_force, int32_t flags, const ys_solve_opts* opts,
                          ys_cloth_stats* stats) {
  if (!b || !(h > 0)) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(b->device));
  ys_batch::Graph& G = b->graph;
  b->v.h = h;
  b->v.ext = nullptr;
  if (ext_force) {
    ys_status s = upload_soa(b, ext_force, b->ext, 5, flags);
    if (s != YS_OK) return s;
    b->v.ext = b->ext;
  }
  const double tol = (opts && opts->tol > 0) ? opts->tol : DBL_EPSILON;
  const int override_max = (opts && opts->maxiter >= 0) ? opts->maxiter : -1;
  // iterations per trip through the loop body; the learned solve converges in
  // a few, so its body is short unless the call asks otherwise
  const bool learned = b->learn.kind == YS_PREC_LEARNED;
  int m = (opts && opts->check_every > 0) ? opts->check_every : learned ? kLearnedCheckEvery : b->check_every;
  m += m & 1;
  const int cap = override_max >= 0 ? override_max : b->max_maxiter;
  b->so.tol = tol;
  if (!G.built || G.h != h || G.has_ext != (ext_force != nullptr) || G.tol != tol ||
      G.override_max != override_max || G.m != m || G.cap != cap || (learned && G.lnet != b->learn.net)) {
    G.drop();
    G.built = true;
    G.h = h;
    G.has_ext = ext_force != nullptr;
    G.tol = tol;
    G.override_max = override_max;
    G.m = m;
    G.cap = cap;
    G.lnet = b->learn.net;
  }
  if (learned) return step_graphed_learned(b, opts, stats, m, cap, override_max);
  if (!G.exec) {
    const ys_status s = graph_build(b, m, cap, override_max);
    if (s != YS_OK) {
      G.drop();
      return s;
    }
  }
  YS_CUDA(cudaGraphLaunch(G.exec, b->stream));
  std::vector<ys::PcgCloth> pc(b->ncloth);
  YS_CUDA(cudaMemcpyAsync(pc.data(), b->so.pc, sizeof(ys::PcgCloth) * b->ncloth, cudaMemcpyDeviceToHost, b->stream));
  if (b->plan.kind == YS_PCG_PHASES)
    YS_CUDA(cudaMemcpyAsync(&G.h_it, G.it_base, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  // kernels the graph ran: 11 (+ geometry) before the loop, 3 per iteration
  // + 1 per trip through the body, 2 after; with the persistent PCG, 9 (+
  // geometry) before the solve, the solve, 2 after
  if (b->plan.kind == YS_PCG_PERSISTENT) b->launches += 12 + (b->geom_n ? 1 : 0);
  else b->launches += 13 + (b->geom_n ? 1 : 0) + 3LL * G.h_it + G.h_it / m;
  return step_result(b, pc, stats);
}

// The schedule tuner: every candidate (whole-step graph or launch by launch;
// phase PCG with its iterations between convergence checks, or the persistent
// per-cloth PCG in one cluster shape) runs the same steps from the same state
// and gives bit-identical results -- the choices only move launches, host
// synchronisations and which threads do the same arithmetic -- so the tuner
// times each on a snapshot of the state, restores it, and keeps the fastest.
ys_status ys_autotune(ys_batch* b, double h, const ys_solve_opts* opts, int32_t steps, ys_schedule* best) {
  if (!b || !(h > 0) || steps < 1) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(b->device));
  const size_t nt = (size_t)b->v.ntot;
  double* const state[6] = {b->v.X, b->v.XF, b->v.V, b->v.UV, b->v.UVB, b->v.UVD};
  const int comps[6] = {3, 3, 3, 2, 2, 2};
  double* snap = nullptr;
  YS_CUDA(cudaMalloc(&snap, sizeof(double) * 15 * nt));
  auto copy_state = [&](bool save) -> cudaError_t {
    size_t off = 0;
    for (int k = 0; k < 6; ++k) {
      const size_t n = comps[k] * nt;
      cudaError_t e = cudaMemcpyAsync(save ? snap + off : state[k], save ? state[k] : snap + off,
                                      sizeof(double) * n, cudaMemcpyDeviceToDevice, b->stream);
      if (e != cudaSuccess) return e;
      off += n;
    }
    return cudaSuccess;
  };
  const bool was_graph = b->graph.enabled, was_prof = b->profiling;
  const ys_batch::PcgPlan was_plan = b->plan;
  const int was_pt = b->producer_threads;
  b->profiling = false;
  // the candidates
  std::vector<ys_schedule> cand;
  int max_nodes = 0;
  for (int c = 0; c < b->ncloth; ++c) max_nodes = std::max(max_nodes, b->cp[c].W * b->cp[c].H);
  for (int g = 0; g < 2; ++g) {
    for (int every : {2, 4, 8, 16, 32}) {
      ys_schedule k{};
      k.graphs = g;
      k.check_every = every;
      k.pcg = YS_PCG_PHASES;
      cand.push_back(k);
    }
    for (int t : {128, 256, 512, 1024})
      for (int cl : {1, 2, 4, 8, 16}) {
        const int cap_nodes = t * cl;
        if (!ys::pcg_cluster_shape_ok(t, cl) || cap_nodes < max_nodes || cap_nodes >= 4 * std::max(max_nodes, 128))
          continue;
        ys_schedule k{};
        k.graphs = g;
        k.check_every = b->check_every;
        k.pcg = YS_PCG_PERSISTENT;
        k.pcg_threads = t;
        k.pcg_cluster = cl;
        cand.push_back(k);
      }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ys_status st = YS_OK;
  ys_schedule top{};
  top.ms_per_step = -1.0;
  std::vector<ys_cloth_stats> stats(b->ncloth);
  cudaError_t ce = copy_state(true);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  b->tuned.clear();
  for (ys_schedule& k : cand) k.producer_threads = was_pt;
  // first the graph / PCG choices at the batch's producer block size, then
  // the producer block sizes under the best of those
  const int pt_c[3] = {64, 128, 256};
  bool widened = false;  // the producer sizes are appended once, after the first pass
  for (size_t ci = 0; ce == cudaSuccess && st == YS_OK; ++ci) {
    if (ci == cand.size() && !widened) {
      widened = true;
      if (top.ms_per_step >= 0)
        for (int q = 0; q < 3; ++q)
          if (pt_c[q] != was_pt) {
            ys_schedule k = top;
            k.producer_threads = pt_c[q];
            cand.push_back(k);
          }
    }
    if (ci >= cand.size()) break;
    const ys_schedule k = cand[ci];
    if (ys_set_pcg_schedule(b, k.pcg, k.pcg_threads, k.pcg_cluster) != YS_OK) continue;  // shape cannot run here
    b->producer_threads = k.producer_threads;
    b->graph.built = false;
    b->graph.enabled = k.graphs == 1;
    ys_solve_opts o = opts ? *opts : ys_solve_opts{0.0, -1, 0};
    o.check_every = k.check_every;
    // one untimed step builds the graph (and warms the caches)
    if ((ce = copy_state(false)) != cudaSuccess) break;
    ys_status s = ys_step(b, h, nullptr, 0, &o, stats.data());
    if (s == YS_ERR_ARG || s == YS_ERR_CUDA) { st = s; break; }
    if ((ce = copy_state(false)) != cudaSuccess) break;
    if ((ce = cudaEventRecord(e0, b->stream)) != cudaSuccess) break;
    for (int j = 0; j < steps && st == YS_OK; ++j) {
      s = ys_step(b, h, nullptr, 0, &o, stats.data());
      if (s == YS_ERR_ARG || s == YS_ERR_CUDA) st = s;
    }
    if (st != YS_OK) break;
    if ((ce = cudaEventRecord(e1, b->stream)) != cudaSuccess) break;
    if ((ce = cudaEventSynchronize(e1)) != cudaSuccess) break;
    float ms = 0.f;
    if ((ce = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
    const double per = ms / steps;
    b->tuned.push_back(k);
    b->tuned.back().ms_per_step = per;
    if (top.ms_per_step < 0 || per < top.ms_per_step) {
      top = k;
      top.ms_per_step = per;
    }
  }
  if (ce == cudaSuccess) ce = copy_state(false);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->stream);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(snap);
  b->profiling = was_prof;
  b->assembled = false;
  if (ce != cudaSuccess || st != YS_OK || top.ms_per_step < 0) {
    b->graph.enabled = was_graph;
    b->plan.kind = was_plan.kind;
    b->plan.threads = was_plan.threads;
    b->plan.csize = was_plan.csize;
    b->producer_threads = was_pt;
    b->graph.built = false;
    if (ce != cudaSuccess) return fail(YS_ERR_CUDA, std::string("ys_autotune: ") + cudaGetErrorString(ce));
    if (st != YS_OK) return st;
    return fail(YS_ERR_CUDA, "ys_autotune: no schedule ran");
  }
  b->graph.enabled = top.graphs != 0;
  b->check_every = top.check_every;
  b->producer_threads = top.producer_threads;
  b->graph.built = false;
  const ys_status sp = ys_set_pcg_schedule(b, top.pcg, top.pcg_threads, top.pcg_cluster);
  if (sp != YS_OK) return sp;
  if (best) *best = top;
  return YS_OK;
}

}  // extern "C"


// ------------------------------------------------------- learned preconditioner
struct ys_gnn {
  int device = 0;
  ys::GnnNet net{};
  float* m = nullptr;  // Adam moments
  float* vv = nullptr;
  int step = 0;
  int objective = YS_GNN_FSAI;
  std::vector<void*> allocs;
  template <class T>
  cudaError_t alloc(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *p = static_cast<T*>(q);
    }
    return e;
  }
  ~ys_gnn() {
    for (void* p : allocs) cudaFree(p);
  }
};

namespace {

// GNN buffers of a batch, sized for its nodes
ys_status learn_ensure(ys_batch* b) {
  ys_batch::Learn& L = b->learn;
  if (L.ready) return YS_OK;
  const int nt = b->ntot;
  ys::GnnBufs& g = L.g;
  g.ntot = nt;
  g.nlblk = (nt + 127) / 128;
  g.nsplit = 296;
  ys_status st = YS_OK;
  auto A = [&](auto** p, size_t cnt) { if (st == YS_OK) st = b->alloc(p, cnt); };
  A(&g.nbr, 4 * (size_t)nt);
  A(&g.pat, 8 * (size_t)nt);
  A(&g.upat, 8 * (size_t)nt);
  A(&g.linv, 15 * (size_t)nt);
  A(&g.chol_ok, nt);
  A(&g.E, 150 * (size_t)nt);
  A(&g.f, (size_t)ys::kGIn * nt);
  A(&g.h, 4 * (size_t)ys::kGHid * nt);
  A(&g.hb, 4 * (size_t)ys::kGHid * nt);
  A(&g.act, 3 * (size_t)ys::kGHid * nt);
  A(&g.o, (size_t)ys::kGOut * nt);
  A(&g.G, (size_t)ys::kGUsed * nt);
  A(&g.Gh, (size_t)ys::kGPairs * nt);
  A(&g.Gn, (size_t)ys::kGUsed * nt);
  A(&g.Nt, (size_t)ys::kGUsed * nt);
  A(&g.vec, 4 * 5 * (size_t)nt);
  A(&g.dob, (size_t)ys::kGOut * nt);
  A(&g.dh, (size_t)ys::kGHid * nt);
  A(&g.dzb, (size_t)ys::kGHid * nt);
  A(&g.dm, (size_t)ys::kGMsg * nt);
  A(&g.wpart, (size_t)g.nsplit * ys::kWgradRows * ys::kGOut);
  A(&g.grad, ys::kGParams);
  A(&g.lpart, 2 * (size_t)g.nlblk + 3);
  A(&g.err, 1);
  A(&L.rf, 5 * (size_t)nt);
  A(&L.z, 5 * (size_t)nt);
  if (st != YS_OK) return st;
  YS_CUDA(cudaMemsetAsync(g.err, 0, sizeof(int), b->stream));
  YS_CUDA(cudaMemsetAsync(g.grad, 0, sizeof(float) * ys::kGParams, b->stream));
  ys::gnn_neighbours(b->v, g, b->stream);
  b->launches += 1;
  YS_CUDA(cudaGetLastError());
  L.ready = true;
  return YS_OK;
}

// the learned PCG's buffers: G (BF16), the FP32 residual, z
ys::LpcgExtra learned_extra(ys_batch* b) {
  const ys_batch::Learn& L = b->learn;
  return ys::LpcgExtra{L.g.Gh, L.rf, L.z};
}

// features, network, G blocks for the assembled system
ys_status learn_infer(ys_batch* b, ys_gnn* net, bool training = false) {
  ys::GnnBufs& g = b->learn.g;
  b->run(YS_PROF_GNN, 2 + 5 + 1, [&] {
    ys::gnn_prepare(b->v, g, b->stream);
    ys::gnn_forward(net->net, g, training, b->stream);
    ys::gnn_make_g(g, training, b->stream);
  });
  YS_CUDA(cudaGetLastError());
  return YS_OK;
}

ys_status read_err(ys_batch* b, int* err) {
  YS_CUDA(cudaMemcpyAsync(err, b->learn.g.err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  return YS_OK;
}

// PCG with M^-1 = G^T G; cloths that stop without converging (iteration cap or
// a breakdown) are solved again by Jacobi-PCG, which also judges the residual
// rule both solvers share: |b - A x| <= tol |b| on the recursively updated
// residual, as in Eigen's ConjugateGradient.
ys_status solve_learned(ys_batch* b, const ys_solve_opts* opts, ys_cloth_stats* stats) {
  ys_batch::Learn& L = b->learn;
  if (!L.net) return fail(YS_ERR_ARG, "learned preconditioner without a network");
  ys_status st = learn_ensure(b);
  if (st != YS_OK) return st;
  if (!L.have_g || ++L.since >= L.refresh_every) {
    if ((st = learn_infer(b, L.net)) != YS_OK) return st;
    L.have_g = true;
    L.since = 0;
  }
  cudaStream_t s = b->stream;
  const ys::View& v = b->v;
  b->so.tol = (opts && opts->tol > 0) ? opts->tol : DBL_EPSILON;
  const int override_max = (opts && opts->maxiter >= 0) ? opts->maxiter : -1;
  const int every = (opts && opts->check_every > 0) ? opts->check_every : kLearnedCheckEvery;
  const int cap = override_max >= 0 ? override_max : b->max_maxiter;
  const ys::LpcgExtra lx = learned_extra(b);
  b->run(YS_PROF_MISC, 1, [&] {
    k_reset_pc<<<(b->ncloth + 127) / 128, 128, 0, s>>>(b->so.pc, b->maxiter_dev, b->ncloth, override_max);
  });
  b->run(YS_PROF_PCG_SETUP, 3, [&] { ys::lpcg_setup(v, b->blk, b->so, lx, s); });
  YS_CUDA(cudaGetLastError());
  int it = 0;
  while (it < cap) {
    const int n = std::min(every, cap - it);
    for (int q = 0; q < n; ++q, ++it) {
      const int par = it & 1;
      b->run(YS_PROF_SPMV, 1, [&] { ys::launch_pcg_spmv(v, b->blk, b->so, s); });
      b->run(YS_PROF_AXPY, 1, [&] { ys::lpcg_axpy(v, b->blk, b->so, lx, par, s); });
      b->run(YS_PROF_PREC, 1, [&] { ys::lpcg_precondition(v, b->blk, b->so, lx, s); });
      b->run(YS_PROF_DIR, 1, [&] { ys::lpcg_dir(v, b->blk, b->so, lx, par, it, s); });
    }
    b->run(YS_PROF_MISC, 1, [&] { ys::launch_count_active(v, b->so, s); });
    YS_CUDA(cudaMemcpyAsync(b->h_nactive, b->so.nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
    YS_CUDA(cudaStreamSynchronize(s));
    if (*b->h_nactive == 0) break;
  }
  YS_CUDA(cudaGetLastError());
  int err = 0;
  if ((st = read_err(b, &err)) != YS_OK) return st;
  std::vector<ys::PcgCloth> pc(b->ncloth);
  YS_CUDA(cudaMemcpyAsync(pc.data(), b->so.pc, sizeof(ys::PcgCloth) * b->ncloth, cudaMemcpyDeviceToHost, s));
  YS_CUDA(cudaStreamSynchronize(s));
  L.solves += 1;
  // fall back on an expired tensor-core wait, a breakdown (bit 3), or the
  // default iteration cap (a cap the caller set is honoured as Jacobi-PCG's)
  bool redo = err != 0;
  for (int c = 0; c < b->ncloth; ++c)
    if (!(pc[c].status & 1) && ((pc[c].status & 8) || ((pc[c].status & 4) && override_max < 0))) redo = true;
  if (redo) {
    // Jacobi-PCG for the whole batch (a cloth that converged keeps an equally
    // valid solution, but one solve keeps the batch's bookkeeping uniform)
    L.fallbacks += 1;
    if (err) YS_CUDA(cudaMemsetAsync(L.g.err, 0, sizeof(int), s));
    return solve_impl(b, v, opts, stats);
  }
  ys_status ret = YS_OK;
  for (int c = 0; c < b->ncloth; ++c) {
    if (pc[c].status & 1) ret = YS_ERR_NONFINITE;
    else if ((pc[c].status & 4) && ret == YS_OK) ret = YS_ERR_MAXITER;
    if (stats) {
      stats[c].ok = (pc[c].status & 3) == 0;
      stats[c].cg_iterations = pc[c].iters;
      stats[c].cg_error = pc[c].bb > 0 ? std::sqrt(pc[c].rr / pc[c].bb) : 0.0;
      stats[c].hit_maxiter = (pc[c].status & 4) ? 1 : 0;
    }
  }
  return ret;
}

// the learned-preconditioner step as a graph: assembly, [the network and G,]
// the learned PCG's set-up, a conditional while node over m iterations (SpMV,
// residual update, z = G^T G r, direction) and the condition,
// then the verdict (hold the update back if the solve must be redone by
// Jacobi-PCG) and the solution check and Cloth::update, which honour it
ys_status graph_build_learned(ys_batch* b, int m, int cap, int override_max, int with_net) {
  ys_batch::Graph& G = b->graph;
  ys_batch::Learn& L = b->learn;
  ys_status st = graph_prepare(b);
  if (st != YS_OK) return st;
  if (with_net) ys::gnn_forward_attrs();  // function attributes are set outside the capture
  ys::Solver so = b->so;
  so.it_base = G.it_base;
  ys::Solver so_post = b->so;
  so_post.hold = G.hold;
  const ys::View& v = b->v;
  const ys::LpcgExtra lx = learned_extra(b);
  return build_loop_graph(
      b,
      [&](cudaStream_t c) {
        capture_assembly(b, c, override_max);
        if (with_net) {
          ys::gnn_prepare(v, L.g, c);
          ys::gnn_forward(L.net->net, L.g, false, c);
          ys::gnn_make_g(L.g, false, c);
        }
        ys::lpcg_setup(v, b->blk, so, lx, c);
        ys::launch_graph_loop_begin(so, c);
      },
      [&](cudaStream_t c, cudaGraphConditionalHandle h) {
        for (int j = 0; j < m; ++j) {
          ys::launch_pcg_spmv(v, b->blk, so, c);
          ys::lpcg_axpy(v, b->blk, so, lx, j & 1, c);
          ys::lpcg_precondition(v, b->blk, so, lx, c);
          ys::lpcg_dir(v, b->blk, so, lx, j & 1, j, c);
        }
        ys::launch_graph_loop_tail(so, b->ncloth, m, cap, h, c);
      },
      [&](cudaStream_t c) {
        ys::launch_learned_verdict(so, b->ncloth, L.g.err, override_max >= 0 ? 1 : 0, G.hold, c);
        ys::launch_update(v, b->blk, so_post, c);
      },
      &G.lmain[with_net], &G.lexec[with_net]);
}

uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int32_t ys_gnn_param_count(void) { return ys::kGParams; }

void ys_gnn_dims(int32_t* outputs, int32_t* blocks) {
  if (outputs) *outputs = ys::kGOut;
  if (blocks) *blocks = ys::kGBlocks;
}

ys_status ys_gnn_set_objective(ys_gnn* g, int32_t objective) {
  if (!g || (objective != YS_GNN_KAPORIN && objective != YS_GNN_FSAI)) return fail(YS_ERR_ARG, "bad argument");
  g->objective = objective;
  return YS_OK;
}

ys_status ys_gnn_create(int32_t device, uint64_t seed, ys_gnn** out) {
  if (!out) return fail(YS_ERR_ARG, "null output");
  YS_CUDA(cudaSetDevice(device));
  ys_gnn* g = new ys_gnn();
  g->device = device;
  ys::GnnNet& n = g->net;
  cudaError_t e = g->alloc(&n.w, ys::kGParams);
  if (e == cudaSuccess) e = g->alloc(&n.W0, (size_t)ys::kGHid * ys::kGIn);
  if (e == cudaSuccess) e = g->alloc(&n.Wl, (size_t)ys::kGLayers * ys::kGHid * ys::kGMsg);
  if (e == cudaSuccess) e = g->alloc(&n.Wh, (size_t)ys::kGOut * ys::kGHid);
  if (e == cudaSuccess) e = g->alloc(&n.WlT, (size_t)ys::kGLayers * ys::kGHid * ys::kGMsg);
  if (e == cudaSuccess) e = g->alloc(&n.WhT, (size_t)ys::kGOut * ys::kGHid);
  if (e == cudaSuccess) e = g->alloc(&g->m, ys::kGParams);
  if (e == cudaSuccess) e = g->alloc(&g->vv, ys::kGParams);
  if (e != cudaSuccess) {
    delete g;
    return fail(YS_ERR_CUDA, std::string("ys_gnn_create: ") + cudaGetErrorString(e));
  }
  // uniform fan-in/fan-out initialisation; the output head starts at zero so
  // an untrained network is the analytic approximate inverse
  std::vector<float> w(ys::kGParams, 0.f);
  uint64_t st = seed;
  auto fill = [&](int off, int rows, int cols, double scale) {
    const double bound = scale * std::sqrt(6.0 / (rows + cols));
    for (int i = 0; i < rows * cols; ++i) {
      const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
      w[off + i] = (float)((2.0 * u - 1.0) * bound);
    }
  };
  fill(ys::kPW0, ys::kGHid, ys::kGIn, 1.0);
  for (int l = 0; l < ys::kGLayers; ++l) fill(ys::kPW(l), ys::kGHid, ys::kGMsg, 0.5);
  e = cudaMemcpy(n.w, w.data(), sizeof(float) * ys::kGParams, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(g->m, 0, sizeof(float) * ys::kGParams);
  if (e == cudaSuccess) e = cudaMemset(g->vv, 0, sizeof(float) * ys::kGParams);
  if (e == cudaSuccess) {
    ys::gnn_refresh_bf16(n, 0);
    e = cudaDeviceSynchronize();
  }
  if (e != cudaSuccess) {
    delete g;
    return fail(YS_ERR_CUDA, std::string("ys_gnn_create: ") + cudaGetErrorString(e));
  }
  *out = g;
  return YS_OK;
}

void ys_gnn_destroy(ys_gnn* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  cudaDeviceSynchronize();
  delete g;
}

ys_status ys_gnn_get_params(ys_gnn* g, float* out) {
  if (!g || !out) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(g->device));
  YS_CUDA(cudaDeviceSynchronize());
  YS_CUDA(cudaMemcpy(out, g->net.w, sizeof(float) * ys::kGParams, cudaMemcpyDeviceToHost));
  return YS_OK;
}

ys_status ys_gnn_set_params(ys_gnn* g, const float* in) {
  if (!g || !in) return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(g->device));
  YS_CUDA(cudaDeviceSynchronize());
  YS_CUDA(cudaMemcpy(g->net.w, in, sizeof(float) * ys::kGParams, cudaMemcpyHostToDevice));
  YS_CUDA(cudaMemset(g->m, 0, sizeof(float) * ys::kGParams));
  YS_CUDA(cudaMemset(g->vv, 0, sizeof(float) * ys::kGParams));
  g->step = 0;
  ys::gnn_refresh_bf16(g->net, 0);
  YS_CUDA(cudaDeviceSynchronize());
  return YS_OK;
}

ys_status ys_gnn_loss_grad(ys_gnn* g, ys_batch* b, const float* probes, uint64_t seed, double* loss, float* grad,
                           float* outputs, float* gblocks) {
  if (!g || !b) return fail(YS_ERR_ARG, "null handle");
  if (g->device != b->device) return fail(YS_ERR_ARG, "network and batch on different devices");
  if (!b->has_system) return fail(YS_ERR_ARG, "no assembled system");
  YS_CUDA(cudaSetDevice(b->device));
  ys_status st = learn_ensure(b);
  if (st != YS_OK) return st;
  YS_CUDA(cudaStreamSynchronize(0));
  if ((st = learn_infer(b, g, true)) != YS_OK) return st;
  b->learn.have_g = false;
  ys::GnnBufs& G = b->learn.g;
  const int nt = b->ntot;
  if (probes) {
    std::vector<float> t(5 * (size_t)nt);
    for (int n = 0; n < nt; ++n)
      for (int c = 0; c < 5; ++c) t[(size_t)c * nt + n] = probes[(size_t)n * 5 + c];
    YS_CUDA(cudaMemcpyAsync(G.vec, t.data(), sizeof(float) * t.size(), cudaMemcpyHostToDevice, b->stream));
    YS_CUDA(cudaStreamSynchronize(b->stream));
  }
  ys::gnn_loss_grad(b->v, g->net, G, seed, probes != nullptr, g->objective, b->stream);
  YS_CUDA(cudaGetLastError());
  int err = 0;
  if ((st = read_err(b, &err)) != YS_OK) return st;
  if (err) {
    cudaMemsetAsync(G.err, 0, sizeof(int), b->stream);
    return fail(YS_ERR_CUDA, "tensor-core wait ran out");
  }
  if (loss) YS_CUDA(cudaMemcpy(loss, G.lpart + 2 * G.nlblk, sizeof(double), cudaMemcpyDeviceToHost));
  if (grad) YS_CUDA(cudaMemcpy(grad, G.grad, sizeof(float) * ys::kGParams, cudaMemcpyDeviceToHost));
  if (outputs) {  // stored component-major on the device
    std::vector<float> t((size_t)ys::kGOut * nt);
    YS_CUDA(cudaMemcpy(t.data(), G.o, sizeof(float) * t.size(), cudaMemcpyDeviceToHost));
    for (int n = 0; n < nt; ++n)
      for (int k = 0; k < ys::kGOut; ++k) outputs[(size_t)n * ys::kGOut + k] = t[(size_t)k * nt + n];
  }
  if (gblocks) {
    std::vector<float> t((size_t)ys::kGUsed * nt);
    YS_CUDA(cudaMemcpy(t.data(), G.G, sizeof(float) * t.size(), cudaMemcpyDeviceToHost));
    for (int n = 0; n < nt; ++n)
      for (int k = 0; k < ys::kGUsed; ++k) gblocks[(size_t)n * ys::kGUsed + k] = t[(size_t)k * nt + n];
  }
  return YS_OK;
}

ys_status ys_gnn_train_step(ys_gnn* g, ys_batch* b, uint64_t seed, float lr, double* loss) {
  if (!g || !b || !(lr > 0)) return fail(YS_ERR_ARG, "bad argument");
  if (g->device != b->device) return fail(YS_ERR_ARG, "network and batch on different devices");
  if (!b->has_system) return fail(YS_ERR_ARG, "no assembled system");
  YS_CUDA(cudaSetDevice(b->device));
  ys_status st = learn_ensure(b);
  if (st != YS_OK) return st;
  if ((st = learn_infer(b, g, true)) != YS_OK) return st;
  b->learn.have_g = false;
  ys::GnnBufs& G = b->learn.g;
  ys::gnn_loss_grad(b->v, g->net, G, seed, false, g->objective, b->stream);
  g->step += 1;
  ys::gnn_adam(g->net, G, g->m, g->vv, lr, g->step, b->stream);
  YS_CUDA(cudaGetLastError());
  int err = 0;
  if ((st = read_err(b, &err)) != YS_OK) return st;
  if (err) {
    cudaMemsetAsync(G.err, 0, sizeof(int), b->stream);
    return fail(YS_ERR_CUDA, "tensor-core wait ran out");
  }
  if (loss) {
    YS_CUDA(cudaMemcpyAsync(loss, G.lpart + 2 * G.nlblk, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    YS_CUDA(cudaStreamSynchronize(b->stream));
  }
  return YS_OK;
}

ys_status ys_set_preconditioner(ys_batch* b, int32_t kind, ys_gnn* g) {
  if (!b || (kind != YS_PREC_JACOBI && kind != YS_PREC_LEARNED)) return fail(YS_ERR_ARG, "bad argument");
  if (kind == YS_PREC_LEARNED && (!g || g->device != b->device)) return fail(YS_ERR_ARG, "bad network");
  b->learn.kind = kind;
  b->learn.net = kind == YS_PREC_LEARNED ? g : nullptr;
  b->learn.have_g = false;
  return YS_OK;
}

ys_status ys_precond_refresh(ys_batch* b, int32_t every) {
  if (!b || every < 1) return fail(YS_ERR_ARG, "bad argument");
  b->learn.refresh_every = every;
  b->learn.have_g = false;
  return YS_OK;
}

ys_status ys_precond_info(ys_batch* b, int64_t* solves, int64_t* fallbacks) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (solves) *solves = b->learn.solves;
  if (fallbacks) *fallbacks = b->learn.fallbacks;
  return YS_OK;
}

ys_status ys_get_system_slots(ys_batch* b, double* slots, double* rhs) {
  if (!b) return fail(YS_ERR_ARG, "null handle");
  if (!b->has_system) return fail(YS_ERR_ARG, "no assembled system");
  YS_CUDA(cudaSetDevice(b->device));
  YS_CUDA(cudaStreamSynchronize(b->stream));
  if (slots) YS_CUDA(cudaMemcpy(slots, b->v.A, sizeof(double) * ys::YS_NUM_SLOTS * b->ntot, cudaMemcpyDeviceToHost));
  if (rhs) YS_CUDA(cudaMemcpy(rhs, b->v.B, sizeof(double) * 5 * b->ntot, cudaMemcpyDeviceToHost));
  return YS_OK;
}

ys_status ys_tc_gemm_bf16(int32_t device, const uint16_t* A, const uint16_t* B, float* C, int32_t M, int32_t N,
                          int32_t K) {
  if (!A || !B || !C || M < 1 || (N != 64 && N != 128 && (N <= 0 || N % 64)) || K < 64 || K % 64)
    return fail(YS_ERR_ARG, "bad argument");
  YS_CUDA(cudaSetDevice(device));
  void *dA = nullptr, *dB = nullptr, *dC = nullptr, *dE = nullptr;
  cudaError_t e = cudaMalloc(&dA, 2 * (size_t)M * K);
  if (e == cudaSuccess) e = cudaMalloc(&dB, 2 * (size_t)N * K);
  if (e == cudaSuccess) e = cudaMalloc(&dC, 4 * (size_t)M * N);
  if (e == cudaSuccess) e = cudaMalloc(&dE, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, 2 * (size_t)M * K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, 2 * (size_t)N * K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dE, 0, sizeof(int));
  int err = 0;
  if (e == cudaSuccess) {
    ys::tc_gemm_bf16(static_cast<const __nv_bfloat16*>(dA), static_cast<const __nv_bfloat16*>(dB),
                     static_cast<float*>(dC), M, N, K, static_cast<int*>(dE), 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(C, dC, 4 * (size_t)M * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&err, dE, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dE);
  if (e != cudaSuccess) return fail(YS_ERR_CUDA, std::string("ys_tc_gemm_bf16: ") + cudaGetErrorString(e));
  if (err) return fail(YS_ERR_CUDA, "tensor-core wait ran out");
  return YS_OK;
}

}  // extern "C"
