/*
 * yarnsim_torch.h -- LibTorch-side binding of the C ABI (yarnsim.h) for C++
 * drivers of the reference (header only; link libyarnsim.so and LibTorch).
 *
 *   yarnsim::ClothDescription  a cloth's construction parameters (the
 *                              reference's Cloth constructor, src/Cloth.h:55-60)
 *   yarnsim::GpuCloth          one cloth on the GPU with the reference's
 *                              ClothState tensors at its interface
 *                              ([N,3,1] / [N,2,1] float64, node u + v*W,
 *                              src/Cloth.h:22-29); step() is SimStep
 *                              (src/TrainHelper.cpp:15-97) and returns its bool
 *   yarnsim::AdjointRollout    a torch::autograd::Function: positions of a
 *                              rollout of a two-yarn cloth as a function of
 *                              (rho, Y, B of each yarn, S, mu); its backward is
 *                              the reverse-mode adjoint (ys_adjoint_step) with a
 *                              checkpoint every k steps -- the gradient the
 *                              reference's loss.backward() takes through its
 *                              rollouts (src/TrainHeter.h:160-231) in
 *                              YS_TANGENT_REFERENCE mode, the derivative of the
 *                              discrete step in YS_TANGENT_EXACT mode
 *
 * With YARNSIM_REFERENCE_CLOTH defined after the reference's Cloth.h and
 * Environment.h are included, describe() reads a reference Cloth (its
 * per-edge yarns, so per-line material carries over) and YarnSimGpu is the
 * drop-in for SimStep(cloth, phy, h) on that Cloth.
 */
#ifndef YARNSIM_TORCH_H
#define YARNSIM_TORCH_H

#include <torch/torch.h>

#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "yarnsim.h"

namespace yarnsim {

inline void check(ys_status s, const char* where) {
  if (s != YS_OK) throw std::runtime_error(std::string(where) + ": " + ys_last_error());
}

// Construction parameters of one cloth; per-line material: warp line v (node
// row) and weft line u (node column) each carry rho, Y, B.
struct ClothDescription {
  ys_cloth_desc d{};
  std::vector<double> warp_rho, warp_Y, warp_B, weft_rho, weft_Y, weft_B;
  std::vector<int32_t> handles;  // (u, v) pairs
  // points d's arrays at the vectors (call after any change to them)
  const ys_cloth_desc& desc() {
    d.warp_rho = warp_rho.data(); d.warp_Y = warp_Y.data(); d.warp_B = warp_B.data();
    d.weft_rho = weft_rho.data(); d.weft_Y = weft_Y.data(); d.weft_B = weft_B.data();
    d.n_handles = (int32_t)(handles.size() / 2);
    d.handles = handles.empty() ? nullptr : handles.data();
    return d;
  }
  // two yarn types, lines alternating by parity (src/Cloth.cpp:195-268)
  void set_two_yarns(const double y0[3], const double y1[3]) {
    warp_rho.clear(); warp_Y.clear(); warp_B.clear(); weft_rho.clear(); weft_Y.clear(); weft_B.clear();
    for (int v = 0; v < d.length; ++v) {
      const double* y = v % 2 ? y1 : y0;
      warp_rho.push_back(y[0]); warp_Y.push_back(y[1]); warp_B.push_back(y[2]);
    }
    for (int u = 0; u < d.width; ++u) {
      const double* y = u % 2 ? y1 : y0;
      weft_rho.push_back(y[0]); weft_Y.push_back(y[1]); weft_B.push_back(y[2]);
    }
  }
  int nodes() const { return d.width * d.length; }
  int dim() const { return 3 * d.width * d.length + 2 * (d.width - 2) * (d.length - 2); }
};

// The reference's ClothState fields.
struct State {
  torch::Tensor LPos, LPosFix, LVel, EPos, EPosBar, EVel;
};

// One cloth on the GPU (device memory owned by its ys_batch).
class GpuCloth {
 public:
  explicit GpuCloth(ClothDescription desc, int device = 0) : desc_(std::move(desc)) {
    check(ys_batch_create(1, &desc_.desc(), device, nullptr, &b_), "ys_batch_create");
  }
  ~GpuCloth() { if (b_) ys_batch_destroy(b_); }
  GpuCloth(const GpuCloth&) = delete;
  GpuCloth& operator=(const GpuCloth&) = delete;

  ys_batch* handle() const { return b_; }
  const ClothDescription& description() const { return desc_; }

  // state as the reference's ClothState: [N,3,1] / [N,2,1] float64 (host)
  void set_state(const State& s) {
    auto c = [](const torch::Tensor& t) { return t.detach().to(torch::kCPU, torch::kFloat64).contiguous(); };
    State h{c(s.LPos), c(s.LPosFix), c(s.LVel), c(s.EPos), c(s.EPosBar), c(s.EVel)};
    check(ys_set_state(b_, h.LPos.data_ptr<double>(), h.LPosFix.data_ptr<double>(), h.LVel.data_ptr<double>(),
                       h.EPos.data_ptr<double>(), h.EPosBar.data_ptr<double>(), h.EVel.data_ptr<double>(), 0),
          "ys_set_state");
  }
  State get_state() const {
    const int64_t N = desc_.nodes();
    auto o = torch::TensorOptions().dtype(torch::kFloat64);
    State s{torch::empty({N, 3, 1}, o), torch::empty({N, 3, 1}, o), torch::empty({N, 3, 1}, o),
            torch::empty({N, 2, 1}, o), torch::empty({N, 2, 1}, o), torch::empty({N, 2, 1}, o)};
    check(ys_get_state(b_, s.LPos.data_ptr<double>(), s.LPosFix.data_ptr<double>(), s.LVel.data_ptr<double>(),
                       s.EPos.data_ptr<double>(), s.EPosBar.data_ptr<double>(), s.EVel.data_ptr<double>(), 0),
          "ys_get_state");
    return s;
  }

  // SimStep (src/TrainHelper.cpp:15-54; with an external force 56-97): false
  // when the system or the new velocity is not finite, as the reference's.
  // ext_force in the reference's DOF layout ([x of all nodes; u, v of
  // interior nodes], [dim] or [dim,1]) or undefined.
  // tol > 0: PCG relative residual (default: Eigen's, the machine epsilon).
  bool step(double h, const torch::Tensor& ext_force = torch::Tensor(), double tol = 0.0) {
    std::vector<double> e5;
    if (ext_force.defined()) e5 = to_node5(ext_force);
    ys_cloth_stats st{};
    const ys_solve_opts o{tol, -1, 0};
    const ys_status r = ys_step(b_, h, e5.empty() ? nullptr : e5.data(), 0, &o, &st);
    if (r == YS_ERR_NONFINITE) return false;
    if (r != YS_OK && r != YS_ERR_MAXITER) check(r, "ys_step");
    return st.ok != 0;
  }

  // reference DOF layout -> node layout [N][5]
  std::vector<double> to_node5(const torch::Tensor& ref) const {
    torch::Tensor r = ref.detach().to(torch::kCPU, torch::kFloat64).contiguous().view({-1});
    const int W = desc_.d.width, H = desc_.d.length, N = W * H;
    if (r.numel() != desc_.dim()) throw std::invalid_argument("ext_force must have the cloth's DOF count");
    const double* p = r.data_ptr<double>();
    std::vector<double> out(5 * (size_t)N, 0.0);
    for (int n = 0; n < N; ++n)
      for (int c = 0; c < 3; ++c) out[5 * n + c] = p[3 * n + c];
    for (int v = 1; v < H - 1; ++v)
      for (int u = 1; u < W - 1; ++u) {
        const int n = u + v * W, e = 3 * N + 2 * ((u - 1) + (v - 1) * (W - 2));
        out[5 * n + 3] = p[e];
        out[5 * n + 4] = p[e + 1];
      }
    return out;
  }

 private:
  ClothDescription desc_;
  ys_batch* b_ = nullptr;
};

// Positions (LPos [steps, N, 3] and EPos [steps, N, 2]) of a rollout of the
// two-yarn cloth `tmpl` from `state0`, differentiable with respect to
// theta = (rho0, Y0, B0, rho1, Y1, B1, S, mu) (float64 [8]).
struct AdjointRollout : public torch::autograd::Function<AdjointRollout> {
  static torch::autograd::variable_list forward(torch::autograd::AutogradContext* ctx, torch::Tensor theta,
                                                ClothDescription tmpl, State state0, int64_t steps, double h,
                                                int64_t mode, int64_t k, double tol = 0.0) {
    torch::Tensor th = theta.detach().to(torch::kCPU, torch::kFloat64).contiguous();
    const double* t = th.data_ptr<double>();
    const double y0[3] = {t[0], t[1], t[2]}, y1[3] = {t[3], t[4], t[5]};
    tmpl.set_two_yarns(y0, y1);
    tmpl.d.S = t[6];
    tmpl.d.mu = t[7];
    // the rollout's cloth lives until backward (which frees it); without a
    // gradient to take it is freed here
    auto* cloth = new GpuCloth(tmpl);
    cloth->set_state(state0);
    std::vector<torch::Tensor> xs, es;
    std::map<int64_t, State> checkpoints;
    for (int64_t s = 0; s < steps; ++s) {
      if (s % k == 0) checkpoints[s] = cloth->get_state();
      cloth->step(h, torch::Tensor(), tol);
      State cur = cloth->get_state();
      xs.push_back(cur.LPos.view({-1, 3}));
      es.push_back(cur.EPos.view({-1, 2}));
    }
    ctx->saved_data["steps"] = steps;
    ctx->saved_data["h"] = h;
    ctx->saved_data["mode"] = mode;
    ctx->saved_data["k"] = k;
    ctx->saved_data["tol"] = tol;
    ctx->saved_data["cloth"] = reinterpret_cast<int64_t>(cloth);
    std::vector<torch::Tensor> flat;
    for (auto& kv : checkpoints) {
      const State& c = kv.second;
      for (const torch::Tensor* f : {&c.LPos, &c.LPosFix, &c.LVel, &c.EPos, &c.EPosBar, &c.EVel}) flat.push_back(*f);
    }
    ctx->saved_data["checkpoints"] = flat;
    if (!theta.requires_grad()) {
      delete cloth;
      ctx->saved_data["cloth"] = (int64_t)0;
    }
    return {torch::stack(xs), torch::stack(es)};
  }

  static torch::autograd::variable_list backward(torch::autograd::AutogradContext* ctx,
                                                 torch::autograd::variable_list grads) {
    auto* cloth = reinterpret_cast<GpuCloth*>(ctx->saved_data["cloth"].toInt());
    const int64_t steps = ctx->saved_data["steps"].toInt(), k = ctx->saved_data["k"].toInt();
    const double h = ctx->saved_data["h"].toDouble(), tol = ctx->saved_data["tol"].toDouble();
    const ys_solve_opts opts{tol, -1, 0};
    const int mode = (int)ctx->saved_data["mode"].toInt();
    std::vector<torch::Tensor> flat = ctx->saved_data["checkpoints"].toTensorVector();
    const ClothDescription& d = cloth->description();
    const int64_t N = d.nodes(), nl = d.d.width + d.d.length;
    torch::Tensor gx = grads[0].to(torch::kCPU, torch::kFloat64).contiguous();
    torch::Tensor ge = grads[1].to(torch::kCPU, torch::kFloat64).contiguous();
    ys_adjoint* adj = nullptr;
    check(ys_adjoint_create(cloth->handle(), mode, 128, &adj), "ys_adjoint_create");
    auto o = torch::TensorOptions().dtype(torch::kFloat64);
    // adjoint of the state after step s: LPos, LVel, EPos, EVel, EPosBar
    std::vector<torch::Tensor> g = {torch::zeros({N, 3}, o), torch::zeros({N, 3}, o), torch::zeros({N, 2}, o),
                                    torch::zeros({N, 2}, o), torch::zeros({N, 2}, o)};
    torch::Tensor gp_line[3] = {torch::zeros({nl}, o), torch::zeros({nl}, o), torch::zeros({nl}, o)};
    torch::Tensor gp_cloth[2] = {torch::zeros({1}, o), torch::zeros({1}, o)};
    g[0] += gx[steps - 1];
    g[2] += ge[steps - 1];
    const int64_t nck = (int64_t)flat.size() / 6;
    for (int64_t ci = nck - 1; ci >= 0; --ci) {
      const int64_t a = ci * k, e = std::min(a + k, steps);
      State cp{flat[6 * ci], flat[6 * ci + 1], flat[6 * ci + 2], flat[6 * ci + 3], flat[6 * ci + 4], flat[6 * ci + 5]};
      cloth->set_state(cp);
      std::vector<State> seg;
      for (int64_t s = a; s < e; ++s) {
        seg.push_back(cloth->get_state());
        if (s + 1 < e) cloth->step(h, torch::Tensor(), tol);
      }
      for (int64_t s = e - 1; s >= a; --s) {
        cloth->set_state(seg[s - a]);
        std::vector<torch::Tensor> out = {torch::empty({N, 3}, o), torch::empty({N, 3}, o), torch::empty({N, 2}, o),
                                          torch::empty({N, 2}, o), torch::empty({N, 2}, o)};
        torch::Tensor pl[3] = {torch::empty({nl}, o), torch::empty({nl}, o), torch::empty({nl}, o)};
        torch::Tensor pc[2] = {torch::empty({1}, o), torch::empty({1}, o)};
        const double* gin[5];
        double* gout[5];
        for (int i = 0; i < 5; ++i) {
          g[i] = g[i].contiguous();
          gin[i] = g[i].data_ptr<double>();
          gout[i] = out[i].data_ptr<double>();
        }
        double* gpar[5] = {pl[0].data_ptr<double>(), pl[1].data_ptr<double>(), pl[2].data_ptr<double>(),
                           pc[0].data_ptr<double>(), pc[1].data_ptr<double>()};
        const ys_status st = ys_adjoint_step(adj, h, nullptr, gin, gout, gpar, nullptr, 0, &opts, nullptr);
        if (st != YS_OK && st != YS_ERR_MAXITER) {
          ys_adjoint_destroy(adj);
          check(st, "ys_adjoint_step");
        }
        for (int i = 0; i < 3; ++i) gp_line[i] += pl[i];
        for (int i = 0; i < 2; ++i) gp_cloth[i] += pc[i];
        g = out;
        if (s >= 1) {
          g[0] += gx[s - 1];
          g[2] += ge[s - 1];
        }
      }
    }
    ys_adjoint_destroy(adj);
    const int64_t length = d.d.length;  // d belongs to the cloth freed next
    delete cloth;
    ctx->saved_data["cloth"] = (int64_t)0;
    // per-line gradients into the two yarn types (warp line v, weft line u: parity)
    torch::Tensor gt = torch::zeros({8}, o);
    auto acc = gt.accessor<double, 1>();
    for (int64_t l = 0; l < nl; ++l) {
      const int64_t pos = l < length ? l : l - length;
      const int type = (int)(pos % 2);
      for (int p = 0; p < 3; ++p) acc[3 * type + p] += gp_line[p][l].item<double>();
    }
    acc[6] = gp_cloth[0][0].item<double>();
    acc[7] = gp_cloth[1][0].item<double>();
    return {gt.to(grads[0].device()), torch::Tensor(), torch::Tensor(), torch::Tensor(), torch::Tensor(),
            torch::Tensor(), torch::Tensor(), torch::Tensor()};
  }
};

// the training loss of src/TrainHeter.h:194-222:
// sum_s (mean_N |x_s - x^_s|^2 + mean_N |e_s - e^_s|^2) / max(steps - 1, 1)
inline torch::Tensor position_loss(const torch::Tensor& x, const torch::Tensor& e, const torch::Tensor& gx,
                                   const torch::Tensor& ge) {
  const int64_t steps = x.size(0);
  torch::Tensor dl = x - gx, de = e - ge;
  torch::Tensor l = (dl * dl).sum(-1).mean(-1).sum() + (de * de).sum(-1).mean(-1).sum();
  return l / (double)std::max<int64_t>(steps - 1, 1);
}

#ifdef YARNSIM_REFERENCE_CLOTH
// A reference Cloth's construction parameters: geometry, the material of
// every yarn line as its edges carry it (src/Cloth.cpp:184-268; a driver
// that set per-line yarns keeps them), kc, kf, df, mu, S, handle stiffness,
// gravity and wind from the Environment.
inline ClothDescription describe(const Cloth& c, const Environment& env,
                                 const std::vector<std::pair<int, int>>& handles) {
  ClothDescription out;
  ys_cloth_desc& d = out.d;
  d.width = c.width; d.length = c.length; d.height = c.hight; d.L = c.L; d.R = c.R;
  d.pose = 0;  // positions come from the Cloth's own state at every step
  d.weave = (int32_t)c.woven_pattern;
  out.warp_rho.assign(c.length, 0.0); out.warp_Y.assign(c.length, 0.0); out.warp_B.assign(c.length, 0.0);
  out.weft_rho.assign(c.width, 0.0); out.weft_Y.assign(c.width, 0.0); out.weft_B.assign(c.width, 0.0);
  for (const Edge& e : c.edges) {
    const bool warp = e.edge_type == "warp";
    const int line = warp ? e.n0->idx_v : e.n0->idx_u;
    (warp ? out.warp_rho : out.weft_rho)[line] = e.yarn.rho.item<double>();
    (warp ? out.warp_Y : out.weft_Y)[line] = e.yarn.Y.item<double>();
    (warp ? out.warp_B : out.weft_B)[line] = e.yarn.B.item<double>();
  }
  d.kc = c.kc.item<double>(); d.kf = c.kf.item<double>(); d.df = c.df.item<double>();
  d.mu = c.mu.item<double>(); d.S = c.S.item<double>(); d.handle_stiffness = c.handle_stiffness.item<double>();
  torch::Tensor G = env.G.detach().to(torch::kFloat64).contiguous().view({-1});
  torch::Tensor w = env.wind.WindVelocity.detach().to(torch::kFloat64).contiguous().view({-1});
  for (int k = 0; k < 3; ++k) { d.G[k] = G[k].item<double>(); d.wind_vel[k] = w[k].item<double>(); }
  d.wind_density = env.wind.WindDensity.item<double>();
  d.wind_drag = env.wind.WindDrag.item<double>();
  for (const auto& p : handles) { out.handles.push_back(p.first); out.handles.push_back(p.second); }
  out.desc();
  return out;
}

// Drop-in for SimStep(cloth, phy, h[, ext_force]) on a reference Cloth: the
// Cloth's state goes to the GPU, one step runs there, the new state comes
// back through Cloth::set_ClothState. Construct once per cloth (after
// set_handles), then call step() where the driver called SimStep.
class YarnSimGpu {
 public:
  YarnSimGpu(const Cloth& c, const Environment& env, const std::vector<std::pair<int, int>>& handles,
             int device = 0)
      : gpu_(describe(c, env, handles), device) {}
  bool step(Cloth& cloth, double h, const torch::Tensor& ext_force = torch::Tensor()) {
    ClothState s = cloth.get_ClothState();
    gpu_.set_state(State{s.LPos, s.LPosFix, s.LVel, s.EPos, s.EPosBar, s.EVel});
    if (!gpu_.step(h, ext_force)) return false;
    State n = gpu_.get_state();
    cloth.set_ClothState(ClothState{n.LPos, n.LPosFix, n.LVel, n.EPos, n.EPosBar, n.EVel});
    return true;
  }
  GpuCloth& gpu() { return gpu_; }

 private:
  GpuCloth gpu_;
};
#endif  // YARNSIM_REFERENCE_CLOTH

}  // namespace yarnsim

#endif  // YARNSIM_TORCH_H
