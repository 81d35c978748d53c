// Test-oracle harness around the reference's own physics sources.
//
// Builds a Cloth (src/Cloth.cpp:3-50), an Environment and a PhysicsCloth
// exactly as the reference drivers do (e.g. src/Simulate.h:34-64), then runs
// the body of SimStep (src/TrainHelper.cpp:15-54) for a number of steps:
//   FillMV -> A = M - h^2 dF/dx - h dF/dv, b = h (F - (dF/dv)^T v) + M v
//   -> solve -> Cloth::update -> ResetMV
// and writes the per-step state (plus, at selected steps, the dense system
// pieces) to a binary record file. The solve uses the Eigen-CG stand-in in
// shim/eigen_cg.cpp (the reference's EigenSolver::apply path) or, on request,
// a dense LU solve (src/Solvers.h:27-29, TorchSolver).
//
// It is test infrastructure only: it produces golden vectors for the oracle
// restatement and for the GPU path.
//
// Usage: ref_harness <config-file>
// Config: key=value lines (see tests/golden/make_golden.py for the keys).
#include <array>
#include <cmath>
#include <cstdio>
#include <set>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "PhysicsCloth.h"
#include "ForceNet.h"
#include "Render.h"
#include "CollisionUtil.h"

void ref_cg_set_options(double tol, long max_iter);
long ref_cg_last_iterations();
double ref_cg_last_error();

namespace {

std::map<std::string, std::string> read_config(const char* path) {
  std::map<std::string, std::string> kv;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    auto eq = line.find('=');
    if (eq == std::string::npos) continue;
    kv[line.substr(0, eq)] = line.substr(eq + 1);
  }
  return kv;
}

std::vector<double> parse_list(const std::string& s) {
  std::vector<double> out;
  std::string tok;
  for (char c : s) {
    if (c == ',' || c == ';' || c == ' ') {
      if (!tok.empty()) out.push_back(std::stod(tok));
      tok.clear();
    } else {
      tok.push_back(c);
    }
  }
  if (!tok.empty()) out.push_back(std::stod(tok));
  return out;
}

double get_d(const std::map<std::string, std::string>& kv, const std::string& k, double dflt) {
  auto it = kv.find(k);
  return it == kv.end() ? dflt : std::stod(it->second);
}
std::string get_s(const std::map<std::string, std::string>& kv, const std::string& k, const std::string& dflt) {
  auto it = kv.find(k);
  return it == kv.end() ? dflt : it->second;
}

struct Writer {
  FILE* f;
  explicit Writer(const std::string& path) { f = std::fopen(path.c_str(), "wb"); }
  ~Writer() { if (f) std::fclose(f); }
  void put(const std::string& name, const std::vector<long>& dims, const double* data) {
    int nl = static_cast<int>(name.size());
    std::fwrite(&nl, sizeof(int), 1, f);
    std::fwrite(name.data(), 1, nl, f);
    int nd = static_cast<int>(dims.size());
    std::fwrite(&nd, sizeof(int), 1, f);
    long total = 1;
    for (long d : dims) { std::fwrite(&d, sizeof(long), 1, f); total *= d; }
    std::fwrite(data, sizeof(double), total, f);
  }
  void put_tensor(const std::string& name, const Tensor& t) {
    Tensor c = t.detach().contiguous().to(torch::kFloat64);
    std::vector<long> dims;
    for (auto d : c.sizes()) dims.push_back(d);
    put(name, dims, c.data_ptr<double>());
  }
};

std::string key(int u, int v) { return std::to_string(u) + "," + std::to_string(v); }

}  // namespace

// ---------------------------------------------------------------------------
// mode=grad: the gradient the reference's parameter learning computes
// (src/TrainHeter.h:160-231 with YarnSimNetHeter, src/YarnSimNetHeter.h):
// two yarn types (lines alternate by parity) whose rho, Y, B and the cloth's
// S and mu are LibTorch leaves; a ground-truth rollout with a second
// parameter set from the same initial state; the loss
//   sum_s (mean_N |x_s - x^_s|^2 + mean_N |e_s - e^_s|^2) / max(steps - 1, 1)
// and loss.backward() through SimStep (src/TrainHelper.cpp:15-54) and
// EigenSolver's backward (shim/eigen_cg.cpp). Writes "loss" and "grad" =
// d loss / d (rho0, Y0, B0, rho1, Y1, B1, S, mu).
struct Sim {
  Cloth cloth;
  Environment env;
  PhysicsCloth phy;
};

int run_grad(std::map<std::string, std::string>& kv) {
  const int W = static_cast<int>(get_d(kv, "width", 5));
  const int Lh = static_cast<int>(get_d(kv, "length", 5));
  const double height = get_d(kv, "height", 5.0);
  const double L = get_d(kv, "L", 1e-3);
  const double R = get_d(kv, "R", 1e-4);
  const int steps = static_cast<int>(get_d(kv, "steps", 2));
  ref_cg_set_options(get_d(kv, "cg_tol", DBL_EPSILON), static_cast<long>(get_d(kv, "cg_maxiter", -1)));
  const std::string weave = get_s(kv, "weave", "plain");
  WovenPattern wp = weave == "twill" ? WovenPattern::Twill : (weave == "satin" ? WovenPattern::Satin : WovenPattern::Plain);
  InitPose ip = get_s(kv, "pose", "flat") == "upright" ? InitPose::Upright : InitPose::Flat;
  std::vector<double> G = parse_list(get_s(kv, "G", "0,0,9.8"));
  std::vector<double> wv = parse_list(get_s(kv, "wind_vel", "0,0,0"));
  std::vector<std::pair<int, int>> handles;
  {
    std::vector<double> hl = parse_list(get_s(kv, "handles", ""));
    for (size_t i = 0; i + 1 < hl.size(); i += 2) handles.emplace_back(static_cast<int>(hl[i]), static_cast<int>(hl[i + 1]));
  }
  const int N = W * Lh;
  std::vector<double> init(N * 15);
  const bool has_init = kv.count("init_state") > 0;
  if (has_init) {
    std::ifstream f(kv["init_state"], std::ios::binary);
    f.read(reinterpret_cast<char*>(init.data()), init.size() * sizeof(double));
  }
  auto T1 = [&](const std::string& k, double d) { return torch::tensor({get_d(kv, k, d)}, opts); };
  // params: rho0 Y0 B0 rho1 Y1 B1 S mu
  auto build = [&](const std::vector<Tensor>& p) {
    std::vector<Yarn> yarns{Yarn{R, p[0], p[1], p[2]}, Yarn{R, p[3], p[4], p[5]}};
    Sim* sim = new Sim{Cloth(W, Lh, height, L, R, yarns, T1("kc", 1.0), T1("kf", 1000.0), T1("df", 1000.0), p[7], p[6],
                             T1("handle_stiffness", 1e4), wp, ip),
                       Environment{}, PhysicsCloth{}};
    sim->cloth.set_handles(handles);
    Wind wind{torch::tensor({wv[0], wv[1], wv[2]}, opts).view({3, 1}), T1("wind_density", 0.0), T1("wind_drag", 0.0)};
    sim->env = Environment{&sim->cloth, torch::tensor({G[0], G[1], G[2]}, opts).view({3, 1}), wind};
    sim->phy = PhysicsCloth{&sim->env};
    if (has_init) {
      const double* lp = init.data();
      const double* lf = lp + 3 * N;
      const double* lv = lf + 3 * N;
      const double* ep = lv + 3 * N;
      const double* eb = ep + 2 * N;
      const double* ev = eb + 2 * N;
      for (int v = 0; v < Lh; ++v)
        for (int u = 0; u < W; ++u) {
          int id = u + v * W;
          Node& n = sim->cloth.nodes[key(u, v)];
          n.LPos = torch::tensor({lp[3 * id], lp[3 * id + 1], lp[3 * id + 2]}, opts).view({3, 1});
          n.LPosFix = torch::tensor({lf[3 * id], lf[3 * id + 1], lf[3 * id + 2]}, opts).view({3, 1});
          n.LVel = torch::tensor({lv[3 * id], lv[3 * id + 1], lv[3 * id + 2]}, opts).view({3, 1});
          n.EPos = torch::tensor({ep[2 * id], ep[2 * id + 1]}, opts).view({2, 1});
          n.EPosBar = torch::tensor({eb[2 * id], eb[2 * id + 1]}, opts).view({2, 1});
          n.EVel = torch::tensor({ev[2 * id], ev[2 * id + 1]}, opts).view({2, 1});
          sim->cloth.warp_nodes[key(u, v)].LPos = n.LPos;
          sim->cloth.weft_nodes[key(u, v)].LPos = n.LPos;
        }
      sim->cloth.UpdateClothUnits();
    }
    sim->phy.InitMV();
    return sim;
  };
  const Tensor h = torch::tensor({get_d(kv, "h", 1e-3)}, opts);
  auto step = [&](Sim* sim) {
    sim->phy.FillMV();
    const Tensor M = sim->phy.get_SpaM();
    const Tensor Kx = sim->phy.get_SpaFPos();
    const Tensor Dv = sim->phy.get_SpaFVel();
    const Tensor A = M - Kx * torch::pow(h, 2) - Dv * h;
    const Tensor b = h * (sim->phy.get_SpaF() - torch::mm(Dv.transpose(0, 1), sim->phy.get_SpaVel())) +
                     torch::mm(M, sim->phy.get_SpaVel());
    Tensor new_vel = EigenSolver::apply(A, b);
    sim->cloth.update(new_vel, sim->phy.F_E_is_Slides[0], h);
    sim->phy.ResetMV();
  };
  auto positions = [&](Sim* sim, bool detach) {
    std::vector<Tensor> xs, es;
    for (int v = 0; v < Lh; ++v)
      for (int u = 0; u < W; ++u) {
        const Node& n = sim->cloth.nodes.at(key(u, v));
        xs.push_back(detach ? n.LPos.detach() : n.LPos);
        es.push_back(detach ? n.EPos.detach() : n.EPos);
      }
    return std::make_pair(torch::stack(xs), torch::stack(es));
  };
  // ground truth
  std::vector<double> gt = parse_list(get_s(kv, "gt_params", ""));
  std::vector<Tensor> gtp;
  for (double x : gt) gtp.push_back(torch::tensor({x}, opts));
  Sim* ref = build(gtp);
  std::vector<std::pair<Tensor, Tensor>> target;
  for (int s = 0; s < steps; ++s) {
    step(ref);
    target.push_back(positions(ref, true));
  }
  // learned parameters as leaves
  std::vector<double> th = parse_list(get_s(kv, "params", ""));
  std::vector<Tensor> leaves;
  for (double x : th) leaves.push_back(torch::tensor({x}, opts).requires_grad_(true));
  Sim* sim = build(leaves);
  Tensor loss = torch::zeros(1, opts);
  std::vector<std::pair<Tensor, Tensor>> traj;
  for (int s = 0; s < steps; ++s) {
    step(sim);
    auto pe = positions(sim, false);
    traj.push_back(std::make_pair(pe.first.detach(), pe.second.detach()));
    Tensor dl = pe.first - target[s].first, de = pe.second - target[s].second;
    Tensor pos_loss = torch::mean(torch::bmm(dl.transpose(2, 1), dl)) + torch::mean(torch::bmm(de.transpose(2, 1), de));
    loss = loss + pos_loss;
  }
  loss = loss / (steps - 1 > 0 ? steps - 1 : 1);
  loss.backward();
  Writer w(get_s(kv, "out", "ref_out.bin"));
  double lv = loss.item<double>();
  w.put("loss", {1}, &lv);
  std::vector<double> g;
  for (auto& t : leaves) g.push_back(t.grad().defined() ? t.grad().item<double>() : 0.0);
  w.put("grad", {static_cast<int>(g.size())}, g.data());
  for (int s = 0; s < steps; ++s) {
    const std::string t = std::to_string(s + 1);
    w.put_tensor("target" + t + ".LPos", target[s].first.reshape({N, 3}));
    w.put_tensor("target" + t + ".EPos", target[s].second.reshape({N, 2}));
    w.put_tensor("traj" + t + ".LPos", traj[s].first.reshape({N, 3}));
    w.put_tensor("traj" + t + ".EPos", traj[s].second.reshape({N, 2}));
  }
  double st = 0;
  w.put("status", {1}, &st);
  delete sim;
  delete ref;
  return 0;
}

// mode=vjp: c^T (db / d state) by autograd at one state, for a probe vector c
// (key "probe", reference DOF layout), with b = h (F - D^T v) + M v as SimStep
// forms it (M, D built without a graph). Writes "g.LPos", "g.LVel" [N][3],
// "g.EPos", "g.EPosBar", "g.EVel" [N][2].
int run_vjp(std::map<std::string, std::string>& kv) {
  const int W = static_cast<int>(get_d(kv, "width", 5));
  const int Lh = static_cast<int>(get_d(kv, "length", 5));
  const double R = get_d(kv, "R", 1e-4);
  std::vector<double> th = parse_list(get_s(kv, "params", ""));
  std::vector<Tensor> p;
  for (double x : th) p.push_back(torch::tensor({x}, opts));
  std::vector<Yarn> yarns{Yarn{R, p[0], p[1], p[2]}, Yarn{R, p[3], p[4], p[5]}};
  const std::string weave = get_s(kv, "weave", "plain");
  WovenPattern wp = weave == "twill" ? WovenPattern::Twill : (weave == "satin" ? WovenPattern::Satin : WovenPattern::Plain);
  InitPose ip = get_s(kv, "pose", "flat") == "upright" ? InitPose::Upright : InitPose::Flat;
  auto T1 = [&](const std::string& k, double d) { return torch::tensor({get_d(kv, k, d)}, opts); };
  Cloth cloth(W, Lh, get_d(kv, "height", 5.0), get_d(kv, "L", 1e-3), R, yarns, T1("kc", 1.0), T1("kf", 1000.0),
              T1("df", 1000.0), p[7], p[6], T1("handle_stiffness", 1e4), wp, ip);
  std::vector<std::pair<int, int>> handles;
  {
    std::vector<double> hl = parse_list(get_s(kv, "handles", ""));
    for (size_t i = 0; i + 1 < hl.size(); i += 2) handles.emplace_back(static_cast<int>(hl[i]), static_cast<int>(hl[i + 1]));
  }
  cloth.set_handles(handles);
  std::vector<double> G = parse_list(get_s(kv, "G", "0,0,9.8"));
  std::vector<double> wv = parse_list(get_s(kv, "wind_vel", "0,0,0"));
  Wind wind{torch::tensor({wv[0], wv[1], wv[2]}, opts).view({3, 1}), T1("wind_density", 0.0), T1("wind_drag", 0.0)};
  Environment env{&cloth, torch::tensor({G[0], G[1], G[2]}, opts).view({3, 1}), wind};
  const int N = W * Lh;
  std::vector<double> init(N * 15);
  {
    std::ifstream f(kv["init_state"], std::ios::binary);
    f.read(reinterpret_cast<char*>(init.data()), init.size() * sizeof(double));
  }
  const double* lp = init.data();
  const double* lf = lp + 3 * N;
  const double* lv = lf + 3 * N;
  const double* ep = lv + 3 * N;
  const double* eb = ep + 2 * N;
  const double* ev = eb + 2 * N;
  std::vector<Tensor> leaves;  // per node: LPos, LVel, EPos, EPosBar, EVel
  for (int v = 0; v < Lh; ++v)
    for (int u = 0; u < W; ++u) {
      int id = u + v * W;
      Node& n = cloth.nodes[key(u, v)];
      n.LPos = torch::tensor({lp[3 * id], lp[3 * id + 1], lp[3 * id + 2]}, opts).view({3, 1}).requires_grad_(true);
      n.LPosFix = torch::tensor({lf[3 * id], lf[3 * id + 1], lf[3 * id + 2]}, opts).view({3, 1});
      n.LVel = torch::tensor({lv[3 * id], lv[3 * id + 1], lv[3 * id + 2]}, opts).view({3, 1}).requires_grad_(true);
      n.EPos = torch::tensor({ep[2 * id], ep[2 * id + 1]}, opts).view({2, 1}).requires_grad_(true);
      n.EPosBar = torch::tensor({eb[2 * id], eb[2 * id + 1]}, opts).view({2, 1}).requires_grad_(true);
      n.EVel = torch::tensor({ev[2 * id], ev[2 * id + 1]}, opts).view({2, 1}).requires_grad_(true);
      leaves.push_back(n.LPos); leaves.push_back(n.LVel); leaves.push_back(n.EPos);
      leaves.push_back(n.EPosBar); leaves.push_back(n.EVel);
      cloth.warp_nodes[key(u, v)].LPos = n.LPos;
      cloth.weft_nodes[key(u, v)].LPos = n.LPos;
    }
  cloth.UpdateClothUnits();
  PhysicsCloth phy{&env};
  phy.InitMV();
  const Tensor h = torch::tensor({get_d(kv, "h", 1e-3)}, opts);
  phy.FillMV();
  const Tensor M = phy.get_SpaM();
  const Tensor Dv = phy.get_SpaFVel();
  const Tensor b = h * (phy.get_SpaF() - torch::mm(Dv.transpose(0, 1), phy.get_SpaVel())) + torch::mm(M, phy.get_SpaVel());
  std::vector<double> c = parse_list(get_s(kv, "probe", ""));
  Tensor phi = torch::sum(b.view({-1}) * torch::tensor(c, opts));
  phi.backward();
  Writer w(get_s(kv, "out", "ref_out.bin"));
  std::vector<double> gl(N * 3), gv(N * 3), ge(N * 2), gb(N * 2), gev(N * 2);
  for (int id = 0; id < N; ++id) {
    auto G3 = [&](const Tensor& t, std::vector<double>& o, int k) {
      for (int r = 0; r < k; ++r) o[k * id + r] = t.grad().defined() ? t.grad()[r][0].item<double>() : 0.0;
    };
    G3(leaves[5 * id], gl, 3); G3(leaves[5 * id + 1], gv, 3); G3(leaves[5 * id + 2], ge, 2);
    G3(leaves[5 * id + 3], gb, 2); G3(leaves[5 * id + 4], gev, 2);
  }
  w.put("g.LPos", {N, 3}, gl.data()); w.put("g.LVel", {N, 3}, gv.data()); w.put("g.EPos", {N, 2}, ge.data());
  w.put("g.EPosBar", {N, 2}, gb.data()); w.put("g.EVel", {N, 2}, gev.data());
  w.put_tensor("b", b);
  double st = 0;
  w.put("status", {1}, &st);
  return 0;
}


// ---------------------------------------------------------------------------
// mode=collide: the broad and narrow phase of the reference's collision
// detection on one cloth state, for golden pair lists and impacts.
// The BVH is the reference's own (src/BVH.cpp, src/CollisionUtil.cpp:3-9:
// AccelStruct = BVHTree(ccd, mesh) over the cloth mesh and the obstacle
// mesh); the traversal restates Collision::for_overlapping_faces and
// collect_upper_nodes (src/Collision.cpp:266-326) and the narrow phase
// comp_face_impacts / vf / ee / collision_test (src/Collision.cpp:210-253,
// 327-419) with the reference's Geometry.cpp, and the cubic solve restates
// src/Solvers.cpp:60-178 (Solvers.cpp needs Eigen). The obstacle mesh is
// built as load_obj builds it (src/Loader.cpp:269-345; Loader.cpp needs HDF5).
// Inputs: cloth width/length (the reference's clothMesh topology) with node
// positions x / x_prev from "cloth_state" ([N][3] x then [N][3] x_prev), an
// optional obstacle from "obstacle" ([No] count, [No][3] x, [No][3] x_prev,
// [Fo] count, [Fo][3] node ids, as doubles), thickness, ccd.
// Writes "pairs" [P][3] (first face, second face, 1 if the second face is an
// obstacle face) in emission order and "impacts" [I][15] (type 0 VF / 1 EE,
// four node ids (obstacle nodes as -1 - id), t, ws[4], n[3], pair index).
namespace collide {

int quad(double a, double b, double c, double& x0, double& x1) {
  const double d = b * b - 4.0 * a * c;
  if (d < 0.0) {
    x0 = -b / (2.0 * a);
    return 0;
  }
  const double q = -(b + std::sqrt(d)) / 2.0, q1 = -(b - std::sqrt(d)) / 2.0;
  if (std::fabs(a) > 1e-12) {
    if (q / a < q1 / a) { x0 = q / a; x1 = q1 / a; }
    else { x0 = q1 / a; x1 = q / a; }
    return 2;
  }
  x0 = -c / b;
  return 1;
}
double newton(double a, double b, double c, double d, double x0, int dir) {
  if (dir != 0) {
    const double y0 = d + x0 * (c + x0 * (b + x0 * a)), ddy0 = 2 * b + (x0 + dir * 1e-6) * (6 * a);
    x0 = x0 + dir * std::sqrt(std::fabs(2 * y0 / ddy0));
  }
  for (int it = 0; it < 100; ++it) {
    const double y = d + x0 * (c + x0 * (b + x0 * a)), dy = c + x0 * (2 * b + x0 * 3 * a);
    if (dy == 0.0) return x0;
    const double x1 = x0 - y / dy;
    if (std::fabs(x0 - x1) < 1e-6) return x0;
    x0 = x1;
  }
  return x0;
}
std::vector<double> cubic(double a, double b, double c, double d) {
  double xc0 = -1.0, xc1 = -1.0, x0 = -1.0, x1 = -1.0, x2 = -1.0;
  const int ncrit = quad(3.0 * a, 2.0 * b, c, xc0, xc1);
  if (ncrit == 0) return {newton(a, b, c, d, xc0, 0)};
  if (ncrit == 1) {
    const int ns = quad(b, c, d, x0, x1);
    if (ns == 1) return {x0};
    if (ns == 2) return {x0, x1};
    return {};
  }
  const double yc0 = d + xc0 * (c + xc0 * (b + xc0 * a)), yc1 = d + xc1 * (c + xc1 * (b + xc1 * a));
  int ns = 0;
  if (yc0 * a >= 0.0) { x0 = newton(a, b, c, d, xc0, -1); ns++; }
  if (yc0 * yc1 <= 0.0) {
    if (std::fabs(yc0) < std::fabs(yc1)) x1 = newton(a, b, c, d, xc0, 1);
    else x1 = newton(a, b, c, d, xc1, -1);
    ns++;
  }
  if (yc1 * a <= 0.0) { x2 = newton(a, b, c, d, xc1, 1); ns++; }
  if (ns == 1) return {x0};
  if (ns == 2) return {x0, x1};
  if (ns == 3) return {x0, x1, x2};
  return {};
}

struct Ctx {
  Mesh* cloth;
  Mesh* obs;
  Tensor thickness;
  bool ccd;
  std::vector<std::array<double, 3>> pairs;
  std::vector<std::array<double, 15>> impacts;
};

double node_id(Ctx& c, const MeshNode* n) {
  if (n->index < (int)c.cloth->nodes.size() && n == &c.cloth->nodes.at(n->index)) return n->index;
  return -1.0 - n->index;
}

bool test(Ctx& c, int type, const MeshNode* n0, const MeshNode* n1, const MeshNode* n2, const MeshNode* n3, int pair) {
  Tensor x0 = n0->x_prev, v0 = n0->x - x0;
  Tensor x1 = n1->x_prev - x0, x2 = n2->x_prev - x0, x3 = n3->x_prev - x0;
  Tensor v1 = n1->x - n1->x_prev - v0, v2 = n2->x - n2->x_prev - v0, v3 = n3->x - n3->x_prev - v0;
  auto dotc = [](const Tensor& a, const Tensor& b, const Tensor& cc) {
    return torch::mm(a.transpose(0, 1), torch::cross(b, cc)).item<double>();
  };
  const double a0 = dotc(x1, x2, x3);
  const double a1 = dotc(v1, x2, x3) + dotc(x1, v2, x3) + dotc(x1, x2, v3);
  const double a2 = dotc(x1, v2, v3) + dotc(v1, x2, v3) + dotc(v1, v2, x3);
  const double a3 = dotc(v1, v2, v3);
  for (double t : cubic(a3, a2, a1, a0)) {
    if (std::isnan(t) || std::isinf(t) || t < 0 || t > 1) continue;
    Tensor tt = torch::tensor({t}, opts);
    Tensor bx1 = x1 + tt * v1, bx2 = x2 + tt * v2, bx3 = x3 + tt * v3;
    Tensor n;
    std::array<Tensor, 4> ws;
    bool over = false, inside = false;
    if (type == 0) {
      sub_signed_vf_distance(bx1, bx2, bx3, n, ws, 1e-12, over);
      inside = std::min(-ws[1].item<double>(), std::min(-ws[2].item<double>(), -ws[3].item<double>())) >= -1e-12;
    } else {
      sub_signed_ee_distance(bx1, bx2, bx3, bx2 - bx1, bx3 - bx1, bx3 - bx2, n, ws, 1e-12, over);
      inside = std::min(std::min(ws[0].item<double>(), ws[1].item<double>()),
                        std::min(-ws[2].item<double>(), -ws[3].item<double>())) >= -1e-12;
    }
    if (over || !inside) continue;
    if (torch::dot(n.squeeze(), (ws[1] * v1 + ws[2] * v2 + ws[3] * v3).squeeze()).item<double>() > 0.0) n = -1 * n;
    std::array<double, 15> r;
    r[0] = type;
    r[1] = node_id(c, n0); r[2] = node_id(c, n1); r[3] = node_id(c, n2); r[4] = node_id(c, n3);
    r[5] = t;
    for (int k = 0; k < 4; ++k) r[6 + k] = ws[k].item<double>();
    for (int k = 0; k < 3; ++k) r[10 + k] = n[k][0].item<double>();
    r[13] = pair;
    r[14] = 0;
    c.impacts.push_back(r);
    return true;
  }
  return false;
}

void face_impacts(Ctx& c, MeshFace* f0, MeshFace* f1, int pair) {
  std::array<kDOP18, 6> nb, eb;
  std::array<kDOP18, 2> fb;
  for (int n = 0; n < 3; ++n) {
    nb[n] = node_box(f0->v[n]->node, c.ccd);
    nb[n + 3] = node_box(f1->v[n]->node, c.ccd);
  }
  for (int a = 0; a < 3; ++a) {
    const int b = a != 2 ? a + 1 : 0;
    eb[a] = nb[a] + nb[b];
    eb[a + 3] = nb[a + 3] + nb[b + 3];
  }
  fb[0] = nb[0] + nb[1] + nb[2];
  fb[1] = nb[3] + nb[4] + nb[5];
  auto vf = [&](const MeshVert* v, const MeshFace* f) {
    const MeshNode* nd = v->node;
    if (nd == f->v[0]->node || nd == f->v[1]->node || nd == f->v[2]->node) return;
    test(c, 0, nd, f->v[0]->node, f->v[1]->node, f->v[2]->node, pair);
  };
  for (int n = 0; n < 3; ++n)
    if (overlap(nb[n], fb[1], c.thickness)) vf(f0->v[n], f1);
  for (int n = 0; n < 3; ++n)
    if (overlap(nb[n + 3], fb[0], c.thickness)) vf(f1->v[n], f0);
  for (int e0 = 0; e0 < 3; ++e0)
    for (int e1 = 0; e1 < 3; ++e1) {
      if (!overlap(eb[e0], eb[e1 + 3], c.thickness)) continue;
      const MeshEdge* a = f0->adj_edges[e0];
      const MeshEdge* b = f1->adj_edges[e1];
      if (a->n0 == b->n0 || a->n0 == b->n1 || a->n1 == b->n0 || a->n1 == b->n1) continue;
      test(c, 1, a->n0, a->n1, b->n0, b->n1, pair);
    }
}

void emit(Ctx& c, MeshFace* f0, MeshFace* f1, bool obs) {
  c.pairs.push_back({(double)f0->index, (double)f1->index, obs ? 1.0 : 0.0});
}
void pair_nodes(Ctx& c, BVHNode* a, BVHNode* b, bool obs) {
  if (!a->_actived && !b->_actived) return;
  if (!overlap(a->_box, b->_box, c.thickness)) return;
  if (a->isLeaf() && b->isLeaf()) emit(c, a->_face, b->_face, obs);
  else if (a->isLeaf()) {
    pair_nodes(c, a, b->_left, obs);
    pair_nodes(c, a, b->_right, obs);
  } else {
    pair_nodes(c, a->_left, b, obs);
    pair_nodes(c, a->_right, b, obs);
  }
}
void self_nodes(Ctx& c, BVHNode* n) {
  if (n->isLeaf() || !n->_actived) return;
  self_nodes(c, n->_left);
  self_nodes(c, n->_right);
  pair_nodes(c, n->_left, n->_right, false);
}

}  // namespace collide

int run_collide(std::map<std::string, std::string>& kv) {
  const int W = static_cast<int>(get_d(kv, "width", 5));
  const int Lh = static_cast<int>(get_d(kv, "length", 5));
  const double R = get_d(kv, "R", 1e-4);
  std::vector<Yarn> yarns{Yarn{R, torch::tensor({1e-3}, opts), torch::tensor({1e3}, opts), torch::tensor({1e-5}, opts)}};
  auto T1 = [&](double d) { return torch::tensor({d}, opts); };
  Cloth cloth(W, Lh, 0.05, get_d(kv, "L", 1e-3), R, yarns, T1(1.0), T1(1000.0), T1(1000.0), T1(0.3), T1(1e-4), T1(1e4),
              WovenPattern::Plain, InitPose::Flat);
  const int N = W * Lh;
  std::vector<double> st(6 * N);
  {
    std::ifstream f(kv["cloth_state"], std::ios::binary);
    f.read(reinterpret_cast<char*>(st.data()), st.size() * sizeof(double));
  }
  for (int n = 0; n < N; ++n) {
    MeshNode& m = cloth.clothMesh.nodes.at(n);
    m.x = torch::tensor({st[3 * n], st[3 * n + 1], st[3 * n + 2]}, opts).view({3, 1});
    m.x_prev = torch::tensor({st[3 * N + 3 * n], st[3 * N + 3 * n + 1], st[3 * N + 3 * n + 2]}, opts).view({3, 1});
  }
  Mesh obs;
  const bool has_obs = kv.count("obstacle") > 0;
  if (has_obs) {
    std::ifstream f(kv["obstacle"], std::ios::binary);
    double cnt;
    f.read(reinterpret_cast<char*>(&cnt), sizeof(double));
    const int No = (int)cnt;
    std::vector<double> xo(3 * No), xp(3 * No);
    f.read(reinterpret_cast<char*>(xo.data()), xo.size() * sizeof(double));
    f.read(reinterpret_cast<char*>(xp.data()), xp.size() * sizeof(double));
    f.read(reinterpret_cast<char*>(&cnt), sizeof(double));
    const int Fo = (int)cnt;
    std::vector<double> fo(3 * Fo);
    f.read(reinterpret_cast<char*>(fo.data()), fo.size() * sizeof(double));
    obs.nodes.reserve(No);
    obs.verts.reserve(No);
    for (int i = 0; i < No; ++i) {
      MeshNode nd(torch::tensor({xo[3 * i], xo[3 * i + 1], xo[3 * i + 2]}, opts).view({3, 1}));
      obs.add(nd);
      obs.nodes.back().x_prev = torch::tensor({xp[3 * i], xp[3 * i + 1], xp[3 * i + 2]}, opts).view({3, 1});
      obs.add(MeshVert(torch::zeros({2, 1}, opts)));
    }
    for (int i = 0; i < No; ++i) connect(&obs.verts.at(i), &obs.nodes.at(i));
    std::set<std::pair<int, int>> en;
    for (int q = 0; q < Fo; ++q)
      for (int a = 0; a < 3; ++a) {
        const int b = a != 2 ? a + 1 : 0;
        const int u = (int)fo[3 * q + a], w = (int)fo[3 * q + b];
        en.insert(u < w ? std::make_pair(u, w) : std::make_pair(w, u));
      }
    obs.edges.reserve(en.size());
    for (auto& e : en) obs.add(MeshEdge(&obs.nodes.at(e.first), &obs.nodes.at(e.second)));
    obs.faces.reserve(Fo);
    for (int q = 0; q < Fo; ++q)
      obs.add(MeshFace(&obs.verts.at((int)fo[3 * q]), &obs.verts.at((int)fo[3 * q + 1]), &obs.verts.at((int)fo[3 * q + 2])));
    obs.add_adjecent();
  }
  collide::Ctx c{&cloth.clothMesh, &obs, torch::tensor({get_d(kv, "thickness", 5e-4)}, opts),
                 get_d(kv, "ccd", 1) != 0, {}, {}};
  AccelStruct cacc(cloth.clothMesh, c.ccd);
  AccelStruct* oacc = has_obs ? new AccelStruct(obs, c.ccd) : nullptr;
  // collect_upper_nodes (src/Collision.cpp:306-326) with NThrd nodes
  std::vector<BVHNode*> nodes{cacc.root};
  while ((int)nodes.size() < NThrd) {
    std::vector<BVHNode*> ch;
    for (BVHNode* n : nodes) {
      if (n->isLeaf()) ch.push_back(n);
      else { ch.push_back(n->_left); ch.push_back(n->_right); }
    }
    if (ch.size() == nodes.size()) break;
    nodes = ch;
  }
  for (int n = 0; n < (int)nodes.size(); ++n) {
    collide::self_nodes(c, nodes[n]);
    for (int m = 0; m < n; ++m) collide::pair_nodes(c, nodes[n], nodes[m], false);
    if (oacc) collide::pair_nodes(c, nodes[n], oacc->root, true);
  }
  for (int p = 0; p < (int)c.pairs.size(); ++p) {
    MeshFace* f0 = &cloth.clothMesh.faces.at((int)c.pairs[p][0]);
    MeshFace* f1 = c.pairs[p][2] != 0 ? &obs.faces.at((int)c.pairs[p][1]) : &cloth.clothMesh.faces.at((int)c.pairs[p][1]);
    collide::face_impacts(c, f0, f1, p);
  }
  Writer w(get_s(kv, "out", "ref_out.bin"));
  std::vector<double> pf;
  for (auto& q : c.pairs) pf.insert(pf.end(), q.begin(), q.end());
  w.put("pairs", {(long)c.pairs.size(), 3}, pf.data());
  std::vector<double> im;
  for (auto& q : c.impacts) im.insert(im.end(), q.begin(), q.end());
  w.put("impacts", {(long)c.impacts.size(), 15}, im.data());
  double stv = 0;
  w.put("status", {1}, &stv);
  delete oacc;
  return 0;
}

// ---------------------------------------------------------------------------
// mode=embed: the reference's control learning step (src/TrainEmbed.h:84-176):
// a ForceNet (src/ForceNet.h, float32, initialised by torch::manual_seed(seed))
// reads the cloth state [LPos, EPos, LVel, EVel] flattened and predicts a
// lift and a drag strength applied at the z / y DOF (first * width + second)
// of each listed pair; the loop of train_embed with its `if (s = 5)` (an
// assignment: after the first step the loop jumps to s = 6 and later steps
// run without force), SimStep with the external force
// (src/TrainHelper.cpp:56-97, restated like run_grad's step), the loss
// |mean(goal) - mean(LPos)|^2 and loss.backward(). Writes the loss, the
// predicted forces, every ForceNet parameter and its gradient, and the
// final positions. One homogeneous cloth (no handles), upright, plain.
int run_embed(std::map<std::string, std::string>& kv) {
  const int W = static_cast<int>(get_d(kv, "width", 5));
  const int Lh = static_cast<int>(get_d(kv, "length", 5));
  const double height = get_d(kv, "height", 5.0);
  const double L = get_d(kv, "L", 1e-3);
  const double R = get_d(kv, "R", 1e-4);
  const int sample = static_cast<int>(get_d(kv, "sample", 10));
  // loop=intended forces steps 0..5 as the comment in train_embed describes
  const bool intended = get_s(kv, "loop", "reference") == "intended";
  ref_cg_set_options(get_d(kv, "cg_tol", DBL_EPSILON), static_cast<long>(get_d(kv, "cg_maxiter", -1)));
  torch::manual_seed(static_cast<uint64_t>(get_d(kv, "seed", 0)));
  std::vector<double> G = parse_list(get_s(kv, "G", "0,0,9.8"));
  std::vector<double> wv = parse_list(get_s(kv, "wind_vel", "0,0,0"));
  std::vector<double> hl = parse_list(get_s(kv, "force_at", "0,0,4,0,0,4,4,4"));
  auto T1 = [&](const std::string& k, double d) { return torch::tensor({get_d(kv, k, d)}, opts); };
  const int N = W * Lh;
  const int force_size = 3 * N + 2 * (W - 2) * (Lh - 2);
  Tensor lift_at = torch::zeros({force_size, 1}, opts), drag_at = torch::zeros({force_size, 1}, opts);
  for (size_t i = 0; i + 1 < hl.size(); i += 2) {
    const int first = static_cast<int>(hl[i]), second = static_cast<int>(hl[i + 1]);
    lift_at.index_put_({(first * W + second) * 3 + 2, 0}, 1.0);
    drag_at.index_put_({(first * W + second) * 3 + 1, 0}, 1.0);
  }
  const Tensor zero_force = torch::zeros({force_size, 1}, opts);
  std::vector<double> goal(3 * N);
  {
    std::ifstream f(kv["goal"], std::ios::binary);
    f.read(reinterpret_cast<char*>(goal.data()), goal.size() * sizeof(double));
  }
  const Tensor goal_t = torch::from_blob(goal.data(), {N, 3, 1}, opts).clone();
  ForceNet net{10 * N, 2};
  std::vector<Yarn> yarns{Yarn{R, T1("rho", 1e-3), T1("Y", 1e3), T1("B", 1e-5)}};
  Cloth cloth(W, Lh, height, L, R, yarns, T1("kc", 1.0), T1("kf", 1000.0), T1("df", 1000.0), T1("mu", 0.3),
              T1("S", 1e-4), T1("handle_stiffness", 1e4), WovenPattern::Plain, InitPose::Upright);
  Wind wind{torch::tensor({wv[0], wv[1], wv[2]}, opts).view({3, 1}), T1("wind_density", 0.0), T1("wind_drag", 0.0)};
  Environment env{&cloth, torch::tensor({G[0], G[1], G[2]}, opts).view({3, 1}), wind};
  PhysicsCloth phy{&env};
  phy.InitMV();
  const Tensor h = torch::tensor({get_d(kv, "h", 1e-3)}, opts);
  auto step = [&](const Tensor& ext) {
    phy.FillMV();
    const Tensor M = phy.get_SpaM();
    const Tensor Kx = phy.get_SpaFPos();
    const Tensor Dv = phy.get_SpaFVel();
    const Tensor A = M - Kx * torch::pow(h, 2) - Dv * h;
    const Tensor b = h * (phy.get_SpaF() + ext - torch::mm(Dv.transpose(0, 1), phy.get_SpaVel())) +
                     torch::mm(M, phy.get_SpaVel());
    Tensor new_vel = EigenSolver::apply(A, b);
    if (!torch::isfinite(new_vel).all().item<bool>()) return false;
    cloth.update(new_vel, phy.F_E_is_Slides[0], h);
    phy.ResetMV();
    return true;
  };
  ClothState bkup = cloth.get_ClothState();
  bool ok = true;
  std::vector<double> forces;
  for (int s = 0; s < sample - 1; ++s) {
    if (s <= 5) {
      ClothState cs = cloth.get_ClothState();
      Tensor in = torch::cat({cs.LPos.flatten(), cs.EPos.flatten(), cs.LVel.flatten(), cs.EVel.flatten()})
                      .unsqueeze(0).to(torch::kFloat32);
      Tensor pred = net->forward(in);
      Tensor ext = lift_at * pred.index({0, 0}) + drag_at * pred.index({0, 1});
      forces.push_back(pred.index({0, 0}).item<double>());
      forces.push_back(pred.index({0, 1}).item<double>());
      ok = step(ext);
      if (intended) {
        if (s == 5) bkup = cloth.get_ClothState();
      } else {
        s = 5;  // the reference's `if (s = force_stop_frame)`
        bkup = cloth.get_ClothState();
      }
      if (!ok) break;
    } else {
      ok = step(zero_force);
      if (!ok) break;
    }
  }
  ClothState fin = ok ? cloth.get_ClothState() : bkup;
  Tensor dc = (torch::mean(goal_t, 0) - torch::mean(fin.LPos, 0)).squeeze();
  Tensor loss = torch::matmul(dc, dc);
  loss.backward();
  Writer w(get_s(kv, "out", "ref_out.bin"));
  double lv = loss.item<double>();
  w.put("loss", {1}, &lv);
  w.put("forces", {static_cast<int>(forces.size())}, forces.data());
  for (auto& p : net->named_parameters()) {
    Tensor v = p.value().detach().to(torch::kFloat64).contiguous();
    std::vector<long> shape(v.sizes().begin(), v.sizes().end());
    std::vector<double> vals(v.data_ptr<double>(), v.data_ptr<double>() + v.numel());
    w.put("param." + p.key(), shape, vals.data());
    Tensor g = p.value().grad().defined() ? p.value().grad().to(torch::kFloat64).contiguous() : torch::zeros_like(v);
    std::vector<double> gv(g.data_ptr<double>(), g.data_ptr<double>() + g.numel());
    w.put("grad." + p.key(), shape, gv.data());
  }
  w.put_tensor("final.LPos", fin.LPos.detach().reshape({N, 3}));
  double st = ok ? 0.0 : 1.0;
  w.put("status", {1}, &st);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s config\n", argv[0]);
    return 2;
  }
  torch::set_num_threads(1);
  auto kv = read_config(argv[1]);
  if (get_s(kv, "mode", "") == "grad") return run_grad(kv);
  if (get_s(kv, "mode", "") == "vjp") return run_vjp(kv);
  if (get_s(kv, "mode", "") == "collide") return run_collide(kv);
  if (get_s(kv, "mode", "") == "embed") return run_embed(kv);

  const int W = static_cast<int>(get_d(kv, "width", 5));
  const int Lh = static_cast<int>(get_d(kv, "length", 5));
  const double height = get_d(kv, "height", 5.0);
  const double L = get_d(kv, "L", 1e-3);
  const double R = get_d(kv, "R", 1e-4);
  const std::string pose = get_s(kv, "pose", "flat");
  const std::string weave = get_s(kv, "weave", "plain");
  const int steps = static_cast<int>(get_d(kv, "steps", 1));
  const std::string solver = get_s(kv, "solver", "cg");
  ref_cg_set_options(get_d(kv, "cg_tol", DBL_EPSILON), static_cast<long>(get_d(kv, "cg_maxiter", -1)));

  std::vector<double> y0 = parse_list(get_s(kv, "yarn0", "1e-3,3.1830988618379e10,318.30988618379"));
  std::vector<Yarn> yarns{Yarn{R, torch::tensor({y0[0]}, opts), torch::tensor({y0[1]}, opts), torch::tensor({y0[2]}, opts)}};
  if (kv.count("yarn1")) {
    std::vector<double> y1 = parse_list(kv["yarn1"]);
    yarns.push_back(Yarn{R, torch::tensor({y1[0]}, opts), torch::tensor({y1[1]}, opts), torch::tensor({y1[2]}, opts)});
  }
  auto T1 = [&](const std::string& k, double d) { return torch::tensor({get_d(kv, k, d)}, opts); };
  WovenPattern wp = weave == "twill" ? WovenPattern::Twill : (weave == "satin" ? WovenPattern::Satin : WovenPattern::Plain);
  InitPose ip = pose == "upright" ? InitPose::Upright : InitPose::Flat;

  Cloth cloth(W, Lh, height, L, R, yarns, T1("kc", 1.0), T1("kf", 1000.0), T1("df", 1000.0), T1("mu", 0.3),
              T1("S", 1e3), T1("handle_stiffness", 1e4), wp, ip);

  // Optional per-yarn-line material: warp line = node row v, weft line = node column u.
  if (kv.count("warp_lines") || kv.count("weft_lines")) {
    std::vector<double> wl = parse_list(get_s(kv, "warp_lines", ""));
    std::vector<double> fl = parse_list(get_s(kv, "weft_lines", ""));
    auto mk = [&](const std::vector<double>& a, int line) {
      return Yarn{R, torch::tensor({a[3 * line]}, opts), torch::tensor({a[3 * line + 1]}, opts),
                  torch::tensor({a[3 * line + 2]}, opts)};
    };
    for (auto& e : cloth.edges) {
      if (e.edge_type == "warp" && !wl.empty()) e.yarn = mk(wl, e.n0->idx_v);
      if (e.edge_type == "weft" && !fl.empty()) e.yarn = mk(fl, e.n0->idx_u);
    }
    for (auto* segs : {&cloth.bend_segs, &cloth.crimp_bend_segs})
      for (auto& b : *segs) {
        if (b.seg_type == "warp" && !wl.empty()) b.yarn = mk(wl, b.n0->idx_v);
        if (b.seg_type == "weft" && !fl.empty()) b.yarn = mk(fl, b.n0->idx_u);
      }
  }

  std::vector<double> G = parse_list(get_s(kv, "G", "0,0,9.8"));
  std::vector<double> wv = parse_list(get_s(kv, "wind_vel", "0,0,0"));
  Wind wind{torch::tensor({wv[0], wv[1], wv[2]}, opts).view({3, 1}), T1("wind_density", 0.0), T1("wind_drag", 0.0)};
  Environment env{&cloth, torch::tensor({G[0], G[1], G[2]}, opts).view({3, 1}), wind};

  std::vector<std::pair<int, int>> handles;
  {
    std::vector<double> hl = parse_list(get_s(kv, "handles", ""));
    for (size_t i = 0; i + 1 < hl.size(); i += 2) handles.emplace_back(static_cast<int>(hl[i]), static_cast<int>(hl[i + 1]));
  }
  cloth.set_handles(handles);

  const int N = W * Lh;
  // Optional initial state (raw doubles, node order u + v*W):
  // LPos[N*3] LPosFix[N*3] LVel[N*3] EPos[N*2] EPosBar[N*2] EVel[N*2]
  if (kv.count("init_state")) {
    std::ifstream f(kv["init_state"], std::ios::binary);
    std::vector<double> buf(N * 15);
    f.read(reinterpret_cast<char*>(buf.data()), buf.size() * sizeof(double));
    const double* lp = buf.data();
    const double* lf = lp + 3 * N;
    const double* lv = lf + 3 * N;
    const double* ep = lv + 3 * N;
    const double* eb = ep + 2 * N;
    const double* ev = eb + 2 * N;
    for (int v = 0; v < Lh; ++v)
      for (int u = 0; u < W; ++u) {
        int id = u + v * W;
        Node& n = cloth.nodes[key(u, v)];
        n.LPos = torch::tensor({lp[3 * id], lp[3 * id + 1], lp[3 * id + 2]}, opts).view({3, 1});
        n.LPosFix = torch::tensor({lf[3 * id], lf[3 * id + 1], lf[3 * id + 2]}, opts).view({3, 1});
        n.LVel = torch::tensor({lv[3 * id], lv[3 * id + 1], lv[3 * id + 2]}, opts).view({3, 1});
        n.EPos = torch::tensor({ep[2 * id], ep[2 * id + 1]}, opts).view({2, 1});
        n.EPosBar = torch::tensor({eb[2 * id], eb[2 * id + 1]}, opts).view({2, 1});
        n.EVel = torch::tensor({ev[2 * id], ev[2 * id + 1]}, opts).view({2, 1});
        cloth.warp_nodes[key(u, v)].LPos = n.LPos;
        cloth.weft_nodes[key(u, v)].LPos = n.LPos;
      }
    cloth.UpdateClothUnits();
  }

  std::vector<double> dump_steps = parse_list(get_s(kv, "dump_steps", ""));
  auto is_dump = [&](int s) {
    for (double d : dump_steps)
      if (static_cast<int>(d) == s) return true;
    return false;
  };

  Writer w(get_s(kv, "out", "ref_out.bin"));
  PhysicsCloth phy{&env};
  phy.InitMV();
  const Tensor h = torch::tensor({get_d(kv, "h", 1e-3)}, opts);

  std::vector<double> ext;
  if (kv.count("ext_force")) ext = parse_list(kv["ext_force"]);
  // ext_steps=K: the force acts in steps 0..K-1 only (SimControl zeroes it
  // once i > 5, src/Simulate.h:290-291); default every step
  const int ext_steps = static_cast<int>(get_d(kv, "ext_steps", 1e9));

  auto dump_state = [&](const std::string& tag) {
    std::vector<double> lp(N * 3), lv(N * 3), lf(N * 3), ep(N * 2), ev(N * 2), eb(N * 2), nrm(N * 3, 0.0);
    for (int v = 0; v < Lh; ++v)
      for (int u = 0; u < W; ++u) {
        int id = u + v * W;
        const Node& n = cloth.nodes.at(key(u, v));
        for (int k = 0; k < 3; ++k) {
          lp[3 * id + k] = n.LPos[k][0].item<double>();
          lv[3 * id + k] = n.LVel[k][0].item<double>();
          lf[3 * id + k] = n.LPosFix[k][0].item<double>();
          if (n.n.defined()) nrm[3 * id + k] = n.n[k][0].item<double>();
        }
        for (int k = 0; k < 2; ++k) {
          ep[2 * id + k] = n.EPos[k][0].item<double>();
          ev[2 * id + k] = n.EVel[k][0].item<double>();
          eb[2 * id + k] = n.EPosBar[k][0].item<double>();
        }
      }
    w.put(tag + ".LPos", {N, 3}, lp.data());
    w.put(tag + ".LVel", {N, 3}, lv.data());
    w.put(tag + ".LPosFix", {N, 3}, lf.data());
    w.put(tag + ".EPos", {N, 2}, ep.data());
    w.put(tag + ".EVel", {N, 2}, ev.data());
    w.put(tag + ".EPosBar", {N, 2}, eb.data());
    w.put(tag + ".normal", {N, 3}, nrm.data());
  };

  dump_state("s0");
  int status = 0;
  for (int s = 0; s < steps; ++s) {
    phy.FillMV();
    const Tensor M = phy.get_SpaM();
    const Tensor Kx = phy.get_SpaFPos();
    const Tensor Dv = phy.get_SpaFVel();
    Tensor F = phy.get_SpaF();
    const Tensor V = phy.get_SpaVel();
    if (!ext.empty() && s < ext_steps) F = F + torch::tensor(ext, opts).view({-1, 1});
    const Tensor A = M - Kx * torch::pow(h, 2) - Dv * h;
    const Tensor b = h * (F - torch::mm(Dv.transpose(0, 1), V)) + torch::mm(M, V);
    if (DetectNaN(A, false) || DetectNaN(b, false) || DetectInf(A, false) || DetectInf(b, false)) {
      status = 1;
      break;
    }
    Tensor new_vel = solver == "lu" ? TorchSolver(A, b) : EigenSolver::apply(A, b);
    if (DetectNaN(new_vel, false) || DetectInf(new_vel, false)) {
      status = 1;
      break;
    }
    if (is_dump(s)) {
      std::string t = "d" + std::to_string(s);
      w.put_tensor(t + ".M", M);
      w.put_tensor(t + ".FPos", Kx);
      w.put_tensor(t + ".FVel", Dv);
      w.put_tensor(t + ".F", F);
      w.put_tensor(t + ".Vel", V);
      w.put_tensor(t + ".A", A);
      w.put_tensor(t + ".b", b);
      w.put_tensor(t + ".new_vel", new_vel);
      w.put_tensor(t + ".slide", phy.F_E_is_Slides[0]);
      double it = static_cast<double>(ref_cg_last_iterations());
      double er = ref_cg_last_error();
      w.put(t + ".cg_iters", {1}, &it);
      w.put(t + ".cg_error", {1}, &er);
    }
    cloth.update(new_vel, phy.F_E_is_Slides[0], h);
    phy.ResetMV();
    dump_state("s" + std::to_string(s + 1));
  }
  double st = status;
  w.put("status", {1}, &st);
  // render=PREFIX: the reference's own OBJ writer (src/Render.cpp) on the
  // final state, in its three forms
  if (kv.count("render")) {
    const std::string pre = kv["render"];
    RenderCloth(cloth, pre + "_tri.obj", RenderType::MeshTriangle);
    RenderCloth(cloth, pre + "_rect.obj", RenderType::MeshRectangle);
    RenderCloth(cloth, pre + "_yarn.obj", RenderType::YarnSpline);
  }
  return 0;
}
