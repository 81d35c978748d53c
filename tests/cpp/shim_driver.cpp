// Test driver of include/yarnsim_torch.h (test infrastructure): a C++
// program on LibTorch that steps a cloth through yarnsim::GpuCloth -- the
// SimHomo loop of src/Simulate.h:78-101 with SimStep replaced -- or takes the
// training loss's gradient through yarnsim::AdjointRollout, reading a
// key=value config and raw float64 files written by tests/test_gpu_shim.py.
//
//   shim_driver <config>
// config keys: mode (traj | grad), width, length, height, L, R, pose, weave,
// kc, kf, df, mu, S, handle_stiffness, G, wind_vel, wind_density, wind_drag,
// handles, warp / weft (files: [lines][3] rho, Y, B), init (file: LPos,
// LPosFix, LVel [N][3], EPos, EPosBar, EVel [N][2]), steps, h, out;
// grad: theta (8 values), targets (file: [steps][N][3] then [steps][N][2]),
// adjoint (0 exact, 1 reference), k, tol (PCG relative residual; default
// Eigen's).
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "yarnsim_torch.h"

namespace {

std::map<std::string, std::string> read_config(const char* path) {
  std::map<std::string, std::string> kv;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    auto eq = line.find('=');
    if (eq != std::string::npos) kv[line.substr(0, eq)] = line.substr(eq + 1);
  }
  return kv;
}
std::vector<double> list(const std::string& s) {
  std::vector<double> out;
  std::stringstream ss(s);
  std::string tok;
  while (std::getline(ss, tok, ','))
    if (!tok.empty()) out.push_back(std::stod(tok));
  return out;
}
std::vector<double> file(const std::string& path, size_t n) {
  std::vector<double> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), n * sizeof(double));
  if (!f) throw std::runtime_error("short file " + path);
  return v;
}
torch::Tensor tensor(const std::vector<double>& v, size_t off, std::vector<int64_t> shape) {
  int64_t n = 1;
  for (auto d : shape) n *= d;
  return torch::from_blob(const_cast<double*>(v.data() + off), {n}, torch::kFloat64).clone().view(shape);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  auto kv = read_config(argv[1]);
  auto d = [&](const char* k) { return std::stod(kv.at(k)); };
  yarnsim::ClothDescription desc;
  ys_cloth_desc& c = desc.d;
  c.width = (int)d("width"); c.length = (int)d("length"); c.height = d("height"); c.L = d("L"); c.R = d("R");
  c.pose = (int)d("pose"); c.weave = (int)d("weave");
  c.kc = d("kc"); c.kf = d("kf"); c.df = d("df"); c.mu = d("mu"); c.S = d("S"); c.handle_stiffness = d("handle_stiffness");
  auto G = list(kv.at("G")), w = list(kv.at("wind_vel"));
  for (int k = 0; k < 3; ++k) { c.G[k] = G[k]; c.wind_vel[k] = w[k]; }
  c.wind_density = d("wind_density"); c.wind_drag = d("wind_drag");
  for (double x : list(kv["handles"])) desc.handles.push_back((int32_t)x);
  const int W = c.width, H = c.length, N = W * H;
  auto wl = file(kv.at("warp"), 3 * (size_t)H), fl = file(kv.at("weft"), 3 * (size_t)W);
  for (int v = 0; v < H; ++v) { desc.warp_rho.push_back(wl[3 * v]); desc.warp_Y.push_back(wl[3 * v + 1]); desc.warp_B.push_back(wl[3 * v + 2]); }
  for (int u = 0; u < W; ++u) { desc.weft_rho.push_back(fl[3 * u]); desc.weft_Y.push_back(fl[3 * u + 1]); desc.weft_B.push_back(fl[3 * u + 2]); }
  auto in = file(kv.at("init"), 15 * (size_t)N);
  yarnsim::State s0{tensor(in, 0, {N, 3, 1}), tensor(in, 3 * N, {N, 3, 1}), tensor(in, 6 * N, {N, 3, 1}),
                    tensor(in, 9 * N, {N, 2, 1}), tensor(in, 11 * N, {N, 2, 1}), tensor(in, 13 * N, {N, 2, 1})};
  const int steps = (int)d("steps");
  const double h = d("h");
  std::FILE* out = std::fopen(kv.at("out").c_str(), "wb");
  if (kv.at("mode") == "traj") {
    yarnsim::GpuCloth cloth(desc);
    cloth.set_state(s0);
    for (int s = 0; s < steps; ++s) {
      if (!cloth.step(h)) { std::fprintf(stderr, "step %d failed\n", s); return 1; }
      yarnsim::State st = cloth.get_state();
      for (const torch::Tensor* t : {&st.LPos, &st.LPosFix, &st.LVel, &st.EPos, &st.EPosBar, &st.EVel})
        std::fwrite(t->data_ptr<double>(), sizeof(double), t->numel(), out);
    }
  } else {
    auto th = list(kv.at("theta"));
    torch::Tensor theta = torch::tensor(th, torch::kFloat64).requires_grad_(true);
    auto tg = file(kv.at("targets"), (size_t)steps * N * 5);
    torch::Tensor gx = tensor(tg, 0, {steps, N, 3}), ge = tensor(tg, (size_t)steps * N * 3, {steps, N, 2});
    const double tol = kv.count("tol") ? d("tol") : 0.0;
    auto xe = yarnsim::AdjointRollout::apply(theta, desc, s0, (int64_t)steps, h, (int64_t)d("adjoint"),
                                             (int64_t)d("k"), tol);
    torch::Tensor loss = yarnsim::position_loss(xe[0], xe[1], gx, ge);
    loss.backward();
    double l = loss.item<double>();
    std::fwrite(&l, sizeof(double), 1, out);
    torch::Tensor g = theta.grad().contiguous();
    std::fwrite(g.data_ptr<double>(), sizeof(double), 8, out);
  }
  std::fclose(out);
  return 0;
}
