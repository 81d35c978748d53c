// Test infrastructure: include/yarnsim_torch.h's reference binding compiled
// against the reference's own Cloth.h / Environment.h and linked with its
// objects (oracle/_ref/obj, built by oracle/ref/build_ref.sh) and
// libyarnsim.so. The SimHomo loop of src/Simulate.h:78-101 with SimStep
// replaced by YarnSimGpu::step; running it needs a GPU.
// Environment.h includes Cloth.h (which has no include guard of its own)
#include "Environment.h"
#define YARNSIM_REFERENCE_CLOTH
#include "yarnsim_torch.h"

int main() {
  Yarn yarn{0.0005, torch::tensor({0.002}, opts), torch::tensor({500000.0}, opts), torch::tensor({0.00014}, opts)};
  auto T = [](double x) { return torch::tensor({x}, opts); };
  Cloth cloth(6, 6, 0.05, 0.001, 0.0005, std::vector<Yarn>{yarn}, T(1.0), T(1000.0), T(1000.0), T(0.5), T(1000.0),
              T(1e4), WovenPattern::Plain, InitPose::Upright);
  Wind wind{torch::tensor({0.0, 5.0, 0.0}, opts).view({3, 1}), T(2.0), T(0.5)};
  Environment env{&cloth, torch::tensor({0.0, 0.0, 9.8}, opts).view({3, 1}), wind};
  std::vector<std::pair<int, int>> handles{{0, 0}, {5, 0}};
  cloth.set_handles(handles);
  yarnsim::YarnSimGpu gpu(cloth, env, handles);
  for (int i = 0; i < 12; ++i)
    if (!gpu.step(cloth, 1e-3)) return 1;
  return 0;
}
