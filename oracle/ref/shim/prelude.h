// Build-side prelude for compiling the reference's own physics sources
// (src/Cloth.cpp, src/PhysicsCloth.cpp, src/MatrixMp.cpp, src/Mesh.cpp,
// src/Geometry.cpp) against the LibTorch that ships with the installed torch
// wheel. The reference sources are compiled unmodified; this header is
// force-included ahead of them.
//
// * <cfloat> is needed by src/BVH.h-style code paths that use DBL_MAX.
// * Without -fopenmp nothing declares the two OpenMP runtime calls used by
//   src/PhysicsCloth.cpp:5,59; the libgomp symbols are declared here so the
//   serial build links against them (outside a parallel region
//   omp_get_thread_num() returns 0, so every per-thread buffer is buffer 0).
// * LibTorch 2.x no longer provides the C++ torch::linalg namespace used by
//   src/Solvers.h:27-29 (TorchSolver); it is mapped onto at::linalg_solve.
#pragma once
#include <cfloat>
#include <cmath>
#include <torch/torch.h>

#ifndef _OPENMP
extern "C" int omp_get_thread_num(void);
extern "C" void omp_set_num_threads(int);
#endif

namespace torch {
namespace linalg {
inline at::Tensor solve(const at::Tensor& A, const at::Tensor& B) {
  return at::linalg_solve(A, B);
}
}  // namespace linalg
}  // namespace torch
