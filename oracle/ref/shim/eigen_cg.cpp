// Stand-in for src/Solvers.cpp:3-58 (EigenSolverForward / EigenSolverBackward),
// used only to build the reference physics as a test oracle.
//
// The reference calls Eigen 3.3.9's
//   ConjugateGradient<SparseMatrix<double>, Lower|Upper>
// with every option left at its default. Eigen is not installed here, so the
// published algorithm of that class is restated below:
//   * preconditioner: DiagonalPreconditioner (z = r / diag(A); a zero diagonal
//     entry is treated as 1),
//   * initial guess x0 = 0,
//   * stop when |r|^2 < max(tol^2 * |b|^2, DBL_MIN) with tol = DBL_EPSILON,
//   * at most 2 * n iterations,
//   * Lower|Upper means the full (possibly non-symmetric) matrix is used in
//     every product A*p.
// The sparse matrix keeps the non-zero entries of the dense tensor (scan at
// src/Solvers.cpp:7-13), and the product accumulates each row in increasing
// column order, as a column-major sparse * dense product does.
//
// The tolerance and iteration cap can be overridden through
// ref_cg_set_options() so a harness can also run tighter or looser solves.
#include <cfloat>
#include <cmath>
#include <vector>
#include "Solvers.h"

static double g_tol = DBL_EPSILON;
static long g_max_iter = -1;  // -1: 2 * n (Eigen default)
static long g_last_iters = 0;
static double g_last_error = 0.0;

void ref_cg_set_options(double tol, long max_iter) {
  g_tol = tol;
  g_max_iter = max_iter;
}
long ref_cg_last_iterations() { return g_last_iters; }
double ref_cg_last_error() { return g_last_error; }

namespace {
struct Csr {
  int n = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
  std::vector<double> diag;
};

Csr dense_to_csr(const at::Tensor& A_in) {
  at::Tensor A = A_in.contiguous();
  Csr m;
  m.n = static_cast<int>(A.size(0));
  const int nc = static_cast<int>(A.size(1));
  const double* a = A.data_ptr<double>();
  m.rowptr.assign(m.n + 1, 0);
  m.diag.assign(m.n, 0.0);
  for (int i = 0; i < m.n; ++i) {
    for (int j = 0; j < nc; ++j) {
      const double v = a[static_cast<long>(i) * nc + j];
      if (v != 0.0) {
        m.col.push_back(j);
        m.val.push_back(v);
        if (i == j) m.diag[i] = v;
      }
    }
    m.rowptr[i + 1] = static_cast<int>(m.col.size());
  }
  return m;
}

void spmv(const Csr& m, const std::vector<double>& x, std::vector<double>& y) {
  for (int i = 0; i < m.n; ++i) {
    double s = 0.0;
    for (int k = m.rowptr[i]; k < m.rowptr[i + 1]; ++k) s += m.val[k] * x[m.col[k]];
    y[i] = s;
  }
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

std::vector<double> pcg(const Csr& m, const std::vector<double>& rhs) {
  const int n = m.n;
  std::vector<double> x(n, 0.0), r(rhs), z(n), p(n), q(n);
  std::vector<double> invdiag(n);
  for (int i = 0; i < n; ++i) invdiag[i] = (m.diag[i] != 0.0) ? 1.0 / m.diag[i] : 1.0;
  const long max_iter = g_max_iter < 0 ? 2L * n : g_max_iter;
  const double rhs_norm2 = dot(rhs, rhs);
  g_last_iters = 0;
  if (rhs_norm2 == 0.0) {
    g_last_error = 0.0;
    return x;
  }
  const double threshold = std::max(g_tol * g_tol * rhs_norm2, DBL_MIN);
  double res_norm2 = dot(r, r);
  if (res_norm2 < threshold) {
    g_last_error = std::sqrt(res_norm2 / rhs_norm2);
    return x;
  }
  for (int i = 0; i < n; ++i) p[i] = invdiag[i] * r[i];
  double abs_new = dot(r, p);
  long it = 0;
  while (it < max_iter) {
    spmv(m, p, q);
    const double alpha = abs_new / dot(p, q);
    for (int i = 0; i < n; ++i) x[i] += alpha * p[i];
    for (int i = 0; i < n; ++i) r[i] -= alpha * q[i];
    res_norm2 = dot(r, r);
    if (res_norm2 < threshold) break;
    for (int i = 0; i < n; ++i) z[i] = invdiag[i] * r[i];
    const double abs_old = abs_new;
    abs_new = dot(r, z);
    const double beta = abs_new / abs_old;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  g_last_iters = it;
  g_last_error = std::sqrt(res_norm2 / rhs_norm2);
  return x;
}

at::Tensor solve_dense(const at::Tensor& A, const at::Tensor& b) {
  Csr m = dense_to_csr(A);
  at::Tensor bc = b.contiguous();
  std::vector<double> rhs(bc.data_ptr<double>(), bc.data_ptr<double>() + m.n);
  std::vector<double> x = pcg(m, rhs);
  at::Tensor out = torch::zeros_like(b, opts);
  double* o = out.data_ptr<double>();
  for (int i = 0; i < m.n; ++i) o[i] = x[i];
  return out;
}
}  // namespace

Tensor EigenSolverForward(const Tensor& A, const Tensor& b, bool) {
  return solve_dense(A.detach(), b.detach());
}

// src/Solvers.cpp:33-58: the backward solves A * dx = dldz (with A, not A^T)
// and returns dA = -dx (x) ans, db = dx.
std::vector<Tensor> EigenSolverBackward(Tensor& dldz, const Tensor& ans, const Tensor& tensor_A,
                                        const Tensor& tensor_b) {
  at::Tensor g = dldz.contiguous().detach().view({tensor_b.size(0), tensor_b.size(1)});
  at::Tensor dx = solve_dense(tensor_A.detach(), g);
  at::Tensor dlda = -torch::ger(dx.squeeze(), ans.squeeze());
  return {dlda, dx};
}
