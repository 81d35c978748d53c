// ys_emu.cpp -- TEST-ONLY host emulation of the GPU step for one cloth.
//
// Runs the product's per-element / per-node device functions
// (csrc/ys_items.cuh, compiled here as plain C++) in host loops that mirror
// the launch order of csrc/ys_api.cu, so the element arithmetic can be
// checked against the CPU oracle on a machine without a GPU. It is built and
// loaded only by tests/test_emu_vs_oracle.py; the package never loads it.
#include <cfloat>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/yarnsim.h"
#include "../../fine-grained-differentiable-physics-a-yarn-level-model-for-fabrics_gb300/csrc/ys_items.cuh"
#include "../../fine-grained-differentiable-physics-a-yarn-level-model-for-fabrics_gb300/csrc/ys_bvh.h"
#include "../../fine-grained-differentiable-physics-a-yarn-level-model-for-fabrics_gb300/csrc/ys_zones.h"

namespace {

struct Emu {
  ys::ClothParams P;
  int N;
  std::vector<int> node_cloth, node_u, node_v;
  std::vector<uint8_t> flags;
  std::vector<double> rho, ks, kb;
  std::vector<double> X, V, XF, UV, UVD, UVB, UV0, NRM, COMP, SLIDE, A, B, EXT, DINV, SOL;
  std::vector<double> RE, RB, RF, RS;  // element records
  ys::View v{};
  ys::Records R{};
  int bad = 0;
  // forward-mode tangents (kTangents directions)
  int tmode = 0;  // 0 exact, 1 reference (M, D, A held constant; transposed solves)
  std::vector<double> dX, dV, dUV, dUVD, dUVB, dNRM, dCOMP, dSLIDE, drho, dks, dkb, dS, dmu, dA, dB, dRE, dRB, dRF,
      dRS, As, Bs, RT, DQ, QS;

  void bind() {
    v.ntot = N;
    v.ncloth = 1;
    v.node_cloth = node_cloth.data(); v.node_u = node_u.data(); v.node_v = node_v.data();
    v.flags = flags.data(); v.cp = &P;
    v.line_rho = rho.data(); v.line_ks = ks.data(); v.line_kb = kb.data();
    v.nlines = (int)rho.size();
    v.X = X.data(); v.V = V.data(); v.XF = XF.data(); v.UV = UV.data(); v.UVD = UVD.data(); v.UVB = UVB.data();
    v.UV0 = UV0.data(); v.NRM = NRM.data(); v.COMP = COMP.data(); v.SLIDE = SLIDE.data();
    v.A = A.data(); v.B = B.data();
    R.edge = RE.data(); R.bend = RB.data(); R.face = RF.data(); R.shear = RS.data();
  }
};

int flip_of(int weave, int i, int j) {
  if (weave == 0) return (i + j) % 2 != 0;
  if (weave == 1) { int rv = j % 4, ru = (i + rv) % 4; return ru < 2; }
  int rv = (j - 1) % 4, q = rv / 2, r = rv % 2, idx = q * 3 + r * 2, ru = (i - 1 + idx) % 4;
  return ru == 0;
}

}  // namespace

extern "C" {

void* emu_create(const ys_cloth_desc* d) {
  Emu* e = new Emu();
  const int W = d->width, H = d->length, N = W * H;
  e->N = N;
  ys::ClothParams& P = e->P;
  P = ys::ClothParams{};
  P.W = W; P.H = H; P.node_off = 0; P.warp_line_off = 0; P.weft_line_off = H;
  P.L = d->L; P.R = d->R; P.kc = d->kc; P.kf = d->kf; P.df = d->df; P.mu = d->mu; P.S = d->S;
  P.kh = d->handle_stiffness; P.jam = 2.0 * std::asin(d->R / d->L);
  for (int k = 0; k < 3; ++k) { P.G[k] = d->G[k]; P.wind[k] = d->wind_vel[k]; }
  P.wind_rho = d->wind_density; P.wind_drag = d->wind_drag;
  P.pb4 = std::pow(ys::kPi / 2, 4);
  P.pb5 = std::pow(ys::kPi / 2, 5);
  for (int i = 0; i < H; ++i) {
    e->rho.push_back(d->warp_rho[i]);
    e->ks.push_back(d->warp_Y[i] * ys::kPi * std::pow(d->R, 2));
    e->kb.push_back(d->warp_B[i] * ys::kPi * std::pow(d->R, 2));
  }
  for (int i = 0; i < W; ++i) {
    e->rho.push_back(d->weft_rho[i]);
    e->ks.push_back(d->weft_Y[i] * ys::kPi * std::pow(d->R, 2));
    e->kb.push_back(d->weft_B[i] * ys::kPi * std::pow(d->R, 2));
  }
  auto Z = [&](std::vector<double>& a, int c) { a.assign((size_t)c * N, 0.0); };
  Z(e->X, 3); Z(e->V, 3); Z(e->XF, 3); Z(e->UV, 2); Z(e->UVD, 2); Z(e->UVB, 2); Z(e->UV0, 2); Z(e->NRM, 3);
  Z(e->COMP, 1); Z(e->SLIDE, 2); Z(e->A, ys::YS_NUM_SLOTS); Z(e->B, 5); Z(e->EXT, 5); Z(e->DINV, 5); Z(e->SOL, 5);
  Z(e->RE, ys::kEdgeFields * 2); Z(e->RB, ys::kBendFields * 2); Z(e->RF, 6); Z(e->RS, ys::kShearFields * 4);
  std::vector<uint8_t> fixed(N, 0);
  for (int h = 0; h < d->n_handles; ++h) fixed[d->handles[2 * h] + d->handles[2 * h + 1] * W] = 1;
  for (int j = 0; j < H; ++j)
    for (int i = 0; i < W; ++i) {
      const int n = i + j * W;
      e->node_cloth.push_back(0); e->node_u.push_back(i); e->node_v.push_back(j);
      const bool in = !(i == 0 || i == W - 1 || j == 0 || j == H - 1);
      uint8_t f = in ? ys::YS_INTERIOR : 0;
      if (in && flip_of(d->weave, i, j)) f |= ys::YS_FLIP;
      if (fixed[n]) f |= ys::YS_FIXED;
      e->flags.push_back(f);
      double x[3];
      if (d->pose == 0) { x[0] = i * d->L; x[1] = 0.0; x[2] = d->height - j * d->L; }
      else { x[0] = i * d->L; x[1] = j * d->L; x[2] = d->height; }
      for (int k = 0; k < 3; ++k) { e->X[k * N + n] = x[k]; e->XF[k * N + n] = x[k]; }
      const double uv[2] = {i * d->L, j * d->L};
      for (int k = 0; k < 2; ++k) { e->UV[k * N + n] = uv[k]; e->UVB[k * N + n] = uv[k]; e->UV0[k * N + n] = uv[k]; }
    }
  e->bind();
  return e;
}

void emu_destroy(void* h) { delete static_cast<Emu*>(h); }

// ---------------------------------------------------------------- tangents
constexpr int KT = ys::kTangents;
void emu_assemble(void* h, double dt, const double* ext);

int emu_tangent_count(void) { return KT; }
void emu_tangent_mode(void* h, int mode) { static_cast<Emu*>(h)->tmode = mode; }

void emu_tangent_init(void* h) {
  Emu* e = static_cast<Emu*>(h);
  const size_t N = e->N, nl = e->rho.size();
  auto Z = [&](std::vector<double>& a, size_t c) { a.assign(c, 0.0); };
  Z(e->dX, 3 * KT * N); Z(e->dV, 3 * KT * N); Z(e->dUV, 2 * KT * N); Z(e->dUVD, 2 * KT * N); Z(e->dUVB, 2 * KT * N);
  Z(e->dNRM, 3 * KT * N); Z(e->dCOMP, KT * N); Z(e->dSLIDE, 2 * KT * N);
  Z(e->drho, KT * nl); Z(e->dks, KT * nl); Z(e->dkb, KT * nl); Z(e->dS, KT); Z(e->dmu, KT);
  Z(e->dA, (size_t)ys::YS_NUM_SLOTS * KT * N); Z(e->dB, 5 * KT * N);
  Z(e->dRE, (size_t)ys::kEdgeFields * 2 * KT * N); Z(e->dRB, (size_t)ys::kBendFields * 2 * KT * N);
  Z(e->dRF, 6 * KT * N); Z(e->dRS, (size_t)ys::kShearFields * 4 * KT * N);
  Z(e->As, (size_t)ys::YS_NUM_SLOTS * N); Z(e->Bs, 5 * N); Z(e->RT, 5 * KT * N); Z(e->DQ, 5 * KT * N); Z(e->QS, 5 * N);
  // buffers every step writes before reading start as NaN, as device memory
  // may hold anything: a read of an unwritten entry shows up in the tests
  const double nan = std::nan("");
  for (auto* a : {&e->dNRM, &e->dCOMP, &e->dSLIDE, &e->dA, &e->dB, &e->dRE, &e->dRB, &e->dRF, &e->dRS, &e->As,
                  &e->Bs, &e->RT})
    std::fill(a->begin(), a->end(), nan);
}

// parameter tangents: [KT][nlines] for rho, Y, B (lines: warp rows then weft
// columns), [KT] for S and mu; Y and B enter as ks, kb = (Y, B) pi R^2
void emu_tangent_seed(void* h, const double* drho, const double* dY, const double* dBm, const double* dS,
                      const double* dmu) {
  Emu* e = static_cast<Emu*>(h);
  const size_t nl = e->rho.size();
  const double a = ys::kPi * std::pow(e->P.R, 2);
  for (size_t i = 0; i < KT * nl; ++i) {
    e->drho[i] = drho ? drho[i] : 0.0;
    e->dks[i] = dY ? dY[i] * a : 0.0;
    e->dkb[i] = dBm ? dBm[i] * a : 0.0;
  }
  for (int k = 0; k < KT; ++k) {
    e->dS[k] = dS ? dS[k] : 0.0;
    e->dmu[k] = dmu ? dmu[k] : 0.0;
  }
}

// state tangents in node layout [KT][N][c]
static void tan_io(Emu* e, double* ext, std::vector<double>& a, int c, bool in) {
  const int N = e->N;
  for (int k = 0; k < KT; ++k)
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < c; ++j) {
        double& t = a[((size_t)j * KT + k) * N + i];
        double& x = ext[((size_t)k * N + i) * c + j];
        if (in) t = x; else x = t;
      }
}
void emu_tangent_state(void* h, double* dlpos, double* dlvel, double* depos, double* deposbar, double* devel, int set) {
  Emu* e = static_cast<Emu*>(h);
  if (dlpos) tan_io(e, dlpos, e->dX, 3, set);
  if (dlvel) tan_io(e, dlvel, e->dV, 3, set);
  if (depos) tan_io(e, depos, e->dUV, 2, set);
  if (deposbar) tan_io(e, deposbar, e->dUVB, 2, set);
  if (devel) tan_io(e, devel, e->dUVD, 2, set);
}

// raw tangent buffers (for diagnosis): 0 dNRM 1 dCOMP 2 dSLIDE 3 dA 4 dB 5 dRE
// 6 dRB 7 dRF 8 dRS 9 DQ; returns the element count, copies when out != 0
long emu_tangent_raw(void* h, int which, double* out) {
  Emu* e = static_cast<Emu*>(h);
  std::vector<double>* t[18] = {&e->dNRM, &e->dCOMP, &e->dSLIDE, &e->dA, &e->dB, &e->dRE, &e->dRB, &e->dRF,
                                &e->dRS, &e->DQ, &e->NRM, &e->COMP, &e->SLIDE, &e->As, &e->Bs, &e->RE, &e->RB, &e->RF};
  if (which < 0 || which > 17) return -1;
  if (out) std::memcpy(out, t[which]->data(), sizeof(double) * t[which]->size());
  return (long)t[which]->size();
}

// Jacobi-PCG as emu_solve on an arbitrary right-hand side
static long pcg(Emu* e, const double* b, double* x, double tol, long maxiter, bool trans = false) {
  ys::View& v = e->v;
  const int N = e->N;
  std::vector<double> r(5 * N), p(5 * N), q(5 * N), z(5 * N);
  double bb = 0, rz = 0;
  for (int i = 0; i < 5 * N; ++i) {
    x[i] = 0; r[i] = b[i]; z[i] = e->DINV[i] * r[i]; p[i] = z[i];
    bb += r[i] * r[i]; rz += r[i] * z[i];
  }
  double rr = bb;
  const double thr = std::max(tol * tol * bb, DBL_MIN);
  if (bb == 0 || rr < thr) return 0;
  long it = 0;
  while (it < maxiter) {
    double pq = 0;
    for (int n = 0; n < N; ++n) {
      double y[5];
      if (trans) ys::spmv_row_t(v, p.data(), n, y);
      else ys::spmv_row(v, p.data(), n, y);
      for (int k = 0; k < 5; ++k) { q[k * N + n] = y[k]; pq += p[k * N + n] * y[k]; }
    }
    const double alpha = rz / pq;
    rr = 0;
    double rzn = 0;
    for (int i = 0; i < 5 * N; ++i) {
      x[i] += alpha * p[i]; r[i] -= alpha * q[i]; rr += r[i] * r[i]; z[i] = e->DINV[i] * r[i]; rzn += r[i] * z[i];
    }
    ++it;
    if (rr < thr) break;
    const double beta = rzn / rz;
    rz = rzn;
    for (int i = 0; i < 5 * N; ++i) p[i] = z[i] + beta * p[i];
  }
  return it;
}

// One step with tangents: the plain step's assemble and solve, the same
// assembly over Dual<KT> (tangents of A, b), kact tangent solves
// A dq = db - dA q, and the update of state and tangents. Returns non-zero if
// the step was not finite.
int emu_step_tangent(void* h, double dt, const double* ext, double tol, int kact) {
  Emu* e = static_cast<Emu*>(h);
  typedef ys::Dual<KT> D;
  const int W = e->P.W, H = e->P.H, N = e->N;
  emu_assemble(h, dt, ext);
  if (e->bad) return 1;
  const long dim = 3L * N + 2L * (W - 2) * (H - 2);
  pcg(e, e->B.data(), e->SOL.data(), tol, 2 * dim);
  for (double s : e->SOL) if (!std::isfinite(s)) return 1;
  // dual pass: values of A, b into shadows, tangents alongside
  ys::View dv = e->v;
  dv.A = e->As.data(); dv.B = e->Bs.data();
  dv.K = KT;
  dv.trunc = e->tmode;
  dv.dX = e->dX.data(); dv.dV = e->dV.data(); dv.dUV = e->dUV.data(); dv.dUVD = e->dUVD.data();
  dv.dUVB = e->dUVB.data(); dv.dNRM = e->dNRM.data(); dv.dCOMP = e->dCOMP.data(); dv.dSLIDE = e->dSLIDE.data();
  dv.dline_rho = e->drho.data(); dv.dline_ks = e->dks.data(); dv.dline_kb = e->dkb.data();
  dv.dS = e->dS.data(); dv.dmu = e->dmu.data(); dv.dA = e->dA.data(); dv.dB = e->dB.data();
  ys::Records R = e->R;
  R.dedge = e->dRE.data(); R.dbend = e->dRB.data(); R.dface = e->dRF.data(); R.dshear = e->dRS.data();
  for (int j = 1; j < H - 1; ++j) for (int i = 1; i < W - 1; ++i) ys::node_normal_dual<KT>(dv, i + j * W, W);
  for (int k = 0; k < 2; ++k)
    for (int n = 0; n < N; ++n) {
      const int i = n % W, j = n / W;
      if (k == 0 ? i >= W - 1 : j >= H - 1) continue;
      ys::EdgeOut<D> o;
      ys::edge_element(dv, n, n + (k == 0 ? 1 : W), k, o);
      ys::edge_store(dv, R.edge, R.dedge, n, k, o);
    }
  for (int k = 0; k < 2; ++k)
    for (int n = 0; n < N; ++n) {
      const int i = n % W, j = n / W;
      const int pos = k == 0 ? i : j, len = k == 0 ? W : H;
      if (pos < 1 || pos > len - 2) continue;
      const int step = k == 0 ? 1 : W;
      ys::bend_element<D>(dv, R.bend, R.dbend, n - step, n, n + step, k, k == 0 ? j : H + i);
    }
  for (int n = 0; n < N; ++n)
    if (n % W < W - 1 && n / W < H - 1) ys::cell_faces<D>(dv, R.face, R.dface, n);
  for (int n = 0; n < N; ++n) ys::gather_elements<D>(dv, R, n);
  for (int seg = 0; seg < 4; ++seg)
    for (int n = 0; n < N; ++n)
      if (e->flags[n] & ys::YS_INTERIOR) ys::shear_element<D>(dv, R.shear, R.dshear, n, seg);
  for (int n = 0; n < N; ++n) ys::gather_shear_finalize<D>(dv, R, n, nullptr);
  // tangent solves
  std::vector<double> rk(5 * N), xk(5 * N);
  for (int k = 0; k < kact && k < KT; ++k) {
    for (int n = 0; n < N; ++n) {
      double r[5];
      ys::tangent_rhs_row(dv, e->SOL.data(), n, k, r);
      for (int c = 0; c < 5; ++c) rk[c * N + n] = r[c];
    }
    pcg(e, rk.data(), xk.data(), tol, 2 * dim, e->tmode == 1);
    for (int c = 0; c < 5; ++c)
      for (int n = 0; n < N; ++n) e->DQ[((size_t)c * KT + k) * N + n] = xk[c * N + n];
  }
  for (int n = 0; n < N; ++n)
    ys::update_node_dual<KT>(dv, e->SOL.data(), e->DQ.data(), e->dX.data(), e->dV.data(), e->dUV.data(),
                             e->dUVD.data(), e->dUVB.data(), n);
  return 0;
}

void emu_set_state(void* h, const double* lpos, const double* lposfix, const double* lvel, const double* epos,
                   const double* eposbar, const double* evel) {
  Emu* e = static_cast<Emu*>(h);
  const int N = e->N;
  auto S = [&](const double* src, std::vector<double>& dst, int c) {
    if (src) for (int i = 0; i < N; ++i) for (int k = 0; k < c; ++k) dst[k * N + i] = src[i * c + k];
  };
  S(lpos, e->X, 3); S(lposfix, e->XF, 3); S(lvel, e->V, 3); S(epos, e->UV, 2); S(eposbar, e->UVB, 2); S(evel, e->UVD, 2);
}

void emu_get_state(void* h, double* lpos, double* lposfix, double* lvel, double* epos, double* eposbar, double* evel) {
  Emu* e = static_cast<Emu*>(h);
  const int N = e->N;
  auto G = [&](double* dst, const std::vector<double>& src, int c) {
    if (dst) for (int i = 0; i < N; ++i) for (int k = 0; k < c; ++k) dst[i * c + k] = src[k * N + i];
  };
  G(lpos, e->X, 3); G(lposfix, e->XF, 3); G(lvel, e->V, 3); G(epos, e->UV, 2); G(eposbar, e->UVB, 2); G(evel, e->UVD, 2);
}

void emu_get_normals(void* h, double* nrm) {
  Emu* e = static_cast<Emu*>(h);
  for (int i = 0; i < e->N; ++i) for (int k = 0; k < 3; ++k) nrm[i * 3 + k] = e->NRM[k * e->N + i];
}

// same pass order as ys_assemble in csrc/ys_api.cu
void emu_assemble(void* h, double dt, const double* ext /* [N][5] or null */) {
  Emu* e = static_cast<Emu*>(h);
  ys::View& v = e->v;
  const int W = e->P.W, H = e->P.H, N = e->N;
  v.h = dt;
  v.ext = nullptr;
  if (ext) {
    for (int i = 0; i < N; ++i) for (int k = 0; k < 5; ++k) e->EXT[k * N + i] = ext[i * 5 + k];
    v.ext = e->EXT.data();
  }
  for (int j = 1; j < H - 1; ++j) for (int i = 1; i < W - 1; ++i) ys::node_normal(v, i + j * W, W);
  // element records, then the two gathers (same order as ys_assemble)
  for (int k = 0; k < 2; ++k)
    for (int n = 0; n < N; ++n) {
      const int i = n % W, j = n / W;
      if (k == 0 ? i >= W - 1 : j >= H - 1) continue;
      ys::EdgeOut<double> o;
      ys::edge_element(v, n, n + (k == 0 ? 1 : W), k, o);
      ys::edge_store(v, e->R.edge, e->R.dedge, n, k, o);
    }
  for (int k = 0; k < 2; ++k)
    for (int n = 0; n < N; ++n) {
      const int i = n % W, j = n / W;
      const int pos = k == 0 ? i : j, len = k == 0 ? W : H;
      if (pos < 1 || pos > len - 2) continue;
      const int step = k == 0 ? 1 : W;
      const int line = k == 0 ? j : H + i;
      ys::bend_element<double>(v, e->R.bend, e->R.dbend, n - step, n, n + step, k, line);
    }
  for (int n = 0; n < N; ++n)
    if (n % W < W - 1 && n / W < H - 1) ys::cell_faces<double>(v, e->R.face, e->R.dface, n);
  for (int n = 0; n < N; ++n) ys::gather_elements<double>(v, e->R, n);
  for (int seg = 0; seg < 4; ++seg)
    for (int n = 0; n < N; ++n)
      if (e->flags[n] & ys::YS_INTERIOR) ys::shear_element<double>(v, e->R.shear, e->R.dshear, n, seg);
  e->bad = 0;
  for (int n = 0; n < N; ++n)
    if (!ys::gather_shear_finalize<double>(v, e->R, n, e->DINV.data())) e->bad = 1;
}

// raw slots [159][N] and rhs [5][N]
void emu_raw(void* h, double* slots, double* rhs) {
  Emu* e = static_cast<Emu*>(h);
  if (slots) std::memcpy(slots, e->A.data(), sizeof(double) * e->A.size());
  if (rhs) std::memcpy(rhs, e->B.data(), sizeof(double) * e->B.size());
}

// Jacobi-PCG on the structured system (Eigen ConjugateGradient algorithm);
// returns iterations, writes the relative residual.
long emu_solve(void* h, double tol, long maxiter, double* err) {
  Emu* e = static_cast<Emu*>(h);
  ys::View& v = e->v;
  const int N = e->N;
  std::vector<double> r(5 * N), p(5 * N), q(5 * N), z(5 * N);
  double* x = e->SOL.data();
  if (tol <= 0) tol = DBL_EPSILON;
  const long dim = 3L * N + 2L * (e->P.W - 2) * (e->P.H - 2);
  if (maxiter < 0) maxiter = 2 * dim;
  double bb = 0, rr = 0, rz = 0;
  for (int i = 0; i < 5 * N; ++i) {
    x[i] = 0; r[i] = e->B[i]; z[i] = e->DINV[i] * r[i]; p[i] = z[i];
    bb += r[i] * r[i]; rz += r[i] * z[i];
  }
  rr = bb;
  long it = 0;
  double thr = std::max(tol * tol * bb, DBL_MIN);
  if (bb == 0 || rr < thr) { *err = bb > 0 ? std::sqrt(rr / bb) : 0; return 0; }
  while (it < maxiter) {
    double pq = 0;
    for (int n = 0; n < N; ++n) {
      double y[5];
      ys::spmv_row(v, p.data(), n, y);
      for (int k = 0; k < 5; ++k) { q[k * N + n] = y[k]; pq += p[k * N + n] * y[k]; }
    }
    const double alpha = rz / pq;
    rr = 0;
    double rzn = 0;
    for (int i = 0; i < 5 * N; ++i) {
      x[i] += alpha * p[i]; r[i] -= alpha * q[i]; rr += r[i] * r[i]; z[i] = e->DINV[i] * r[i]; rzn += r[i] * z[i];
    }
    if (rr < thr) break;
    const double beta = rzn / rz;
    rz = rzn;
    for (int i = 0; i < 5 * N; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  *err = std::sqrt(rr / bb);
  return it;
}

void emu_apply(void* h, const double* xin /* [5][N] */, double* yout /* [5][N] */) {
  Emu* e = static_cast<Emu*>(h);
  for (int n = 0; n < e->N; ++n) {
    double y[5];
    ys::spmv_row(e->v, xin, n, y);
    for (int k = 0; k < 5; ++k) yout[k * e->N + n] = y[k];
  }
}

int emu_update(void* h) {
  Emu* e = static_cast<Emu*>(h);
  if (e->bad) return 1;
  for (double s : e->SOL) if (!std::isfinite(s)) return 1;
  for (int n = 0; n < e->N; ++n) ys::update_node(e->v, e->SOL.data(), n);
  return 0;
}


// ---------------------------------------------------------------- collision
// Host restatement of the reference's traversal (src/Collision.cpp:266-326)
// over the product's tree (ys_bvh.h) and narrow phase (ys_collide.cuh), in
// the reference's emission order. faces / face_edges: cloth mesh; obstacle
// faces given by node ids. Writes pairs [P][3] and impacts [I][15] (type,
// four node ids, t, w[4], n[3], pair index, 0); returns 0, or 1 if a buffer
// was too small.
namespace {
struct HostColl {
  const ys::BvhTree* t[2];
  std::vector<ys::Kdop> box[2];
  std::vector<uint8_t> act[2];  // BVHNode::_actived, used when masked
  bool masked = false;
  std::vector<ys::CFace> faces[2];
  ys::CMesh m;
  double thick;
  bool ccd;
  std::vector<int> pairs;
};
void hc_refit(HostColl& h, int which, int n) {
  const ys::BvhTree& t = *h.t[which];
  if (t.face[n] >= 0) {
    const ys::CFace& f = h.faces[which][t.face[n]];
    ys::Kdop b, nb;
    ys::kdop_node(b, ys::cc_pos(h.m, f.v[0], false), ys::cc_pos(h.m, f.v[0], true), h.ccd);
    for (int k = 1; k < 3; ++k) {
      ys::kdop_node(nb, ys::cc_pos(h.m, f.v[k], false), ys::cc_pos(h.m, f.v[k], true), h.ccd);
      ys::kdop_add(b, nb);
    }
    h.box[which][n] = b;
  } else {
    hc_refit(h, which, t.left[n]);
    hc_refit(h, which, t.right[n]);
    h.box[which][n] = h.box[which][t.left[n]];
    ys::kdop_add(h.box[which][n], h.box[which][t.right[n]]);
  }
}
void hc_pair(HostColl& h, int a, int wb, int b) {  // a: cloth node, b: node of tree wb
  if (h.masked && !h.act[0][a] && !h.act[wb][b]) return;
  if (!ys::kdop_overlap(h.box[0][a], h.box[wb][b], h.thick)) return;
  const ys::BvhTree& ta = *h.t[0];
  const ys::BvhTree& tb = *h.t[wb];
  if (ta.face[a] >= 0 && tb.face[b] >= 0) {
    h.pairs.push_back(ta.face[a]);
    h.pairs.push_back(tb.face[b]);
    h.pairs.push_back(wb);
  } else if (ta.face[a] >= 0) {
    hc_pair(h, a, wb, tb.left[b]);
    hc_pair(h, a, wb, tb.right[b]);
  } else {
    hc_pair(h, ta.left[a], wb, b);
    hc_pair(h, ta.right[a], wb, b);
  }
}
void hc_self(HostColl& h, int n) {
  const ys::BvhTree& t = *h.t[0];
  if (t.face[n] >= 0 || (h.masked && !h.act[0][n])) return;
  hc_self(h, t.left[n]);
  hc_self(h, t.right[n]);
  hc_pair(h, t.left[n], 0, t.right[n]);
}
}  // namespace

int emu_collide(int nn, const double* x, const double* xp, int nf, const int* fv, const int* fe, int no,
                const double* ox, const double* oxp, int nof, const int* ofv, double thick, int ccd, int* pairs,
                long pcap, double* impacts, long icap, long* np, long* ni) {
  HostColl h;
  h.m = ys::CMesh{x, xp, ox, oxp};
  h.thick = thick;
  h.ccd = ccd != 0;
  h.faces[0].resize(nf);
  for (int f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) {
      h.faces[0][f].v[k] = fv[3 * f + k];
      h.faces[0][f].e[k][0] = fe[6 * f + 2 * k];
      h.faces[0][f].e[k][1] = fe[6 * f + 2 * k + 1];
    }
  h.faces[1].resize(nof);
  for (int f = 0; f < nof; ++f)
    for (int k = 0; k < 3; ++k) {
      const int b = k != 2 ? k + 1 : 0;
      int e0 = ofv[3 * f + k], e1 = ofv[3 * f + b];
      if (e0 > e1) std::swap(e0, e1);
      h.faces[1][f].v[k] = -1 - ofv[3 * f + k];
      h.faces[1][f].e[k][0] = -1 - e0;
      h.faces[1][f].e[k][1] = -1 - e1;
    }
  std::vector<int> cv(nn), ov(no);
  for (int i = 0; i < nn; ++i) cv[i] = i;
  for (int i = 0; i < no; ++i) ov[i] = i;
  ys::BvhTree ct = ys::bvh_build(nf, fv, nn, cv.data(), x, xp, h.ccd);
  ys::BvhTree ot = ys::bvh_build(nof, ofv, no, ov.data(), ox, oxp, h.ccd);
  h.t[0] = &ct;
  h.t[1] = &ot;
  h.box[0].resize(ct.face.size());
  h.box[1].resize(ot.face.size());
  hc_refit(h, 0, 0);
  if (nof) {
    // obstacle boxes use obstacle ids: refit with the obstacle faces (ids < 0)
    hc_refit(h, 1, 0);
  }
  std::vector<int> up{0};
  while (up.size() < 8) {
    std::vector<int> ch;
    for (int n : up) {
      if (ct.face[n] >= 0) ch.push_back(n);
      else { ch.push_back(ct.left[n]); ch.push_back(ct.right[n]); }
    }
    if (ch.size() == up.size()) break;
    up = ch;
  }
  for (size_t n = 0; n < up.size(); ++n) {
    hc_self(h, up[n]);
    for (size_t q = 0; q < n; ++q) hc_pair(h, up[n], 0, up[q]);
    if (nof) hc_pair(h, up[n], 1, 0);
  }
  const long P = (long)h.pairs.size() / 3;
  *np = P;
  std::vector<double> imp;
  for (long p = 0; p < P; ++p) {
    const ys::CFace& f0 = h.faces[0][h.pairs[3 * p]];
    const ys::CFace& f1 = h.faces[h.pairs[3 * p + 2]][h.pairs[3 * p + 1]];
    ys::Impact out[15];
    const int c = ys::cc_face_pair(h.m, f0, f1, thick, h.ccd, out);
    for (int k = 0; k < c; ++k) {
      const ys::Impact& s = out[k];
      const double r[15] = {(double)s.type, (double)s.node[0], (double)s.node[1], (double)s.node[2], (double)s.node[3],
                            s.t, s.w[0], s.w[1], s.w[2], s.w[3], s.n[0], s.n[1], s.n[2], (double)p, 0.0};
      imp.insert(imp.end(), r, r + 15);
    }
  }
  *ni = (long)imp.size() / 15;
  if (P > pcap || *ni > icap) return 1;
  std::memcpy(pairs, h.pairs.data(), sizeof(int) * h.pairs.size());
  std::memcpy(impacts, imp.data(), sizeof(double) * imp.size());
  return 0;
}

// ---------------------------------------------------------------- response
// The product's response loop (ys_zones.h) driven by host detection: the
// trees built once from the positions before the response, refit every
// round, traversed as the reference does with its active flags.
namespace {
ys::ZoneResponse g_resp;
std::vector<double> g_resp_x0;
double g_resp_k = 0.0;

void hc_mark(HostColl& h, const ys::BvhTree& t, const uint8_t* fa, int n, bool& on) {
  if (t.face[n] >= 0) {
    on = fa[t.face[n]] != 0;
  } else {
    bool l = false, r = false;
    hc_mark(h, t, fa, t.left[n], l);
    hc_mark(h, t, fa, t.right[n], r);
    on = l || r;
  }
  h.act[0][n] = on ? 1 : 0;
}
}  // namespace

// x [nn][3] in/out, v [nn][3] in/out (may be null), mass [nn] (may be null);
// info[9]: rounds, converged, changed, zones, infeasible, impacts,
// projections, zone overflow, reverted projections
static int g_max_zone_impacts = -1;  // < 0: the response's default

// zone limit of the next emu_respond calls (< 0: the default)
int emu_set_max_zone_impacts(int n) {
  g_max_zone_impacts = n;
  return 0;
}

int emu_respond(int nn, double* x, const double* xp, int nf, const int* fv, const int* fe, int no, const double* ox,
                const double* oxp, int nof, const int* ofv, double thick, int ccd, const double* mass, double hstep,
                double damp, int max_iter, double* v, long* info) {
  HostColl h;
  h.thick = thick;
  h.ccd = ccd != 0;
  h.faces[0].resize(nf);
  for (int f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) {
      h.faces[0][f].v[k] = fv[3 * f + k];
      h.faces[0][f].e[k][0] = fe[6 * f + 2 * k];
      h.faces[0][f].e[k][1] = fe[6 * f + 2 * k + 1];
    }
  h.faces[1].resize(nof);
  for (int f = 0; f < nof; ++f)
    for (int k = 0; k < 3; ++k) {
      const int b = k != 2 ? k + 1 : 0;
      int e0 = ofv[3 * f + k], e1 = ofv[3 * f + b];
      if (e0 > e1) std::swap(e0, e1);
      h.faces[1][f].v[k] = -1 - ofv[3 * f + k];
      h.faces[1][f].e[k][0] = -1 - e0;
      h.faces[1][f].e[k][1] = -1 - e1;
    }
  std::vector<int> cv(nn), ov(no);
  for (int i = 0; i < nn; ++i) cv[i] = i;
  for (int i = 0; i < no; ++i) ov[i] = i;
  ys::BvhTree ct = ys::bvh_build(nf, fv, nn, cv.data(), x, xp, h.ccd);
  ys::BvhTree ot = ys::bvh_build(nof, ofv, no, ov.data(), ox, oxp, h.ccd);
  h.t[0] = &ct;
  h.t[1] = &ot;
  h.box[0].resize(ct.face.size());
  h.box[1].resize(ot.face.size());
  h.act[0].assign(ct.face.size(), 1);
  h.act[1].assign(ot.face.size(), 1);
  std::vector<int> up{0};
  while (up.size() < 8) {
    std::vector<int> ch;
    for (int n : up) {
      if (ct.face[n] >= 0) ch.push_back(n);
      else { ch.push_back(ct.left[n]); ch.push_back(ct.right[n]); }
    }
    if (ch.size() == up.size()) break;
    up = ch;
  }
  auto detect = [&](const double* xc, const uint8_t* mask, std::vector<ys::ZImpact>& out) -> int {
    h.m = ys::CMesh{xc, xp, ox, oxp};
    hc_refit(h, 0, 0);
    if (nof) hc_refit(h, 1, 0);
    h.masked = mask != nullptr;
    if (mask) {
      bool on = false;
      hc_mark(h, ct, mask, 0, on);
      std::fill(h.act[1].begin(), h.act[1].end(), 0);
    }
    h.pairs.clear();
    for (size_t n = 0; n < up.size(); ++n) {
      hc_self(h, up[n]);
      for (size_t q = 0; q < n; ++q) hc_pair(h, up[n], 0, up[q]);
      if (nof) hc_pair(h, up[n], 1, 0);
    }
    out.clear();
    for (size_t p = 0; p < h.pairs.size() / 3; ++p) {
      const ys::CFace& f0 = h.faces[0][h.pairs[3 * p]];
      const ys::CFace& f1 = h.faces[h.pairs[3 * p + 2]][h.pairs[3 * p + 1]];
      ys::Impact im[15];
      const int c = ys::cc_face_pair(h.m, f0, f1, thick, h.ccd, im);
      for (int k = 0; k < c; ++k) {
        ys::ZImpact z;
        z.type = im[k].type;
        z.t = im[k].t;
        for (int q = 0; q < 4; ++q) {
          z.node[q] = im[k].node[q];
          z.w[q] = im[k].w[q];
        }
        for (int q = 0; q < 3; ++q) z.n[q] = im[k].n[q];
        out.push_back(z);
      }
    }
    return 0;
  };
  g_resp = ys::ZoneResponse();
  g_resp.n_nodes = nn;
  g_resp.n_faces = nf;
  g_resp.faces = fv;
  static std::vector<double> obs;  // kept for the backward
  obs.assign(ox, ox + 3 * (size_t)no);
  g_resp.obs_x = obs.data();
  static std::vector<double> xprev, obsprev;
  xprev.assign(xp, xp + 3 * (size_t)nn);
  obsprev.assign(oxp, oxp + 3 * (size_t)no);
  g_resp.xprev = xprev.data();
  g_resp.obs_xprev = obsprev.data();
  g_resp.thickness = thick;
  g_resp.max_iter = max_iter;
  if (g_max_zone_impacts >= 0) g_resp.max_zone_impacts = g_max_zone_impacts;
  g_resp_x0.assign(x, x + 3 * (size_t)nn);
  ys::zone_respond(g_resp, x, mass, detect);
  g_resp.faces = nullptr;
  if (v && g_resp.changed)
    for (size_t i = 0; i < 3 * (size_t)nn; ++i) v[i] = v[i] + (damp * (x[i] - g_resp_x0[i])) / hstep;
  g_resp_k = damp / hstep;
  info[0] = g_resp.rounds;
  info[1] = g_resp.converged;
  info[2] = g_resp.changed;
  info[3] = g_resp.zones;
  info[4] = g_resp.infeasible;
  info[5] = (long)g_resp.accepted.size();
  info[6] = (long)g_resp.tape.size();
  info[7] = g_resp.zone_overflow;
  info[8] = g_resp.reverted;
  return 0;
}

// accepted impacts [A][15] as emu_collide's rows (the pair column holds the
// round); multipliers of every projection are not exported
int emu_response_impacts(double* out, long cap) {
  if ((long)g_resp.accepted.size() > cap) return 1;
  for (size_t i = 0; i < g_resp.accepted.size(); ++i) {
    const ys::ZImpact& s = g_resp.accepted[i];
    const double r[15] = {(double)s.type, (double)s.node[0], (double)s.node[1], (double)s.node[2], (double)s.node[3],
                          s.t, s.w[0], s.w[1], s.w[2], s.w[3], s.n[0], s.n[1], s.n[2],
                          (double)g_resp.accepted_round[i], 0.0};
    std::memcpy(out + 15 * i, r, sizeof(r));
  }
  return 0;
}

// backward of the last emu_respond; gx [nn][3] in: dL/dx out, out: dL/dx in;
// gv [nn][3] dL/dv out (may be null); gw [A][4], gn [A][3] out
int emu_respond_backward(double* gx, const double* gv, double* gw, double* gn, int flags, double* gxp) {
  const size_t n3 = 3 * (size_t)g_resp.n_nodes, na = g_resp.accepted.size();
  std::vector<double> w(4 * std::max<size_t>(na, 1), 0.0), nn(3 * std::max<size_t>(na, 1), 0.0), p(n3, 0.0);
  if (gv && g_resp.changed)
    for (size_t i = 0; i < n3; ++i) gx[i] += g_resp_k * gv[i];
  ys::zone_backward(g_resp, gx, w.data(), nn.data(), flags, p.data());
  if (gv && g_resp.changed)
    for (size_t i = 0; i < n3; ++i) gx[i] -= g_resp_k * gv[i];
  if (na) {
    std::memcpy(gw, w.data(), 4 * na * sizeof(double));
    std::memcpy(gn, nn.data(), 3 * na * sizeof(double));
  }
  if (gxp) std::memcpy(gxp, p.data(), n3 * sizeof(double));
  return 0;
}

// the least-distance solver alone: min |u| s.t. G u >= h (G [k][n])
int emu_ldp(int n, int k, const double* G, const double* h, double* u, double* lam) {
  return ys::ldp(n, k, G, h, u, lam);
}

// the large-zone solver on the same programme, G given by sparse rows
// (cols [k][4], coef [k][4][3])
int emu_ldp_sparse(int n, int k, const int* cols, const double* coef, const double* h, double* u, double* lam) {
  return ys::ldp_sparse(n, k, cols, coef, h, u, lam);
}

// one detection round as the response runs it: trees built from xb (the
// positions before the response) and x_prev, refit to x, traversed with the
// active flags of face_active (null: all active); impacts [I][15] as
// emu_collide's rows (pair column 0)
int emu_detect(int nn, const double* xb, const double* x, const double* xp, int nf, const int* fv, const int* fe, int no,
               const double* ox, const double* oxp, int nof, const int* ofv, double thick, int ccd,
               const unsigned char* face_active, double* impacts, long icap, long* ni) {
  std::vector<double> xc(x, x + 3 * (size_t)nn);
  std::vector<double> xbb(xb, xb + 3 * (size_t)nn);
  HostColl h;
  h.thick = thick;
  h.ccd = ccd != 0;
  h.faces[0].resize(nf);
  for (int f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) {
      h.faces[0][f].v[k] = fv[3 * f + k];
      h.faces[0][f].e[k][0] = fe[6 * f + 2 * k];
      h.faces[0][f].e[k][1] = fe[6 * f + 2 * k + 1];
    }
  h.faces[1].resize(nof);
  for (int f = 0; f < nof; ++f)
    for (int k = 0; k < 3; ++k) {
      const int b = k != 2 ? k + 1 : 0;
      int e0 = ofv[3 * f + k], e1 = ofv[3 * f + b];
      if (e0 > e1) std::swap(e0, e1);
      h.faces[1][f].v[k] = -1 - ofv[3 * f + k];
      h.faces[1][f].e[k][0] = -1 - e0;
      h.faces[1][f].e[k][1] = -1 - e1;
    }
  std::vector<int> cv(nn), ov(no);
  for (int i = 0; i < nn; ++i) cv[i] = i;
  for (int i = 0; i < no; ++i) ov[i] = i;
  ys::BvhTree ct = ys::bvh_build(nf, fv, nn, cv.data(), xbb.data(), xp, h.ccd);
  ys::BvhTree ot = ys::bvh_build(nof, ofv, no, ov.data(), ox, oxp, h.ccd);
  h.t[0] = &ct;
  h.t[1] = &ot;
  h.box[0].resize(ct.face.size());
  h.box[1].resize(ot.face.size());
  h.act[0].assign(ct.face.size(), 1);
  h.act[1].assign(ot.face.size(), nof ? 1 : 0);
  h.m = ys::CMesh{xc.data(), xp, ox, oxp};
  hc_refit(h, 0, 0);
  if (nof) hc_refit(h, 1, 0);
  h.masked = face_active != nullptr;
  if (face_active) {
    bool on = false;
    hc_mark(h, ct, face_active, 0, on);
    std::fill(h.act[1].begin(), h.act[1].end(), 0);
  }
  std::vector<int> up{0};
  while (up.size() < 8) {
    std::vector<int> ch;
    for (int n : up) {
      if (ct.face[n] >= 0) ch.push_back(n);
      else { ch.push_back(ct.left[n]); ch.push_back(ct.right[n]); }
    }
    if (ch.size() == up.size()) break;
    up = ch;
  }
  for (size_t n = 0; n < up.size(); ++n) {
    hc_self(h, up[n]);
    for (size_t q = 0; q < n; ++q) hc_pair(h, up[n], 0, up[q]);
    if (nof) hc_pair(h, up[n], 1, 0);
  }
  long cnt = 0;
  for (size_t p = 0; p < h.pairs.size() / 3; ++p) {
    const ys::CFace& f0 = h.faces[0][h.pairs[3 * p]];
    const ys::CFace& f1 = h.faces[h.pairs[3 * p + 2]][h.pairs[3 * p + 1]];
    ys::Impact im[15];
    const int c = ys::cc_face_pair(h.m, f0, f1, thick, h.ccd, im);
    for (int k = 0; k < c; ++k, ++cnt) {
      if (cnt >= icap) continue;
      const ys::Impact& s = im[k];
      const double r[15] = {(double)s.type, (double)s.node[0], (double)s.node[1], (double)s.node[2],
                            (double)s.node[3], s.t, s.w[0], s.w[1], s.w[2], s.w[3], s.n[0], s.n[1], s.n[2],
                            (double)p, 0.0};
      std::memcpy(impacts + 15 * cnt, r, sizeof(r));
    }
  }
  *ni = cnt;
  return cnt > icap ? 1 : 0;
}

// impact_jacobian for tests: J [7][24]
int emu_impact_jacobian(int type, const double* x, const double* xp, double t, int sign, double* J) {
  double Jl[7][24];
  if (!ys::impact_jacobian(type, x, xp, t, sign, Jl)) return 1;
  std::memcpy(J, Jl, sizeof(Jl));
  return 0;
}

}  // extern "C"
