/*
 * yarn_oracle.c -- CPU restatement of the reference's per-step yarn solve.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle the GPU path is checked
 * against and the CPU baseline that bench.py times; nothing in the product
 * links or calls it.
 *
 * Each routine restates one reference routine and cites it as path:line
 * relative to the reference project root. The restatement keeps the
 * reference's arithmetic *as written*, including its quirks, because parity
 * is defined against what the reference computes, not against the exact
 * derivatives. The quirks kept on purpose are listed where they occur:
 *   - 3x3 node-node (LL) blocks are written transposed into the dense matrix
 *     (src/MatrixMp.cpp:54-65),
 *   - MDotVDot_D_Pos ADDS its Jacobian while MDotVDot_F subtracts the force
 *     (src/PhysicsCloth.cpp:2231-2235 vs 1936-1937),
 *   - Inertia_D_Pos builds its (x, uv) mixed block with a sign-asymmetric
 *     4x4 block (src/PhysicsCloth.cpp:1357-1361),
 *   - Bending_D writes the (n0,n2) E-L coupling at (E of n0, L of n2)
 *     (src/PhysicsCloth.cpp:780-795),
 *   - jamming Shear_D omits PI in the second derivative of kx and broadcasts a
 *     scalar 1 over 3x3 matrices (src/PhysicsCloth.cpp:2962-2992),
 *   - ConSlideFriction's velocity derivative uses tanh(10*fric_lim - F)
 *     (src/PhysicsCloth.cpp:2630-2631),
 *   - crimp bending segments keep the EPos of the build (src/Cloth.cpp:107),
 *   - EPS = DBL_MIN makes the theta clamp a no-op (src/Constants.h:25).
 */
#include "yarn_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define YO_PI 3.1415926535897 /* src/Constants.h:24 */

typedef struct {
  int n0, n1, k, line, in0, in1;
  double rho, ks, kb;
  double du, dx[3], w[3], l, d[3], P[3][3], q[8];
} edge_t;

typedef struct {
  int n2, n0, n1, k, in2, in0, in1;
  double kb, du, l1, l2, d1[3], d2[3], P1[3][3], P2[3][3], theta;
} bend_t;

struct yo_cloth {
  int W, H, N, Nc, dim;
  double L, R, height;
  int pose, weave;
  double *rho_warp, *ks_warp, *kb_warp, *rho_weft, *ks_weft, *kb_weft;
  double kc, kf, df, mu, S, kh, G[3], wind_v[3], wind_rho, wind_drag, jam;
  /* state, node order */
  double *x, *v, *xfix, *uv, *uvdot, *uvbar, *uv0;
  unsigned char *fixed, *flip;
  double *nrm, *xw, *xf, *comp;
  /* sparse storage, reference DOF order */
  int nnz;
  int *rowptr, *col;
  double *Mv, *Kv, *Dv;
  double *F, *slide, *CL, *CLE;
};

/* ------------------------------------------------------------------ */
/* small helpers                                                       */
/* ------------------------------------------------------------------ */
static int nid(const yo_cloth *c, int u, int v) { return u + v * c->W; }
static int is_int(const yo_cloth *c, int n) {
  int u = n % c->W, v = n / c->W;
  return !(u == 0 || u == c->W - 1 || v == 0 || v == c->H - 1);
}
static int eidx(const yo_cloth *c, int n) {
  int u = n % c->W, v = n / c->W;
  return (u - 1) + (v - 1) * (c->W - 2);
}
static int erow(const yo_cloth *c, int n) { return 3 * c->N + 2 * eidx(c, n); }

static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double norm3(const double *a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
static void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
static void proj(const double *d, double P[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P[i][j] = (i == j ? 1.0 : 0.0) - d[i] * d[j];
}
static void mv3(double P[3][3], const double *a, double *o) {
  for (int i = 0; i < 3; ++i) o[i] = P[i][0] * a[0] + P[i][1] * a[1] + P[i][2] * a[2];
}
static void outer3(const double *a, const double *b, double O[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) O[i][j] = a[i] * b[j];
}
static void mm3(double A[3][3], double B[3][3], double O[3][3]) {
  double T[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
  memcpy(O, T, sizeof(T));
}

/* sparse entry lookup (binary search inside the row) */
static double *at(yo_cloth *c, double *vals, int r, int col) {
  int lo = c->rowptr[r], hi = c->rowptr[r + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    if (c->col[mid] == col) return &vals[mid];
    if (c->col[mid] < col) lo = mid + 1; else hi = mid - 1;
  }
  abort(); /* pattern miss: a write outside the 13-point stencil */
}
/* X_LL[find_index(f, d, "LL")] += blk, written transposed into the dense
 * matrix by To_Sparse_Mat (src/PhysicsCloth.cpp:202, src/MatrixMp.cpp:54-65). */
static void add_LL(yo_cloth *c, double *A, int f, int d, double blk[3][3], double s) {
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) *at(c, A, 3 * f + r, 3 * d + q) += s * blk[q][r];
}
/* X_LE[find_index(l, e, "EL") + k] += vec -> A[L(l)][E(e)+k]
 * (src/PhysicsCloth.cpp:204, src/MatrixMp.cpp:67-76). */
static void add_LE(yo_cloth *c, double *A, int l, int e, int k, const double *vec, double s) {
  for (int r = 0; r < 3; ++r) *at(c, A, 3 * l + r, erow(c, e) + k) += s * vec[r];
}
/* X_EL[find_index(l, e, "EL") + k] += row -> A[E(e)+k][L(l)]
 * (src/MatrixMp.cpp:78-87). */
static void add_EL(yo_cloth *c, double *A, int l, int e, int k, const double *row, double s) {
  for (int q = 0; q < 3; ++q) *at(c, A, erow(c, e) + k, 3 * l + q) += s * row[q];
}
/* X_EE[find_index(f, d, "EE", "uu"|"vv")] += val (src/PhysicsCloth.cpp:205-209). */
static void add_EE(yo_cloth *c, double *A, int f, int d, int k, double val) {
  *at(c, A, erow(c, f) + k, erow(c, d) + k) += val;
}

/* ------------------------------------------------------------------ */
/* topology and storage                                                */
/* ------------------------------------------------------------------ */
static int cmp_int(const void *a, const void *b) { return (*(const int *)a) - (*(const int *)b); }

static void build_pattern(yo_cloth *c) {
  static const int off[13][2] = {{0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-2, 0}, {2, 0},
                                 {0, -2}, {0, 2}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  int dim = c->dim;
  int *cnt = (int *)calloc(dim + 1, sizeof(int));
  int *tmp = (int *)malloc(sizeof(int) * 13 * 5);
  /* count */
  for (int n = 0; n < c->N; ++n) {
    int u = n % c->W, v = n / c->W, m = 0;
    for (int s = 0; s < 13; ++s) {
      int uu = u + off[s][0], vv = v + off[s][1];
      if (uu < 0 || uu >= c->W || vv < 0 || vv >= c->H) continue;
      m += 3 + (is_int(c, nid(c, uu, vv)) ? 2 : 0);
    }
    for (int r = 0; r < 3; ++r) cnt[3 * n + r + 1] = m;
    if (is_int(c, n)) { cnt[erow(c, n) + 1] = m; cnt[erow(c, n) + 2] = m; }
  }
  for (int r = 0; r < dim; ++r) cnt[r + 1] += cnt[r];
  c->rowptr = cnt;
  c->nnz = cnt[dim];
  c->col = (int *)malloc(sizeof(int) * c->nnz);
  for (int n = 0; n < c->N; ++n) {
    int u = n % c->W, v = n / c->W, m = 0;
    for (int s = 0; s < 13; ++s) {
      int uu = u + off[s][0], vv = v + off[s][1];
      if (uu < 0 || uu >= c->W || vv < 0 || vv >= c->H) continue;
      int j = nid(c, uu, vv);
      for (int q = 0; q < 3; ++q) tmp[m++] = 3 * j + q;
      if (is_int(c, j)) { tmp[m++] = erow(c, j); tmp[m++] = erow(c, j) + 1; }
    }
    qsort(tmp, m, sizeof(int), cmp_int);
    int rows[5], nr = 0;
    for (int r = 0; r < 3; ++r) rows[nr++] = 3 * n + r;
    if (is_int(c, n)) { rows[nr++] = erow(c, n); rows[nr++] = erow(c, n) + 1; }
    for (int r = 0; r < nr; ++r) memcpy(&c->col[c->rowptr[rows[r]]], tmp, sizeof(int) * m);
  }
  free(tmp);
  c->Mv = (double *)calloc(c->nnz, sizeof(double));
  c->Kv = (double *)calloc(c->nnz, sizeof(double));
  c->Dv = (double *)calloc(c->nnz, sizeof(double));
}

/* Node normal: smallest right singular vector of the centred 5x3 stencil
 * (src/Cloth.cpp:440-463). Restated as the eigenvector of the smallest
 * eigenvalue of the 3x3 scatter matrix (cyclic Jacobi rotations). */
static void sym3_min_eigvec(double A[3][3], double out[3]) {
  double a[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  memcpy(a, A, sizeof(a));
  /* off-diagonal entries below 1e-24 of the diagonal scale are treated as zero */
  const double tiny = 1e-24 * (fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]));
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    if (off <= tiny) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (fabs(a[p][q]) <= tiny) continue;
        double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < 3; ++k) {
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = cs * akp - sn * akq;
          a[k][q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = cs * apk - sn * aqk;
          a[q][k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = cs * vkp - sn * vkq;
          V[k][q] = sn * vkp + cs * vkq;
        }
      }
  }
  int m = 0;
  if (a[1][1] < a[m][m]) m = 1;
  if (a[2][2] < a[m][m]) m = 2;
  for (int k = 0; k < 3; ++k) out[k] = V[k][m];
}

static void node_normal(yo_cloth *c, int u, int v, double *nrm) {
  int ids[5] = {nid(c, u, v), nid(c, u - 1, v), nid(c, u + 1, v), nid(c, u, v - 1), nid(c, u, v + 1)};
  double mean[3] = {0, 0, 0}, S[3][3] = {{0}};
  for (int i = 0; i < 5; ++i)
    for (int k = 0; k < 3; ++k) mean[k] += c->x[3 * ids[i] + k];
  for (int k = 0; k < 3; ++k) mean[k] /= 5.0;
  for (int i = 0; i < 5; ++i) {
    double r[3];
    for (int k = 0; k < 3; ++k) r[k] = c->x[3 * ids[i] + k] - mean[k];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) S[a][b] += r[a] * r[b];
  }
  double n[3];
  sym3_min_eigvec(S, n);
  double nn = norm3(n);
  for (int k = 0; k < 3; ++k) n[k] /= nn;
  double vw[3], vf[3], cr[3];
  for (int k = 0; k < 3; ++k) {
    vw[k] = c->x[3 * ids[2] + k] - c->x[3 * ids[1] + k];
    vf[k] = c->x[3 * ids[4] + k] - c->x[3 * ids[3] + k];
  }
  cross3(vw, vf, cr);
  double cosv = dot3(cr, n) / (norm3(cr) * norm3(n));
  if (cosv < 0) for (int k = 0; k < 3; ++k) n[k] = -n[k];
  if (c->flip[ids[0]]) for (int k = 0; k < 3; ++k) n[k] = -n[k];
  memcpy(nrm, n, sizeof(n));
}

/* UpdateClothUnits (src/Cloth.cpp:307-348): normals and crimp offsets; the
 * element geometry itself is evaluated on demand from the node state. */
static void update_units(yo_cloth *c) {
  for (int n = 0; n < c->N; ++n) {
    memcpy(&c->xw[3 * n], &c->x[3 * n], sizeof(double) * 3);
    memcpy(&c->xf[3 * n], &c->x[3 * n], sizeof(double) * 3);
  }
  for (int u = 1; u < c->W - 1; ++u)
    for (int v = 1; v < c->H - 1; ++v) {
      int n = nid(c, u, v);
      node_normal(c, u, v, &c->nrm[3 * n]);
      for (int k = 0; k < 3; ++k) {
        c->xw[3 * n + k] = c->x[3 * n + k] - c->R * c->nrm[3 * n + k];
        c->xf[3 * n + k] = c->x[3 * n + k] + c->R * c->nrm[3 * n + k];
      }
    }
}

/* Edge geometry (src/ClothUnit.h:134-154). k = 0 warp, 1 weft. */
static void edge_geom(const yo_cloth *c, int n0, int n1, int k, int line, edge_t *e) {
  e->n0 = n0; e->n1 = n1; e->k = k; e->line = line;
  e->in0 = is_int(c, n0); e->in1 = is_int(c, n1);
  if (k == 0) { e->rho = c->rho_warp[line]; e->ks = c->ks_warp[line]; e->kb = c->kb_warp[line]; }
  else { e->rho = c->rho_weft[line]; e->ks = c->ks_weft[line]; e->kb = c->kb_weft[line]; }
  e->du = c->uv[2 * n1 + k] - c->uv[2 * n0 + k];
  for (int i = 0; i < 3; ++i) e->dx[i] = c->x[3 * n1 + i] - c->x[3 * n0 + i];
  for (int i = 0; i < 3; ++i) e->w[i] = e->dx[i] / e->du;
  e->l = norm3(e->dx);
  for (int i = 0; i < 3; ++i) e->d[i] = e->dx[i] / e->l;
  proj(e->d, e->P);
  for (int i = 0; i < 3; ++i) { e->q[i] = c->v[3 * n0 + i]; e->q[4 + i] = c->v[3 * n1 + i]; }
  e->q[3] = c->uvdot[2 * n0 + k];
  e->q[7] = c->uvdot[2 * n1 + k];
}

/* Bend segment geometry (src/ClothUnit.h:197-210). pos = node positions to
 * use (real nodes or crimp-offset nodes), uvsrc = EPos source. */
static void bend_geom(const yo_cloth *c, const double *pos, const double *uvsrc, int n2, int n0, int n1,
                      int k, double kb, bend_t *b) {
  b->n2 = n2; b->n0 = n0; b->n1 = n1; b->k = k; b->kb = kb;
  b->in2 = is_int(c, n2); b->in0 = is_int(c, n0); b->in1 = is_int(c, n1);
  b->du = uvsrc[2 * n1 + k] - uvsrc[2 * n2 + k];
  double a1[3], a2[3];
  for (int i = 0; i < 3; ++i) { a1[i] = pos[3 * n1 + i] - pos[3 * n0 + i]; a2[i] = pos[3 * n2 + i] - pos[3 * n0 + i]; }
  b->l1 = norm3(a1); b->l2 = norm3(a2);
  for (int i = 0; i < 3; ++i) { b->d1[i] = a1[i] / b->l1; b->d2[i] = a2[i] / b->l2; }
  proj(b->d1, b->P1); proj(b->d2, b->P2);
  double cth = -dot3(b->d1, b->d2);
  const double lo = -1.0 + DBL_MIN, hi = 1.0 - DBL_MIN;
  if (cth < lo) cth = lo;
  if (cth > hi) cth = hi;
  b->theta = acos(cth);
}

/* ------------------------------------------------------------------ */
/* 8x8 helpers for the edge kinetic-energy terms                       */
/* ------------------------------------------------------------------ */
typedef double m8[8][8];
/* B = [[z*I3, p], [q^T, s]] */
static void blk4(double B[4][4], double z, const double *p, const double *q, double s) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) B[i][j] = (i == j) ? z : 0.0;
    B[i][3] = p[i];
    B[3][i] = q[i];
  }
  B[3][3] = s;
}
/* out = scale * [[2B, B], [B, 2B]] */
static void big8(m8 out, double B[4][4], double scale) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      out[i][j] = scale * (2.0 * B[i][j]);
      out[i][j + 4] = scale * B[i][j];
      out[i + 4][j] = scale * B[i][j];
      out[i + 4][j + 4] = scale * (2.0 * B[i][j]);
    }
}
static void lin8(m8 out, double a, m8 A, double b, m8 B) {
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) out[i][j] = a * A[i][j] + b * B[i][j];
}
static void scal8(m8 out, double a, m8 A) {
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) out[i][j] = a * A[i][j];
}
/* 0.5 * q^T M q */
static double hquad8(m8 M, const double *q) {
  double s = 0.0;
  for (int j = 0; j < 8; ++j) {
    double r = 0.0;
    for (int i = 0; i < 8; ++i) r += q[i] * M[i][j];
    s += r * q[j];
  }
  return 0.5 * s;
}
static void mv8(m8 M, const double *q, double *o) {
  for (int i = 0; i < 8; ++i) {
    double s = 0.0;
    for (int j = 0; j < 8; ++j) s += M[i][j] * q[j];
    o[i] = s;
  }
}

/* Writes the 8x8 (force-DOF x derivative-DOF) edge Jacobian C into matrix X
 * with the sign s, following the write pattern shared by Inertia_D_Pos,
 * Inertia_D_Vel, MDotVDot_D_Pos and MDotVDot_D_Vel
 * (e.g. src/PhysicsCloth.cpp:1544-1600, 2226-2308, 2505-2577).
 * DOF order inside C: x0(0..2) uv0(3) x1(4..6) uv1(7). */
static void write_edge_jac(yo_cloth *c, double *X, const edge_t *e, m8 C, double s) {
  double L0L0[3][3], L0L1[3][3], L1L0[3][3], L1L1[3][3];
  double L0E0[3], L0E1[3], L1E0[3], L1E1[3], E0L0[3], E0L1[3], E1L0[3], E1L1[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      L0L0[i][j] = C[i][j]; L0L1[i][j] = C[i][4 + j];
      L1L0[i][j] = C[4 + i][j]; L1L1[i][j] = C[4 + i][4 + j];
    }
    L0E0[i] = C[i][3]; L0E1[i] = C[i][7]; L1E0[i] = C[4 + i][3]; L1E1[i] = C[4 + i][7];
    E0L0[i] = C[3][i]; E0L1[i] = C[3][4 + i]; E1L0[i] = C[7][i]; E1L1[i] = C[7][4 + i];
  }
  int n0 = e->n0, n1 = e->n1, k = e->k;
  add_LL(c, X, n0, n0, L0L0, s);
  add_LL(c, X, n0, n1, L0L1, s);
  add_LL(c, X, n1, n0, L1L0, s);
  add_LL(c, X, n1, n1, L1L1, s);
  if (e->in0) {
    add_EL(c, X, n0, n0, k, E0L0, s);
    add_LE(c, X, n0, n0, k, L0E0, s);
    add_EE(c, X, n0, n0, k, s * C[3][3]);
  }
  if (e->in1) {
    add_EL(c, X, n1, n1, k, E1L1, s);
    add_LE(c, X, n1, n1, k, L1E1, s);
    add_EE(c, X, n1, n1, k, s * C[7][7]);
  }
  if (e->in0 && e->in1) {
    add_LE(c, X, n1, n0, k, L1E0, s);
    add_LE(c, X, n0, n1, k, L0E1, s);
    add_EL(c, X, n1, n0, k, E0L1, s);
    add_EL(c, X, n0, n1, k, E1L0, s);
    add_EE(c, X, n0, n1, k, s * C[3][7]);
    add_EE(c, X, n1, n0, k, s * C[7][3]);
  }
}

/* ------------------------------------------------------------------ */
/* element terms                                                        */
/* ------------------------------------------------------------------ */

/* Mass (src/PhysicsCloth.cpp:250-338). */
static void t_mass(yo_cloth *c, const edge_t *e) {
  double coeff = (1.0 / 6.0) * e->rho * e->du;
  double I2[3][3] = {{0}}, I1[3][3] = {{0}};
  for (int i = 0; i < 3; ++i) { I2[i][i] = 2.0 * coeff; I1[i][i] = coeff; }
  double wTw = dot3(e->w, e->w);
  double LE2[3], LE1[3];
  for (int i = 0; i < 3; ++i) { LE2[i] = -2.0 * coeff * e->w[i]; LE1[i] = -1.0 * coeff * e->w[i]; }
  double EE2 = 2.0 * coeff * wTw, EE1 = 0.5 * EE2;
  int n0 = e->n0, n1 = e->n1, k = e->k;
  add_LL(c, c->Mv, n0, n0, I2, 1.0);
  add_LL(c, c->Mv, n1, n0, I1, 1.0);
  add_LL(c, c->Mv, n0, n1, I1, 1.0);
  add_LL(c, c->Mv, n1, n1, I2, 1.0);
  if (e->in0) { add_LE(c, c->Mv, n0, n0, k, LE2, 1.0); add_EL(c, c->Mv, n0, n0, k, LE2, 1.0); add_EE(c, c->Mv, n0, n0, k, EE2); }
  if (e->in1) { add_LE(c, c->Mv, n1, n1, k, LE2, 1.0); add_EL(c, c->Mv, n1, n1, k, LE2, 1.0); add_EE(c, c->Mv, n1, n1, k, EE2); }
  if (e->in0 && e->in1) {
    add_LE(c, c->Mv, n1, n0, k, LE1, 1.0);
    add_LE(c, c->Mv, n0, n1, k, LE1, 1.0);
    add_EL(c, c->Mv, n1, n0, k, LE1, 1.0);
    add_EL(c, c->Mv, n0, n1, k, LE1, 1.0);
    add_EE(c, c->Mv, n0, n1, k, EE1);
    add_EE(c, c->Mv, n1, n0, k, EE1);
  }
}

/* Gravity_F / Gravity_D (src/PhysicsCloth.cpp:340-425). */
static void t_gravity(yo_cloth *c, const edge_t *e) {
  int n0 = e->n0, n1 = e->n1, k = e->k;
  for (int i = 0; i < 3; ++i) {
    double g = 0.5 * e->rho * c->G[i] * e->du;
    c->F[3 * n0 + i] -= g;
    c->F[3 * n1 + i] -= g;
  }
  double sx[3];
  for (int i = 0; i < 3; ++i) sx[i] = c->x[3 * n0 + i] + c->x[3 * n1 + i];
  double gx = dot3(c->G, sx);
  if (e->in0) c->F[erow(c, n0) + k] -= (-0.5) * e->rho * gx;
  if (e->in1) c->F[erow(c, n1) + k] -= 0.5 * e->rho * gx;
  double g0[3], g1[3];
  for (int i = 0; i < 3; ++i) { g0[i] = 0.5 * e->rho * c->G[i]; g1[i] = -g0[i]; }
  if (e->in0) { add_EL(c, c->Kv, n0, n0, k, g0, 1.0); add_LE(c, c->Kv, n0, n0, k, g0, 1.0); }
  if (e->in1) { add_EL(c, c->Kv, n1, n1, k, g1, 1.0); add_LE(c, c->Kv, n1, n1, k, g1, 1.0); }
  if (e->in0 && e->in1) {
    add_LE(c, c->Kv, n1, n0, k, g0, 1.0); /* L1E0 */
    add_LE(c, c->Kv, n0, n1, k, g1, 1.0); /* L0E1 */
    add_EL(c, c->Kv, n1, n0, k, g0, 1.0); /* E0L1 */
    add_EL(c, c->Kv, n0, n1, k, g1, 1.0); /* E1L0 */
  }
}

/* Stretch_F / Stretch_D (src/PhysicsCloth.cpp:427-577); also the crimp
 * compression accumulators StrhBend_C_L / StrhBend_C_LE (self entries). */
static void t_stretch(yo_cloth *c, const edge_t *e) {
  int n0 = e->n0, n1 = e->n1, k = e->k;
  double nw = norm3(e->w);
  double sgn = (k == 0) ? 1.0 : -1.0;
  for (int i = 0; i < 3; ++i) {
    double f = e->ks * (nw - 1) * e->d[i];
    c->F[3 * n0 + i] += f;
    c->F[3 * n1 + i] -= f;
    c->CL[3 * n0 + i] += sgn * f;
    c->CL[3 * n1 + i] -= sgn * f;
  }
  double fe = 0.5 * e->ks * (nw * nw - 1);
  if (e->in0) c->F[erow(c, n0) + k] -= fe;
  if (e->in1) c->F[erow(c, n1) + k] += fe;

  double LL[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) LL[i][j] = (e->ks / e->l) * e->P[i][j] - (e->ks / e->du) * (i == j ? 1.0 : 0.0);
  double EE = -e->ks * ((nw * nw) / e->du);
  double LE[3], ELr[3];
  for (int i = 0; i < 3; ++i) { LE[i] = e->ks * (nw / e->du) * e->d[i]; ELr[i] = e->ks / e->du * e->w[i]; }
  add_LL(c, c->Kv, n0, n0, LL, 1.0);
  add_LL(c, c->Kv, n1, n0, LL, -1.0);
  add_LL(c, c->Kv, n0, n1, LL, -1.0);
  add_LL(c, c->Kv, n1, n1, LL, 1.0);
  if (e->in0) {
    add_LE(c, c->Kv, n0, n0, k, LE, 1.0);
    add_EL(c, c->Kv, n0, n0, k, ELr, 1.0);
    add_EE(c, c->Kv, n0, n0, k, EE);
    for (int i = 0; i < 3; ++i) c->CLE[6 * eidx(c, n0) + 3 * k + i] += sgn * LE[i];
  }
  if (e->in1) {
    add_LE(c, c->Kv, n1, n1, k, LE, 1.0);
    add_EL(c, c->Kv, n1, n1, k, ELr, 1.0);
    add_EE(c, c->Kv, n1, n1, k, EE);
    for (int i = 0; i < 3; ++i) c->CLE[6 * eidx(c, n1) + 3 * k + i] += sgn * LE[i];
  }
  if (e->in0 && e->in1) {
    add_LE(c, c->Kv, n1, n0, k, LE, -1.0);
    add_LE(c, c->Kv, n0, n1, k, LE, -1.0);
    add_EL(c, c->Kv, n1, n0, k, ELr, -1.0);
    add_EL(c, c->Kv, n0, n1, k, ELr, -1.0);
    add_EE(c, c->Kv, n0, n1, k, -EE);
    add_EE(c, c->Kv, n1, n0, k, -EE);
  }
}

/* ParaColli_F / ParaColli_D (src/PhysicsCloth.cpp:989-1069). */
static void t_paracolli(yo_cloth *c, const edge_t *e) {
  int n0 = e->n0, n1 = e->n1, k = e->k;
  double d = (c->flip[n0] != c->flip[n1]) ? 4.0 * c->R : 2.0 * c->R;
  double rl = d - e->du;
  if (rl < 0) rl = 0.0;
  double fu0 = c->kc * c->L * rl;
  if (e->in0) c->F[erow(c, n0) + k] += fu0;
  if (e->in1) c->F[erow(c, n1) + k] += -fu0;
  double ee = -c->kc * c->L * rl;
  if (e->in0) add_EE(c, c->Kv, n0, n0, k, ee);
  if (e->in1) add_EE(c, c->Kv, n1, n1, k, ee);
  if (e->in0 && e->in1) { add_EE(c, c->Kv, n0, n1, k, ee); add_EE(c, c->Kv, n1, n0, k, ee); }
}

/* mass-matrix derivative building blocks shared by the inertia terms:
 * M_matrix (unscaled), M_x0_j blocks (src/PhysicsCloth.cpp:1076-1105). */
static void mass_matrix_unscaled(const edge_t *e, m8 Mm) {
  double B[4][4], mw[3];
  for (int i = 0; i < 3; ++i) mw[i] = -1.0 * e->w[i];
  blk4(B, 1.0, mw, mw, dot3(e->w, e->w));
  big8(Mm, B, 1.0);
}
static void mx0_block_unscaled(const edge_t *e, int j, m8 out) {
  /* w_x0 = (-1/du) I, column j; wTw_x0 = (-2/(du*du)) (x1 - x0), entry j */
  double col[3] = {0, 0, 0}, B[4][4];
  col[j] = -(-1.0 / e->du);
  double wtw_j = (-2.0 / (e->du * e->du) * e->dx[j]);
  blk4(B, 0.0, col, col, wtw_j);
  big8(out, B, 1.0);
}

/* Inertia_F (src/PhysicsCloth.cpp:1071-1186). */
static void t_inertia_F(yo_cloth *c, const edge_t *e) {
  double sc = 1.0 / 6.0 * e->rho * e->du;
  m8 Mm, T, Mx, Muv0, Bb;
  mass_matrix_unscaled(e, Mm);
  double T0[3], T1[3];
  for (int j = 0; j < 3; ++j) {
    mx0_block_unscaled(e, j, T);
    scal8(Mx, sc, T);
    T0[j] = hquad8(Mx, e->q);
    scal8(Mx, -1.0, Mx);
    T1[j] = hquad8(Mx, e->q);
  }
  double B[4][4], p[3];
  double wTw = dot3(e->w, e->w);
  for (int i = 0; i < 3; ++i) p[i] = (-1.0 / e->du) * e->w[i];
  blk4(B, 0.0, p, p, (2.0 / e->du) * wTw);
  big8(Bb, B, 1.0);
  lin8(Muv0, -(1.0 / 6.0) * e->rho, Mm, (1.0 / 6.0) * e->rho * e->du, Bb);
  double Tuv0 = hquad8(Muv0, e->q);
  scal8(Muv0, -1.0, Muv0);
  double Tuv1 = hquad8(Muv0, e->q);
  for (int i = 0; i < 3; ++i) { c->F[3 * e->n0 + i] += T0[i]; c->F[3 * e->n1 + i] += T1[i]; }
  if (e->in0) c->F[erow(c, e->n0) + e->k] += Tuv0;
  if (e->in1) c->F[erow(c, e->n1) + e->k] += Tuv1;
}

/* Inertia_D_Pos (src/PhysicsCloth.cpp:1188-1601). */
static void t_inertia_Dpos(yo_cloth *c, const edge_t *e) {
  const double rho = e->rho, du = e->du;
  m8 C, A, Bm, Mx0[3], Mx0uv0[3], tmp;
  memset(C, 0, sizeof(C));
  for (int j = 0; j < 3; ++j) mx0_block_unscaled(e, j, Mx0[j]);
  /* second derivative w.r.t. x0_j x0_j: only the uv-uv corner 2/(du*du) */
  {
    double B[4][4], z[3] = {0, 0, 0};
    blk4(B, 0.0, z, z, 2 / (du * du));
    big8(A, B, (1.0 / 6.0) * rho);
  }
  double T00 = hquad8(A, e->q);
  scal8(tmp, -1.0, A);
  double T01 = hquad8(tmp, e->q);       /* M_x0_1_x1_1 = -M_x0_1_x0_1 */
  double T10 = hquad8(tmp, e->q);       /* M_x1_1_x0_1 = -M_x0_1_x0_1 */
  scal8(tmp, -1.0, tmp);
  double T11 = hquad8(tmp, e->q);       /* M_x1_1_x1_1 = -M_x1_1_x0_1 */
  for (int i = 0; i < 3; ++i) {
    C[i][i] = T00; C[i][4 + i] = T01; C[4 + i][i] = T10; C[4 + i][4 + i] = T11;
  }
  /* mixed x / uv blocks; the bottom-left entry carries -(-w)^T (sign kept as
   * written at src/PhysicsCloth.cpp:1357-1361) */
  const double wTw = dot3(e->w, e->w);
  for (int j = 0; j < 3; ++j) {
    double top[3] = {0, 0, 0}, bot[3] = {0, 0, 0}, B[4][4];
    double wx0uv0_j = (1.0 / (du * du)); /* w_x0_uv_0 = (1/du^2) I */
    top[j] = -wx0uv0_j;
    bot[j] = -(-wx0uv0_j);
    blk4(B, 0.0, top, bot, (-4.0 / (du * du)) * e->w[j]);
    big8(Mx0uv0[j], B, 1.0);
  }
  double Tx0uv0[3], Tx0uv1[3], Tx1uv0[3], Tx1uv1[3], Tuv0x0[3], Tuv0x1[3], Tuv1x0[3], Tuv1x1[3];
  for (int j = 0; j < 3; ++j) {
    m8 M;
    lin8(M, (-1.0 / 6.0) * rho, Mx0[j], (1.0 / 6.0) * rho * du, Mx0uv0[j]); /* M_x0_j_uv_0 */
    Tx0uv0[j] = hquad8(M, e->q);
    scal8(tmp, -1.0, M);
    Tx0uv1[j] = hquad8(tmp, e->q); /* M_x0_j_uv_1 = -M_x0_j_uv_0 */
    Tx1uv0[j] = hquad8(tmp, e->q); /* M_x1_j_uv_0 = -M_x0_j_uv_0 */
    scal8(tmp, -1.0, tmp);
    Tx1uv1[j] = hquad8(tmp, e->q); /* M_x1_j_uv_1 = -M_x1_j_uv_0 */
    m8 Mneg;
    scal8(Mneg, -1.0, Mx0uv0[j]);
    lin8(M, (-1.0 / 6.0) * rho, Mx0[j], (1.0 / 6.0) * rho * du, Mneg); /* M_uv_0_x0_j */
    Tuv0x0[j] = hquad8(M, e->q);
    scal8(tmp, -1.0, M);
    Tuv0x1[j] = hquad8(tmp, e->q); /* M_uv_0_x1_j = -M_uv_0_x0_j */
    Tuv1x0[j] = hquad8(tmp, e->q); /* M_uv_1_x0_j = -M_uv_0_x0_j */
    scal8(tmp, -1.0, tmp);
    Tuv1x1[j] = hquad8(tmp, e->q); /* M_uv_1_x1_j = -M_uv_1_x0_j */
  }
  /* uv-uv */
  {
    double B[4][4], p[3], mw2[3];
    for (int i = 0; i < 3; ++i) p[i] = (-1.0 / du) * e->w[i];
    blk4(B, 0.0, p, p, (2.0 / du) * wTw);
    big8(A, B, 1.0); /* M_matrix_uv_0 */
    for (int i = 0; i < 3; ++i) mw2[i] = -((2 / (du * du)) * e->w[i]);
    blk4(B, 0.0, mw2, mw2, (6 / (du * du)) * wTw);
    big8(Bm, B, 1.0); /* M_matrix_uv_0_uv_0 */
  }
  m8 Muu;
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j)
      Muu[i][j] = (-1.0 / 6.0) * rho * A[i][j] - (1.0 / 6.0) * rho * A[i][j] + (1.0 / 6.0) * rho * du * Bm[i][j];
  double Tuu = hquad8(Muu, e->q);
  scal8(tmp, -1.0, Muu);
  double Tu01 = hquad8(tmp, e->q), Tu10 = hquad8(tmp, e->q);
  scal8(tmp, -1.0, tmp);
  double Tu11 = hquad8(tmp, e->q);
  for (int j = 0; j < 3; ++j) {
    C[j][3] = Tx0uv0[j]; C[j][7] = Tx0uv1[j]; C[4 + j][3] = Tx1uv0[j]; C[4 + j][7] = Tx1uv1[j];
    C[3][j] = Tuv0x0[j]; C[3][4 + j] = Tuv0x1[j]; C[7][j] = Tuv1x0[j]; C[7][4 + j] = Tuv1x1[j];
  }
  C[3][3] = Tuu; C[3][7] = Tu01; C[7][3] = Tu10; C[7][7] = Tu11;
  write_edge_jac(c, c->Kv, e, C, 1.0);
}

/* Inertia_D_Vel (src/PhysicsCloth.cpp:1602-1901): row j of block (x_j, X) is
 * (M_xj qdot)_X. */
static void t_inertia_Dvel(yo_cloth *c, const edge_t *e) {
  double sc = (1.0 / 6.0) * e->rho * e->du;
  m8 Mm, T, M, C, Bb;
  mass_matrix_unscaled(e, Mm);
  double r[8];
  for (int j = 0; j < 3; ++j) {
    mx0_block_unscaled(e, j, T);
    scal8(M, sc, T);
    mv8(M, e->q, r);
    for (int a = 0; a < 8; ++a) C[j][a] = r[a];
    scal8(M, -1.0, M);
    mv8(M, e->q, r);
    for (int a = 0; a < 8; ++a) C[4 + j][a] = r[a];
  }
  double B[4][4], p[3];
  for (int i = 0; i < 3; ++i) p[i] = (-1.0 / e->du) * e->w[i];
  blk4(B, 0.0, p, p, (2.0 / e->du) * dot3(e->w, e->w));
  big8(Bb, B, 1.0);
  lin8(M, -(1.0 / 6.0) * e->rho, Mm, (1.0 / 6.0) * e->rho * e->du, Bb);
  mv8(M, e->q, r);
  for (int a = 0; a < 8; ++a) C[3][a] = r[a];
  scal8(M, -1.0, M);
  mv8(M, e->q, r);
  for (int a = 0; a < 8; ++a) C[7][a] = r[a];
  write_edge_jac(c, c->Dv, e, C, 1.0);
}

/* M_dot (src/PhysicsCloth.cpp:1916-1932): common to the MDotVDot terms. */
static void mdot_matrix(const edge_t *e, double dud, double *wdot, m8 Mdot) {
  m8 Mm, Bb;
  mass_matrix_unscaled(e, Mm);
  for (int i = 0; i < 3; ++i)
    wdot[i] = (e->q[4 + i] - e->q[i]) * e->du - e->dx[i] * dud;
  for (int i = 0; i < 3; ++i) wdot[i] /= (e->du * e->du);
  double wTwd = dot3(e->w, wdot) + dot3(wdot, e->w);
  double B[4][4], mwd[3];
  for (int i = 0; i < 3; ++i) mwd[i] = -wdot[i];
  blk4(B, 0.0, mwd, mwd, wTwd);
  big8(Bb, B, 1.0);
  lin8(Mdot, (1.0 / 6.0) * e->rho * dud, Mm, (1.0 / 6.0) * e->rho * e->du, Bb);
}

/* MDotVDot_F (src/PhysicsCloth.cpp:1903-1961). */
static void t_mdot_F(yo_cloth *c, const edge_t *e) {
  double dud = e->q[7] - e->q[3], wdot[3], r[8];
  m8 Mdot;
  mdot_matrix(e, dud, wdot, Mdot);
  mv8(Mdot, e->q, r);
  for (int i = 0; i < 3; ++i) { c->F[3 * e->n0 + i] -= r[i]; c->F[3 * e->n1 + i] -= r[4 + i]; }
  if (e->in0) c->F[erow(c, e->n0) + e->k] -= r[3];
  if (e->in1) c->F[erow(c, e->n1) + e->k] -= r[7];
}

/* MDotVDot_D_Pos (src/PhysicsCloth.cpp:1963-2309); ADDED into dF/dx. */
static void t_mdot_Dpos(yo_cloth *c, const edge_t *e) {
  const double rho = e->rho, du = e->du, dud = e->q[7] - e->q[3];
  double wdot[3], r[8];
  m8 Mdot, C, Mx, Mdx, M;
  mdot_matrix(e, dud, wdot, Mdot);
  for (int side = 0; side < 2; ++side) {
    double sw = side == 0 ? -1.0 : 1.0; /* w_x0 = (-1/du) I, w_x1 = (1/du) I */
    for (int j = 0; j < 3; ++j) {
      double B[4][4], top[3] = {0, 0, 0};
      double wxj = sw * (1.0 / du);
      top[j] = -wxj;
      double wtwx = (sw * 2.0 / (du * du) * e->dx[j]);
      blk4(B, 0.0, top, top, wtwx);
      big8(Mx, B, 1.0);
      double wdxj = side == 0 ? (dud / (du * du)) : -(dud / (du * du));
      double wtwdx = 2 * (wxj * wdot[j]) + 2 * (e->w[j] * wdxj);
      double top2[3] = {0, 0, 0};
      top2[j] = -wdxj;
      blk4(B, 0.0, top2, top2, wtwdx);
      big8(Mdx, B, 1.0);
      lin8(M, (1.0 / 6.0) * rho * dud, Mx, (1.0 / 6.0) * rho * du, Mdx);
      mv8(M, e->q, r);
      for (int a = 0; a < 8; ++a) C[a][4 * side + j] = r[a];
    }
    /* uv derivative column */
    double wuv[3], wduv[3], B[4][4], mwduv[3];
    double s2 = side == 0 ? -1.0 : 1.0;
    for (int i = 0; i < 3; ++i) wuv[i] = s2 * e->w[i] / du;
    double wTwuv = s2 * (2 / du) * dot3(e->w, e->w);
    for (int i = 0; i < 3; ++i)
      wduv[i] = (e->q[4 + i] - e->q[i]) / (du * du) - (4 * e->dx[i] * dud) / (du * du * du);
    if (side == 1) for (int i = 0; i < 3; ++i) wduv[i] = -wduv[i];
    double wTwduv = 2 * dot3(wuv, wdot) + 2 * dot3(wduv, e->w);
    blk4(B, 0.0, wuv, wuv, wTwuv); /* no negation here (src/PhysicsCloth.cpp:2159-2161) */
    big8(Mx, B, 1.0);
    for (int i = 0; i < 3; ++i) mwduv[i] = -wduv[i];
    blk4(B, 0.0, mwduv, mwduv, wTwduv);
    big8(Mdx, B, 1.0);
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b)
        M[a][b] = (1.0 / 6.0) * rho * dud * Mx[a][b] - (1.0 / 6.0) * rho * Mdot[a][b] +
                  (1.0 / 6.0) * rho * du * Mdx[a][b];
    mv8(M, e->q, r);
    for (int a = 0; a < 8; ++a) C[a][4 * side + 3] = r[a];
  }
  write_edge_jac(c, c->Kv, e, C, 1.0);
}

/* MDotVDot_D_Vel (src/PhysicsCloth.cpp:2310-2577); SUBTRACTED from dF/dv. */
static void t_mdot_Dvel(yo_cloth *c, const edge_t *e) {
  const double rho = e->rho, du = e->du, dud = e->q[7] - e->q[3];
  double wdot[3], r[8];
  m8 Mdot, Mm, C, Md, M;
  mdot_matrix(e, dud, wdot, Mdot);
  mass_matrix_unscaled(e, Mm);
  for (int side = 0; side < 2; ++side) {
    double sw = side == 0 ? -1.0 : 1.0;
    for (int j = 0; j < 3; ++j) {
      double B[4][4], top[3] = {0, 0, 0};
      double wdj = sw * (1.0 / du);         /* w_dot_x{0,1}_dot */
      double wtw = 2 * (e->w[j] * wdj);     /* 2 w^T w_dot_x_dot_j */
      top[j] = -wdj;
      blk4(B, 0.0, top, top, wtw);
      big8(Md, B, 1.0);
      mv8(Md, e->q, r);
      double mcol[8];
      for (int a = 0; a < 8; ++a) mcol[a] = Mdot[a][4 * side + j];
      for (int a = 0; a < 8; ++a) C[a][4 * side + j] = (1.0 / 6.0) * rho * du * r[a] + mcol[a];
    }
    double wd[3], B[4][4], mwd[3];
    for (int i = 0; i < 3; ++i) wd[i] = (side == 0 ? (1.0 / du) : (-1.0 / du)) * e->w[i];
    double wtwd = 2 * dot3(e->w, wd);
    for (int i = 0; i < 3; ++i) mwd[i] = -wd[i];
    blk4(B, 0.0, mwd, mwd, wtwd);
    big8(Md, B, 1.0);
    lin8(M, (side == 0 ? -1.0 : 1.0) * (1.0 / 6.0) * rho, Mm, (1.0 / 6.0) * rho * du, Md);
    mv8(M, e->q, r);
    for (int a = 0; a < 8; ++a) C[a][4 * side + 3] = r[a] + Mdot[a][4 * side + 3];
  }
  write_edge_jac(c, c->Dv, e, C, -1.0);
}

/* Bending_F / Bending_D (src/PhysicsCloth.cpp:579-822) on real nodes. */
static void bend_terms(const bend_t *b, double Fx1[3], double Fx2[3], double L11[3][3], double L12[3][3],
                       double L21[3][3], double L22[3][3], double L1E1[3], double L2E1[3], double E1L1[3],
                       double E1L2[3]) {
  memset(Fx1, 0, 3 * sizeof(double)); memset(Fx2, 0, 3 * sizeof(double));
  memset(L11, 0, 9 * sizeof(double)); memset(L12, 0, 9 * sizeof(double));
  memset(L21, 0, 9 * sizeof(double)); memset(L22, 0, 9 * sizeof(double));
  memset(L1E1, 0, 3 * sizeof(double)); memset(L2E1, 0, 3 * sizeof(double));
  memset(E1L1, 0, 3 * sizeof(double)); memset(E1L2, 0, 3 * sizeof(double));
  double th = b->theta, s = sin(th);
  if (s == 0) return;
  double co = cos(th), kb = b->kb, du = b->du;
  double a[3], bb[3];
  mv3((double (*)[3])b->P1, b->d2, a);
  mv3((double (*)[3])b->P2, b->d1, bb);
  double c1 = (-2 * kb * th) / (b->l1 * du * s), c2 = (-2 * kb * th) / (b->l2 * du * s);
  for (int i = 0; i < 3; ++i) { Fx1[i] = c1 * a[i]; Fx2[i] = c2 * bb[i]; }
  double k11 = (2 * kb) / ((b->l1 * b->l1) * du * s), k12 = (-2 * kb) / (b->l1 * b->l2 * du * s);
  double k22 = (2 * kb) / ((b->l2 * b->l2) * du * s);
  double cs2 = co / (s * s), is = 1 / s;
  double ad1[3][3], aa[3][3], d1a[3][3], bd2[3][3], bbo[3][3], d2b[3][3], T[3][3];
  outer3(a, b->d1, ad1); outer3(a, a, aa); outer3(b->d1, a, d1a);
  outer3(bb, b->d2, bd2); outer3(bb, bb, bbo); outer3(b->d2, bb, d2b);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      L11[i][j] = k11 * (th * (ad1[i][j] + cs2 * aa[i][j] + co * b->P1[i][j] + d1a[i][j]) - is * aa[i][j]);
      L22[i][j] = k22 * (th * (bd2[i][j] + cs2 * bbo[i][j] + co * b->P2[i][j] + d2b[i][j]) - is * bbo[i][j]);
      T[i][j] = th * (b->P1[i][j] - cs2 * ad1[i][j]) + is * ad1[i][j];
    }
  mm3(T, (double (*)[3])b->P2, L12);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) L12[i][j] *= k12;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T[i][j] = th * (b->P2[i][j] - cs2 * bd2[i][j]) + is * bd2[i][j];
  mm3(T, (double (*)[3])b->P1, L21);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) L21[i][j] *= k12;
  double e1 = (2 * kb * th) / (b->l1 * (du * du) * s), e2 = (2 * kb * th) / (b->l2 * (du * du) * s);
  for (int i = 0; i < 3; ++i) { L1E1[i] = e1 * a[i]; L2E1[i] = e2 * bb[i]; E1L1[i] = e1 * a[i]; E1L2[i] = e2 * bb[i]; }
}

static void t_bend(yo_cloth *c, const bend_t *b) {
  double Fx1[3], Fx2[3], L11[3][3], L12[3][3], L21[3][3], L22[3][3], L1E1[3], L2E1[3], E1L1[3], E1L2[3];
  bend_terms(b, Fx1, Fx2, L11, L12, L21, L22, L1E1, L2E1, E1L1, E1L2);
  int n2 = b->n2, n0 = b->n0, n1 = b->n1, k = b->k;
  double du = b->du, th = b->theta;
  double Fu2 = (-b->kb * th) / (du * du), Fu1 = -1 * Fu2;
  for (int i = 0; i < 3; ++i) {
    double Fx0 = -(Fx1[i] + Fx2[i]);
    c->F[3 * n2 + i] += Fx2[i];
    c->F[3 * n0 + i] += Fx0;
    c->F[3 * n1 + i] += Fx1[i];
  }
  if (b->in2) c->F[erow(c, n2) + k] += Fu2;
  if (b->in0) c->F[erow(c, n0) + k] += 0.0;
  if (b->in1) c->F[erow(c, n1) + k] += Fu1;

  double L10[3][3], L20[3][3], L01[3][3], L02[3][3], L00[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      L10[i][j] = -(L11[i][j] + L12[i][j]);
      L20[i][j] = -(L21[i][j] + L22[i][j]);
      L01[i][j] = -(L11[i][j] + L21[i][j]);
      L02[i][j] = -(L12[i][j] + L22[i][j]);
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) L00[i][j] = -(L10[i][j] + L20[i][j]);
  double E1E1 = (-2 * b->kb * (th * th)) / (du * du * du);
  double L2E2[3], L0E1[3], L0E2[3], E2L2[3], E1L0[3], E2L0[3];
  for (int i = 0; i < 3; ++i) {
    L2E2[i] = -L2E1[i];
    L0E1[i] = -(L1E1[i] + L2E1[i]);
    L0E2[i] = -L0E1[i];
    E2L2[i] = -E1L2[i];
    E1L0[i] = -(E1L1[i] + E1L2[i]);
    E2L0[i] = -E1L0[i];
  }
  add_LL(c, c->Kv, n2, n2, L22, 1.0);
  add_LL(c, c->Kv, n2, n0, L20, 1.0);
  add_LL(c, c->Kv, n2, n1, L21, 1.0);
  add_LL(c, c->Kv, n0, n2, L02, 1.0);
  add_LL(c, c->Kv, n0, n0, L00, 1.0);
  add_LL(c, c->Kv, n0, n1, L01, 1.0);
  add_LL(c, c->Kv, n1, n2, L12, 1.0);
  add_LL(c, c->Kv, n1, n0, L10, 1.0);
  add_LL(c, c->Kv, n1, n1, L11, 1.0);
  if (b->in2) { add_LE(c, c->Kv, n2, n2, k, L2E2, 1.0); add_EL(c, c->Kv, n2, n2, k, E2L2, 1.0); add_EE(c, c->Kv, n2, n2, k, E1E1); }
  if (b->in1) { add_LE(c, c->Kv, n1, n1, k, L1E1, 1.0); add_EL(c, c->Kv, n1, n1, k, E1L1, 1.0); add_EE(c, c->Kv, n1, n1, k, E1E1); }
  if (b->in2 && b->in0) {
    add_LE(c, c->Kv, n0, n2, k, L0E2, 1.0); /* F_LE_Pos[find_index(n0,n2)] */
    add_EL(c, c->Kv, n2, n0, k, E2L0, 1.0); /* F_EL_Pos[find_index(n2,n0)] */
  }
  if (b->in0 && b->in1) {
    add_LE(c, c->Kv, n0, n1, k, L0E1, 1.0);
    add_EL(c, c->Kv, n0, n1, k, E1L0, 1.0);
  }
}

/* Crimp_Bending_F / Crimp_Bending_D (src/PhysicsCloth.cpp:824-987): only the
 * compression accumulators; only the self E-L entries are ever read. */
static void t_crimp(yo_cloth *c, const bend_t *b) {
  double Fx1[3], Fx2[3], L11[3][3], L12[3][3], L21[3][3], L22[3][3], L1E1[3], L2E1[3], E1L1[3], E1L2[3];
  bend_terms(b, Fx1, Fx2, L11, L12, L21, L22, L1E1, L2E1, E1L1, E1L2);
  double sgn = (b->k == 0) ? 1.0 : -1.0;
  for (int i = 0; i < 3; ++i) {
    double Fx0 = -(Fx1[i] + Fx2[i]);
    c->CL[3 * b->n2 + i] += sgn * Fx2[i];
    c->CL[3 * b->n0 + i] += sgn * Fx0;
    c->CL[3 * b->n1 + i] += sgn * Fx1[i];
  }
  if (b->in2)
    for (int i = 0; i < 3; ++i) c->CLE[6 * eidx(c, b->n2) + 3 * b->k + i] += sgn * (-L2E1[i]);
  if (b->in1)
    for (int i = 0; i < 3; ++i) c->CLE[6 * eidx(c, b->n1) + 3 * b->k + i] += sgn * L1E1[i];
}

/* Wind_F (src/PhysicsCloth.cpp:3091-3107). */
static void t_wind(yo_cloth *c, int n1, int n2, int n3) {
  double e1[3], e2[3], cr[3], n[3];
  for (int i = 0; i < 3; ++i) { e1[i] = c->x[3 * n2 + i] - c->x[3 * n1 + i]; e2[i] = c->x[3 * n3 + i] - c->x[3 * n1 + i]; }
  cross3(e1, e2, cr);
  double nc = norm3(cr);
  double area = 0.5 * nc; /* src/ClothUnit.h:268-273 */
  for (int i = 0; i < 3; ++i) n[i] = (nc == 0.0) ? cr[i] : cr[i] / nc;
  double fv[3], rel[3];
  for (int i = 0; i < 3; ++i) { fv[i] = (c->v[3 * n1 + i] + c->v[3 * n2 + i] + c->v[3 * n3 + i]) / 3.0; rel[i] = c->wind_v[i] - fv[i]; }
  double vn = dot3(n, rel);
  for (int i = 0; i < 3; ++i) {
    double tang = rel[i] - vn * n[i];
    double f = c->wind_rho * area * fabs(vn) * vn * n[i] + c->wind_drag * area * tang;
    c->F[3 * n1 + i] += f / 3.0;
    c->F[3 * n2 + i] += f / 3.0;
    c->F[3 * n3 + i] += f / 3.0;
  }
}

/* ConSlideFriction (src/PhysicsCloth.cpp:2579-2641). Runs after all edge and
 * bend terms; reads this node's no-slide force and EE diagonals. */
static void t_friction(yo_cloth *c, int n) {
  int fe = eidx(c, n), er = erow(c, n);
  double uvm[2] = {c->uv[2 * n] - c->uvbar[2 * n], c->uv[2 * n + 1] - c->uvbar[2 * n + 1]};
  double EEp[2] = {*at(c, c->Kv, er, er), *at(c, c->Kv, er + 1, er + 1)};
  double EEv[2] = {*at(c, c->Dv, er, er), *at(c, c->Dv, er + 1, er + 1)};
  double FEns[2] = {c->F[er], c->F[er + 1]};
  const double *nn = &c->nrm[3 * n];
  double comp = 0.5 * dot3(nn, &c->CL[3 * n]);
  if (comp < 0) comp = 0.0;
  double compEE[2] = {0.5 * dot3(nn, &c->CLE[6 * fe]), 0.5 * dot3(nn, &c->CLE[6 * fe + 3])};
  c->comp[n] = comp;
  const double mu = c->mu, kf = c->kf, df = c->df;
  double lim = 1.0 * comp * mu;
  for (int k = 0; k < 2; ++k) {
    double slide = 1.0 / (1.0 + exp(-(1e4 * (fabs(FEns[k]) - lim))));
    double t = tanh(10 * uvm[k]);
    double tl = tanh(10 * (lim - FEns[k]));
    double force = (-0.5 * (kf * uvm[k] - t * comp * mu) * tl + 0.5 * (kf * uvm[k] + t * comp * mu)) - df * c->uvdot[2 * n + k];
    double pos = (-0.5 * (kf - (1.0 - t * t) * mu * comp - t * mu * compEE[k])) * tl -
                 (0.5 * (kf * uvm[k] - t * mu * comp)) * (1.0 - tl * tl) * (EEp[k] - mu * compEE[k]) -
                 (0.5 * (kf + (1.0 - t * t) * mu * comp + t * mu * compEE[k]));
    double tq = tanh(10 * lim - FEns[k]);
    double vel = (-0.5 * (kf * uvm[k] - t * mu * comp)) * (1.0 - tq * tq) * EEv[k] - df;
    c->slide[2 * fe + k] = slide;
    c->F[er + k] += force;
    *at(c, c->Kv, er + k, er + k) += pos;
    *at(c, c->Dv, er + k, er + k) += vel;
  }
}

/* Shear_F / Shear_D (src/PhysicsCloth.cpp:2643-3089). n0 = crossing node,
 * n1 = warp neighbour, n3 = weft neighbour. */
static void t_shear(yo_cloth *c, int n0, int n1, int n3) {
  const double Lc = c->L, R = c->R, S = c->S;
  const double comp = c->comp[n0];
  double a1v[3], a3v[3], d1[3], d3[3], P1[3][3], P3[3][3];
  for (int i = 0; i < 3; ++i) { a1v[i] = c->x[3 * n1 + i] - c->x[3 * n0 + i]; a3v[i] = c->x[3 * n3 + i] - c->x[3 * n0 + i]; }
  double l1 = norm3(a1v), l3 = norm3(a3v);
  for (int i = 0; i < 3; ++i) { d1[i] = a1v[i] / l1; d3[i] = a3v[i] / l3; }
  proj(d1, P1); proj(d3, P3);
  double phi = acos(dot3(d1, d3));
  double s = sin(phi), co = cos(phi);
  double a3[3], a1[3]; /* a3 = P1 d3, a1 = P3 d1 */
  mv3(P1, d3, a3); mv3(P3, d1, a1);
  int jam = (c->flip[n0] != c->flip[n1]) && (c->flip[n0] != c->flip[n3]);
  double Fx1[3], Fx3[3], J11[3][3], J13[3][3], J31[3][3], J33[3][3];
  double cs2 = co / (s * s), is = 1 / s;
  if (!jam) {
    double kx = (comp + 1.0) * S * R * R * YO_PI;
    double cf1 = (kx * Lc * (phi - YO_PI / 2)) / (l1 * s), cf3 = (kx * Lc * (phi - YO_PI / 2)) / (l3 * s);
    for (int i = 0; i < 3; ++i) { Fx1[i] = cf1 * a3[i]; Fx3[i] = cf3 * a1[i]; }
    double ph = phi - YO_PI / 2;
    double a3d1[3][3], a3a3[3][3], d1a3[3][3], a1d3[3][3], a1a1[3][3], d3a1[3][3], T[3][3];
    outer3(a3, d1, a3d1); outer3(a3, a3, a3a3); outer3(d1, a3, d1a3);
    outer3(a1, d3, a1d3); outer3(a1, a1, a1a1); outer3(d3, a1, d3a1);
    double k11 = (kx * Lc) / ((l1 * l1) * s), k33 = (kx * Lc) / ((l3 * l3) * s);
    double k13 = (kx * Lc) / (l3 * l1 * s), k31 = (kx * Lc) / (l1 * l3 * s);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        J11[i][j] = k11 * (ph * (-1 * a3d1[i][j] + cs2 * a3a3[i][j] - co * P1[i][j] - d1a3[i][j]) - is * a3a3[i][j]);
        J33[i][j] = k33 * (ph * (-1 * a1d3[i][j] + cs2 * a1a1[i][j] - co * P3[i][j] - d3a1[i][j]) - is * a1a1[i][j]);
        T[i][j] = ph * (cs2 * a3d1[i][j] - is * a3d1[i][j]);
      }
    mm3(T, P3, J13);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) { J13[i][j] *= k13; T[i][j] = ph * (cs2 * a1d3[i][j] - is * a1d3[i][j]); }
    mm3(T, P1, J31);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) J31[i][j] *= k31;
  } else {
    const double pb = YO_PI / 2, pl = c->jam, sig = 0.6;
    const int cc = 3;
    const double LR = Lc / R;
    double px1[3], px3[3];
    for (int i = 0; i < 3; ++i) { px1[i] = -a3[i] / (l1 * s); px3[i] = -a1[i] / (l3 * s); }
    double gamma = (Lc * sqrt(2.0) - 2 * Lc * sin(0.5 * phi)) / R;
    double gx1[3], gx3[3];
    for (int i = 0; i < 3; ++i) { gx1[i] = -LR * cos(0.5 * phi) * px1[i]; gx3[i] = -LR * cos(0.5 * phi) * px3[i]; }
    double A = phi - pl, Bq = phi - pb;
    double phs = phi * A * Bq;
    double phs1[3], phs3[3];
    for (int i = 0; i < 3; ++i) {
      phs1[i] = px1[i] * A * Bq + phi * px1[i] * Bq + phi * A * px1[i];
      phs3[i] = px3[i] * A * Bq + phi * px3[i] * Bq + phi * A * px3[i];
    }
    double pb5 = pow(pb, 5), pb4 = pow(pb, 4);
    double num = pb5 * A, den = phs * phs + pb4 * sig * sig;
    double cfx = num / den, cf = tanh(cfx);
    double num1[3], num3[3], den1[3], den3[3], cfx1n[3], cfx3n[3], cfx1[3], cfx3[3];
    double den2 = den * den;
    for (int i = 0; i < 3; ++i) {
      num1[i] = pb5 * px1[i]; num3[i] = pb5 * px3[i];
      den1[i] = 2 * phs * phs1[i]; den3[i] = 2 * phs * phs3[i];
      cfx1n[i] = num1[i] * den - num * den1[i];
      cfx3n[i] = num3[i] * den - num * den3[i];
      cfx1[i] = cfx1n[i] / den2;
      cfx3[i] = cfx3n[i] / den2;
    }
    double g3 = gamma * gamma * gamma, g2 = gamma * gamma, g1 = gamma;
    double base = 0.5 * (comp + 1.0) * S * YO_PI * (R * R);
    double kx = base * ((1 + g3) + (1 - g3) * cf);
    double kx1[3], kx3[3];
    for (int i = 0; i < 3; ++i) {
      kx1[i] = base * (cc * g2 * gx1[i] - cc * g2 * gx1[i] * cf + (1 - g3) * (1 - cf * cf * cfx1[i]));
      kx3[i] = base * (cc * g2 * gx3[i] - cc * g2 * gx3[i] * cf + (1 - g3) * (1 - cf * cf * cfx3[i]));
    }
    double Bq2 = Bq * Bq;
    double cf1 = (kx * Lc * Bq) / (l1 * s), cf3 = (kx * Lc * Bq) / (l3 * s);
    for (int i = 0; i < 3; ++i) {
      Fx1[i] = -0.5 * kx1[i] * Lc * Bq2 + cf1 * a3[i];
      Fx3[i] = -0.5 * kx3[i] * Lc * Bq2 + cf3 * a1[i];
    }
    /* second derivatives */
    double a3d1[3][3], d1a3[3][3], a3a3[3][3], a1d3[3][3], d3a1[3][3], a1a1[3][3], a3a1[3][3], a1a3[3][3];
    double P1P3[3][3], P3P1[3][3], P3d3o[3][3];
    outer3(a3, d1, a3d1); outer3(d1, a3, d1a3); outer3(a3, a3, a3a3);
    outer3(a1, d3, a1d3); outer3(d3, a1, d3a1); outer3(a1, a1, a1a1);
    outer3(a3, a1, a3a1); outer3(a1, a3, a1a3);
    mm3(P1, P3, P1P3); mm3(P3, P1, P3P1);
    { /* outer(P3 d1, d3) P3 as written (src/PhysicsCloth.cpp:2775-2777) */
      double o[3][3];
      outer3(a1, d3, o);
      mm3(o, P3, P3d3o);
    }
    double px11[3][3], px33[3][3], px13[3][3], px31[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        px11[i][j] = (a3d1[i][j] + d1a3[i][j] - (cs2 * a3a3[i][j]) + co * P1[i][j]) / ((l1 * l1) * s);
        px33[i][j] = (a1d3[i][j] + d3a1[i][j] - (cs2 * a1a1[i][j]) + co * P3[i][j]) / ((l3 * l3) * s);
        px13[i][j] = -(cs2 * a3a1[i][j] + P1P3[i][j]) / (l1 * l3 * s);
        px31[i][j] = -(cs2 * P3d3o[i][j] + P3P1[i][j]) / (l3 * l1 * s);
      }
    double sh = sin(0.5 * phi), ch = cos(0.5 * phi);
    double gx11[3][3], gx33[3][3], gx13[3][3], gx31[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        gx11[i][j] = (0.5 * LR * sh * a3a3[i][j]) / ((l1 * s) * (l1 * s)) - LR * ch * px11[i][j];
        gx33[i][j] = (0.5 * LR * sh * a1a1[i][j]) / ((l3 * s) * (l3 * s)) - LR * ch * px33[i][j];
        gx13[i][j] = (0.5 * LR * sh * a3a1[i][j]) / (l1 * l3 * (s * s)) - LR * ch * px13[i][j];
        gx31[i][j] = (0.5 * LR * sh * a1a3[i][j]) / (l3 * l1 * (s * s)) - LR * ch * px31[i][j];
      }
    double O11[3][3], O33[3][3], O13[3][3], O31[3][3];
    outer3(px1, px1, O11); outer3(px3, px3, O33); outer3(px1, px3, O13); outer3(px3, px1, O31);
    double ps11[3][3], ps33[3][3], ps13[3][3], ps31[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        ps11[i][j] = px11[i][j] * A * Bq + O11[i][j] * Bq + O11[i][j] * A + O11[i][j] * Bq + phi * px11[i][j] * Bq +
                     phi * O11[i][j] + O11[i][j] * A + phi * O11[i][j] + phi * A * px11[i][j];
        ps33[i][j] = px33[i][j] * A * Bq + O33[i][j] * Bq + O33[i][j] * A + O33[i][j] * Bq + phi * px33[i][j] * Bq +
                     phi * O33[i][j] + O33[i][j] * A + phi * O33[i][j] + phi * A * px33[i][j];
        ps13[i][j] = px13[i][j] * A * Bq + O13[i][j] * Bq + O13[i][j] * A + O31[i][j] * Bq + phi * px13[i][j] * Bq +
                     phi * O13[i][j] + O31[i][j] * A + phi * O31[i][j] + phi * A * px13[i][j];
        ps31[i][j] = px31[i][j] * A * Bq + O31[i][j] * Bq + O31[i][j] * A + O31[i][j] * Bq + phi * px31[i][j] * Bq +
                     phi * O31[i][j] + O31[i][j] * A + phi * O31[i][j] + phi * A * px31[i][j];
      }
    double cfx11[3][3], cfx33[3][3], cfx13[3][3], cfx31[3][3];
    {
      double Pp11[3][3], Pp33[3][3], Pn1s3[3][3], Pn3s1[3][3], Ps1s3[3][3], Ps3s1[3][3], Oc11[3][3], Oc33[3][3],
          Oc13[3][3], Oc31[3][3];
      outer3(phs1, phs1, Pp11); outer3(phs3, phs3, Pp33);
      outer3(num1, phs3, Pn1s3); outer3(num3, phs1, Pn3s1);
      outer3(phs1, phs3, Ps1s3); outer3(phs3, phs1, Ps3s1);
      double dd1[3], dd3[3];
      for (int i = 0; i < 3; ++i) { dd1[i] = 2 * den * den1[i]; dd3[i] = 2 * den * den3[i]; }
      outer3(cfx1n, dd1, Oc11); outer3(cfx3n, dd3, Oc33); outer3(cfx1n, dd3, Oc13); outer3(cfx3n, dd1, Oc31);
      double Pn3s1b[3][3], Pn1s3b[3][3];
      outer3(num3, phs1, Pn3s1b); /* outer(con_func_x_num_x3, phi_s_x1) */
      outer3(num1, phs3, Pn1s3b); /* outer(con_func_x_num_x1, phi_s_x3) */
      double den22 = den2 * den2;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double n11 = (pb5 * px11[i][j]) * den - 2 * num * Pp11[i][j] - 2 * num * phs * ps11[i][j];
          double n33 = (pb5 * px33[i][j]) * den - 2 * num * Pp33[i][j] - 2 * num * phs * ps33[i][j];
          double n13 = ((pb5 * px13[i][j]) * den + 2 * phs * Pn1s3[i][j] - 2 * phs * Pn3s1[i][j] -
                        2 * num * Ps1s3[i][j] - 2 * num * phs * ps13[i][j]);
          double n31 = ((pb5 * px31[i][j]) * den + 2 * phs * Pn3s1b[i][j] - 2 * phs * Pn1s3b[i][j] -
                        2 * num * Ps3s1[i][j] - 2 * num * phs * ps31[i][j]);
          cfx11[i][j] = (n11 * den2 - Oc11[i][j]) / den22;
          cfx33[i][j] = (n33 * den2 - Oc33[i][j]) / den22;
          cfx13[i][j] = (n13 * den2 - Oc13[i][j]) / den22;
          cfx31[i][j] = (n31 * den2 - Oc31[i][j]) / den22;
        }
    }
    double cfd1[3], cfd3[3];
    for (int i = 0; i < 3; ++i) { cfd1[i] = (1.0 - cf * cf) * cfx1[i]; cfd3[i] = (1.0 - cf * cf) * cfx3[i]; }
    double cf11[3][3], cf33[3][3], cf13[3][3], cf31[3][3];
    {
      double o11[3][3], o33[3][3], o31[3][3], o13[3][3];
      outer3(cfx1, cfx1, o11); outer3(cfx3, cfx3, o33); outer3(cfx3, cfx1, o31); outer3(cfx1, cfx3, o13);
      double q = -2 * cf * (1 - cf * cf);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          cf11[i][j] = q * o11[i][j] + (1 - cf * cf * cfx11[i][j]);
          cf33[i][j] = q * o33[i][j] + (1 - cf * cf * cfx33[i][j]);
          cf13[i][j] = q * o31[i][j] + (1 - cf * cf) * cfx13[i][j];
          cf31[i][j] = q * o13[i][j] + (1 - cf * cf) * cfx31[i][j];
        }
    }
    double kx11[3][3], kx33[3][3], kx13[3][3], kx31[3][3];
    {
      double G11[3][3], G33[3][3], G13[3][3], G31[3][3], GC11[3][3], GC33[3][3], GC13[3][3], GC31[3][3];
      double CG13[3][3], CG31[3][3];
      outer3(gx1, gx1, G11); outer3(gx3, gx3, G33); outer3(gx1, gx3, G13); outer3(gx3, gx1, G31);
      outer3(gx1, cfd1, GC11); outer3(gx3, cfd3, GC33); outer3(gx1, cfd3, GC13); outer3(gx3, cfd1, GC31);
      outer3(cfd1, gx3, CG13); outer3(cfd3, gx1, CG31);
      double c1 = cc * (cc - 1) * g1, c2 = cc * g2; /* c(c-1) g^(c-2), c g^(c-1) */
      double base2 = 0.5 * (comp + 1.0) * S * (R * R);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double t1, t2, t3;
          t1 = c1 * G11[i][j] + c2 * gx11[i][j];
          t2 = c1 * G11[i][j] * cf + c2 * gx11[i][j] * cf + c2 * GC11[i][j];
          t3 = -c2 * GC11[i][j] + (1 - g3) * cf11[i][j];
          kx11[i][j] = base2 * (t1 - t2 + t3);
          t1 = c1 * G33[i][j] + c2 * gx33[i][j];
          t2 = c1 * G33[i][j] * cf + c2 * gx33[i][j] * cf + c2 * GC33[i][j];
          t3 = -c2 * GC33[i][j] + (1 - g3) * cf33[i][j];
          kx33[i][j] = base2 * (t1 - t2 + t3);
          t1 = c1 * G13[i][j] + c2 * gx13[i][j];
          t2 = c1 * G13[i][j] * cf + c2 * gx13[i][j] * cf + c2 * GC13[i][j];
          t3 = -c2 * CG13[i][j] + (1 - g3) * cf13[i][j];
          kx13[i][j] = base2 * (t1 - t2 + t3);
          t1 = c1 * G31[i][j] + c2 * gx31[i][j];
          t2 = c1 * G31[i][j] * cf + c2 * gx31[i][j] * cf + c2 * GC31[i][j];
          t3 = -c2 * CG31[i][j] + (1 - g3) * cf31[i][j];
          kx31[i][j] = base2 * (t1 - t2 + t3);
        }
    }
    double K1x1[3][3], K1x3[3][3], P1x3[3][3], K3x1[3][3], K3x3[3][3], P3x1[3][3];
    outer3(kx1, px1, K1x1); outer3(kx1, px3, K1x3); outer3(px1, kx3, P1x3);
    outer3(kx3, px1, K3x1); outer3(kx3, px3, K3x3); outer3(px3, kx1, P3x1);
    double o11a[3][3], o13a[3][3], o31a[3][3], o33a[3][3];
    { double o[3][3]; outer3(a1, d3, o); mm3(o, P1, o31a); } /* outer(P3 d1, d3) P1 */
    { double o[3][3]; outer3(a3, d3, o); mm3(o, P1, o11a); } /* outer(P1 d3, d3) P1 */
    { double o[3][3]; outer3(a1, d1, o); mm3(o, P3, o33a); } /* outer(P3 d1, d1) P3 */
    { double o[3][3]; outer3(a3, d1, o); mm3(o, P3, o13a); } /* outer(P1 d3, d1) P3 */
    double kL = kx * Lc;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double f11o = (kL / ((l1 * l1) * s)) *
                      (Bq * (-a3d1[i][j] + cs2 * o11a[i][j] - co * P1[i][j] - d1a3[i][j]) - (1.0 / s) * o11a[i][j]);
        double f33o = (kL / ((l3 * l3) * s)) *
                      (Bq * (-a1d3[i][j] + cs2 * o33a[i][j] - co * P3[i][j] - d3a1[i][j]) - (1.0 / s) * o33a[i][j]);
        double f13o = (kL / (l1 * l3 * s)) * (Bq * (cs2 * o13a[i][j] + P1P3[i][j]) - (1.0 / s) * o13a[i][j]);
        double f31o = (kL / (l3 * l1 * s)) * (Bq * (cs2 * o31a[i][j] + P3P1[i][j]) - (1.0 / s) * o31a[i][j]);
        J11[i][j] = -0.5 * kx11[i][j] * Lc * Bq2 - 2 * Lc * Bq * K1x1[i][j] + f11o;
        J33[i][j] = -0.5 * kx33[i][j] * Lc * Bq2 - 2 * Lc * Bq * K3x3[i][j] + f33o;
        J13[i][j] = (-0.5 * kx13[i][j] * Lc * Bq2 - Lc * Bq * K1x3[i][j] - Lc * Bq * P1x3[i][j] + f13o);
        J31[i][j] = (-0.5 * kx31[i][j] * Lc * Bq2 - Lc * Bq * K3x1[i][j] - Lc * Bq * P3x1[i][j] + f31o);
      }
  }
  for (int i = 0; i < 3; ++i) {
    double Fx0 = -1 * (Fx1[i] + Fx3[i]);
    c->F[3 * n0 + i] += Fx0;
    c->F[3 * n1 + i] += Fx1[i];
    c->F[3 * n3 + i] += Fx3[i];
  }
  double J10[3][3], J30[3][3], J01[3][3], J03[3][3], J00[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      J10[i][j] = -(J11[i][j] + J13[i][j]);
      J30[i][j] = -(J31[i][j] + J33[i][j]);
      J01[i][j] = -(J11[i][j] + J31[i][j]);
      J03[i][j] = -(J13[i][j] + J33[i][j]);
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J00[i][j] = -(J10[i][j] + J30[i][j]);
  add_LL(c, c->Kv, n0, n0, J00, 1.0);
  add_LL(c, c->Kv, n0, n1, J01, 1.0);
  add_LL(c, c->Kv, n0, n3, J03, 1.0);
  add_LL(c, c->Kv, n1, n0, J10, 1.0);
  add_LL(c, c->Kv, n1, n1, J11, 1.0);
  add_LL(c, c->Kv, n1, n3, J13, 1.0);
  add_LL(c, c->Kv, n3, n0, J30, 1.0);
  add_LL(c, c->Kv, n3, n1, J31, 1.0);
  add_LL(c, c->Kv, n3, n3, J33, 1.0);
}

/* ------------------------------------------------------------------ */
/* FillMV                                                               */
/* ------------------------------------------------------------------ */
void yo_fill(yo_cloth *c) {
  memset(c->Mv, 0, sizeof(double) * c->nnz);
  memset(c->Kv, 0, sizeof(double) * c->nnz);
  memset(c->Dv, 0, sizeof(double) * c->nnz);
  memset(c->F, 0, sizeof(double) * c->dim);
  memset(c->CL, 0, sizeof(double) * 3 * c->N);
  memset(c->CLE, 0, sizeof(double) * 6 * (c->Nc > 0 ? c->Nc : 1));
  memset(c->slide, 0, sizeof(double) * 2 * (c->Nc > 0 ? c->Nc : 1));
  const int W = c->W, H = c->H;
  /* Constraint_F / Constraint_D (src/PhysicsCloth.cpp:232-248) */
  for (int i = 0; i < W; ++i)
    for (int j = 0; j < H; ++j) {
      int n = nid(c, i, j);
      if (!c->fixed[n]) continue;
      for (int k = 0; k < 3; ++k) c->F[3 * n + k] -= c->kh * (c->x[3 * n + k] - c->xfix[3 * n + k]);
      double I[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      add_LL(c, c->Kv, n, n, I, -c->kh);
    }
  /* edges in construction order (src/Cloth.cpp:189-228) */
  edge_t e;
  for (int pass = 0; pass < 2; ++pass) {
    int outer = pass == 0 ? H : W, inner = pass == 0 ? W - 1 : H - 1;
    for (int i = 0; i < outer; ++i)
      for (int j = 0; j < inner; ++j) {
        if (pass == 0) edge_geom(c, nid(c, j, i), nid(c, j + 1, i), 0, i, &e);
        else edge_geom(c, nid(c, i, j), nid(c, i, j + 1), 1, i, &e);
        /* Mass, forces, then Jacobians (src/PhysicsCloth.cpp:67-79) */
        t_mass(c, &e);
        t_gravity(c, &e);
        t_stretch(c, &e);
        t_inertia_F(c, &e);
        t_mdot_F(c, &e);
        t_paracolli(c, &e);
        t_inertia_Dpos(c, &e);
        t_inertia_Dvel(c, &e);
        t_mdot_Dpos(c, &e);
        t_mdot_Dvel(c, &e);
      }
  }
  /* bend + crimp segments (src/Cloth.cpp:229-270, src/PhysicsCloth.cpp:82-89) */
  bend_t b;
  for (int pass = 0; pass < 2; ++pass) {
    int outer = pass == 0 ? H : W, inner = pass == 0 ? W - 2 : H - 2;
    for (int i = 0; i < outer; ++i)
      for (int j = 0; j < inner; ++j) {
        int n2, n0, n1;
        double kb;
        if (pass == 0) { n2 = nid(c, j, i); n0 = nid(c, j + 1, i); n1 = nid(c, j + 2, i); kb = c->kb_warp[i]; }
        else { n2 = nid(c, i, j); n0 = nid(c, i, j + 1); n1 = nid(c, i, j + 2); kb = c->kb_weft[i]; }
        bend_geom(c, c->x, c->uv, n2, n0, n1, pass, kb, &b);
        t_bend(c, &b);
        bend_geom(c, pass == 0 ? c->xw : c->xf, c->uv0, n2, n0, n1, pass, kb, &b);
        t_crimp(c, &b);
      }
  }
  /* faces (src/Cloth.cpp:271-296) */
  for (int i = 0; i < W - 1; ++i)
    for (int j = 0; j < H - 1; ++j) {
      int tl = nid(c, i, j), tr = nid(c, i + 1, j), bl = nid(c, i, j + 1), br = nid(c, i + 1, j + 1);
      if ((i + j) % 2 == 0) { t_wind(c, tl, tr, br); t_wind(c, tl, br, bl); }
      else { t_wind(c, tl, tr, bl); t_wind(c, tr, br, bl); }
    }
  /* friction (src/PhysicsCloth.cpp:114-123) */
  for (int i = 1; i < H - 1; ++i)
    for (int j = 1; j < W - 1; ++j) t_friction(c, nid(c, j, i));
  /* shear (src/Cloth.cpp:170-181, src/PhysicsCloth.cpp:125-131) */
  for (int i = 1; i < W - 1; ++i)
    for (int j = 1; j < H - 1; ++j) {
      int n = nid(c, i, j), lf = nid(c, i - 1, j), rt = nid(c, i + 1, j), tp = nid(c, i, j - 1), bt = nid(c, i, j + 1);
      t_shear(c, n, lf, bt);
      t_shear(c, n, lf, tp);
      t_shear(c, n, rt, bt);
      t_shear(c, n, rt, tp);
    }
}

/* ------------------------------------------------------------------ */
/* construction / state                                                 */
/* ------------------------------------------------------------------ */
yo_cloth *yo_create(const yo_desc *d) {
  if (d->width < 3 || d->length < 3) return NULL;
  yo_cloth *c = (yo_cloth *)calloc(1, sizeof(yo_cloth));
  c->W = d->width; c->H = d->length; c->N = c->W * c->H; c->Nc = (c->W - 2) * (c->H - 2);
  c->dim = 3 * c->N + 2 * c->Nc;
  c->L = d->L; c->R = d->R; c->height = d->height; c->pose = d->pose; c->weave = d->weave;
  c->kc = d->kc; c->kf = d->kf; c->df = d->df; c->mu = d->mu; c->S = d->S; c->kh = d->handle_stiffness;
  for (int k = 0; k < 3; ++k) { c->G[k] = d->G[k]; c->wind_v[k] = d->wind_vel[k]; }
  c->wind_rho = d->wind_density; c->wind_drag = d->wind_drag;
  c->jam = 2.0 * asin(c->R / c->L); /* src/Cloth.cpp:29 */
  c->rho_warp = (double *)malloc(sizeof(double) * c->H); c->ks_warp = (double *)malloc(sizeof(double) * c->H);
  c->kb_warp = (double *)malloc(sizeof(double) * c->H);
  c->rho_weft = (double *)malloc(sizeof(double) * c->W); c->ks_weft = (double *)malloc(sizeof(double) * c->W);
  c->kb_weft = (double *)malloc(sizeof(double) * c->W);
  for (int i = 0; i < c->H; ++i) {
    c->rho_warp[i] = d->warp_rho[i];
    c->ks_warp[i] = d->warp_Y[i] * YO_PI * pow(c->R, 2); /* src/Yarn.h:14-15 */
    c->kb_warp[i] = d->warp_B[i] * YO_PI * pow(c->R, 2);
  }
  for (int i = 0; i < c->W; ++i) {
    c->rho_weft[i] = d->weft_rho[i];
    c->ks_weft[i] = d->weft_Y[i] * YO_PI * pow(c->R, 2);
    c->kb_weft[i] = d->weft_B[i] * YO_PI * pow(c->R, 2);
  }
  int N = c->N;
  c->x = (double *)calloc(3 * N, sizeof(double)); c->v = (double *)calloc(3 * N, sizeof(double));
  c->xfix = (double *)calloc(3 * N, sizeof(double)); c->uv = (double *)calloc(2 * N, sizeof(double));
  c->uvdot = (double *)calloc(2 * N, sizeof(double)); c->uvbar = (double *)calloc(2 * N, sizeof(double));
  c->uv0 = (double *)calloc(2 * N, sizeof(double));
  c->fixed = (unsigned char *)calloc(N, 1); c->flip = (unsigned char *)calloc(N, 1);
  c->nrm = (double *)calloc(3 * N, sizeof(double)); c->xw = (double *)calloc(3 * N, sizeof(double));
  c->xf = (double *)calloc(3 * N, sizeof(double)); c->comp = (double *)calloc(N, sizeof(double));
  c->F = (double *)calloc(c->dim, sizeof(double));
  int nc = c->Nc > 0 ? c->Nc : 1;
  c->slide = (double *)calloc(2 * nc, sizeof(double));
  c->CL = (double *)calloc(3 * N, sizeof(double));
  c->CLE = (double *)calloc(6 * nc, sizeof(double));
  /* Cloth::build (src/Cloth.cpp:52-109) */
  for (int j = 0; j < c->H; ++j)
    for (int i = 0; i < c->W; ++i) {
      int n = nid(c, i, j);
      if (c->pose == 0) { c->x[3 * n] = i * c->L; c->x[3 * n + 1] = 0.0; c->x[3 * n + 2] = c->height - j * c->L; }
      else { c->x[3 * n] = i * c->L; c->x[3 * n + 1] = j * c->L; c->x[3 * n + 2] = c->height; }
      c->uv[2 * n] = i * c->L; c->uv[2 * n + 1] = j * c->L;
      memcpy(&c->xfix[3 * n], &c->x[3 * n], sizeof(double) * 3);
      memcpy(&c->uvbar[2 * n], &c->uv[2 * n], sizeof(double) * 2);
      memcpy(&c->uv0[2 * n], &c->uv[2 * n], sizeof(double) * 2);
      if (!is_int(c, n)) continue;
      int f = 0;
      if (c->weave == 0) {
        f = ((i + j) % 2 != 0);
      } else if (c->weave == 1) {
        int rv = j % 4, ru = (i + rv) % 4;
        f = ru < 2;
      } else {
        int rv = (j - 1) % 4, q = rv / 2, r = rv % 2, idx = q * 3 + r * 2, ru = (i - 1 + idx) % 4;
        f = ru == 0;
      }
      c->flip[n] = (unsigned char)f;
    }
  for (int h = 0; h < d->n_handles; ++h) {
    int u = d->handles[2 * h], v = d->handles[2 * h + 1];
    if (u >= 0 && u < c->W && v >= 0 && v < c->H) c->fixed[nid(c, u, v)] = 1;
  }
  build_pattern(c);
  update_units(c);
  return c;
}

void yo_destroy(yo_cloth *c) {
  if (!c) return;
  free(c->rho_warp); free(c->ks_warp); free(c->kb_warp); free(c->rho_weft); free(c->ks_weft); free(c->kb_weft);
  free(c->x); free(c->v); free(c->xfix); free(c->uv); free(c->uvdot); free(c->uvbar); free(c->uv0);
  free(c->fixed); free(c->flip); free(c->nrm); free(c->xw); free(c->xf); free(c->comp);
  free(c->rowptr); free(c->col); free(c->Mv); free(c->Kv); free(c->Dv);
  free(c->F); free(c->slide); free(c->CL); free(c->CLE);
  free(c);
}

int yo_num_nodes(const yo_cloth *c) { return c->N; }
int yo_dim(const yo_cloth *c) { return c->dim; }

void yo_set_state(yo_cloth *c, const double *lpos, const double *lposfix, const double *lvel, const double *epos,
                  const double *eposbar, const double *evel) {
  int N = c->N;
  if (lpos) memcpy(c->x, lpos, sizeof(double) * 3 * N);
  if (lposfix) memcpy(c->xfix, lposfix, sizeof(double) * 3 * N);
  if (lvel) memcpy(c->v, lvel, sizeof(double) * 3 * N);
  if (epos) memcpy(c->uv, epos, sizeof(double) * 2 * N);
  if (eposbar) memcpy(c->uvbar, eposbar, sizeof(double) * 2 * N);
  if (evel) memcpy(c->uvdot, evel, sizeof(double) * 2 * N);
  update_units(c);
}

void yo_get_state(const yo_cloth *c, double *lpos, double *lposfix, double *lvel, double *epos, double *eposbar,
                  double *evel) {
  int N = c->N;
  if (lpos) memcpy(lpos, c->x, sizeof(double) * 3 * N);
  if (lposfix) memcpy(lposfix, c->xfix, sizeof(double) * 3 * N);
  if (lvel) memcpy(lvel, c->v, sizeof(double) * 3 * N);
  if (epos) memcpy(epos, c->uv, sizeof(double) * 2 * N);
  if (eposbar) memcpy(eposbar, c->uvbar, sizeof(double) * 2 * N);
  if (evel) memcpy(evel, c->uvdot, sizeof(double) * 2 * N);
}

void yo_get_normals(const yo_cloth *c, double *normals) { memcpy(normals, c->nrm, sizeof(double) * 3 * c->N); }

void yo_set_wind(yo_cloth *c, const double wind_vel[3]) {
  for (int k = 0; k < 3; ++k) c->wind_v[k] = wind_vel[k];
}

static void vel_vector(const yo_cloth *c, double *V) {
  for (int n = 0; n < c->N; ++n)
    for (int k = 0; k < 3; ++k) V[3 * n + k] = c->v[3 * n + k];
  for (int n = 0; n < c->N; ++n)
    if (is_int(c, n))
      for (int k = 0; k < 2; ++k) V[erow(c, n) + k] = c->uvdot[2 * n + k];
}

void yo_export_dense(const yo_cloth *c, double *M, double *K, double *D, double *F, double *V, double *slide) {
  size_t dim = (size_t)c->dim;
  if (M) memset(M, 0, sizeof(double) * dim * dim);
  if (K) memset(K, 0, sizeof(double) * dim * dim);
  if (D) memset(D, 0, sizeof(double) * dim * dim);
  for (int r = 0; r < c->dim; ++r)
    for (int p = c->rowptr[r]; p < c->rowptr[r + 1]; ++p) {
      size_t o = (size_t)r * dim + c->col[p];
      if (M) M[o] = c->Mv[p];
      if (K) K[o] = c->Kv[p];
      if (D) D[o] = c->Dv[p];
    }
  if (F) memcpy(F, c->F, sizeof(double) * dim);
  if (V) vel_vector(c, V);
  if (slide) memcpy(slide, c->slide, sizeof(double) * 2 * c->Nc);
}

/* A (CSR values over the pattern) and b */
static void assemble(const yo_cloth *c, double h, const double *ext, double *Av, double *b) {
  int dim = c->dim;
  double *V = (double *)malloc(sizeof(double) * dim);
  vel_vector(c, V);
  double h2 = h * h;
  for (int p = 0; p < c->nnz; ++p) Av[p] = c->Mv[p] - c->Kv[p] * h2 - c->Dv[p] * h;
  double *DtV = (double *)calloc(dim, sizeof(double)), *MV = (double *)calloc(dim, sizeof(double));
  for (int r = 0; r < dim; ++r)
    for (int p = c->rowptr[r]; p < c->rowptr[r + 1]; ++p) {
      DtV[c->col[p]] += c->Dv[p] * V[r];
      MV[r] += c->Mv[p] * V[c->col[p]];
    }
  for (int r = 0; r < dim; ++r) b[r] = h * ((c->F[r] + (ext ? ext[r] : 0.0)) - DtV[r]) + MV[r];
  free(V); free(DtV); free(MV);
}

void yo_export_system(const yo_cloth *c, double h, const double *ext_force, double *A, double *b) {
  double *Av = (double *)malloc(sizeof(double) * c->nnz);
  double *bb = (double *)malloc(sizeof(double) * c->dim);
  assemble(c, h, ext_force, Av, bb);
  size_t dim = (size_t)c->dim;
  if (A) {
    memset(A, 0, sizeof(double) * dim * dim);
    for (int r = 0; r < c->dim; ++r)
      for (int p = c->rowptr[r]; p < c->rowptr[r + 1]; ++p) A[(size_t)r * dim + c->col[p]] = Av[p];
  }
  if (b) memcpy(b, bb, sizeof(double) * dim);
  free(Av); free(bb);
}

/* Eigen ConjugateGradient<SparseMatrix, Lower|Upper> defaults restated:
 * Jacobi preconditioner (zero diagonal -> 1), x0 = 0, stop when
 * |r|^2 < max(tol^2 |b|^2, DBL_MIN), tol = DBL_EPSILON, at most 2n steps
 * (used by src/Solvers.cpp:22-24). */
static long csr_pcg(int n, const int *rowptr, const int *col, const double *val, const double *rhs, double *x,
                    double tol, long maxiter, double *err) {
  double *r = (double *)malloc(sizeof(double) * n), *z = (double *)malloc(sizeof(double) * n);
  double *p = (double *)malloc(sizeof(double) * n), *q = (double *)malloc(sizeof(double) * n);
  double *id = (double *)malloc(sizeof(double) * n);
  for (int i = 0; i < n; ++i) {
    double dg = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (col[k] == i) dg = val[k];
    id[i] = dg != 0.0 ? 1.0 / dg : 1.0;
    x[i] = 0.0;
    r[i] = rhs[i];
  }
  if (tol <= 0) tol = DBL_EPSILON;
  if (maxiter < 0) maxiter = 2L * n;
  double bn = 0.0;
  for (int i = 0; i < n; ++i) bn += rhs[i] * rhs[i];
  long it = 0;
  if (bn == 0.0) { *err = 0.0; goto done; }
  double thr = tol * tol * bn;
  if (thr < DBL_MIN) thr = DBL_MIN;
  double rn = bn;
  if (rn < thr) { *err = sqrt(rn / bn); goto done; }
  double an = 0.0;
  for (int i = 0; i < n; ++i) { p[i] = id[i] * r[i]; an += r[i] * p[i]; }
  while (it < maxiter) {
    double pq = 0.0;
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += val[k] * p[col[k]];
      q[i] = s;
      pq += p[i] * s;
    }
    double alpha = an / pq;
    rn = 0.0;
    for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; rn += r[i] * r[i]; }
    if (rn < thr) break;
    double ao = an;
    an = 0.0;
    for (int i = 0; i < n; ++i) { z[i] = id[i] * r[i]; an += r[i] * z[i]; }
    double beta = an / ao;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  *err = sqrt(rn / bn);
done:
  free(r); free(z); free(p); free(q); free(id);
  return it;
}

long yo_dense_pcg(int n, const double *A, const double *b, double *x, double tol, long maxiter, double *err_out) {
  int *rowptr = (int *)malloc(sizeof(int) * (n + 1));
  int nnz = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) nnz += A[(size_t)i * n + j] != 0.0;
  int *col = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
  double *val = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
  nnz = 0;
  rowptr[0] = 0;
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j)
      if (A[(size_t)i * n + j] != 0.0) { col[nnz] = j; val[nnz] = A[(size_t)i * n + j]; ++nnz; }
    rowptr[i + 1] = nnz;
  }
  double err = 0.0;
  long it = csr_pcg(n, rowptr, col, val, b, x, tol, maxiter, &err);
  if (err_out) *err_out = err;
  free(rowptr); free(col); free(val);
  return it;
}

static int all_finite(const double *a, long n) {
  for (long i = 0; i < n; ++i)
    if (!isfinite(a[i])) return 0;
  return 1;
}

/* Cloth::update (src/Cloth.cpp:111-148). */
static void cloth_update(yo_cloth *c, const double *nv, double h) {
  for (int i = 0; i < c->W; ++i)
    for (int j = 0; j < c->H; ++j) {
      int n = nid(c, i, j);
      for (int k = 0; k < 3; ++k) {
        c->v[3 * n + k] = nv[3 * n + k];
        c->x[3 * n + k] = c->x[3 * n + k] + c->v[3 * n + k] * h;
      }
      if (!c->fixed[n]) memcpy(&c->xfix[3 * n], &c->x[3 * n], sizeof(double) * 3);
      if (is_int(c, n)) {
        int fe = eidx(c, n), er = erow(c, n);
        for (int k = 0; k < 2; ++k) {
          c->uvdot[2 * n + k] = nv[er + k];
          c->uv[2 * n + k] = c->uv[2 * n + k] + c->uvdot[2 * n + k] * h;
          c->uvbar[2 * n + k] = c->uvbar[2 * n + k] + c->slide[2 * fe + k] * c->uvdot[2 * n + k] * h;
        }
      }
    }
  update_units(c);
}

int yo_step(yo_cloth *c, double h, const double *ext_force, double cg_tol, long cg_maxiter, yo_stats *st) {
  yo_stats local;
  if (!st) st = &local;
  memset(st, 0, sizeof(*st));
  yo_fill(c);
  double *Av = (double *)malloc(sizeof(double) * c->nnz);
  double *b = (double *)malloc(sizeof(double) * c->dim);
  double *x = (double *)malloc(sizeof(double) * c->dim);
  assemble(c, h, ext_force, Av, b);
  if (!all_finite(Av, c->nnz) || !all_finite(b, c->dim)) {
    st->status = 1;
  } else {
    st->cg_iterations = csr_pcg(c->dim, c->rowptr, c->col, Av, b, x, cg_tol, cg_maxiter, &st->cg_error);
    if (!all_finite(x, c->dim)) st->status = 1;
    else cloth_update(c, x, h);
  }
  free(Av); free(b); free(x);
  return st->status;
}
