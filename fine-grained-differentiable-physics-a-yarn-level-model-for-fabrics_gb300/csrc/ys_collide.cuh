// ys_collide.cuh -- continuous collision detection of cloth meshes: 18-DOP
// boxes, the broad-phase overlap test and the narrow phase (vertex-face and
// edge-edge coplanarity in [0, 1] of the step), as functions of one pair.
//
// The arithmetic restates the reference: kDOP18 (src/BVH.h:28-230), dilate
// and overlap (src/BVH.cpp:268-291), comp_face_impacts (src/Collision.cpp:
// 210-253), vf / ee / collision_test (src/Collision.cpp:327-419), the cubic
// solver (src/Solvers.cpp:60-178) and sub_signed_vf / ee_distance
// (src/Geometry.cpp:15-83), including the solver's return of x0 when its
// only root landed in x1 or x2.
#pragma once

#include <float.h>
#include <math.h>

#include "ys_common.cuh"

namespace ys {

// ------------------------------------------------------------------ kDOP18
// d[0..8] lower bounds, d[9..17] upper bounds along x, y, z, x+y, x+z, y+z,
// x-y, x-z, y-z.
struct Kdop {
  double d[18];
};

YS_HD double kmin(double a, double b) { return a < b ? a : b; }  // MIN (src/BVH.h:18-21)
YS_HD double kmax(double a, double b) { return a > b ? a : b; }  // MAX (src/BVH.h:13-16)

YS_HD void kdop_diag(const double* p, double* q) {
  q[0] = p[0] + p[1];
  q[1] = p[0] + p[2];
  q[2] = p[1] + p[2];
  q[3] = p[0] - p[1];
  q[4] = p[0] - p[2];
  q[5] = p[1] - p[2];
}
YS_HD void kdop_empty(Kdop& b) {
  for (int i = 0; i < 9; ++i) {
    b.d[i] = FLT_MAX;
    b.d[i + 9] = -FLT_MAX;
  }
}
YS_HD void kdop_point(Kdop& b, const double* p) {  // kDOP18(const vec3f&)
  double q[6];
  kdop_diag(p, q);
  for (int i = 0; i < 3; ++i) b.d[i] = b.d[i + 9] = p[i];
  for (int i = 0; i < 6; ++i) b.d[3 + i] = b.d[12 + i] = q[i];
}
YS_HD void kdop_add_point(Kdop& b, const double* p) {  // operator+=(const vec3f&)
  double q[6];
  kdop_diag(p, q);
  for (int i = 0; i < 3; ++i) {
    b.d[i] = kmin(p[i], b.d[i]);
    b.d[i + 9] = kmax(p[i], b.d[i + 9]);
  }
  for (int i = 0; i < 6; ++i) {
    b.d[3 + i] = kmin(q[i], b.d[3 + i]);
    b.d[12 + i] = kmax(q[i], b.d[12 + i]);
  }
}
YS_HD void kdop_add(Kdop& a, const Kdop& b) {  // operator+=(const kDOP18&)
  for (int i = 0; i < 9; ++i) {
    a.d[i] = kmin(b.d[i], a.d[i]);
    a.d[i + 9] = kmax(b.d[i + 9], a.d[i + 9]);
  }
}
// node_box: the node's position, and its previous position under CCD
YS_HD void kdop_node(Kdop& b, const double* x, const double* xp, bool ccd) {
  kdop_point(b, x);
  if (ccd) kdop_add_point(b, xp);
}
// box0.overlaps(dilate(box1, d)) (src/BVH.cpp:268-291, src/BVH.h:110-118)
YS_HD bool kdop_overlap(const Kdop& a, const Kdop& b, double d) {
  const double s2 = sqrt(2.0) * d;
  for (int i = 0; i < 9; ++i) {
    const double dd = i < 3 ? d : s2;
    const double lo = b.d[i] - dd, hi = b.d[i + 9] + dd;
    if (a.d[i] > hi) return false;
    if (a.d[i + 9] < lo) return false;
  }
  return true;
}
// a test that accepts every pair of boxes inside a and b that kdop_overlap
// accepts (the inner-node prune of a traversal)
YS_HD bool kdop_overlap_loose(const Kdop& a, const Kdop& b, double d) {
  const double s2 = sqrt(2.0) * d * (1.0 + 1e-12) + 1e-300;
  const double d1 = d * (1.0 + 1e-12) + 1e-300;
  for (int i = 0; i < 9; ++i) {
    const double dd = i < 3 ? d1 : s2;
    const double slack = 1e-12 * (fabs(b.d[i]) + fabs(b.d[i + 9]) + fabs(a.d[i]) + fabs(a.d[i + 9]));
    if (a.d[i] > b.d[i + 9] + dd + slack) return false;
    if (a.d[i + 9] < b.d[i] - dd - slack) return false;
  }
  return true;
}

// ------------------------------------------------------------ cubic solve
YS_HD int cc_quad(double a, double b, double c, double& x0, double& x1) {
  const double d = b * b - 4.0 * a * c;
  if (d < 0.0) {
    x0 = -b / (2.0 * a);
    return 0;
  }
  const double sd = sqrt(d);
  const double q = -(b + sd) / 2.0, q1 = -(b - sd) / 2.0;
  if (fabs(a) > 1e-12) {
    if (q / a < q1 / a) {
      x0 = q / a;
      x1 = q1 / a;
    } else {
      x0 = q1 / a;
      x1 = q / a;
    }
    return 2;
  }
  x0 = -c / b;
  return 1;
}
YS_HD double cc_newton(double a, double b, double c, double d, double x0, int dir) {
  if (dir != 0) {
    const double y0 = d + x0 * (c + x0 * (b + x0 * a)), ddy0 = 2 * b + (x0 + dir * 1e-6) * (6 * a);
    x0 = x0 + dir * sqrt(fabs(2 * y0 / ddy0));
  }
  for (int it = 0; it < 100; ++it) {
    const double y = d + x0 * (c + x0 * (b + x0 * a));
    const double dy = c + x0 * (2 * b + x0 * 3 * a);
    if (dy == 0.0) return x0;
    const double x1 = x0 - y / dy;
    if (fabs(x0 - x1) < 1e-6) return x0;
    x0 = x1;
  }
  return x0;
}
// roots of a t^3 + b t^2 + c t + d as the reference returns them; count in r
YS_HD int cc_cubic(double a, double b, double c, double d, double r[3]) {
  double xc0 = -1.0, xc1 = -1.0, x0 = -1.0, x1 = -1.0, x2 = -1.0;
  const int ncrit = cc_quad(3.0 * a, 2.0 * b, c, xc0, xc1);
  if (ncrit == 0) {
    r[0] = cc_newton(a, b, c, d, xc0, 0);
    return 1;
  }
  if (ncrit == 1) {
    const int ns = cc_quad(b, c, d, x0, x1);
    r[0] = x0;
    r[1] = x1;
    return ns == 1 ? 1 : ns == 2 ? 2 : 0;
  }
  const double yc0 = d + xc0 * (c + xc0 * (b + xc0 * a)), yc1 = d + xc1 * (c + xc1 * (b + xc1 * a));
  int ns = 0;
  if (yc0 * a >= 0.0) {
    x0 = cc_newton(a, b, c, d, xc0, -1);
    ns++;
  }
  if (yc0 * yc1 <= 0.0) {
    if (fabs(yc0) < fabs(yc1)) x1 = cc_newton(a, b, c, d, xc0, 1);
    else x1 = cc_newton(a, b, c, d, xc1, -1);
    ns++;
  }
  if (yc1 * a <= 0.0) {
    x2 = cc_newton(a, b, c, d, xc1, 1);
    ns++;
  }
  r[0] = x0;  // the reference returns x0 (, x1 (, x2)) by count, whichever were set
  r[1] = x1;
  r[2] = x2;
  return ns > 3 ? 0 : ns;
}

// ---------------------------------------------------------- narrow phase
YS_HD void cc_cross(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
YS_HD double cc_dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
YS_HD double cc_triple(const double* a, const double* b, const double* c) {
  double t[3];
  cc_cross(b, c, t);
  return cc_dot(a, t);
}

struct Impact {
  int type;     // 0 vertex-face, 1 edge-edge
  int node[4];  // cloth node id, or -1 - id for an obstacle node
  double t;
  double w[4];
  double n[3];
};

// sub_signed_vf_distance / sub_signed_ee_distance with thres 1e-12; returns
// false when the reference sets `over`
YS_HD bool cc_vf_distance(const double* y0, const double* y1, const double* y2, double* n, double* w) {
  double a[3], b[3];
  for (int i = 0; i < 3; ++i) { a[i] = y1[i] - y0[i]; b[i] = y2[i] - y0[i]; }
  cc_cross(a, b, n);
  for (int k = 0; k < 4; ++k) w[k] = 0.0;
  if (cc_dot(n, n) < 1e-12) return false;
  const double l = sqrt(cc_dot(n, n));
  if (l != 0.0)
    for (int i = 0; i < 3; ++i) n[i] /= l;
  const double h = -cc_dot(y0, n);
  if (fabs(h) > 1e-12) return false;
  double t[3];
  cc_cross(y2, n, t);
  const double b0 = cc_dot(y1, t);
  cc_cross(y0, n, t);
  const double b1 = cc_dot(y2, t);
  cc_cross(y1, n, t);
  const double b2 = cc_dot(y0, t);
  const double sum = 1.0 / (b0 + b1 + b2);
  w[0] = 1.0;
  w[1] = -b0 * sum;
  w[2] = -b1 * sum;
  w[3] = -b2 * sum;
  return true;
}
YS_HD bool cc_ee_distance(const double* x1mx0, const double* y0mx0, const double* y1mx0, const double* y0mx1,
                          const double* y1mx1, const double* y1my0, double* n, double* w) {
  cc_cross(x1mx0, y1my0, n);
  for (int k = 0; k < 4; ++k) w[k] = 0.0;
  if (cc_dot(n, n) < 1e-12) return false;
  const double l = sqrt(cc_dot(n, n));
  if (l != 0.0)
    for (int i = 0; i < 3; ++i) n[i] /= l;
  const double h = -cc_dot(y0mx0, n);
  if (fabs(h) > 1e-12) return false;
  double t[3];
  cc_cross(y0mx1, n, t);
  const double a0 = cc_dot(y1mx1, t);
  cc_cross(y1mx0, n, t);
  const double a1 = cc_dot(y0mx0, t);
  cc_cross(y1mx0, n, t);
  const double b0 = cc_dot(y1mx1, t);
  cc_cross(y0mx1, n, t);
  const double b1 = cc_dot(y0mx0, t);
  const double suma = 1.0 / (a0 + a1), sumb = 1.0 / (b0 + b1);
  w[0] = a0 * suma;
  w[1] = a1 * suma;
  w[2] = -b0 * sumb;
  w[3] = -b1 * sumb;
  return true;
}

// collision_test for nodes p[4] (previous positions xp[k], current x[k])
YS_HD bool cc_test(int type, const double* const x[4], const double* const xp[4], Impact& im) {
  double x1[3], x2[3], x3[3], v0[3], v1[3], v2[3], v3[3];
  for (int i = 0; i < 3; ++i) {
    v0[i] = x[0][i] - xp[0][i];
    x1[i] = xp[1][i] - xp[0][i];
    x2[i] = xp[2][i] - xp[0][i];
    x3[i] = xp[3][i] - xp[0][i];
    v1[i] = x[1][i] - xp[1][i] - v0[i];
    v2[i] = x[2][i] - xp[2][i] - v0[i];
    v3[i] = x[3][i] - xp[3][i] - v0[i];
  }
  const double a0 = cc_triple(x1, x2, x3);
  const double a1 = cc_triple(v1, x2, x3) + cc_triple(x1, v2, x3) + cc_triple(x1, x2, v3);
  const double a2 = cc_triple(x1, v2, v3) + cc_triple(v1, x2, v3) + cc_triple(v1, v2, x3);
  const double a3 = cc_triple(v1, v2, v3);
  double r[3];
  const int nr = cc_cubic(a3, a2, a1, a0, r);
  for (int k = 0; k < nr; ++k) {
    const double t = r[k];
    if (isnan(t) || isinf(t) || t < 0 || t > 1) continue;
    double b1[3], b2[3], b3[3];
    for (int i = 0; i < 3; ++i) {
      b1[i] = x1[i] + t * v1[i];
      b2[i] = x2[i] + t * v2[i];
      b3[i] = x3[i] + t * v3[i];
    }
    double n[3], w[4];
    bool ok, inside;
    if (type == 0) {
      ok = cc_vf_distance(b1, b2, b3, n, w);
      inside = kmin(-w[1], kmin(-w[2], -w[3])) >= -1e-12;
    } else {
      double d21[3], d31[3], d32[3];
      for (int i = 0; i < 3; ++i) { d21[i] = b2[i] - b1[i]; d31[i] = b3[i] - b1[i]; d32[i] = b3[i] - b2[i]; }
      ok = cc_ee_distance(b1, b2, b3, d21, d31, d32, n, w);
      inside = kmin(kmin(w[0], w[1]), kmin(-w[2], -w[3])) >= -1e-12;
    }
    if (!ok || !inside) continue;
    double rv[3];
    for (int i = 0; i < 3; ++i) rv[i] = w[1] * v1[i] + w[2] * v2[i] + w[3] * v3[i];
    if (cc_dot(n, rv) > 0.0)
      for (int i = 0; i < 3; ++i) n[i] = -1 * n[i];
    im.type = type;
    im.t = t;
    for (int i = 0; i < 4; ++i) im.w[i] = w[i];
    for (int i = 0; i < 3; ++i) im.n[i] = n[i];
    return true;
  }
  return false;
}

// A face: three node ids and its three edges (each an oriented node pair),
// ids < 0 denote obstacle nodes (-1 - id).
struct CFace {
  int v[3];
  int e[3][2];
};
struct CMesh {
  const double* x;   // cloth nodes [n][3]
  const double* xp;
  const double* ox;  // obstacle nodes [no][3]
  const double* oxp;
};
YS_HD const double* cc_pos(const CMesh& m, int id, bool prev) {
  return id >= 0 ? (prev ? m.xp : m.x) + 3 * (int64_t)id : (prev ? m.oxp : m.ox) + 3 * (int64_t)(-1 - id);
}

// comp_face_impacts for the pair (f0, f1): up to 15 impacts in out, in the
// reference's order (3 + 3 vertex-face, 9 edge-edge); returns the count
// The 15 tests of a face pair in cc_face_pair's order -- t 0..2: node t of f0
// against f1; 3..5: node t - 3 of f1 against f0; 6..14: edge (t - 6) / 3 of
// f0 against edge (t - 6) % 3 of f1 -- and the nodes each one takes.
YS_HD void cc_pair_test_nodes(const CFace& f0, const CFace& f1, int t, int& type, int ids[4]) {
  if (t < 3) {
    type = 0;
    ids[0] = f0.v[t]; ids[1] = f1.v[0]; ids[2] = f1.v[1]; ids[3] = f1.v[2];
  } else if (t < 6) {
    type = 0;
    ids[0] = f1.v[t - 3]; ids[1] = f0.v[0]; ids[2] = f0.v[1]; ids[3] = f0.v[2];
  } else {
    type = 1;
    const int* e0 = f0.e[(t - 6) / 3];
    const int* e1 = f1.e[(t - 6) % 3];
    ids[0] = e0[0]; ids[1] = e0[1]; ids[2] = e1[0]; ids[3] = e1[1];
  }
}

// Bit t set when cc_face_pair would run test t: the k-DOP overlap and
// shared-node rules of comp_face_impacts (src/Collision.cpp:327-419). nk(id)
// gives node id's k-DOP (kdop_node of its two positions); the face and edge
// boxes are their unions, formed in cc_face_pair's order (min / max: exact).
template <class NodeBox>
YS_HD int cc_face_pair_mask(const NodeBox& nk, const CFace& f0, const CFace& f1, double thickness) {
  int mask = 0;
  {
    Kdop fb = nk(f1.v[0]);
    kdop_add(fb, nk(f1.v[1]));
    kdop_add(fb, nk(f1.v[2]));
    for (int k = 0; k < 3; ++k) {
      const int nd = f0.v[k];
      if (nd == f1.v[0] || nd == f1.v[1] || nd == f1.v[2]) continue;
      if (kdop_overlap(nk(nd), fb, thickness)) mask |= 1 << k;
    }
  }
  {
    Kdop fb = nk(f0.v[0]);
    kdop_add(fb, nk(f0.v[1]));
    kdop_add(fb, nk(f0.v[2]));
    for (int k = 0; k < 3; ++k) {
      const int nd = f1.v[k];
      if (nd == f0.v[0] || nd == f0.v[1] || nd == f0.v[2]) continue;
      if (kdop_overlap(nk(nd), fb, thickness)) mask |= 1 << (3 + k);
    }
  }
  for (int a = 0; a < 3; ++a) {
    const int an = a != 2 ? a + 1 : 0;
    Kdop ea = nk(f0.v[a]);
    kdop_add(ea, nk(f0.v[an]));
    for (int b = 0; b < 3; ++b) {
      const int* e0 = f0.e[a];
      const int* e1 = f1.e[b];
      if (e0[0] == e1[0] || e0[0] == e1[1] || e0[1] == e1[0] || e0[1] == e1[1]) continue;
      const int bn = b != 2 ? b + 1 : 0;
      Kdop eb = nk(f1.v[b]);
      kdop_add(eb, nk(f1.v[bn]));
      if (kdop_overlap(ea, eb, thickness)) mask |= 1 << (6 + 3 * a + b);
    }
  }
  return mask;
}

YS_HD int cc_face_pair(const CMesh& m, const CFace& f0, const CFace& f1, double thickness, bool ccd, Impact* out) {
  Kdop nb[6], eb[6], fb[2];
  for (int k = 0; k < 3; ++k) {
    kdop_node(nb[k], cc_pos(m, f0.v[k], false), cc_pos(m, f0.v[k], true), ccd);
    kdop_node(nb[k + 3], cc_pos(m, f1.v[k], false), cc_pos(m, f1.v[k], true), ccd);
  }
  for (int a = 0; a < 3; ++a) {
    const int b = a != 2 ? a + 1 : 0;
    eb[a] = nb[a];
    kdop_add(eb[a], nb[b]);
    eb[a + 3] = nb[a + 3];
    kdop_add(eb[a + 3], nb[b + 3]);
  }
  fb[0] = nb[0];
  kdop_add(fb[0], nb[1]);
  kdop_add(fb[0], nb[2]);
  fb[1] = nb[3];
  kdop_add(fb[1], nb[4]);
  kdop_add(fb[1], nb[5]);
  int cnt = 0;
  auto run = [&](int type, int a, int b, int c, int d) {
    const int ids[4] = {a, b, c, d};
    const double* xs[4];
    const double* xps[4];
    for (int k = 0; k < 4; ++k) {
      xs[k] = cc_pos(m, ids[k], false);
      xps[k] = cc_pos(m, ids[k], true);
    }
    Impact im;
    if (cc_test(type, xs, xps, im)) {
      for (int k = 0; k < 4; ++k) im.node[k] = ids[k];
      out[cnt++] = im;
    }
  };
  for (int k = 0; k < 3; ++k) {  // nodes of f0 against f1
    if (!kdop_overlap(nb[k], fb[1], thickness)) continue;
    const int nd = f0.v[k];
    if (nd == f1.v[0] || nd == f1.v[1] || nd == f1.v[2]) continue;
    run(0, nd, f1.v[0], f1.v[1], f1.v[2]);
  }
  for (int k = 0; k < 3; ++k) {  // nodes of f1 against f0
    if (!kdop_overlap(nb[k + 3], fb[0], thickness)) continue;
    const int nd = f1.v[k];
    if (nd == f0.v[0] || nd == f0.v[1] || nd == f0.v[2]) continue;
    run(0, nd, f0.v[0], f0.v[1], f0.v[2]);
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      if (!kdop_overlap(eb[a], eb[b + 3], thickness)) continue;
      const int* e0 = f0.e[a];
      const int* e1 = f1.e[b];
      if (e0[0] == e1[0] || e0[0] == e1[1] || e0[1] == e1[0] || e0[1] == e1[1]) continue;
      run(1, e0[0], e0[1], e1[0], e1[1]);
    }
  return cnt;
}

}  // namespace ys
