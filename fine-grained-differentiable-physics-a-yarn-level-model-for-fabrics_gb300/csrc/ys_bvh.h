// ys_bvh.h -- host construction of the face BVH of a mesh, the same tree the
// reference builds (BVHTree::Construct and the splitting BVHNode constructor,
// src/BVH.cpp:54-231): the root splits the faces at the centre of the box of
// all vertices along its longest axis, every other node at the centre of the
// box of its faces, with the reference's partition order and its fallback to
// halves. The tree is returned flattened in preorder, with what the device
// traversal and refit need: children, leaf faces, depths, and per leaf its
// left-to-right rank and the index of the upper node above it (the frontier
// of at least NThrd = 8 nodes that Collision::collect_upper_nodes forms,
// src/Collision.cpp:306-326), which fix the orientation of every pair the
// reference reports.
#pragma once

#include <algorithm>
#include <cstdint>
#include <future>
#include <vector>

#include "ys_collide.cuh"
#include "ys_pool.h"

namespace ys {

struct BvhTree {
  std::vector<int> left, right, face, depth;  // per node; face = -1 for inner nodes
  std::vector<int> leaf_of_face;              // node of each face
  std::vector<int> rank;                      // per face: leaf order left to right
  std::vector<int> upper;                     // per face: index of its upper node
  int max_depth = 0;
};

namespace bvh_detail {

struct Aap {  // the split plane (class aap, src/BVH.cpp:25-50)
  int xyz;
  double p;
  explicit Aap(const Kdop& t) {
    const double c[3] = {(t.d[0] + t.d[9]) * 0.5, (t.d[1] + t.d[10]) * 0.5, (t.d[2] + t.d[11]) * 0.5};
    const double w = t.d[9] - t.d[0], h = t.d[10] - t.d[1], dd = t.d[11] - t.d[2];
    xyz = 2;
    if (w >= h && w >= dd) xyz = 0;
    else if (h >= w && h >= dd) xyz = 1;
    p = c[xyz];
  }
  bool inside(const double* mid) const { return mid[xyz] > p; }
};

// the split plane of a box given by its x, y, z extents (lo, hi): the same
// arithmetic as Aap(const Kdop&), which reads only those six bounds
inline Aap aap_of(const double* lo, const double* hi) {
  Kdop t;
  for (int i = 0; i < 3; ++i) {
    t.d[i] = lo[i];
    t.d[i + 9] = hi[i];
  }
  return Aap(t);
}

// The reference's recursive construction (BVHNode(parent, lst, lst_num, ...),
// src/BVH.cpp:178-223) with the nodes numbered as its depth-first creation
// numbers them: a subtree of num faces takes 2 num - 1 consecutive indices
// (itself, then its left subtree, then its right one), so disjoint subtrees
// can be built on separate host threads and give the same tree.
struct Builder {
  const std::vector<double>& ext;      // [F][6] x, y, z minima then maxima of each face's box
  const std::vector<double>& centers;  // [F][3]
  BvhTree& t;
  void leaf(int f, int dep, int idx) {
    t.face[idx] = f;
    t.depth[idx] = dep;
    t.leaf_of_face[f] = idx;
  }
  // the node's own work for num >= 3 faces: its box, split plane and
  // partition of lst; fills its entry and returns the left child's face count
  int split_node(int* lst, int num, int dep, int idx) {
    t.depth[idx] = dep;
    double lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int q = 0; q < num; ++q) {
      const double* e = &ext[6 * (size_t)lst[q]];
      for (int i = 0; i < 3; ++i) {
        lo[i] = kmin(e[i], lo[i]);
        hi[i] = kmax(e[3 + i], hi[i]);
      }
    }
    const Aap pln = aap_of(lo, hi);
    unsigned left_idx = 0, right_idx = (unsigned)num - 1;
    for (int q = 0; q < num; ++q) {
      const int i = lst[left_idx];
      if (pln.inside(&centers[3 * (size_t)i])) {
        left_idx++;
      } else {
        const int tmp = lst[left_idx];
        lst[left_idx] = lst[right_idx];
        lst[right_idx--] = tmp;
      }
    }
    const int hal = num / 2;
    const int split = (left_idx == 0 || (int)left_idx == num) ? hal : (int)left_idx;
    t.left[idx] = idx + 1;
    t.right[idx] = idx + 2 * split;
    return split;
  }
  void node(int* lst, int num, int dep, int idx, int threads) {
    if (num == 1) {
      leaf(lst[0], dep, idx);
      return;
    }
    if (num == 2) {
      t.depth[idx] = dep;
      t.left[idx] = idx + 1;
      t.right[idx] = idx + 2;
      leaf(lst[0], dep + 1, idx + 1);
      leaf(lst[1], dep + 1, idx + 2);
      return;
    }
    const int split = split_node(lst, num, dep, idx);
    if (threads > 1 && num > 8192) {
      auto lf = std::async(std::launch::async, [=] { node(lst, split, dep + 1, idx + 1, threads / 2); });
      node(lst + split, num - split, dep + 1, idx + 2 * split, threads - threads / 2);
      lf.get();
    } else {
      node(lst, split, dep + 1, idx + 1, 1);
      node(lst + split, num - split, dep + 1, idx + 2 * split, 1);
    }
  }
  // the subtrees under the first levels, for a pool: splits nodes of more
  // than `min_faces` faces until depth `top`, recording each subtree left
  struct Task {
    int* lst;
    int num, dep, idx;
  };
  void top(int* lst, int num, int dep, int idx, int depth_left, int min_faces, std::vector<Task>& out) {
    if (depth_left == 0 || num <= min_faces || num < 3) {
      out.push_back({lst, num, dep, idx});
      return;
    }
    const int split = split_node(lst, num, dep, idx);
    top(lst, split, dep + 1, idx + 1, depth_left - 1, min_faces, out);
    top(lst + split, num - split, dep + 1, idx + 2 * split, depth_left - 1, min_faces, out);
  }
};

}  // namespace bvh_detail

// Builds the tree of faces [F] with nodes at x / xp ([n][3] each, xp used
// under CCD); face v[k] are node ids into x (this routine never sees
// obstacle ids). verts: the mesh's vertex order for the root box (node ids).
inline BvhTree bvh_build(int nfaces, const int* fv, int nverts, const int* verts, const double* x, const double* xp,
                         bool ccd, BuildPool* pool = nullptr) {
  BvhTree t;
  t.leaf_of_face.assign(nfaces, -1);
  t.rank.assign(nfaces, 0);
  t.upper.assign(nfaces, 0);
  if (nfaces == 0) return t;
  // with a pool (and enough faces) the vertex box, the faces' geometry and
  // the subtrees below the first levels are computed on its threads: min /
  // max bounds do not depend on the grouping, the root's partition stays a
  // pass in face order, and disjoint subtrees give the same tree
  const bool par = pool && pool->size() > 1 && nfaces >= 2048;
  const int nch = par ? pool->size() : 1;
  auto chunk = [&](int ch, int n, int& lo, int& hi) {
    lo = (int)((int64_t)n * ch / nch);
    hi = (int)((int64_t)n * (ch + 1) / nch);
  };
  Kdop total;
  kdop_empty(total);
  {
    std::vector<Kdop> part(nch);
    auto vbox = [&](int ch) {
      int lo, hi;
      chunk(ch, nverts, lo, hi);
      kdop_empty(part[ch]);
      for (int i = lo; i < hi; ++i) {
        kdop_add_point(part[ch], x + 3 * (size_t)verts[i]);
        if (ccd) kdop_add_point(part[ch], xp + 3 * (size_t)verts[i]);
      }
    };
    if (par) pool->run(nch, vbox);
    else vbox(0);
    for (int ch = 0; ch < nch; ++ch) kdop_add(total, part[ch]);
  }
  std::vector<double> ext(6 * (size_t)nfaces);
  std::vector<double> centers(3 * (size_t)nfaces);
  const bvh_detail::Aap pln(total);
  auto face_geom = [&](int ch) {
    int lo, hi;
    chunk(ch, nfaces, lo, hi);
    for (int f = lo; f < hi; ++f) {
      const double* p[3];
      const double* pp[3];
      for (int k = 0; k < 3; ++k) {
        p[k] = x + 3 * (size_t)fv[3 * f + k];
        pp[k] = xp + 3 * (size_t)fv[3 * f + k];
      }
      double mid[3], midp[3];
      for (int i = 0; i < 3; ++i) {  // middle_xyz (src/BVH.cpp:3-13)
        mid[i] = 0.5 * (kmin(kmin(p[0][i], p[1][i]), p[2][i]) + kmax(kmax(p[0][i], p[1][i]), p[2][i]));
        midp[i] = 0.5 * (kmin(kmin(pp[0][i], pp[1][i]), pp[2][i]) + kmax(kmax(pp[0][i], pp[1][i]), pp[2][i]));
      }
      for (int i = 0; i < 3; ++i) centers[3 * (size_t)f + i] = ccd ? (mid[i] + midp[i]) * 0.5 : mid[i];
      // the face box's x, y, z bounds (kDOP18 of its points, and of their
      // previous positions under CCD)
      double* e = &ext[6 * (size_t)f];
      for (int i = 0; i < 3; ++i) {
        e[i] = e[3 + i] = p[0][i];
        for (int k = 1; k < 3; ++k) {
          e[i] = kmin(p[k][i], e[i]);
          e[3 + i] = kmax(p[k][i], e[3 + i]);
        }
        if (ccd)
          for (int k = 0; k < 3; ++k) {
            e[i] = kmin(pp[k][i], e[i]);
            e[3 + i] = kmax(pp[k][i], e[3 + i]);
          }
      }
    }
  };
  if (par) pool->run(nch, face_geom);
  else face_geom(0);
  std::vector<int> buf(nfaces);
  unsigned left_idx = 0, right_idx = (unsigned)nfaces;
  for (int f = 0; f < nfaces; ++f) {
    if (pln.inside(&centers[3 * (size_t)f])) buf[left_idx++] = f;
    else buf[--right_idx] = f;
  }
  const size_t nn = 2 * (size_t)nfaces - 1;
  t.left.assign(nn, -1);
  t.right.assign(nn, -1);
  t.face.assign(nn, -1);
  t.depth.assign(nn, 0);
  bvh_detail::Builder b{ext, centers, t};
  const int root = 0;
  if (nfaces == 1) {
    t.face[root] = buf[0];
    t.leaf_of_face[buf[0]] = root;
  } else {
    int split = (int)left_idx;
    if (left_idx == 0 || (int)left_idx == nfaces) split = nfaces / 2;
    t.left[root] = 1;
    t.right[root] = 2 * split;
    if (par) {
      std::vector<bvh_detail::Builder::Task> tasks;
      b.top(buf.data(), split, 1, 1, 2, 256, tasks);
      b.top(buf.data() + split, nfaces - split, 1, 2 * split, 2, 256, tasks);
      pool->run((int)tasks.size(), [&](int i) {
        const bvh_detail::Builder::Task& k = tasks[i];
        b.node(k.lst, k.num, k.dep, k.idx, 1);
      });
    } else {
      const int threads = nfaces > 16384 ? 8 : 1;
      auto lf = std::async(threads > 1 ? std::launch::async : std::launch::deferred,
                           [&] { b.node(buf.data(), split, 1, 1, threads / 2); });
      b.node(buf.data() + split, nfaces - split, 1, 2 * split, threads - threads / 2);
      lf.get();
    }
  }
  for (int d : t.depth) t.max_depth = d > t.max_depth ? d : t.max_depth;
  // leaf ranks (left to right) and upper nodes
  std::vector<int> stack{root};
  int r = 0;
  while (!stack.empty()) {
    const int n = stack.back();
    stack.pop_back();
    if (t.face[n] >= 0) {
      t.rank[t.face[n]] = r++;
    } else {
      stack.push_back(t.right[n]);
      stack.push_back(t.left[n]);
    }
  }
  std::vector<int> up{root};
  while ((int)up.size() < 8) {
    std::vector<int> ch;
    for (int n : up) {
      if (t.face[n] >= 0) ch.push_back(n);
      else { ch.push_back(t.left[n]); ch.push_back(t.right[n]); }
    }
    if (ch.size() == up.size()) break;
    up = ch;
  }
  for (int u = 0; u < (int)up.size(); ++u) {
    std::vector<int> st{up[u]};
    while (!st.empty()) {
      const int n = st.back();
      st.pop_back();
      if (t.face[n] >= 0) t.upper[t.face[n]] = u;
      else { st.push_back(t.left[n]); st.push_back(t.right[n]); }
    }
  }
  return t;
}

// Is face a the first of the pair (a, b) the reference reports (both cloth
// faces)? Inside one upper node the first lies in the left subtree of the
// two faces' lowest common ancestor (for_overlapping_faces(node)); across two
// upper nodes the first lies under the later one (the m < n loop of
// src/Collision.cpp:269-281).
YS_HD bool bvh_first(int upper_a, int rank_a, int upper_b, int rank_b) {
  return upper_a == upper_b ? rank_a < rank_b : upper_a > upper_b;
}

}  // namespace ys
