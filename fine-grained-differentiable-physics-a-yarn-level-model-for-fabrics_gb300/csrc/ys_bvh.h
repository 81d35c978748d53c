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

#include <cstdint>
#include <vector>

#include "ys_collide.cuh"

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

struct Builder {
  const std::vector<Kdop>& boxes;
  const std::vector<double>& centers;  // [F][3]
  BvhTree& t;
  int add_node(int dep) {
    t.left.push_back(-1);
    t.right.push_back(-1);
    t.face.push_back(-1);
    t.depth.push_back(dep);
    if (dep > t.max_depth) t.max_depth = dep;
    return (int)t.face.size() - 1;
  }
  int leaf(int f, int dep) {
    const int n = add_node(dep);
    t.face[n] = f;
    t.leaf_of_face[f] = n;
    return n;
  }
  // BVHNode(parent, lst, lst_num, ...) (src/BVH.cpp:178-223)
  int node(int* lst, int num, int dep) {
    if (num == 1) return leaf(lst[0], dep);
    const int n = add_node(dep);
    if (num == 2) {
      const int l = leaf(lst[0], dep + 1);
      const int r = leaf(lst[1], dep + 1);
      t.left[n] = l;
      t.right[n] = r;
      return n;
    }
    Kdop box;
    kdop_empty(box);
    for (int q = 0; q < num; ++q) kdop_add(box, boxes[lst[q]]);
    const Aap pln(box);
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
    const int l = node(lst, split, dep + 1);
    const int r = node(lst + split, num - split, dep + 1);
    t.left[n] = l;
    t.right[n] = r;
    return n;
  }
};

}  // namespace bvh_detail

// Builds the tree of faces [F] with nodes at x / xp ([n][3] each, xp used
// under CCD); face v[k] are node ids into x (this routine never sees
// obstacle ids). verts: the mesh's vertex order for the root box (node ids).
inline BvhTree bvh_build(int nfaces, const int* fv, int nverts, const int* verts, const double* x, const double* xp,
                         bool ccd) {
  BvhTree t;
  t.leaf_of_face.assign(nfaces, -1);
  t.rank.assign(nfaces, 0);
  t.upper.assign(nfaces, 0);
  if (nfaces == 0) return t;
  Kdop total;
  kdop_empty(total);
  for (int i = 0; i < nverts; ++i) {
    kdop_add_point(total, x + 3 * (size_t)verts[i]);
    if (ccd) kdop_add_point(total, xp + 3 * (size_t)verts[i]);
  }
  std::vector<Kdop> boxes(nfaces);
  std::vector<double> centers(3 * (size_t)nfaces);
  const bvh_detail::Aap pln(total);
  std::vector<int> buf(nfaces);
  unsigned left_idx = 0, right_idx = (unsigned)nfaces;
  for (int f = 0; f < nfaces; ++f) {
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
    if (pln.inside(&centers[3 * (size_t)f])) buf[left_idx++] = f;
    else buf[--right_idx] = f;
    kdop_empty(boxes[f]);
    for (int k = 0; k < 3; ++k) kdop_add_point(boxes[f], p[k]);
    if (ccd)
      for (int k = 0; k < 3; ++k) kdop_add_point(boxes[f], pp[k]);
  }
  bvh_detail::Builder b{boxes, centers, t};
  const int root = b.add_node(0);
  if (nfaces == 1) {
    t.face[root] = buf[0];
    t.leaf_of_face[buf[0]] = root;
  } else {
    int split = (int)left_idx;
    if (left_idx == 0 || (int)left_idx == nfaces) split = nfaces / 2;
    const int l = b.node(buf.data(), split, 1);
    const int r = b.node(buf.data() + split, nfaces - split, 1);
    t.left[root] = l;
    t.right[root] = r;
  }
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
