"""OBJ output of a cloth's state: the reference's RenderCloth
(src/Render.cpp:3-131) with its three forms and its exact text layout, fed
from the device state (positions from get_state, node normals from
ys_get_normals).

- MeshTriangle: "v" positions, "vt" grid texture coordinates, "vn" the mean
  of the unit normals of each node's adjacent cloth faces, "f v/vt/vn"
  triangles split along alternating diagonals (the cloth faces of
  src/Cloth.cpp:271-286).
- MeshRectangle: "v" positions and one quad "f" per grid cell.
- YarnSpline: the crimped yarn centre lines, warp nodes x - R n and weft nodes
  x + R n (src/Cloth.cpp:323-325; the node itself at the cloth border), as
  "l" polylines.

Numbers are written as the reference's streams write them: positions and
normals fixed with 5 decimals, texture coordinates with std::to_string's 6.
The reference computes its texture step 1 / (max(W, L) - 1) once per process
(a function-local static); here it is computed per call unless given.
"""
from __future__ import annotations

import enum
from typing import Optional

import numpy as np


class RenderType(enum.IntEnum):
    """src/Render.h:4-8"""
    MeshTriangle = 0
    MeshRectangle = 1
    YarnSpline = 2


def _f5(x: float) -> str:
    return "%.5f" % x


def cloth_faces(width: int, length: int):
    """Cloth faces [F, 3] (node ids u + v W) in the reference's order
    (src/Cloth.cpp:271-286): per cell (i, j) with i over u outer and j over v
    inner, the diagonal alternating with (i + j) % 2."""
    out = []
    for i in range(width - 1):
        for j in range(length - 1):
            tl, tr = i + j * width, i + 1 + j * width
            bl, br = i + (j + 1) * width, i + 1 + (j + 1) * width
            if (i + j) % 2 == 0:
                out += [(tl, tr, br), (tl, br, bl)]
            else:
                out += [(tl, tr, bl), (tr, br, bl)]
    return np.array(out, dtype=np.int64)


def vertex_normals(width: int, length: int, lpos: np.ndarray) -> np.ndarray:
    """Mean of the unit face normals of every node's adjacent faces, summed in
    face order (the reference keeps them in a set ordered by address, which is
    their order in the face vector)."""
    faces = cloth_faces(width, length)
    p = np.asarray(lpos, np.float64)
    c = np.cross(p[faces[:, 1]] - p[faces[:, 0]], p[faces[:, 2]] - p[faces[:, 0]])
    nrm = np.sqrt((c * c).sum(1))
    fn = np.where(nrm[:, None] == 0.0, c, c / np.where(nrm == 0.0, 1.0, nrm)[:, None])
    acc = np.zeros((width * length, 3))
    cnt = np.zeros(width * length, dtype=np.int64)
    for f, tri in enumerate(faces):
        for node in sorted(set(int(t) for t in tri)):
            acc[node] += fn[f]
            cnt[node] += 1
    return acc / np.maximum(cnt, 1)[:, None]


def obj_text(width: int, length: int, lpos: np.ndarray, kind: RenderType, normals: Optional[np.ndarray] = None,
             R: float = 0.0, unit_uv: Optional[float] = None) -> str:
    """The OBJ text RenderCloth writes for positions lpos [W L, 3] (node
    u + v W); YarnSpline needs the node normals and the yarn radius R."""
    W, L = int(width), int(length)
    p = np.asarray(lpos, np.float64).reshape(W * L, 3)
    out = ["o cloth\n"]
    if kind == RenderType.MeshTriangle:
        uv = 1.0 / (max(W, L) - 1) if unit_uv is None else unit_uv
        for i in range(L):
            for j in range(W):
                out.append("v " + "".join(_f5(x) + " " for x in p[j + i * W]) + "\n")
        for i in range(L):
            for j in range(W):
                out.append("vt %f %f\n" % (j * uv, i * uv))
        vn = vertex_normals(W, L, p)
        for i in range(L):
            for j in range(W):
                out.append("vn " + "".join(_f5(x) + " " for x in vn[j + i * W]) + "\n")
        for i in range(L - 1):
            for j in range(W - 1):
                tl, tr = j + i * W + 1, j + 1 + i * W + 1
                bl, br = j + (i + 1) * W + 1, j + 1 + (i + 1) * W + 1
                tri = [(tl, tr, br), (tl, br, bl)] if (i + j) % 2 == 0 else [(tl, tr, bl), (tr, br, bl)]
                for t in tri:
                    out.append("f " + " ".join("%d/%d/%d" % (k, k, k) for k in t) + "\n")
    elif kind == RenderType.MeshRectangle:
        for i in range(L):
            for j in range(W):
                out.append("v " + "".join(_f5(x) + " " for x in p[j + i * W]) + "\n")
        for i in range(L - 1):
            for j in range(W - 1):
                tl, tr = j + i * W + 1, j + 1 + i * W + 1
                bl, br = j + (i + 1) * W + 1, j + 1 + (i + 1) * W + 1
                out.append("f %d %d %d %d\n" % (tl, tr, br, bl))
    else:
        if normals is None:
            raise ValueError("YarnSpline needs the node normals")
        n = np.asarray(normals, np.float64).reshape(W * L, 3)

        def crimp(u, v, sign):
            i = u + v * W
            if 1 <= u <= W - 2 and 1 <= v <= L - 2:
                return p[i] + sign * R * n[i]
            return p[i]
        for v in range(1, L - 1):
            for u in range(W):
                out.append("v " + "".join(_f5(x) + " " for x in crimp(u, v, -1.0)) + "\n")
        for u in range(1, W - 1):
            for v in range(L):
                out.append("v " + "".join(_f5(x) + " " for x in crimp(u, v, 1.0)) + "\n")
        for v in range(1, L - 1):
            for u in range(W - 1):
                out.append("l %d %d \n" % ((v - 1) * W + u + 1, (v - 1) * W + u + 2))
        for u in range(1, W - 1):
            for v in range(L - 1):
                out.append("l %d %d \n" % ((L - 2) * W + (u - 1) * L + v + 1, (L - 2) * W + (u - 1) * L + v + 2))
    return "".join(out)


def render_batch_cloth(batch, c: int, save_path: str, kind: RenderType, unit_uv: Optional[float] = None):
    """Writes cloth c of a ClothBatch as RenderCloth would."""
    sl = batch.node_slice(c)
    spec = batch.specs[c]
    st = batch.get_state()
    normals = batch.normals()[sl] if kind == RenderType.YarnSpline else None
    text = obj_text(spec.width, spec.length, st["LPos"][sl], kind, normals, spec.R, unit_uv)
    with open(save_path, "w") as f:
        f.write(text)
    return text


def RenderCloth(cloth, save_path: str, type: RenderType = RenderType.MeshTriangle):  # noqa: A002
    """src/Render.cpp:3: the reference's entry point for a Cloth whose
    PhysicsCloth has been built (its state lives on the GPU)."""
    if cloth._batch is None:
        raise RuntimeError("RenderCloth needs the cloth's PhysicsCloth (its state lives on the GPU)")
    return render_batch_cloth(cloth._batch, 0, save_path, RenderType(type))
