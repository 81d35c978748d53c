"""Continuous collision detection of a cloth mesh against itself and an
obstacle mesh on the GPU: the reference's Collision::find_impacts
(src/Collision.cpp:184-208) -- its 18-DOP BVH broad phase and the
vertex-face / edge-edge narrow phase -- behind the C ABI's ys_collider_*,
and the impact-zone response around it (Collision::collision_response,
src/Collision.cpp:73-156) with the backward of its projections.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _native as N


def cloth_mesh_topology(width: int, length: int):
    """(faces [F, 3], face_edges [F, 3, 2]) of a width x length cloth's mesh in
    the reference's order (src/Cloth.cpp:271-294)."""
    F = 2 * (width - 1) * (length - 1)
    faces = np.zeros((F, 3), np.int32)
    edges = np.zeros((F, 3, 2), np.int32)
    N.check(N.load().ys_cloth_mesh_topology(int(width), int(length), ctypes.c_void_p(faces.ctypes.data),
                                            ctypes.c_void_p(edges.ctypes.data)), "ys_cloth_mesh_topology")
    return faces, edges


def icosphere(radius: float, levels: int, center=(0.0, 0.0, 0.0)):
    """An obstacle mesh: vertices [V, 3] and faces [F, 3] (int32) of an
    icosahedron subdivided `levels` times onto a sphere (F = 20 * 4^levels)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [np.array(p, float) / np.linalg.norm(p) for p in
         [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
          (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(levels):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                p = v[a] + v[b]
                v.append(p / np.linalg.norm(p))
                mid[k] = len(v) - 1
            return mid[k]
        nf = []
        for (a, b, c) in f:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.asarray(center, float) + radius * np.array(v), np.array(f, np.int32)


class Collider:
    """Broad and narrow phase for one cloth of width x length nodes
    (node u + v * width) and an optional obstacle (vertices [No, 3], faces
    [Fo, 3]). thickness dilates the boxes (Collision::thickness); ccd = True
    makes every box span the step's start and end positions."""

    def __init__(self, width: int, length: int, obstacle_faces: Optional[np.ndarray] = None,
                 n_obstacle_nodes: int = 0, thickness: float = 5e-4, ccd: bool = True, device: int = 0,
                 stream: Optional[int] = None):
        self.width, self.length = int(width), int(length)
        self.n_nodes = self.width * self.length
        self.faces, self.face_edges = cloth_mesh_topology(self.width, self.length)
        of = np.zeros((0, 3), np.int32) if obstacle_faces is None else np.ascontiguousarray(obstacle_faces, np.int32)
        self.obstacle_faces = of
        self.n_obs_nodes = int(n_obstacle_nodes)
        h = ctypes.c_void_p()
        N.check(N.load().ys_collider_create(self.n_nodes, len(self.faces), ctypes.c_void_p(self.faces.ctypes.data),
                                            ctypes.c_void_p(self.face_edges.ctypes.data), self.n_obs_nodes, len(of),
                                            ctypes.c_void_p(of.ctypes.data) if len(of) else None, float(thickness),
                                            int(bool(ccd)), int(device), ctypes.c_void_p(stream) if stream else None,
                                            ctypes.byref(h)), "ys_collider_create")
        self._h = h
        self._n_received = 0

    def close(self):
        if getattr(self, "_h", None):
            N.load().ys_collider_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_positions(self, x, x_prev, obs_x=None, obs_x_prev=None):
        """Node positions at the end / start of the step, [n, 3] float64 (host)."""
        arrs = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (x, x_prev, obs_x, obs_x_prev)]
        ptr = [ctypes.c_void_p(a.ctypes.data) if a is not None else None for a in arrs]
        N.check(N.load().ys_collider_set_positions(self._h, *ptr, 0), "ys_collider_set_positions")

    def pairs(self) -> np.ndarray:
        """Broad phase: [P, 3] int32 (first face, second face, 1 if obstacle)."""
        n = ctypes.c_int64()
        N.check(N.load().ys_collider_find_pairs(self._h, ctypes.byref(n)), "ys_collider_find_pairs")
        out = np.zeros((n.value, 3), np.int32)
        N.check(N.load().ys_collider_get_pairs(self._h, ctypes.c_void_p(out.ctypes.data), n.value),
                "ys_collider_get_pairs")
        return out

    def impacts(self) -> dict:
        """Narrow phase over the last pair list: dict of arrays type [I],
        nodes [I, 4] (obstacle nodes as -1 - id), t [I], w [I, 4], n [I, 3],
        pair [I]."""
        n = ctypes.c_int64()
        N.check(N.load().ys_collider_find_impacts(self._h, ctypes.byref(n)), "ys_collider_find_impacts")
        buf = (N.Impact * max(n.value, 1))()
        N.check(N.load().ys_collider_get_impacts(self._h, buf, n.value), "ys_collider_get_impacts")
        a = np.ctypeslib.as_array(buf)[:n.value]
        return dict(type=a["type"].copy(), nodes=a["nodes"].copy(), t=a["t"].copy(), w=a["w"].copy(),
                    n=a["n"].copy(), pair=a["pair"].copy())

    def set_max_zone_impacts(self, n: int):
        """The response stops (zone_overflow) when a zone gathers more than n
        impacts (default 256)."""
        N.check(N.load().ys_collider_set_max_zone_impacts(self._h, int(n)), "ys_collider_set_max_zone_impacts")

    def respond(self, v=None, mass=None, h: float = 1e-3, damp: float = 0.1, max_iter: int = 100,
                check: bool = True) -> dict:
        """collision_response(damp) over the positions of the last
        set_positions: rounds of GPU detection, independent impacts, impact
        zones and their exact inelastic projections, then v + damp (x - x_before)
        / h when a zone moved. v [n, 3] and mass [n] are optional. Returns
        dict(x, v, rounds, converged, changed, zones, infeasible, zone_overflow,
        impacts, projections, reverted); raises when max_iter rounds still found impacts
        (where the reference exits) or a zone outgrew the zone limit
        (set_max_zone_impacts), unless check=False."""
        x = np.zeros((self.n_nodes, 3))
        vv = None if v is None else np.array(v, np.float64).reshape(self.n_nodes, 3).copy()
        m = None if mass is None else np.ascontiguousarray(mass, np.float64).reshape(self.n_nodes)
        info = N.ResponseInfo()
        st = N.load().ys_collider_respond(self._h, ctypes.c_void_p(m.ctypes.data) if m is not None else None,
                                          float(h), float(damp), int(max_iter), ctypes.c_void_p(x.ctypes.data),
                                          ctypes.c_void_p(vv.ctypes.data) if vv is not None else None,
                                          ctypes.byref(info))
        if st != N.YS_ERR_MAXITER or check:
            N.check(st, "ys_collider_respond")
        self._n_received = int(info.impacts)
        return dict(x=x, v=vv, rounds=info.rounds, converged=bool(info.converged), changed=bool(info.changed),
                    zones=info.zones, infeasible=info.infeasible, zone_overflow=bool(info.zone_overflow),
                    impacts=info.impacts, projections=info.projections, reverted=info.reverted,
                    detect_ms=info.detect_ms, zones_ms=info.zones_ms)

    def response_impacts(self) -> dict:
        """The impacts the zones of the last response received, in order
        (arrays as impacts(); "round" = the round that found each)."""
        n = self._n_received
        buf = (N.Impact * max(n, 1))()
        N.check(N.load().ys_collider_response_impacts(self._h, buf, n), "ys_collider_response_impacts")
        a = np.ctypeslib.as_array(buf)[:n]
        return dict(type=a["type"].copy(), nodes=a["nodes"].copy(), t=a["t"].copy(), w=a["w"].copy(),
                    n=a["n"].copy(), round=a["pair"].copy())

    def respond_backward(self, dl_dx=None, dl_dv=None, impacts: bool = False, exact_root: bool = False) -> dict:
        """Backward of the last respond(): gradients of x and v before it and
        of every received impact's weights [I, 4] and normal [I, 3]. With
        impacts=True those are carried on into the positions the impacts were
        computed from (x and x_prev, the reference's full autograd; the cubic
        root's derivative as the reference's CubicSolver backward unless
        exact_root)."""
        n3 = (self.n_nodes, 3)
        gx = None if dl_dx is None else np.ascontiguousarray(dl_dx, np.float64).reshape(n3)
        gv = None if dl_dv is None else np.ascontiguousarray(dl_dv, np.float64).reshape(n3)
        ni = self._n_received
        ox, ov, op = np.zeros(n3), np.zeros(n3), np.zeros(n3)
        gw, gn = np.zeros((max(ni, 1), 4)), np.zeros((max(ni, 1), 3))
        flags = (1 if impacts else 0) | (2 if exact_root else 0)
        p = lambda a: ctypes.c_void_p(a.ctypes.data) if a is not None else None
        N.check(N.load().ys_collider_respond_backward(self._h, p(gx), p(gv), flags, p(ox), p(ov), p(op), p(gw), p(gn)),
                "ys_collider_respond_backward")
        return dict(x=ox, v=ov, x_prev=op, w=gw[:ni], n=gn[:ni])

class Collision:
    """src/Collision.h:64-131 for one Cloth (a W x L cloth mesh) against one
    obstacle mesh (vertices [No, 3], faces [Fo, 3]; the reference's table and
    ground meshes merged into one report the same pairs, src/Collision.cpp:
    286-287). Obstacles are static: their positions before and after a step
    are the same. collision_response(damp, x, x_prev, v) runs the response on
    the GPU collider and returns whether anything moved; the result is in
    .last (respond()'s dict)."""
    max_iter = 100

    def __init__(self, cloth, obstacle_x=None, obstacle_faces=None, thickness: float = 5e-4, h: float = 1e-3,
                 ccd: bool = True, device: int = 0):
        self.thickness, self.h, self.ccd = float(thickness), float(h), bool(ccd)
        self.obs_x = np.zeros((0, 3)) if obstacle_x is None else np.ascontiguousarray(obstacle_x, np.float64)
        of = None if obstacle_faces is None else np.ascontiguousarray(obstacle_faces, np.int32)
        self.collider = Collider(cloth.width, cloth.length, obstacle_faces=of, n_obstacle_nodes=len(self.obs_x),
                                 thickness=self.thickness, ccd=self.ccd, device=device)
        self.last = None

    def collision_response(self, damp_fac: float, x, x_prev, v) -> bool:
        ox = self.obs_x if len(self.obs_x) else None
        self.collider.set_positions(x, x_prev, ox, ox)
        self.last = self.collider.respond(v=v, h=self.h, damp=damp_fac, max_iter=self.max_iter)
        return self.last["changed"]

    def close(self):
        self.collider.close()
