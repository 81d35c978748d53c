"""Scenes for the impact-zone response tests and ctypes helpers around the
test-only emulator's response (tests/emu)."""
import ctypes
import os

import numpy as np

import goldens
from emu_py import lib
from pkg import ys

_dp, _ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)


def topology(W, H):
    """The cloth mesh's faces and edges in the reference's order
    (src/Cloth.cpp:288-293: every cell split along tl-br, unlike the yarn
    faces)."""
    F, E = [], []
    for i in range(W - 1):
        for j in range(H - 1):
            tl = i + j * W
            tr, bl, br = tl + 1, tl + W, tl + W + 1
            for tri in ((tl, tr, br), (tl, br, bl)):
                F.append(tri)
                E.append([sorted((tri[a], tri[(a + 1) % 3])) for a in range(3)])
    return np.array(F, np.int32), np.array(E, np.int32)


def icosphere(radius, levels):
    return ys.collide.icosphere(radius, levels)


def drop_scene(W, depth=1e-3, spacing=1e-3, radius=0.02, levels=3, h=1e-3, seed=0):
    """A flat W x W cloth 2 mm above a sphere moving down 2 mm + depth in one
    step (small jitter), so its middle passes the sphere's top by depth."""
    ox, of = icosphere(radius, levels)
    u, v = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    xp = np.zeros((W * W, 3))
    xp[:, 0] = (u.reshape(-1) - (W - 1) / 2) * spacing
    xp[:, 1] = (v.reshape(-1) - (W - 1) / 2) * spacing
    xp[:, 2] = radius + 2e-3
    x = xp.copy()
    x[:, 2] -= 2e-3 + depth
    x += np.random.default_rng(seed).normal(0.0, 1e-5, x.shape)
    return dict(W=W, H=W, x=x, x_prev=xp, obs_x=ox, obs_faces=of, thickness=5e-4, h=h, v=(x - xp) / h)


def fixture_scene(name, h=1e-3):
    """A collision-detection fixture (tests/golden/collide_*.npz) as a scene."""
    g = dict(np.load(os.path.join(goldens.GOLDEN_DIR, name + ".npz")))
    W, H = int(g["width"]), int(g["length"])
    s = dict(W=W, H=H, x=g["x"], x_prev=g["x_prev"], thickness=float(g["thickness"]), h=h,
             v=(g["x"] - g["x_prev"]) / h)
    if "obs_x" in g:
        s["obs_x"], s["obs_faces"] = g["obs_x"], g["obs_faces"].astype(np.int32)
    else:
        s["obs_x"], s["obs_faces"] = np.zeros((0, 3)), np.zeros((0, 3), np.int32)
    return s


def _arrays(s):
    F, E = topology(s["W"], s["H"])
    c = lambda a, t=np.float64: np.ascontiguousarray(a, t)
    return F, E, c(s["x"]), c(s["x_prev"]), c(s["obs_x"]), c(s["obs_faces"], np.int32)


def _lib():
    L = lib()
    if not getattr(L, "_resp_types", False):
        c_l, c_d, c_i = ctypes.c_long, ctypes.c_double, ctypes.c_int
        L.emu_detect.argtypes = [c_i, _dp, _dp, _dp, c_i, _ip, _ip, c_i, _dp, _dp, c_i, _ip, c_d, c_i,
                                 ctypes.POINTER(ctypes.c_ubyte), _dp, c_l, ctypes.POINTER(c_l)]
        L.emu_respond.argtypes = [c_i, _dp, _dp, c_i, _ip, _ip, c_i, _dp, _dp, c_i, _ip, c_d, c_i, _dp, c_d, c_d, c_i,
                                  _dp, ctypes.POINTER(c_l)]
        L.emu_response_impacts.argtypes = [_dp, c_l]
        L.emu_respond_backward.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int, _dp]
        L.emu_ldp.argtypes = [c_i, c_i, _dp, _dp, _dp, _dp]
        L.emu_set_max_zone_impacts.argtypes = [c_i]
        L.emu_ldp_sparse.argtypes = [c_i, c_i, _ip, _dp, _dp, _dp, _dp]
        L.emu_ldp_sparse.restype = c_i
        for f in ("emu_detect", "emu_respond", "emu_response_impacts", "emu_respond_backward", "emu_ldp",
                  "emu_set_max_zone_impacts"):
            getattr(L, f).restype = c_i
        L._resp_types = True
    return L


def emu_detector(s):
    """detect(x, face_active) of the response's rounds, on the emulator."""
    L = _lib()
    F, E, x0, xp, ox, of = _arrays(s)
    n = s["W"] * s["H"]

    def detect(x, mask):
        xc = np.ascontiguousarray(x, np.float64)
        cap = 1 << 16
        while True:
            buf = np.zeros(15 * cap)
            ni = ctypes.c_long()
            m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
            L.emu_detect(n, x0.ctypes.data_as(_dp), xc.ctypes.data_as(_dp), xp.ctypes.data_as(_dp), len(F),
                         F.ctypes.data_as(_ip), E.ctypes.data_as(_ip), len(ox), ox.ctypes.data_as(_dp),
                         ox.ctypes.data_as(_dp), len(of), of.ctypes.data_as(_ip), s["thickness"], 1,
                         m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)) if m is not None else None,
                         buf.ctypes.data_as(_dp), cap, ctypes.byref(ni))
            if ni.value <= cap:
                break
            cap = ni.value
        rows = buf[:15 * ni.value].reshape(-1, 15)
        return [(int(r[0]), tuple(int(a) for a in r[1:5]), float(r[5]), tuple(r[6:10]), tuple(r[10:13]))
                for r in rows]
    return detect


def emu_respond(s, damp=0.1, max_iter=100, mass=None):
    """The product's response loop (csrc/ys_zones.h) on the emulator's
    detection: dict(x, v, info, impacts)."""
    L = _lib()
    F, E, x0, xp, ox, of = _arrays(s)
    n = s["W"] * s["H"]
    x = x0.copy()
    v = np.ascontiguousarray(s["v"], np.float64).copy()
    info = (ctypes.c_long * 9)()
    m = None if mass is None else np.ascontiguousarray(mass, np.float64)
    L.emu_respond(n, x.ctypes.data_as(_dp), xp.ctypes.data_as(_dp), len(F), F.ctypes.data_as(_ip),
                  E.ctypes.data_as(_ip), len(ox), ox.ctypes.data_as(_dp), ox.ctypes.data_as(_dp), len(of),
                  of.ctypes.data_as(_ip), ctypes.c_double(s["thickness"]), 1,
                  m.ctypes.data_as(_dp) if m is not None else None, ctypes.c_double(s["h"]), ctypes.c_double(damp),
                  int(max_iter), v.ctypes.data_as(_dp), info)
    na = info[5]
    imp = np.zeros(15 * max(na, 1))
    L.emu_response_impacts(imp.ctypes.data_as(_dp), na)
    return dict(x=x, v=v, info=list(info), impacts=imp[:15 * na].reshape(-1, 15))


def emu_respond_backward(gx, gv, n_impacts, flags=0):
    """Backward of the last emu_respond: (dL/dx before, dL/dw [I, 4],
    dL/dn [I, 3], dL/dx_prev)."""
    L = _lib()
    g = np.ascontiguousarray(gx, np.float64).copy()
    gvv = None if gv is None else np.ascontiguousarray(gv, np.float64)
    gw, gn = np.zeros((max(n_impacts, 1), 4)), np.zeros((max(n_impacts, 1), 3))
    gp = np.zeros_like(g)
    L.emu_respond_backward(g.ctypes.data_as(_dp), gvv.ctypes.data_as(_dp) if gvv is not None else None,
                           gw.ctypes.data_as(_dp), gn.ctypes.data_as(_dp), int(flags), gp.ctypes.data_as(_dp))
    return g, gw[:n_impacts], gn[:n_impacts], gp


def emu_ldp(G, h):
    L = _lib()
    G = np.ascontiguousarray(G, np.float64)
    h = np.ascontiguousarray(h, np.float64)
    k, n = G.shape
    u, lam = np.zeros(n), np.zeros(k)
    st = L.emu_ldp(n, k, G.ctypes.data_as(_dp), h.ctypes.data_as(_dp), u.ctypes.data_as(_dp), lam.ctypes.data_as(_dp))
    return u, lam, st


def emu_ldp_sparse(cols, coef, h, n):
    """The large-zone solver: cols [k, 4] (column blocks, -1 unused),
    coef [k, 4, 3]; returns (u, lam, status)."""
    L = _lib()
    cols = np.ascontiguousarray(cols, np.int32)
    coef = np.ascontiguousarray(coef, np.float64)
    h = np.ascontiguousarray(h, np.float64)
    k = len(h)
    u, lam = np.zeros(n), np.zeros(k)
    st = L.emu_ldp_sparse(n, k, cols.ctypes.data_as(_ip), coef.ctypes.data_as(_dp), h.ctypes.data_as(_dp),
                          u.ctypes.data_as(_dp), lam.ctypes.data_as(_dp))
    return u, lam, st
