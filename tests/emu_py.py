"""TEST-ONLY ctypes binding of tests/emu (host emulation of the GPU step)."""
import ctypes
import os
import subprocess

import numpy as np

from layout import slots_to_dense

HERE = os.path.dirname(os.path.abspath(__file__))
EMU_DIR = os.path.join(HERE, "emu")
_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


class CDesc(ctypes.Structure):
    """ys_cloth_desc (include/yarnsim.h)."""
    _fields_ = [
        ("width", ctypes.c_int32), ("length", ctypes.c_int32),
        ("height", ctypes.c_double), ("L", ctypes.c_double), ("R", ctypes.c_double),
        ("pose", ctypes.c_int32), ("weave", ctypes.c_int32),
        ("warp_rho", _dp), ("warp_Y", _dp), ("warp_B", _dp),
        ("weft_rho", _dp), ("weft_Y", _dp), ("weft_B", _dp),
        ("kc", ctypes.c_double), ("kf", ctypes.c_double), ("df", ctypes.c_double),
        ("mu", ctypes.c_double), ("S", ctypes.c_double), ("handle_stiffness", ctypes.c_double),
        ("G", ctypes.c_double * 3), ("wind_vel", ctypes.c_double * 3),
        ("wind_density", ctypes.c_double), ("wind_drag", ctypes.c_double),
        ("n_handles", ctypes.c_int32), ("handles", ctypes.POINTER(ctypes.c_int32)),
    ]


def make_desc(kw, keep):
    W, H = kw["width"], kw["length"]
    warp = np.ascontiguousarray(np.asarray(kw["warp"], float).reshape(H, 3).T.copy())
    weft = np.ascontiguousarray(np.asarray(kw["weft"], float).reshape(W, 3).T.copy())
    hd = np.asarray(kw.get("handles", []), dtype=np.int32).reshape(-1)
    keep += [warp, weft, hd]
    d = CDesc()
    d.width, d.length = W, H
    d.height, d.L, d.R = kw.get("height", 0.05), kw.get("L", 1e-3), kw.get("R", 1e-4)
    d.pose, d.weave = kw.get("pose", 1), kw.get("weave", 0)
    p = lambda a: a.ctypes.data_as(_dp)
    d.warp_rho, d.warp_Y, d.warp_B = p(warp[0]), p(warp[1]), p(warp[2])
    d.weft_rho, d.weft_Y, d.weft_B = p(weft[0]), p(weft[1]), p(weft[2])
    d.kc, d.kf, d.df = kw.get("kc", 1.0), kw.get("kf", 1000.0), kw.get("df", 1000.0)
    d.mu, d.S, d.handle_stiffness = kw.get("mu", 0.3), kw.get("S", 1e-4), kw.get("handle_stiffness", 1e4)
    d.G = (ctypes.c_double * 3)(*kw.get("G", (0, 0, 9.8)))
    d.wind_vel = (ctypes.c_double * 3)(*kw.get("wind_vel", (0, 0, 0)))
    d.wind_density, d.wind_drag = kw.get("wind_density", 0.0), kw.get("wind_drag", 0.0)
    d.n_handles = len(hd) // 2
    d.handles = hd.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if len(hd) else None
    return d


def lib():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", EMU_DIR], check=True)
        L = ctypes.CDLL(os.path.join(EMU_DIR, "_build", "libys_emu.so"))
        L.emu_create.restype = ctypes.c_void_p
        L.emu_create.argtypes = [ctypes.POINTER(CDesc)]
        L.emu_destroy.argtypes = [ctypes.c_void_p]
        L.emu_set_state.argtypes = [ctypes.c_void_p] + [_dp] * 6
        L.emu_get_state.argtypes = [ctypes.c_void_p] + [_dp] * 6
        L.emu_get_normals.argtypes = [ctypes.c_void_p, _dp]
        L.emu_assemble.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp]
        L.emu_raw.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.emu_solve.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_long, _dp]
        L.emu_solve.restype = ctypes.c_long
        L.emu_apply.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.emu_update.argtypes = [ctypes.c_void_p]
        L.emu_update.restype = ctypes.c_int
        L.emu_tangent_count.restype = ctypes.c_int
        L.emu_tangent_init.argtypes = [ctypes.c_void_p]
        L.emu_tangent_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.emu_tangent_seed.argtypes = [ctypes.c_void_p] + [_dp] * 5
        L.emu_tangent_state.argtypes = [ctypes.c_void_p] + [_dp] * 5 + [ctypes.c_int]
        L.emu_step_tangent.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, ctypes.c_double, ctypes.c_int]
        L.emu_step_tangent.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


class EmuCloth:
    def __init__(self, **kw):
        self.keep = []
        self.W, self.H = kw["width"], kw["length"]
        self.N = self.W * self.H
        self.d = make_desc(kw, self.keep)
        self.h = lib().emu_create(ctypes.byref(self.d))

    def __del__(self):
        if getattr(self, "h", None):
            lib().emu_destroy(self.h)

    def set_state(self, st):
        arr = [None if st.get(k) is None else np.ascontiguousarray(st[k], float)
               for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")]
        lib().emu_set_state(self.h, *[_p(a) for a in arr])

    def get_state(self):
        N = self.N
        a = {k: np.zeros((N, 3)) for k in ("LPos", "LPosFix", "LVel")}
        a.update({k: np.zeros((N, 2)) for k in ("EPos", "EPosBar", "EVel")})
        lib().emu_get_state(self.h, *[_p(a[k]) for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")])
        return a

    def normals(self):
        n = np.zeros((self.N, 3))
        lib().emu_get_normals(self.h, _p(n))
        return n

    def assemble(self, h, ext5=None):
        e = None if ext5 is None else np.ascontiguousarray(ext5, float)
        lib().emu_assemble(self.h, h, _p(e))

    def system(self):
        slots = np.zeros((159, self.N))
        rhs = np.zeros((5, self.N))
        lib().emu_raw(self.h, _p(slots), _p(rhs))
        return slots_to_dense(slots, rhs, self.W, self.H)

    def solve(self, tol=0.0, maxiter=-1):
        err = ctypes.c_double()
        it = lib().emu_solve(self.h, tol, maxiter, ctypes.byref(err))
        return it, err.value

    def update(self):
        return lib().emu_update(self.h)

    # ---- forward-mode tangents (K directions per step)
    @property
    def K(self):
        return int(lib().emu_tangent_count())

    def tangent_init(self, mode=0):
        """mode 0: exact tangents; 1: the reference's gradient path (M, D, A
        held constant, transposed solves)."""
        lib().emu_tangent_init(self.h)
        lib().emu_tangent_mode(self.h, int(mode))

    def tangent_seed(self, drho=None, dY=None, dB=None, dS=None, dmu=None):
        """drho, dY, dB: [K][lines] (warp rows then weft columns); dS, dmu: [K]."""
        a = [None if x is None else np.ascontiguousarray(x, float) for x in (drho, dY, dB, dS, dmu)]
        lib().emu_tangent_seed(self.h, *[_p(x) for x in a])

    def tangent_set_state(self, dlpos=None, dlvel=None, depos=None, deposbar=None, devel=None):
        a = [None if x is None else np.ascontiguousarray(x, float) for x in (dlpos, dlvel, depos, deposbar, devel)]
        lib().emu_tangent_state(self.h, *[_p(x) for x in a], 1)

    def tangent_get_state(self):
        K, N = self.K, self.N
        out = dict(LPos=np.zeros((K, N, 3)), LVel=np.zeros((K, N, 3)), EPos=np.zeros((K, N, 2)),
                   EPosBar=np.zeros((K, N, 2)), EVel=np.zeros((K, N, 2)))
        lib().emu_tangent_state(self.h, *[_p(out[k]) for k in ("LPos", "LVel", "EPos", "EPosBar", "EVel")], 0)
        return out

    def step_tangent(self, h, ext5=None, tol=1e-14, kact=None):
        kact = self.K if kact is None else kact
        e = None if ext5 is None else np.ascontiguousarray(ext5, float)
        return lib().emu_step_tangent(self.h, h, _p(e), tol, kact)

    def step(self, h, ext5=None, tol=0.0, maxiter=-1):
        self.assemble(h, ext5)
        it, err = self.solve(tol, maxiter)
        st = self.update()
        return dict(cg_iterations=it, cg_error=err, status=st)
