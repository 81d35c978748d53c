"""ctypes binding for the CPU oracle (oracle/yarn_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker, and by ``bench.py`` for the CPU-baseline leg. The GPU product
never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libyarn_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)


class _Desc(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("length", ctypes.c_int),
        ("height", ctypes.c_double), ("L", ctypes.c_double), ("R", ctypes.c_double),
        ("pose", ctypes.c_int), ("weave", ctypes.c_int),
        ("warp_rho", _dp), ("warp_Y", _dp), ("warp_B", _dp),
        ("weft_rho", _dp), ("weft_Y", _dp), ("weft_B", _dp),
        ("kc", ctypes.c_double), ("kf", ctypes.c_double), ("df", ctypes.c_double),
        ("mu", ctypes.c_double), ("S", ctypes.c_double), ("handle_stiffness", ctypes.c_double),
        ("G", ctypes.c_double * 3), ("wind_vel", ctypes.c_double * 3),
        ("wind_density", ctypes.c_double), ("wind_drag", ctypes.c_double),
        ("n_handles", ctypes.c_int), ("handles", ctypes.POINTER(ctypes.c_int)),
    ]


class _Stats(ctypes.Structure):
    _fields_ = [("cg_iterations", ctypes.c_long), ("cg_error", ctypes.c_double), ("status", ctypes.c_int)]


def build():
    """Compile oracle/_build/libyarn_oracle.so (plain C, a second or two)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "yarn_oracle.c")):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.yo_create.restype = ctypes.c_void_p
        L.yo_create.argtypes = [ctypes.POINTER(_Desc)]
        L.yo_destroy.argtypes = [ctypes.c_void_p]
        L.yo_num_nodes.argtypes = [ctypes.c_void_p]
        L.yo_dim.argtypes = [ctypes.c_void_p]
        L.yo_set_state.argtypes = [ctypes.c_void_p] + [_dp] * 6
        L.yo_get_state.argtypes = [ctypes.c_void_p] + [_dp] * 6
        L.yo_get_normals.argtypes = [ctypes.c_void_p, _dp]
        L.yo_set_wind.argtypes = [ctypes.c_void_p, _dp]
        L.yo_fill.argtypes = [ctypes.c_void_p]
        L.yo_export_dense.argtypes = [ctypes.c_void_p] + [_dp] * 6
        L.yo_export_system.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp]
        L.yo_step.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, ctypes.c_double, ctypes.c_long,
                              ctypes.POINTER(_Stats)]
        L.yo_step.restype = ctypes.c_int
        L.yo_dense_pcg.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_long, _dp]
        L.yo_dense_pcg.restype = ctypes.c_long
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp) if a is not None else None


@dataclass
class ClothSpec:
    """Construction parameters, in the reference's own units.

    Mirrors ``Cloth(width, length, height, L, R, yarns, kc, kf, df, mu, S,
    handle_stiffness, WovenPattern, InitPose)`` (src/Cloth.h:55-60) plus the
    Environment's gravity and wind (src/Environment.h, src/Wind.h). Yarn
    material is given per yarn line: warp lines are node rows (length
    entries), weft lines are node columns (width entries); each entry is
    (rho, Y, B) with ks = Y*PI*R^2 and kb = B*PI*R^2 (src/Yarn.h:12-16).
    """
    width: int
    length: int
    warp: np.ndarray  # [length, 3] (rho, Y, B)
    weft: np.ndarray  # [width, 3]
    height: float = 0.05
    L: float = 1e-3
    R: float = 1e-4
    pose: int = 1          # 0 upright, 1 flat
    weave: int = 0         # 0 plain, 1 twill, 2 satin
    kc: float = 1.0
    kf: float = 1000.0
    df: float = 1000.0
    mu: float = 0.3
    S: float = 1e-4
    handle_stiffness: float = 1e4
    G: tuple = (0.0, 0.0, 9.8)
    wind_vel: tuple = (0.0, 0.0, 0.0)
    wind_density: float = 0.0
    wind_drag: float = 0.0
    handles: list = field(default_factory=list)


class OracleCloth:
    """One cloth simulated by the CPU oracle."""

    def __init__(self, spec: ClothSpec):
        self.spec = spec
        L = lib()
        self._keep = []
        warp = np.ascontiguousarray(np.asarray(spec.warp, dtype=np.float64).reshape(spec.length, 3).T.copy())
        weft = np.ascontiguousarray(np.asarray(spec.weft, dtype=np.float64).reshape(spec.width, 3).T.copy())
        self._keep += [warp, weft]
        h = np.asarray(spec.handles, dtype=np.int32).reshape(-1)
        self._keep.append(h)
        d = _Desc()
        d.width, d.length = spec.width, spec.length
        d.height, d.L, d.R = spec.height, spec.L, spec.R
        d.pose, d.weave = spec.pose, spec.weave
        d.warp_rho, d.warp_Y, d.warp_B = _p(warp[0]), _p(warp[1]), _p(warp[2])
        d.weft_rho, d.weft_Y, d.weft_B = _p(weft[0]), _p(weft[1]), _p(weft[2])
        d.kc, d.kf, d.df, d.mu, d.S = spec.kc, spec.kf, spec.df, spec.mu, spec.S
        d.handle_stiffness = spec.handle_stiffness
        d.G = (ctypes.c_double * 3)(*spec.G)
        d.wind_vel = (ctypes.c_double * 3)(*spec.wind_vel)
        d.wind_density, d.wind_drag = spec.wind_density, spec.wind_drag
        d.n_handles = len(h) // 2
        d.handles = h.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if len(h) else None
        self._h = L.yo_create(ctypes.byref(d))
        if not self._h:
            raise ValueError("oracle rejected the cloth description")
        self.N = L.yo_num_nodes(self._h)
        self.dim = L.yo_dim(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().yo_destroy(self._h)
            self._h = None

    def get_state(self):
        N = self.N
        a = {k: np.zeros((N, 3)) for k in ("LPos", "LPosFix", "LVel")}
        a.update({k: np.zeros((N, 2)) for k in ("EPos", "EPosBar", "EVel")})
        lib().yo_get_state(self._h, _p(a["LPos"]), _p(a["LPosFix"]), _p(a["LVel"]),
                           _p(a["EPos"]), _p(a["EPosBar"]), _p(a["EVel"]))
        return a

    def set_state(self, st):
        arrs = [np.ascontiguousarray(st[k], dtype=np.float64) if st.get(k) is not None else None
                for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")]
        lib().yo_set_state(self._h, *[_p(a) for a in arrs])

    def normals(self):
        n = np.zeros((self.N, 3))
        lib().yo_get_normals(self._h, _p(n))
        return n

    def set_wind(self, v):
        a = np.asarray(v, dtype=np.float64)
        lib().yo_set_wind(self._h, _p(a))

    def fill(self):
        lib().yo_fill(self._h)

    def dense(self):
        d = self.dim
        nc = (self.spec.width - 2) * (self.spec.length - 2)
        out = dict(M=np.zeros((d, d)), K=np.zeros((d, d)), D=np.zeros((d, d)), F=np.zeros(d), V=np.zeros(d),
                   slide=np.zeros(max(2 * nc, 1)))
        lib().yo_export_dense(self._h, _p(out["M"]), _p(out["K"]), _p(out["D"]), _p(out["F"]), _p(out["V"]),
                              _p(out["slide"]))
        return out

    def system(self, h, ext=None):
        d = self.dim
        A, b = np.zeros((d, d)), np.zeros(d)
        e = None if ext is None else np.ascontiguousarray(ext, dtype=np.float64)
        lib().yo_export_system(self._h, h, _p(e), _p(A), _p(b))
        return A, b

    def step(self, h, ext=None, cg_tol=0.0, cg_maxiter=-1):
        st = _Stats()
        e = None if ext is None else np.ascontiguousarray(ext, dtype=np.float64)
        lib().yo_step(self._h, h, _p(e), cg_tol, cg_maxiter, ctypes.byref(st))
        return dict(cg_iterations=st.cg_iterations, cg_error=st.cg_error, status=st.status)


def dense_pcg(A, b, tol=0.0, maxiter=-1):
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    err = ctypes.c_double()
    it = lib().yo_dense_pcg(len(b), _p(A), _p(b), _p(x), tol, maxiter, ctypes.byref(err))
    return x, it, err.value
