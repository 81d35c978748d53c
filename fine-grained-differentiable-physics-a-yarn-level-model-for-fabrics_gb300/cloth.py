"""Host-side mirror of the reference's cloth interface over the C ABI.

``ClothBatch`` is the native object: any number of cloths of uneven sizes
stepped together on one GPU. ``Cloth``, ``Environment``, ``PhysicsCloth``,
``SimStep`` and ``EigenSolver`` keep the reference's names and argument
meaning (src/Cloth.h, src/Environment.h, src/PhysicsCloth.h,
src/TrainHelper.h:10-14, src/Solvers.h:35-52) for a single cloth, so a driver
loop like SimHomo (src/Simulate.h:78-101) reads the same.
"""
from __future__ import annotations

import collections.abc
import ctypes
import enum
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N

PI = 3.1415926535897  # src/Constants.h:24


class StepStats(collections.abc.Sequence):
    """Per-cloth results of a solve or step (the C ABI's ys_cloth_stats
    array): a sequence of dicts {ok, cg_iterations, cg_error, hit_maxiter},
    each built when it is read, and whole-batch aggregates computed over the
    array, so a step of many cloths costs no per-cloth Python work unless
    its entries are read."""

    _dtype = None

    def __init__(self, arr):
        if StepStats._dtype is None:
            StepStats._dtype = np.ctypeslib.as_array(arr).dtype
        self._a = np.frombuffer(arr, dtype=StepStats._dtype)

    def __len__(self):
        return len(self._a)

    def _one(self, s):
        return dict(ok=bool(s["ok"]), cg_iterations=int(s["cg_iterations"]), cg_error=float(s["cg_error"]),
                    hit_maxiter=bool(s["hit_maxiter"]))

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self._one(s) for s in self._a[i]]
        return self._one(self._a[i])

    def __eq__(self, other):
        return list(self) == list(other)

    def __repr__(self):
        return repr(list(self))

    @property
    def all_ok(self) -> bool:
        return bool(np.all(self._a["ok"] != 0))

    @property
    def max_iterations(self) -> int:
        return int(self._a["cg_iterations"].max()) if len(self._a) else 0

    @property
    def max_error(self) -> float:
        return float(self._a["cg_error"].max()) if len(self._a) else 0.0

    @property
    def iterations(self) -> np.ndarray:
        return self._a["cg_iterations"].copy()


class WovenPattern(enum.IntEnum):
    Plain = 0
    Twill = 1
    Satin = 2


class InitPose(enum.IntEnum):
    Upright = 0
    Flat = 1


@dataclass
class Yarn:
    """src/Yarn.h:6-17: ks = Y*PI*R^2, kb = B*PI*R^2."""
    R: float
    rho: float
    Y: float
    B: float

    @property
    def ks(self):
        return self.Y * PI * self.R ** 2

    @property
    def kb(self):
        return self.B * PI * self.R ** 2


@dataclass
class Wind:
    """src/Wind.h:6-17"""
    WindVelocity: Sequence[float] = (0.0, 0.0, 0.0)
    WindDensity: float = 0.0
    WindDrag: float = 0.0


@dataclass
class ClothState:
    """src/Cloth.h:22-29, node order u + v*W."""
    LPos: np.ndarray
    LPosFix: np.ndarray
    LVel: np.ndarray
    EPos: np.ndarray
    EPosBar: np.ndarray
    EVel: np.ndarray

    def as_dict(self):
        return dict(LPos=self.LPos, LPosFix=self.LPosFix, LVel=self.LVel, EPos=self.EPos, EPosBar=self.EPosBar,
                    EVel=self.EVel)


@dataclass
class ClothSpec:
    """Construction parameters of one cloth (src/Cloth.h:55-60 plus gravity and
    wind). ``warp``: [length, 3] (rho, Y, B) per warp yarn line (node row v);
    ``weft``: [width, 3] per weft yarn line (node column u)."""
    width: int
    length: int
    warp: np.ndarray
    weft: np.ndarray
    height: float = 0.05
    L: float = 1e-3
    R: float = 1e-4
    pose: int = InitPose.Flat
    weave: int = WovenPattern.Plain
    kc: float = 1.0
    kf: float = 1000.0
    df: float = 1000.0
    mu: float = 0.3
    S: float = 1e-4
    handle_stiffness: float = 1e4
    G: Sequence[float] = (0.0, 0.0, 9.8)
    wind_vel: Sequence[float] = (0.0, 0.0, 0.0)
    wind_density: float = 0.0
    wind_drag: float = 0.0
    handles: List = field(default_factory=list)

    @staticmethod
    def from_yarns(width, length, height, L, R, yarns: Sequence[Yarn], kc, kf, df, mu, S, handle_stiffness,
                   woven_pattern=WovenPattern.Plain, init_pose=InitPose.Flat) -> "ClothSpec":
        """The reference's constructor arguments; one yarn -> homogeneous, two
        yarns -> lines alternate by parity (src/Cloth.cpp:195-222, 240-268)."""
        def line(i):
            y = yarns[0] if len(yarns) == 1 or i % 2 == 0 else yarns[1]
            return (y.rho, y.Y, y.B)
        warp = np.array([line(i) for i in range(length)], dtype=np.float64)
        weft = np.array([line(i) for i in range(width)], dtype=np.float64)
        return ClothSpec(width=width, length=length, warp=warp, weft=weft, height=height, L=L, R=R,
                         pose=int(init_pose), weave=int(woven_pattern), kc=kc, kf=kf, df=df, mu=mu, S=S,
                         handle_stiffness=handle_stiffness)

    @property
    def num_nodes(self):
        return self.width * self.length

    @property
    def dim(self):
        return 3 * self.width * self.length + 2 * (self.width - 2) * (self.length - 2)


def _ptr(a):
    """(pointer, flags) for a numpy array (host) or a CUDA torch tensor (device)."""
    if a is None:
        return None, 0
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
            raise TypeError("expected a C-contiguous float64 array")
        return a.ctypes.data, 0
    # torch tensor
    if str(a.dtype) != "torch.float64" or not a.is_contiguous():
        raise TypeError("expected a contiguous float64 tensor")
    return a.data_ptr(), (N.YS_ON_DEVICE if a.is_cuda else 0)


class ClothBatch:
    """A batch of cloths stepped together on one GPU (one ys_batch handle)."""

    def __init__(self, specs: Sequence[ClothSpec], device: int = 0, stream: Optional[int] = None):
        L = N.load()
        self.specs = list(specs)
        self._keep = []
        descs = (N.ClothDesc * len(self.specs))()
        for d, s in zip(descs, self.specs):
            warp = np.ascontiguousarray(np.asarray(s.warp, dtype=np.float64).reshape(s.length, 3).T.copy())
            weft = np.ascontiguousarray(np.asarray(s.weft, dtype=np.float64).reshape(s.width, 3).T.copy())
            hd = np.asarray(s.handles, dtype=np.int32).reshape(-1)
            self._keep += [warp, weft, hd]
            p = lambda x: x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            d.width, d.length, d.height, d.L, d.R = s.width, s.length, s.height, s.L, s.R
            d.pose, d.weave = int(s.pose), int(s.weave)
            d.warp_rho, d.warp_Y, d.warp_B = p(warp[0]), p(warp[1]), p(warp[2])
            d.weft_rho, d.weft_Y, d.weft_B = p(weft[0]), p(weft[1]), p(weft[2])
            d.kc, d.kf, d.df, d.mu, d.S, d.handle_stiffness = s.kc, s.kf, s.df, s.mu, s.S, s.handle_stiffness
            d.G = (ctypes.c_double * 3)(*s.G)
            d.wind_vel = (ctypes.c_double * 3)(*s.wind_vel)
            d.wind_density, d.wind_drag = s.wind_density, s.wind_drag
            d.n_handles = len(hd) // 2
            d.handles = hd.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if len(hd) else None
        h = ctypes.c_void_p()
        N.check(L.ys_batch_create(len(self.specs), descs, device, ctypes.c_void_p(stream or 0), ctypes.byref(h)),
                "ys_batch_create")
        self._h = h
        info = N.BatchInfo()
        N.check(L.ys_batch_get_info(self._h, ctypes.byref(info)), "ys_batch_get_info")
        self.n_cloths = info.n_cloths
        self.total_nodes = info.total_nodes
        self.device_bytes = info.device_bytes
        self.offsets = [L.ys_cloth_node_offset(self._h, c) for c in range(self.n_cloths)]

    # -------------------------------------------------------------- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            N.load().ys_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ state
    def node_slice(self, c):
        o = self.offsets[c]
        return slice(o, o + self.specs[c].num_nodes)

    def set_state(self, LPos=None, LPosFix=None, LVel=None, EPos=None, EPosBar=None, EVel=None):
        """Whole-batch arrays [total_nodes, 3|2]: numpy (host) or CUDA tensors."""
        args, flags = [], 0
        for a in (LPos, LPosFix, LVel, EPos, EPosBar, EVel):
            p, f = _ptr(a)
            args.append(ctypes.c_void_p(p) if p else None)
            flags |= f
        N.check(N.load().ys_set_state(self._h, *args, flags), "ys_set_state")

    def get_state(self, out=None):
        """Returns dict of numpy arrays, or fills ``out`` (dict of CUDA tensors)."""
        T = self.total_nodes
        if out is None:
            out = {k: np.zeros((T, 3)) for k in ("LPos", "LPosFix", "LVel")}
            out.update({k: np.zeros((T, 2)) for k in ("EPos", "EPosBar", "EVel")})
        args, flags = [], 0
        for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel"):
            p, f = _ptr(out.get(k))
            args.append(ctypes.c_void_p(p) if p else None)
            flags |= f
        N.check(N.load().ys_get_state(self._h, *args, flags), "ys_get_state")
        return out

    def set_wind(self, cloth: int, velocity):
        v = (ctypes.c_double * 3)(*velocity)
        N.check(N.load().ys_set_wind(self._h, cloth, v), "ys_set_wind")

    def set_winds(self, velocities):
        """Wind velocity of every cloth: [n_cloths, 3] numpy (host) or CUDA tensor."""
        p, f = _ptr(velocities)
        N.check(N.load().ys_set_winds(self._h, ctypes.c_void_p(p), f), "ys_set_winds")

    # ------------------------------------------------------------------- step
    @staticmethod
    def _opts(tol, maxiter, check_every):
        o = N.SolveOpts()
        o.tol, o.maxiter, o.check_every = tol, maxiter, check_every
        return o

    def _stats(self, arr):
        return StepStats(arr)

    def assemble(self, h, ext_force=None):
        """FillMV + system formation; ext_force: [total_nodes, 5] (x,y,z,u,v)."""
        p, f = _ptr(ext_force)
        N.check(N.load().ys_assemble(self._h, h, ctypes.c_void_p(p) if p else None, f), "ys_assemble")

    def solve(self, tol=0.0, maxiter=-1, check_every=0):
        st = (N.ClothStats * self.n_cloths)()
        r = N.load().ys_solve(self._h, ctypes.byref(self._opts(tol, maxiter, check_every)), st)
        if r not in (N.YS_OK, N.YS_ERR_NONFINITE, N.YS_ERR_MAXITER):
            N.check(r, "ys_solve")
        return self._stats(st)

    def solution(self):
        x = np.zeros((self.total_nodes, 5))
        N.check(N.load().ys_get_solution(self._h, ctypes.c_void_p(x.ctypes.data), 0), "ys_get_solution")
        return x

    def step(self, h, ext_force=None, tol=0.0, maxiter=-1, check_every=0):
        """One SimStep for every cloth; returns per-cloth stats (ok = SimStep's bool)."""
        p, f = _ptr(ext_force)
        st = (N.ClothStats * self.n_cloths)()
        r = N.load().ys_step(self._h, h, ctypes.c_void_p(p) if p else None, f,
                             ctypes.byref(self._opts(tol, maxiter, check_every)), st)
        if r not in (N.YS_OK, N.YS_ERR_NONFINITE, N.YS_ERR_MAXITER):
            N.check(r, "ys_step")
        return self._stats(st)

    def use_graphs(self, enable: bool = True):
        """Run step() as one CUDA graph launch per step (see ys_use_graphs)."""
        N.check(N.load().ys_use_graphs(self._h, int(bool(enable))), "ys_use_graphs")

    def set_producer_threads(self, threads: int):
        """Block size of the element-record producers and the gather (64..256;
        results do not depend on it; see ys_set_producer_threads)."""
        N.check(N.load().ys_set_producer_threads(self._h, int(threads)), "ys_set_producer_threads")

    def set_pcg_schedule(self, persistent: bool, threads: int = 0, cluster: int = 0):
        """Phase PCG (three launches per iteration, the default) or the
        persistent per-cloth PCG (one launch per solve, `cluster` CTAs of
        `threads` threads per cloth; threads * cluster >= the largest cloth's
        nodes). Both give the same bits (see ys_set_pcg_schedule)."""
        N.check(N.load().ys_set_pcg_schedule(self._h, 1 if persistent else 0, int(threads), int(cluster)),
                "ys_set_pcg_schedule")

    def normals(self) -> np.ndarray:
        """Node normals [total_nodes, 3] of the current positions (zero on boundary nodes)."""
        out = np.zeros((self.total_nodes, 3))
        N.check(N.load().ys_get_normals(self._h, ctypes.c_void_p(out.ctypes.data), 0), "ys_get_normals")
        return out

    def set_preconditioner(self, kind: str = "jacobi", net=None):
        """'jacobi' (Eigen's default, src/Solvers.cpp:22-24) or 'learned' with a
        precond.LearnedPreconditioner, which the batch borrows."""
        if kind == "jacobi":
            N.check(N.load().ys_set_preconditioner(self._h, N.YS_PREC_JACOBI, None), "ys_set_preconditioner")
            self._precond = None
        elif kind == "learned":
            if net is None:
                raise ValueError("learned preconditioner needs a network")
            N.check(N.load().ys_set_preconditioner(self._h, N.YS_PREC_LEARNED, net._h), "ys_set_preconditioner")
            self._precond = net  # keep it alive while the batch uses it
        else:
            raise ValueError(kind)

    def precond_refresh(self, every: int):
        """Evaluate the learned preconditioner's network once per `every` solves."""
        N.check(N.load().ys_precond_refresh(self._h, int(every)), "ys_precond_refresh")

    def precond_info(self) -> dict:
        s, f = ctypes.c_int64(), ctypes.c_int64()
        N.check(N.load().ys_precond_info(self._h, ctypes.byref(s), ctypes.byref(f)), "ys_precond_info")
        return dict(learned_solves=s.value, fallbacks=f.value)

    def system_slots(self):
        """The last assembled system: coefficient slots [159, n] and right-hand
        side [5, n] (component-major, batch node order)."""
        n = self.total_nodes
        a = np.zeros((159, n))
        b = np.zeros((5, n))
        N.check(N.load().ys_get_system_slots(self._h, ctypes.c_void_p(a.ctypes.data), ctypes.c_void_p(b.ctypes.data)),
                "ys_get_system_slots")
        return a, b

    def autotune(self, h, tol=0.0, maxiter=-1, steps=5) -> dict:
        """Time each step schedule from the current state (restored afterwards)
        and make the fastest the default (see ys_autotune)."""
        sc = N.Schedule()
        N.check(N.load().ys_autotune(self._h, h, ctypes.byref(self._opts(tol, maxiter, 0)), int(steps),
                                     ctypes.byref(sc)), "ys_autotune")
        L = N.load()
        n = L.ys_autotune_results(self._h, None, 0)
        arr = (N.Schedule * max(n, 1))()
        L.ys_autotune_results(self._h, ctypes.cast(arr, ctypes.c_void_p), n)

        def d(x):
            return dict(graphs=bool(x.graphs), check_every=x.check_every, ms_per_step=x.ms_per_step,
                        pcg="persistent" if x.pcg == 1 else "phases", pcg_threads=x.pcg_threads,
                        pcg_cluster=x.pcg_cluster, producer_threads=x.producer_threads)
        out = d(sc)
        out["candidates"] = [d(arr[i]) for i in range(n)]
        return out

    # ---- forward-mode sensitivities
    @property
    def n_tangents(self):
        return int(N.load().ys_tangent_count())

    @property
    def n_lines(self):
        return sum(s.length + s.width for s in self.specs)

    def tangent_enable(self, mode=0):
        """Allocates and zeroes the tangents (mode 0: exact derivatives of the step)."""
        N.check(N.load().ys_tangent_enable(self._h, int(mode)), "ys_tangent_enable")

    def tangent_seed(self, drho=None, dY=None, dB=None, dS=None, dmu=None):
        """Parameter directions: drho, dY, dB [K, lines] (cloth by cloth, warp
        lines then weft lines); dS, dmu [K, n_cloths]."""
        K, nl, nc = self.n_tangents, self.n_lines, self.n_cloths
        arrs = []
        for x, shape in ((drho, (K, nl)), (dY, (K, nl)), (dB, (K, nl)), (dS, (K, nc)), (dmu, (K, nc))):
            arrs.append(None if x is None else np.ascontiguousarray(np.broadcast_to(np.asarray(x, float), shape)))
        ptr = [ctypes.c_void_p(a.ctypes.data) if a is not None else None for a in arrs]
        N.check(N.load().ys_tangent_seed(self._h, *ptr), "ys_tangent_seed")

    def tangent_set_state(self, dlpos=None, dlvel=None, depos=None, deposbar=None, devel=None):
        """State tangents [K, total_nodes, 3|2] (numpy or CUDA tensors; None = 0)."""
        ps = [_ptr(a) for a in (dlpos, dlvel, depos, deposbar, devel)]
        flags = max([f for _, f in ps] + [0])
        N.check(N.load().ys_tangent_set_state(self._h, *[ctypes.c_void_p(p) if p else None for p, _ in ps], flags),
                "ys_tangent_set_state")

    def tangent_get_state(self):
        """dict of state tangents [K, total_nodes, 3|2] (numpy)."""
        K, T = self.n_tangents, self.total_nodes
        out = dict(LPos=np.zeros((K, T, 3)), LVel=np.zeros((K, T, 3)), EPos=np.zeros((K, T, 2)),
                   EPosBar=np.zeros((K, T, 2)), EVel=np.zeros((K, T, 2)))
        N.check(N.load().ys_tangent_get_state(self._h, *[ctypes.c_void_p(out[k].ctypes.data) for k in
                                                         ("LPos", "LVel", "EPos", "EPosBar", "EVel")], 0),
                "ys_tangent_get_state")
        return out

    def step_tangent(self, h, ext_force=None, tol=0.0, maxiter=-1, check_every=0, kact=None, dext_force=None):
        """step() that also advances the first kact tangent directions;
        dext_force [K, total_nodes, 5] (numpy) are the external force's
        tangents (ys_step_tangent_ext)."""
        kact = self.n_tangents if kact is None else int(kact)
        p, f = _ptr(ext_force)
        st = (N.ClothStats * self.n_cloths)()
        if dext_force is not None:
            if f:
                raise ValueError("dext_force with a device ext_force: pass both on the host")
            d = np.ascontiguousarray(dext_force, np.float64)
            if d.shape != (self.n_tangents, self.total_nodes, 5):
                raise ValueError("dext_force must be [%d, %d, 5]" % (self.n_tangents, self.total_nodes))
            r = N.load().ys_step_tangent_ext(self._h, h, ctypes.c_void_p(p) if p else None,
                                             ctypes.c_void_p(d.ctypes.data), 0,
                                             ctypes.byref(self._opts(tol, maxiter, check_every)), kact, st)
        else:
            r = N.load().ys_step_tangent(self._h, h, ctypes.c_void_p(p) if p else None, f,
                                         ctypes.byref(self._opts(tol, maxiter, check_every)), kact, st)
        if r not in (N.YS_OK, N.YS_ERR_NONFINITE, N.YS_ERR_MAXITER):
            N.check(r, "ys_step_tangent")
        return self._stats(st)

    def export_system(self, c):
        """Dense (A, b) of cloth c in the reference's DOF layout."""
        dim = self.specs[c].dim
        A = np.zeros((dim, dim))
        b = np.zeros(dim)
        N.check(N.load().ys_export_system(self._h, c, A.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          b.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "ys_export_system")
        return A, b

    def apply(self, x):
        """y = A x with the assembled matrices, node layout [total_nodes, 5]."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        N.check(N.load().ys_apply_system(self._h, ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(y.ctypes.data), 0),
                "ys_apply_system")
        return y

    def synchronize(self):
        N.check(N.load().ys_synchronize(self._h), "ys_synchronize")

    def profile(self, enable: bool):
        """Brackets every launch with CUDA events (per kernel class)."""
        N.check(N.load().ys_profile(self._h, int(bool(enable))), "ys_profile")

    def profile_read(self, reset=True):
        """{'ms': {class: ms}, 'launches': {class: n}, 'total_launches': n}"""
        k = len(N.PROF_KINDS)
        ms = (ctypes.c_double * k)()
        nl = (ctypes.c_int64 * k)()
        tot = ctypes.c_int64()
        N.check(N.load().ys_profile_read(self._h, ms, nl, ctypes.byref(tot), int(bool(reset))), "ys_profile_read")
        return dict(ms={n: ms[i] for i, n in enumerate(N.PROF_KINDS)},
                    launches={n: nl[i] for i, n in enumerate(N.PROF_KINDS)}, total_launches=tot.value)


STATE_KEYS = ("LPos", "LVel", "EPos", "EVel", "EPosBar")


class Adjoint:
    """Reverse-mode step of a batch (ys_adjoint_*): turns dL/d(state after a
    step) into dL/d(state before it), dL/d(material) and dL/d(external force),
    at a cost independent of how many inputs the gradient is taken for.
    mode: "exact" (the derivative of the discrete step) or "reference" (the
    gradient the reference's loss.backward() takes). copies: workspace size
    (128 copies = one pass per step; fewer copies, more passes)."""

    def __init__(self, batch: ClothBatch, mode="exact", copies: int = 128):
        self.batch = batch
        m = {"exact": N.YS_TANGENT_EXACT, "reference": N.YS_TANGENT_REFERENCE}[mode] if isinstance(mode, str) else mode
        h = ctypes.c_void_p()
        N.check(N.load().ys_adjoint_create(batch._h, int(m), int(copies), ctypes.byref(h)), "ys_adjoint_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            N.load().ys_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step_back(self, h, g_next=None, ext_force=None, tol=0.0, maxiter=-1, want_ext=False):
        """One step backwards from the batch's current state (the state at the
        start of the step; it is left unchanged). g_next: dict of dL/d(state
        after the step) for STATE_KEYS ([total_nodes, 3|2] numpy; missing = 0).
        Returns (g_state, g_params, g_ext): g_state the same keys before the
        step; g_params dict rho, Y, B [total lines] (ys_tangent_seed's line
        order) and S, mu [n_cloths]; g_ext [total_nodes, 5] or None."""
        b = self.batch
        T = b.total_nodes
        comps = dict(LPos=3, LVel=3, EPos=2, EVel=2, EPosBar=2)
        keep = []
        gin = (ctypes.c_void_p * 5)()
        gout = (ctypes.c_void_p * 5)()
        out = {}
        for i, k in enumerate(STATE_KEYS):
            a = None if g_next is None else g_next.get(k)
            if a is not None:
                a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(T, comps[k]))
                keep.append(a)
                gin[i] = a.ctypes.data
            out[k] = np.zeros((T, comps[k]))
            gout[i] = out[k].ctypes.data
        nl = sum(sp.width + sp.length for sp in b.specs)
        gp = dict(rho=np.zeros(nl), Y=np.zeros(nl), B=np.zeros(nl), S=np.zeros(b.n_cloths), mu=np.zeros(b.n_cloths))
        gpp = (ctypes.c_void_p * 5)(*[gp[k].ctypes.data for k in ("rho", "Y", "B", "S", "mu")])
        gext = np.zeros((T, 5)) if want_ext else None
        p, f = _ptr(ext_force)
        if f:
            raise TypeError("ext_force must be a host array here")
        st = (N.ClothStats * b.n_cloths)()
        N.check(N.load().ys_adjoint_step(self._h, float(h), ctypes.c_void_p(p) if p else None, gin, gout, gpp,
                                         ctypes.c_void_p(gext.ctypes.data) if want_ext else None, 0,
                                         ctypes.byref(ClothBatch._opts(tol, maxiter, 0)), st), "ys_adjoint_step")
        return out, gp, gext


# ---------------------------------------------------------------------------
# the reference's single-cloth interface
# ---------------------------------------------------------------------------
class Cloth:
    """src/Cloth.h:31-84. Geometry and state live on the GPU once a
    PhysicsCloth has been built for it."""

    def __init__(self, width, length, height, L, R, yarns, kc, kf, df, mu, S, handle_stiffness,
                 woven_pattern=WovenPattern.Plain, init_pose=InitPose.Upright):
        self.spec = ClothSpec.from_yarns(width, length, height, L, R, yarns, kc, kf, df, mu, S, handle_stiffness,
                                         woven_pattern, init_pose)
        self.width, self.length = width, length
        self._batch: Optional[ClothBatch] = None

    def set_handles(self, idxs):
        """src/Cloth.cpp:386-394; call before building the PhysicsCloth."""
        if self._batch is not None:
            raise RuntimeError("set_handles must precede PhysicsCloth construction")
        self.spec.handles = [tuple(p) for p in idxs]

    def get_ClothState(self) -> ClothState:
        return ClothState(**self._batch.get_state())

    def set_ClothState(self, state: ClothState):
        self._batch.set_state(**state.as_dict())


class Environment:
    """src/Environment.h:6-22 (cloth, gravity, wind)."""

    def __init__(self, cloth: Cloth, G=(0.0, 0.0, 9.8), wind: Wind = Wind()):
        self.cloth = cloth
        self.G = tuple(float(g) for g in np.asarray(G, dtype=np.float64).reshape(-1))
        self.wind = wind
        cloth.spec.G = self.G
        cloth.spec.wind_vel = tuple(float(w) for w in np.asarray(wind.WindVelocity, dtype=np.float64).reshape(-1))
        cloth.spec.wind_density = float(wind.WindDensity)
        cloth.spec.wind_drag = float(wind.WindDrag)


class PhysicsCloth:
    """src/PhysicsCloth.h:6-78. Construction allocates the device batch
    (the role of InitMV, src/PhysicsCloth.cpp:3-44)."""

    def __init__(self, env: Environment, device: int = 0):
        self.env = env
        self.batch = ClothBatch([env.cloth.spec], device=device)
        env.cloth._batch = self.batch
        self.h = None

    def InitMV(self):
        return None  # storage is allocated once at construction

    def FillMV(self, h=1e-3, ext_force=None):
        """FillMV plus the A, b formation of SimStep (needs the step size)."""
        self.h = h
        self.batch.assemble(h, ext_force)

    def ResetMV(self):
        return None  # the next FillMV overwrites the system in place

    def get_system(self):
        return self.batch.export_system(0)


def SimStep(cloth: Cloth, phy: PhysicsCloth, h, ext_force=None, tol=0.0, maxiter=-1, collision=None) -> bool:
    """src/TrainHelper.cpp:15-54 (and 56-97 with ext_force): False if the
    system or the new velocity is non-finite (the cloth is left unchanged).
    With a collide.Collision -- SimStep(cloth, phy, collision, h) as the
    reference calls it, or collision=... -- the step is followed by
    collision_response(0.1) and, when that moved anything, cloth.update()
    (src/TrainHelper.cpp:99-158): positions and velocities written back, the
    fixed positions of non-handle nodes following them."""
    from .collide import Collision
    if isinstance(h, Collision):
        collision, h, ext_force = h, ext_force, None
    h = float(h)
    before = phy.batch.get_state() if collision is not None else None
    stats = phy.batch.step(h, ext_force, tol=tol, maxiter=maxiter)
    if not stats[0]["ok"] or collision is None:
        return bool(stats[0]["ok"])
    st = phy.batch.get_state()
    if collision.collision_response(0.1, st["LPos"], before["LPos"], st["LVel"]):
        r = collision.last
        fixed = np.zeros(len(st["LPos"]), bool)
        for (u, v) in cloth.spec.handles:
            fixed[u + v * cloth.width] = True
        fix = st["LPosFix"].copy()
        fix[~fixed] = r["x"][~fixed]
        phy.batch.set_state(LPos=r["x"], LPosFix=fix, LVel=r["v"], EPos=st["EPos"], EPosBar=st["EPosBar"],
                            EVel=st["EVel"])
    return True


class EigenSolver:
    """src/Solvers.h:35-52 for the system assembled by the last FillMV: returns
    the new velocity in node layout [num_nodes, 5]."""

    @staticmethod
    def apply(phy: PhysicsCloth, tol=0.0, maxiter=-1):
        phy.batch.solve(tol=tol, maxiter=maxiter)
        return phy.batch.solution()
