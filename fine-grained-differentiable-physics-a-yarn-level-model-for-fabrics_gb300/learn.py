"""Differentiable rollouts and the parameter-learning interface of the
reference (YarnSimNetHeter + constraint_para + the training loss), on the GPU
step's forward-mode sensitivities.

The reference learns 8 scalars of a two-yarn cloth -- rho, Y, B of each yarn
type, S and mu (src/YarnSimNetHeter.h:4-120) -- through LibTorch autograd over
whole rollouts (src/TrainHeter.h:160-231). Here a rollout runs on the device
with ys_step_tangent carrying d(state)/d(theta) for all 8 parameters (two
copies of the cloth in one batch, each carrying ys_tangent_count() = 4
directions), and `Rollout` exposes the trajectory as a torch.autograd.Function
whose backward contracts the incoming gradient with that Jacobian. Nothing
of the trajectory has to be kept for the backward pass beyond the Jacobian of
the returned states.

Two gradient definitions (`mode`):
  "exact"     -- the derivative of the discrete step (A dq = db - dA q),
                 checked against central finite differences;
  "reference" -- what the reference's loss.backward() computes: A, M and
                 dF/dv enter without a graph (src/MatrixMp.cpp:40-99), the
                 solve's backward is A^-1 g (src/Solvers.cpp:33-58), and the
                 (phi - PI/2) factor of Shear_F is taken by .item()
                 (src/PhysicsCloth.cpp:2720-2721); checked against gradients
                 of the reference itself.
"""
from __future__ import annotations

import math
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import _native as N
from .cloth import STATE_KEYS, Adjoint, ClothBatch, ClothSpec, InitPose, WovenPattern

PARAM_NAMES = ("rho0", "Y0", "B0", "rho1", "Y1", "B1", "S", "mu")
MODES = {"exact": N.YS_TANGENT_EXACT, "reference": N.YS_TANGENT_REFERENCE}


def constraint_para(para, upper: float = 1.0, lower: float = 0.0):
    """(upper - lower) * sigmoid(para) + lower (src/TrainHelper.cpp:3-7); note
    the reference's call sites pass (range.first = upper, range.second = lower)."""
    import torch
    return (upper - lower) * torch.sigmoid(para) + lower


def invert_constraint_para(para: float, upper: float = 1.0, lower: float = 0.0) -> float:
    """Inverse of constraint_para (src/TrainHelper.cpp:9-13)."""
    return -math.log((upper - lower) / (para - lower) - 1.0)


def two_yarn_spec(template: Dict, theta: Sequence[float]) -> ClothSpec:
    """ClothSpec of a two-yarn cloth: warp line j and weft line i use yarn
    (j % 2) and (i % 2) (src/Cloth.cpp:195-268); theta in PARAM_NAMES order."""
    W, H = int(template["width"]), int(template["length"])
    y = [np.array(theta[0:3], float), np.array(theta[3:6], float)]
    kw = dict(template)
    kw.update(warp=np.array([y[j % 2] for j in range(H)]), weft=np.array([y[i % 2] for i in range(W)]),
              S=float(theta[6]), mu=float(theta[7]))
    return ClothSpec(**kw)


def position_loss(traj_x, traj_e, gt_x, gt_e):
    """sum_s (mean_N |x_s - x^_s|^2 + mean_N |e_s - e^_s|^2) / max(steps - 1, 1)
    (src/TrainHeter.h:194-222); traj_*: [steps, N, 3|2] torch tensors."""
    steps = traj_x.shape[0]
    dl = traj_x - gt_x
    de = traj_e - gt_e
    loss = (dl * dl).sum(-1).mean(-1).sum() + (de * de).sum(-1).mean(-1).sum()
    return loss / max(steps - 1, 1)


def rollout_with_jacobian(template: Dict, theta: Sequence[float], state0: Dict, steps: int, h: float = 1e-3,
                          mode: str = "exact", tol: float = 0.0, maxiter: int = -1, device: int = 0):
    """Runs `steps` steps of the two-yarn cloth from state0 and returns
    (traj_x [steps, N, 3], traj_e [steps, N, 2], J_x [steps, N, 3, 8],
    J_e [steps, N, 2, 8], stats), J = d state / d theta."""
    spec = two_yarn_spec(template, theta)
    K = int(N.load().ys_tangent_count())
    P = len(PARAM_NAMES)
    copies = (P + K - 1) // K
    batch = ClothBatch([spec] * copies, device=device)
    try:
        Nn = spec.num_nodes
        st = {k: np.concatenate([np.asarray(state0[k], float)] * copies) for k in
              ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel") if k in state0}
        batch.set_state(**st)
        batch.tangent_enable(MODES[mode])
        nl = spec.length + spec.width
        parity = np.array([j % 2 for j in range(spec.length)] + [i % 2 for i in range(spec.width)])
        drho = np.zeros((K, copies * nl)); dY = np.zeros_like(drho); dB = np.zeros_like(drho)
        dS = np.zeros((K, copies)); dmu = np.zeros((K, copies))
        for c in range(copies):
            for k in range(K):
                p = c * K + k
                if p >= P:
                    continue
                if p < 6:
                    [drho, dY, dB][p % 3][k, c * nl:(c + 1) * nl] = (parity == p // 3)
                elif p == 6:
                    dS[k, c] = 1.0
                else:
                    dmu[k, c] = 1.0
        batch.tangent_seed(drho, dY, dB, dS, dmu)
        tx = np.zeros((steps, Nn, 3)); te = np.zeros((steps, Nn, 2))
        Jx = np.zeros((steps, Nn, 3, P)); Je = np.zeros((steps, Nn, 2, P))
        stats = []
        for s in range(steps):
            stats.append(batch.step_tangent(h, tol=tol, maxiter=maxiter, kact=K))
            cur = batch.get_state()
            tan = batch.tangent_get_state()
            tx[s] = cur["LPos"][:Nn]
            te[s] = cur["EPos"][:Nn]
            for c in range(copies):
                for k in range(K):
                    p = c * K + k
                    if p < P:
                        Jx[s, :, :, p] = tan["LPos"][k, c * Nn:(c + 1) * Nn]
                        Je[s, :, :, p] = tan["EPos"][k, c * Nn:(c + 1) * Nn]
        return tx, te, Jx, Je, stats
    finally:
        batch.close()


def _rollout_function():
    import torch

    class Rollout(torch.autograd.Function):
        """traj_x, traj_e = Rollout.apply(theta, template, state0, steps, h, mode, tol):
        the states of a rollout as a differentiable function of theta
        (PARAM_NAMES order, a float64 tensor of 8)."""

        @staticmethod
        def forward(ctx, theta, template, state0, steps, h, mode, tol):
            th = theta.detach().cpu().numpy().astype(np.float64)
            tx, te, Jx, Je, stats = rollout_with_jacobian(template, th, state0, steps, h, mode, tol)
            ctx.stats = stats
            dev = theta.device
            Jx_t = torch.as_tensor(Jx, device=dev)
            Je_t = torch.as_tensor(Je, device=dev)
            ctx.save_for_backward(Jx_t, Je_t)
            return torch.as_tensor(tx, device=dev), torch.as_tensor(te, device=dev)

        @staticmethod
        def backward(ctx, gx, ge):
            Jx, Je = ctx.saved_tensors
            g = torch.einsum("snc,sncp->p", gx, Jx) + torch.einsum("snc,sncp->p", ge, Je)
            return g, None, None, None, None, None, None

    return Rollout


_ROLLOUT = None


def rollout(theta, template: Dict, state0: Dict, steps: int, h: float = 1e-3, mode: str = "exact",
            tol: float = 0.0) -> Tuple:
    """Differentiable rollout (see Rollout)."""
    global _ROLLOUT
    if _ROLLOUT is None:
        _ROLLOUT = _rollout_function()
    return _ROLLOUT.apply(theta, template, state0, steps, h, mode, tol)


class CheckpointedRollout:
    """A rollout of a batch whose gradient is taken in reverse mode
    (ys_adjoint_step) with checkpoints: the forward pass keeps the state every
    `checkpoint_every` steps (plus the trajectory it returns); the backward
    pass steps each segment again from its checkpoint, last segment first,
    and runs the adjoint steps of the segment backwards. Memory: one state
    per checkpoint and the states of one segment, whatever the rollout's
    length. The reference's loss.backward() keeps the graph of every step
    instead (src/TrainHeter.h:160-231).

    ext_forces: None, or a list of [total_nodes, 5] arrays (None entries: no
    force) for steps 0..steps-1 -- per-node control forces.

    collision: a collide.Collision of the batch's (single) cloth: every step
    is then SimStep with collision (src/TrainHelper.cpp:99-149): the step,
    collision_response(damp) and, when it moved anything, the write-back of
    positions and velocities (fixed positions follow the nodes that are not
    in `fixed`, a [total_nodes] bool mask of the handles). The backward pass
    runs the response's backward (impacts' weights and normals carried into
    the positions, as the reference's autograd does; exact_root: the CCD
    root's exact derivative instead of the reference's CubicSolver backward)
    before each step's adjoint."""

    FULL = ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")

    def __init__(self, batch: ClothBatch, state0: Dict, steps: int, h: float = 1e-3, ext_forces=None,
                 mode: str = "exact", checkpoint_every: int = 20, tol: float = 0.0, copies: int = 128,
                 collision=None, damp: float = 0.1, fixed=None, exact_root: bool = False):
        self.batch, self.steps, self.h, self.mode, self.tol = batch, int(steps), float(h), mode, tol
        self.k = max(1, int(checkpoint_every))
        self.ext = ext_forces
        self.state0 = {k: np.array(state0[k], dtype=np.float64) for k in self.FULL if k in state0}
        self.copies = copies
        self.collision, self.damp, self.exact_root = collision, float(damp), bool(exact_root)
        self.fixed = np.zeros(batch.total_nodes, bool) if fixed is None else np.asarray(fixed, bool)
        self.checkpoints = {}
        self.ok = True

    def _advance(self, s):
        """Step s from the batch's state (with the collision response when
        given); returns whether the response moved anything."""
        b = self.batch
        before = b.get_state() if self.collision is not None else None
        st = b.step(self.h, self._ext(s), tol=self.tol)
        self.ok = self.ok and all(x["ok"] for x in st)
        if self.collision is None or not st[0]["ok"]:
            return False
        cur = b.get_state()
        if not self.collision.collision_response(self.damp, cur["LPos"], before["LPos"], cur["LVel"]):
            return False
        r = self.collision.last
        fix = cur["LPosFix"].copy()
        fix[~self.fixed] = r["x"][~self.fixed]
        b.set_state(LPos=r["x"], LPosFix=fix, LVel=r["v"], EPos=cur["EPos"], EPosBar=cur["EPosBar"],
                    EVel=cur["EVel"])
        return True

    def _ext(self, s):
        if self.ext is None:
            return None
        e = self.ext[s]
        return None if e is None else np.ascontiguousarray(np.asarray(e, dtype=np.float64))

    def forward(self) -> Dict[str, np.ndarray]:
        """Runs the rollout; returns the state after every step, dict of
        [steps, total_nodes, 3|2] arrays for STATE_KEYS."""
        b = self.batch
        b.set_state(**self.state0)
        traj = {k: [] for k in STATE_KEYS}
        for s in range(self.steps):
            if s % self.k == 0:
                self.checkpoints[s] = b.get_state()
            self._advance(s)
            cur = b.get_state()
            for k in STATE_KEYS:
                traj[k].append(cur[k])
        return {k: np.array(v) for k, v in traj.items()}

    def backward(self, g_traj: Dict[str, np.ndarray], want_ext: bool = False):
        """g_traj: dL/d(state after step s) as [steps, total_nodes, 3|2]
        arrays (missing keys: 0). Returns dict(state0=..., rho, Y, B [lines],
        S, mu [cloths] summed over the steps, ext=[steps, total_nodes, 5] or
        None)."""
        b = self.batch
        adj = Adjoint(b, self.mode, self.copies)
        try:
            T = b.total_nodes
            comps = dict(LPos=3, LVel=3, EPos=2, EVel=2, EPosBar=2)
            nl = sum(sp.width + sp.length for sp in b.specs)
            acc = dict(rho=np.zeros(nl), Y=np.zeros(nl), B=np.zeros(nl), S=np.zeros(b.n_cloths),
                       mu=np.zeros(b.n_cloths))
            gext = np.zeros((self.steps, T, 5)) if want_ext else None

            def injected(s):  # dL/d(state after step s), s = 1..steps
                return {k: np.asarray(g_traj[k][s - 1], dtype=np.float64) for k in STATE_KEYS if k in g_traj}

            g = {k: np.zeros((T, comps[k])) for k in STATE_KEYS}
            for k, v in injected(self.steps).items():
                g[k] = g[k] + v
            for a in reversed(sorted(self.checkpoints)):
                e = min(a + self.k, self.steps)
                # states at the start of steps a .. e-1, stepped again from the checkpoint
                b.set_state(**self.checkpoints[a])
                seg = []
                for s in range(a, e):
                    seg.append(b.get_state())
                    if s + 1 < e:
                        self._advance(s)
                for s in range(e - 1, a - 1, -1):
                    g_prev = None
                    if self.collision is not None:
                        # the step and its response again, then the response's backward
                        b.set_state(**seg[s - a])
                        if self._advance(s):
                            rb = self.collision.collider.respond_backward(dl_dx=g["LPos"], dl_dv=g["LVel"],
                                                                         impacts=True, exact_root=self.exact_root)
                            g = dict(g, LPos=rb["x"], LVel=rb["v"])
                            g_prev = rb["x_prev"]
                    b.set_state(**seg[s - a])
                    gs, gp, ge = adj.step_back(self.h, g, self._ext(s), tol=self.tol, want_ext=want_ext)
                    if g_prev is not None:
                        gs["LPos"] = gs["LPos"] + g_prev
                    for k in acc:
                        acc[k] += gp[k]
                    if want_ext:
                        gext[s] = ge
                    g = gs
                    if s >= 1:
                        for k, v in injected(s).items():
                            g[k] = g[k] + v
            out = dict(acc)
            out["state0"] = g
            out["ext"] = gext
            return out
        finally:
            adj.close()


def two_yarn_param_grad(spec: ClothSpec, g: Dict[str, np.ndarray]) -> np.ndarray:
    """Per-line material gradients of a two-yarn cloth (one cloth) gathered
    into PARAM_NAMES order: yarn type t's rho, Y, B sum the lines of parity t
    (warp line j, weft line i take type j % 2, i % 2)."""
    parity = np.array([j % 2 for j in range(spec.length)] + [i % 2 for i in range(spec.width)])
    out = []
    for t in (0, 1):
        for k in ("rho", "Y", "B"):
            out.append(float(g[k][parity == t].sum()))
    out.append(float(g["S"].sum()))
    out.append(float(g["mu"].sum()))
    return np.array(out)


def _adjoint_rollout_function():
    import torch

    class AdjointRollout(torch.autograd.Function):
        """traj_x, traj_e = AdjointRollout.apply(theta, template, state0, steps, h, mode, tol, k):
        the rollout's positions as a differentiable function of theta
        (PARAM_NAMES order), with the gradient taken in reverse mode
        (CheckpointedRollout, a checkpoint every k steps)."""

        @staticmethod
        def forward(ctx, theta, template, state0, steps, h, mode, tol, k):
            th = theta.detach().cpu().numpy().astype(np.float64)
            spec = two_yarn_spec(template, th)
            batch = ClothBatch([spec])
            ro = CheckpointedRollout(batch, state0, steps, h, mode=mode, checkpoint_every=k, tol=tol)
            traj = ro.forward()
            ctx.ro, ctx.spec = ro, spec
            dev = theta.device
            return torch.as_tensor(traj["LPos"], device=dev), torch.as_tensor(traj["EPos"], device=dev)

        @staticmethod
        def backward(ctx, gx, ge):
            ro = ctx.ro
            try:
                g = ro.backward({"LPos": gx.detach().cpu().numpy(), "EPos": ge.detach().cpu().numpy()})
            finally:
                ro.batch.close()
            gt = torch.as_tensor(two_yarn_param_grad(ctx.spec, g), dtype=gx.dtype, device=gx.device)
            return gt, None, None, None, None, None, None, None

    return AdjointRollout


_ADJ_ROLLOUT = None


def rollout_adjoint(theta, template: Dict, state0: Dict, steps: int, h: float = 1e-3, mode: str = "exact",
                    tol: float = 0.0, checkpoint_every: int = 20):
    """Differentiable rollout whose backward is the reverse-mode adjoint with
    checkpoints (see AdjointRollout); same outputs as rollout()."""
    global _ADJ_ROLLOUT
    if _ADJ_ROLLOUT is None:
        _ADJ_ROLLOUT = _adjoint_rollout_function()
    return _ADJ_ROLLOUT.apply(theta, template, state0, steps, h, mode, tol, checkpoint_every)


def _module_base():
    import torch
    return torch.nn.Module


class YarnSimNetHeter(_module_base()):
    """The reference's YarnSimNetHeter (src/YarnSimNetHeter.h:4-120): raw
    parameters rho_1, rho_2, Y_1, Y_2, B_1, B_2, S, mu mapped into their ranges
    by constraint_para (ranges given as (upper, lower) pairs, as the reference
    passes them), a two-yarn cloth (upright, handles) and its step.

    rollout(state0, steps) returns the trajectory, differentiable w.r.t. the
    parameters; forward(state) is one step without a graph (the reference's
    forward(ClothState, bool&))."""

    def __init__(self, width: int, length: int, R: float, L: float, raw: Dict[str, float],
                 ranges: Dict[str, Tuple[float, float]], handles: Sequence[Tuple[int, int]], h: float = 1e-3,
                 kf: float = 1000.0, df: float = 1000.0, kc: float = 1.0, handle_stiffness: float = 1e4,
                 gravity: float = 9.8, wind_vel=(0.0, 0.0, 0.0), wind_density: float = 0.0, wind_drag: float = 0.0,
                 woven_pattern: int = WovenPattern.Plain, height: float = 5.0, mode: str = "reference"):
        import torch
        super().__init__()
        names = ("rho_1", "rho_2", "Y_1", "Y_2", "B_1", "B_2", "S", "mu")
        for n in names:
            self.register_parameter(n, torch.nn.Parameter(torch.tensor([float(raw[n])], dtype=torch.float64)))
        self.ranges = dict(ranges)
        self.h = h
        self.mode = mode
        self.template = dict(width=width, length=length, height=height, L=L, R=R, pose=InitPose.Upright,
                             weave=int(woven_pattern), kc=kc, kf=kf, df=df, handle_stiffness=handle_stiffness,
                             G=(0.0, 0.0, gravity), wind_vel=tuple(wind_vel), wind_density=wind_density,
                             wind_drag=wind_drag, handles=list(handles))

    def theta(self):
        """Constrained parameters in PARAM_NAMES order (a float64 tensor of 8)."""
        import torch
        p = {n: constraint_para(getattr(self, n), *self.ranges[n]) for n in self.ranges}
        return torch.cat([p["rho_1"], p["Y_1"], p["B_1"], p["rho_2"], p["Y_2"], p["B_2"], p["S"], p["mu"]])

    def rollout(self, state0: Dict, steps: int, tol: float = 0.0):
        return rollout(self.theta(), self.template, state0, steps, self.h, self.mode, tol)

    def forward(self, state: Dict, tol: float = 0.0) -> Tuple[Dict, bool]:
        th = self.theta().detach().cpu().numpy()
        b = ClothBatch([two_yarn_spec(self.template, th)])
        try:
            b.set_state(**state)
            ok = b.step(self.h, tol=tol)[0]["ok"]
            return b.get_state(), ok
        finally:
            b.close()


def _homo_theta(net, names=("rho", "Y", "B")):
    """The 8-vector of two_yarn_spec for a one-yarn cloth: both yarn types
    carry the same constrained rho, Y, B (the lines of a homogeneous cloth);
    S and mu are the module's parameter or constant."""
    import torch
    p = {}
    for n in ("rho", "Y", "B", "S", "mu"):
        if n in net.ranges and isinstance(getattr(net, n, None), torch.nn.Parameter):
            p[n] = constraint_para(getattr(net, n), *net.ranges[n])
        else:
            p[n] = torch.tensor([float(net.const[n])], dtype=torch.float64)
    return torch.cat([p["rho"], p["Y"], p["B"], p["rho"], p["Y"], p["B"], p["S"], p["mu"]])


class YarnSimNetHomo(_module_base()):
    """The reference's YarnSimNetHomo (src/YarnSimNetHomo.h:4-111): raw
    parameters rho, Y, B, S of one yarn type mapped into their ranges by
    constraint_para ((upper, lower) pairs, as the reference passes them),
    mu, kf, df, kc fixed, an upright cloth at height 0 with handles, and its
    step. rollout(state0, steps) is differentiable w.r.t. the four raw
    parameters (forward-mode tangents; rollout_adjoint: the reverse adjoint
    with checkpoints); forward(state) is one step without a graph (the
    reference's forward(ClothState, bool&))."""

    def __init__(self, width: int, length: int, R: float, L: float, raw: Dict[str, float],
                 ranges: Dict[str, Tuple[float, float]], handles: Sequence[Tuple[int, int]], h: float = 1e-3,
                 mu: float = 0.5, kf: float = 1000.0, df: float = 1000.0, kc: float = 1.0,
                 handle_stiffness: float = 1e4, gravity: float = 9.8, wind_vel=(0.0, 0.0, 0.0),
                 wind_density: float = 0.0, wind_drag: float = 0.0, woven_pattern: int = WovenPattern.Plain,
                 height: float = 0.0, mode: str = "reference"):
        import torch
        super().__init__()
        for n in ("rho", "Y", "B", "S"):
            self.register_parameter(n, torch.nn.Parameter(torch.tensor([float(raw[n])], dtype=torch.float64)))
        self.ranges = {n: ranges[n] for n in ("rho", "Y", "B", "S")}
        self.const = dict(mu=float(mu))
        self.h, self.mode = float(h), mode
        self.template = dict(width=width, length=length, height=height, L=L, R=R, pose=InitPose.Upright,
                             weave=int(woven_pattern), kc=kc, kf=kf, df=df, handle_stiffness=handle_stiffness,
                             G=(0.0, 0.0, gravity), wind_vel=tuple(wind_vel), wind_density=wind_density,
                             wind_drag=wind_drag, handles=list(handles))

    def theta(self):
        """The constrained parameters in PARAM_NAMES order (both yarn types equal)."""
        return _homo_theta(self)

    def spec(self) -> ClothSpec:
        return two_yarn_spec(self.template, self.theta().detach().cpu().numpy())

    def rollout(self, state0: Dict, steps: int, tol: float = 0.0):
        return rollout(self.theta(), self.template, state0, steps, self.h, self.mode, tol)

    def rollout_adjoint(self, state0: Dict, steps: int, checkpoint_every: int = 20, tol: float = 0.0):
        return rollout_adjoint(self.theta(), self.template, state0, steps, self.h, self.mode, tol, checkpoint_every)

    def forward(self, state: Dict, tol: float = 0.0) -> Tuple[Dict, bool]:
        b = ClothBatch([self.spec()])
        try:
            b.set_state(**state)
            ok = b.step(self.h, tol=tol)[0]["ok"]
            return b.get_state(), ok
        finally:
            b.close()


def _colli_rollout_function():
    import torch

    class CollisionRollout(torch.autograd.Function):
        """traj_x, traj_e = CollisionRollout.apply(theta, net, state0, steps, k):
        a rollout with the collision response at every step, differentiable
        w.r.t. theta (PARAM_NAMES order) through the reverse adjoint and the
        response's backward (CheckpointedRollout with a collision)."""

        @staticmethod
        def forward(ctx, theta, net, state0, steps, k):
            from .collide import Collision
            spec = two_yarn_spec(net.template, theta.detach().cpu().numpy().astype(np.float64))
            batch = ClothBatch([spec])
            W = spec.width
            fixed = np.zeros(spec.num_nodes, bool)
            for (u, v) in spec.handles:
                fixed[u + v * W] = True
            col = Collision(_Shape(spec), net.obstacle_x, net.obstacle_faces, thickness=net.thickness, h=net.h)
            ro = CheckpointedRollout(batch, state0, steps, net.h, mode=net.mode, checkpoint_every=k,
                                     collision=col, damp=0.1, fixed=fixed, exact_root=net.mode == "exact")
            traj = ro.forward()
            ctx.ro, ctx.spec, ctx.col = ro, spec, col
            dev = theta.device
            return torch.as_tensor(traj["LPos"], device=dev), torch.as_tensor(traj["EPos"], device=dev)

        @staticmethod
        def backward(ctx, gx, ge):
            ro = ctx.ro
            try:
                g = ro.backward({"LPos": gx.detach().cpu().numpy(), "EPos": ge.detach().cpu().numpy()})
            finally:
                ro.batch.close()
                ctx.col.close()
            gt = torch.as_tensor(two_yarn_param_grad(ctx.spec, g), dtype=gx.dtype, device=gx.device)
            return gt, None, None, None, None

    return CollisionRollout


class _Shape:
    """width / length holder for collide.Collision."""

    def __init__(self, spec):
        self.width, self.length = spec.width, spec.length


_COLLI_ROLLOUT = None


class YarnSimNetColli(_module_base()):
    """The reference's YarnSimNetColli (src/YarnSimNetColli.h:4-116): raw
    rho, Y, B of one yarn type (constraint_para into their ranges), S, mu,
    kf, df, kc fixed, an upright plain cloth at `height` with handles, and
    SimStep with collision against the table and ground meshes (merged into
    one obstacle, as the reference's collision reports their pairs; thickness
    0.5 mm) -- src/TrainHelper.cpp:99-149. forward(state) is one step;
    rollout(state0, steps) is differentiable w.r.t. the three raw
    parameters through the reverse adjoint and the collision response's
    backward."""

    def __init__(self, width: int, length: int, height: float, R: float, L: float, raw: Dict[str, float],
                 ranges: Dict[str, Tuple[float, float]], handles: Sequence[Tuple[int, int]], obstacle_x,
                 obstacle_faces, h: float = 1e-3, S: float = 1000.0, mu: float = 0.5, kf: float = 1000.0,
                 df: float = 1000.0, kc: float = 1.0, handle_stiffness: float = 1e4, gravity: float = 9.8,
                 wind_vel=(0.0, 0.0, 0.0), wind_density: float = 0.0, wind_drag: float = 0.0,
                 thickness: float = 0.0005, mode: str = "reference"):
        import torch
        super().__init__()
        for n in ("rho", "Y", "B"):
            self.register_parameter(n, torch.nn.Parameter(torch.tensor([float(raw[n])], dtype=torch.float64)))
        self.ranges = {n: ranges[n] for n in ("rho", "Y", "B")}
        self.const = dict(S=float(S), mu=float(mu))
        self.h, self.mode, self.thickness = float(h), mode, float(thickness)
        self.obstacle_x = np.ascontiguousarray(obstacle_x, np.float64)
        self.obstacle_faces = np.ascontiguousarray(obstacle_faces, np.int32)
        self.template = dict(width=width, length=length, height=height, L=L, R=R, pose=InitPose.Upright,
                             weave=int(WovenPattern.Plain), kc=kc, kf=kf, df=df, handle_stiffness=handle_stiffness,
                             G=(0.0, 0.0, gravity), wind_vel=tuple(wind_vel), wind_density=wind_density,
                             wind_drag=wind_drag, handles=list(handles))

    def theta(self):
        return _homo_theta(self)

    def spec(self) -> ClothSpec:
        return two_yarn_spec(self.template, self.theta().detach().cpu().numpy())

    def rollout(self, state0: Dict, steps: int, checkpoint_every: int = 20):
        global _COLLI_ROLLOUT
        if _COLLI_ROLLOUT is None:
            _COLLI_ROLLOUT = _colli_rollout_function()
        return _COLLI_ROLLOUT.apply(self.theta(), self, state0, steps, checkpoint_every)

    def forward(self, state: Dict, tol: float = 0.0) -> Tuple[Dict, bool]:
        from .collide import Collision
        spec = self.spec()
        b = ClothBatch([spec])
        col = Collision(_Shape(spec), self.obstacle_x, self.obstacle_faces, thickness=self.thickness, h=self.h)
        try:
            fixed = np.zeros(spec.num_nodes, bool)
            for (u, v) in spec.handles:
                fixed[u + v * spec.width] = True
            ro = CheckpointedRollout(b, state, 1, self.h, collision=col, damp=0.1, fixed=fixed, tol=tol)
            b.set_state(**ro.state0)
            ro._advance(0)
            return b.get_state(), ro.ok
        finally:
            col.close()
            b.close()


def _control_rollout_function():
    import torch

    class ControlRollout(torch.autograd.Function):
        """traj_x, traj_e = ControlRollout.apply(forces, net, state0, schedule, k):
        forces [6, 2] (lift, drag) of the six force settings; schedule[s] the
        setting of step s (6: no force). Differentiable w.r.t. the forces
        through the reverse adjoint's dL/d(ext force)."""

        @staticmethod
        def forward(ctx, forces, net, state0, schedule, k):
            f = forces.detach().cpu().numpy().astype(np.float64)
            exts = [net.ext_force(int(i), f) for i in schedule]
            batch = ClothBatch([net.spec()])
            ro = CheckpointedRollout(batch, state0, len(schedule), net.h, ext_forces=exts, mode=net.mode,
                                     checkpoint_every=k)
            traj = ro.forward()
            ctx.ro, ctx.schedule, ctx.net = ro, list(schedule), net
            dev = forces.device
            return torch.as_tensor(traj["LPos"], device=dev), torch.as_tensor(traj["EPos"], device=dev)

        @staticmethod
        def backward(ctx, gx, ge):
            ro = ctx.ro
            try:
                g = ro.backward({"LPos": gx.detach().cpu().numpy(), "EPos": ge.detach().cpu().numpy()},
                                want_ext=True)
            finally:
                ro.batch.close()
            gf = np.zeros((6, 2))
            nodes = ctx.net.force_nodes()
            for s, i in enumerate(ctx.schedule):
                if 0 <= i < 6:
                    gf[i, 0] += g["ext"][s][nodes, 2].sum()
                    gf[i, 1] += g["ext"][s][nodes, 1].sum()
            return torch.as_tensor(gf, dtype=gx.dtype, device=gx.device), None, None, None, None

    return ControlRollout


_CONTROL_ROLLOUT = None
FORCE_NAMES = ("one", "two", "three", "four", "five", "six")


class YarnSimNetControl(_module_base()):
    """The reference's YarnSimNetControl (src/YarnSimNet.h:132-245): six
    settings of a lift (z) and a drag (y) force applied at the `handles`
    nodes, twelve parameters lift_force_one .. drag_force_six; a free
    (unpinned) upright plain cloth at height 5 with fixed material; forward
    (state, idx) is one step under setting idx (6: no force). The force's
    node for handle (a, b) is a * width + b, as the reference indexes it.
    rollout(state0, schedule) is differentiable w.r.t. the twelve forces
    (reverse adjoint, dL/d(ext force) contracted with the force positions)."""

    def __init__(self, width: int, length: int, R: float, L: float, material: Dict[str, float],
                 forces: Sequence[Tuple[float, float]], handles: Sequence[Tuple[int, int]], h: float = 1e-3,
                 mode: str = "exact"):
        import torch
        super().__init__()
        for i, (lift, drag) in enumerate(forces):
            self.register_parameter("lift_force_" + FORCE_NAMES[i],
                                    torch.nn.Parameter(torch.tensor([float(lift)], dtype=torch.float64)))
            self.register_parameter("drag_force_" + FORCE_NAMES[i],
                                    torch.nn.Parameter(torch.tensor([float(drag)], dtype=torch.float64)))
        m = dict(material)
        self.h, self.mode, self.handles = float(h), mode, list(handles)
        yarn = np.array([[m["rho"], m["Y"], m["B"]]])
        self._spec = ClothSpec(width=width, length=length, warp=yarn.repeat(length, 0), weft=yarn.repeat(width, 0),
                               height=5.0, L=L, R=R, pose=InitPose.Upright, weave=int(WovenPattern.Plain),
                               kc=m.get("kc", 1.0), kf=m.get("kf", 1000.0), df=m.get("df", 1000.0),
                               mu=m.get("mu", 0.5), S=m.get("S", 1000.0),
                               handle_stiffness=m.get("handle_stiffness", 1e4),
                               G=(0.0, 0.0, m.get("gravity", 9.8)), wind_vel=tuple(m.get("wind_vel", (0, 0, 0))),
                               wind_density=m.get("wind_density", 0.0), wind_drag=m.get("wind_drag", 0.0),
                               handles=[])

    def spec(self) -> ClothSpec:
        return self._spec

    def forces(self):
        """[6, 2] tensor of (lift, drag) per setting."""
        import torch
        return torch.stack([torch.cat([getattr(self, "lift_force_" + n), getattr(self, "drag_force_" + n)])
                            for n in FORCE_NAMES])

    def force_nodes(self) -> np.ndarray:
        return np.array([a * self._spec.width + b for (a, b) in self.handles], dtype=np.int64)

    def ext_force(self, idx: int, forces=None) -> Optional[np.ndarray]:
        """[N, 5] external force of setting idx (None for 6, the zero force)."""
        if idx == 6:
            return None
        if not 0 <= idx < 6:
            raise ValueError("invalid force index %d" % idx)
        f = self.forces().detach().cpu().numpy() if forces is None else np.asarray(forces)
        e = np.zeros((self._spec.num_nodes, 5))
        for nd in self.force_nodes():
            e[nd, 2] += f[idx, 0]
            e[nd, 1] += f[idx, 1]
        return e

    def rollout(self, state0: Dict, schedule: Sequence[int], checkpoint_every: int = 20):
        global _CONTROL_ROLLOUT
        if _CONTROL_ROLLOUT is None:
            _CONTROL_ROLLOUT = _control_rollout_function()
        return _CONTROL_ROLLOUT.apply(self.forces(), self, state0, list(schedule), checkpoint_every)

    def forward(self, state: Dict, idx: int, tol: float = 0.0) -> Tuple[Dict, bool]:
        b = ClothBatch([self._spec])
        try:
            b.set_state(**state)
            ok = b.step(self.h, self.ext_force(idx), tol=tol)[0]["ok"]
            return b.get_state(), ok
        finally:
            b.close()
