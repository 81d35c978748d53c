"""Learned preconditioner for the implicit step's linear systems.

The reference solves every step with Eigen's Jacobi-preconditioned conjugate
gradient (src/Solvers.cpp:3-31); that stays the default and the fallback. This
module adds a graph network over the crossing graph that reads each assembled
system and emits the blocks of a block lower-triangular G in M^-1 = G^T G over
seven blocks of each node (self, left, down, left-down, right-down, left-2,
down-2). Untrained (output head at zero) it is the first-order approximate
inverse G = (I - E_lower) L^-1; it is trained to predict the exact factorised
sparse approximate inverse of the pattern -- the G that minimises the Kaporin
condition number of G A G^T, which a kernel computes per node from the
assembled system as the training target -- or, optionally, on the stochastic
Kaporin number itself (see ys_gnn.cuh for the network and include/yarnsim.h
for the C ABI). Training runs on the GPU with the
library's own BF16 tensor-core forward and backward kernels, on systems the
simulator generates from seeded batches of cloths like the plain method's
workloads: sizes 5..50, plain / twill / satin weaves, per-line material within
+-20 % of (rho 1e-3, Y 1e3, B 1e-5), blended warp / weft sets 1.5-3x apart,
S and mu within +-20 %, gravity and wind.
"""
from __future__ import annotations

import ctypes
import math
import os
from typing import Optional

import numpy as np

from . import _native as N
from .cloth import ClothBatch, ClothSpec

PARAMS_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "precond_params.npy")


OBJECTIVES = {"kaporin": 0, "fsai": 1}


def param_count() -> int:
    return int(N.load().ys_gnn_param_count())


def dims():
    """(network outputs per node, blocks of G per node)"""
    o, b = ctypes.c_int32(), ctypes.c_int32()
    N.load().ys_gnn_dims(ctypes.byref(o), ctypes.byref(b))
    return o.value, b.value


class LearnedPreconditioner:
    """The network (FP32 master parameters on the device, BF16 copies for the
    tensor cores, Adam state)."""

    def __init__(self, seed: int = 0, device: int = 0, params: Optional[np.ndarray] = None):
        h = ctypes.c_void_p()
        N.check(N.load().ys_gnn_create(int(device), int(seed), ctypes.byref(h)), "ys_gnn_create")
        self._h = h
        self.device = int(device)
        if params is not None:
            self.set_params(params)

    @classmethod
    def pretrained(cls, device: int = 0, path: str = PARAMS_FILE) -> "LearnedPreconditioner":
        """The parameters shipped with the package, trained by main() (the
        FSAI objective, selected by held-out convergence)."""
        return cls(device=device, params=np.load(path))

    def close(self):
        if getattr(self, "_h", None):
            N.load().ys_gnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(param_count(), np.float32)
        N.check(N.load().ys_gnn_get_params(self._h, ctypes.c_void_p(out.ctypes.data)), "ys_gnn_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        if p.shape != (param_count(),):
            raise ValueError("expected %d parameters" % param_count())
        N.check(N.load().ys_gnn_set_params(self._h, ctypes.c_void_p(p.ctypes.data)), "ys_gnn_set_params")

    def save(self, path: str):
        np.save(path, self.params())

    def set_objective(self, name: str):
        """"fsai" (distance to the exact FSAI's blocks; the default) or "kaporin"."""
        N.check(N.load().ys_gnn_set_objective(self._h, OBJECTIVES[name]), "ys_gnn_set_objective")

    def train_step(self, batch: ClothBatch, seed: int, lr: float) -> float:
        """One Adam step on the objective over the systems `batch` assembled
        last; returns the loss before the step."""
        loss = ctypes.c_double()
        N.check(N.load().ys_gnn_train_step(self._h, batch._h, int(seed), float(lr), ctypes.byref(loss)),
                "ys_gnn_train_step")
        return loss.value

    def loss_grad(self, batch: ClothBatch, probes: Optional[np.ndarray] = None, seed: int = 1) -> dict:
        """Loss, parameter gradient, network outputs [n][outputs] and G blocks
        [n][25 blocks] (pattern order) for the batch's last system (no update)."""
        n = batch.total_nodes
        n_out, n_blk = dims()
        loss = ctypes.c_double()
        grad = np.zeros(param_count(), np.float32)
        out = np.zeros((n, n_out), np.float32)
        gb = np.zeros((n, 25 * n_blk), np.float32)
        pr = None
        if probes is not None:
            pr = np.ascontiguousarray(probes, np.float32)
            if pr.shape != (n, 5):
                raise ValueError("probes must be [total_nodes, 5]")
        N.check(N.load().ys_gnn_loss_grad(self._h, batch._h, ctypes.c_void_p(pr.ctypes.data) if pr is not None else None,
                                          int(seed), ctypes.byref(loss), ctypes.c_void_p(grad.ctypes.data),
                                          ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(gb.ctypes.data)),
                "ys_gnn_loss_grad")
        return dict(loss=loss.value, grad=grad, outputs=out, G=gb)


def training_specs(rng: np.random.Generator, n_cloths: int, min_side: int = 5, max_side: int = 50):
    """Seeded cloths of the plain method's workloads (see the module doc)."""
    base = np.array([1e-3, 1e3, 1e-5])
    specs = []
    for _ in range(n_cloths):
        W = int(rng.integers(min_side, max_side + 1))
        blend = rng.random() < 0.5
        scale = np.ones(3)
        if blend:
            scale = 1.5 + 1.5 * rng.random(3)
            scale = np.where(rng.random(3) < 0.5, scale, 1.0 / scale)

        def lines(n, odd_scale):
            out = base * (1.0 + 0.2 * (2.0 * rng.random((n, 3)) - 1.0))
            if blend:
                out[1::2] *= odd_scale
            return out
        wind = (0.0, float(2.0 * rng.random() - 1.0), 0.0)
        specs.append(ClothSpec(width=W, length=W, warp=lines(W, scale), weft=lines(W, scale), height=0.05, L=1e-3,
                               R=1e-4, pose=int(rng.integers(0, 2)), weave=int(rng.integers(0, 3)),
                               mu=0.3 * (1 + 0.2 * (2 * rng.random() - 1)),
                               S=1e-4 * (1 + 0.2 * (2 * rng.random() - 1)), G=(0.0, 0.0, 9.8), wind_vel=wind,
                               wind_density=1.0, wind_drag=0.5, handles=[(0, 0), (W - 1, 0)]))
    return specs


def validation_residual(net: LearnedPreconditioner, batch: ClothBatch, k: int = 5, h: float = 1e-3) -> float:
    """Mean log10 of the relative residual |r| / |b| after k learned PCG
    iterations on the systems `batch` assembles at its current state: the
    conjugate-gradient speed the preconditioner is for."""
    batch.assemble(h)
    batch.set_preconditioner("learned", net)
    st = batch.solve(tol=1e-10, maxiter=k)
    batch.set_preconditioner("jacobi")
    return float(np.mean([np.log10(max(x["cg_error"], 1e-300)) for x in st]))


def train(net: LearnedPreconditioner, systems: int = 20000, cloths_per_batch: int = 64, steps_per_batch: int = 40,
          lr: float = 1e-3, seed: int = 0, h: float = 1e-3, val_every: int = 25, select: bool = True,
          objective: str = "fsai", log=None) -> dict:
    """Trains on `systems` linear systems the simulator generates: batches of
    `cloths_per_batch` seeded cloths are stepped with Jacobi-PCG for
    `steps_per_batch` steps, and every step's systems (one per cloth) feed one
    Adam step on `objective` ("fsai" or "kaporin"). The rate decays by
    cosine to 5 % of lr. Every `val_every` steps (and before the first) the
    network is scored on held-out systems by validation_residual, and the
    best-scoring parameters -- possibly the starting ones -- are kept (with
    select=False the final parameters are).
    Returns {"loss": [...], "validation": [(step, score)], "best_step": s}."""
    net.set_objective(objective)
    rng = np.random.default_rng(seed)
    vrng = np.random.default_rng(seed + 7919)
    vbatch = ClothBatch(training_specs(vrng, 8, 10, 40), device=net.device)
    for _ in range(5):
        vbatch.step(h, tol=1e-10)
    total_steps = max(1, math.ceil(systems / cloths_per_batch))
    hist, val = [], []
    best, best_step, best_params = np.inf, 0, net.params()

    def validate(k):
        nonlocal best, best_step, best_params
        score = validation_residual(net, vbatch, h=h)
        val.append((k, score))
        if score < best:
            best, best_step, best_params = score, k, net.params()
        if log is not None:
            log("step %d validation %.3f (best %.3f at %d)" % (k, score, best, best_step))

    validate(0)
    k = 0
    while k < total_steps:
        batch = ClothBatch(training_specs(rng, cloths_per_batch), device=net.device)
        for _ in range(steps_per_batch):
            if k >= total_steps:
                break
            st = batch.step(h, tol=1e-10)
            if not all(s["ok"] for s in st):
                break
            rate = lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * k / total_steps)))
            loss = net.train_step(batch, seed=(seed << 20) + k + 1, lr=rate)
            hist.append(loss)
            k += 1
            if k % val_every == 0:
                validate(k)
        batch.close()
    if k % val_every:
        validate(k)
    vbatch.close()
    if select:
        net.set_params(best_params)
    return {"loss": hist, "validation": val, "best_step": best_step}


def main(argv=None):
    """Trains the shipped parameters: python -m <package>.precond --out FILE"""
    import argparse
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=800000)
    ap.add_argument("--cloths", type=int, default=64)
    ap.add_argument("--steps-per-batch", type=int, default=40)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=PARAMS_FILE)
    a = ap.parse_args(argv)
    net = LearnedPreconditioner(seed=a.seed)
    t0 = time.time()
    res = train(net, systems=a.systems, cloths_per_batch=a.cloths, steps_per_batch=a.steps_per_batch, lr=a.lr,
                seed=a.seed, log=print)
    hist = res["loss"]
    print("trained on %d systems in %.1f s; kept the parameters of step %d (validation %.3f)" % (
        len(hist) * a.cloths, time.time() - t0, res["best_step"], min(v for _, v in res["validation"])))
    net.save(a.out)
    np.save(os.path.splitext(a.out)[0] + "_loss.npy", np.asarray(hist))
    np.save(os.path.splitext(a.out)[0] + "_validation.npy", np.asarray(res["validation"]))


if __name__ == "__main__":
    main()
