"""Control learning through the simulator: the reference's ForceNet
(src/ForceNet.h:4-24) and one step of its train_embed loop
(src/TrainEmbed.h:84-176), with the gradient of the loss through the GPU
steps taken by forward-mode tangents of the external force
(ys_step_tangent_ext) and the network's own gradient by torch autograd.

ForceNet reads the cloth state [LPos, EPos, LVel, EVel] flattened (float32)
and predicts two strengths, a lift along z and a drag along y, applied at
node (first * width + second) of each listed pair (the reference's index;
for its four corners of a square cloth the same four corners). The loss is
|mean(goal LPos) - mean(final LPos)|^2, the distance of the mass centres.

With loop="reference" the steps are those train_embed actually runs: its
`if (s = force_stop_frame)` is an assignment, so after the forced first step
the loop jumps to s = 6 and the remaining sample - 7 steps run without
force. loop="intended" applies the network at steps 0..5 as the comment
there describes; the network's input at a later forced step depends on the
earlier forces, and that dependence is carried too.
"""
from __future__ import annotations

import math
from typing import Dict, List, Sequence

import numpy as np

from .cloth import ClothBatch, ClothSpec


def _torch():
    import torch
    return torch


def ForceNet(n_in: int, n_out: int = 2):
    """src/ForceNet.h:4-24: Linear(n_in, 125) - relu - Linear(125, 60) - relu -
    Linear(60, n_out) - 0.004 sigmoid (float32, torch's default init)."""
    torch = _torch()

    class _ForceNet(torch.nn.Module):
        def __init__(self):
            super().__init__()
            self.fc1 = torch.nn.Linear(n_in, 125)
            self.fc2 = torch.nn.Linear(125, 60)
            self.fc3 = torch.nn.Linear(60, n_out)

        def forward(self, x):
            x = torch.relu(self.fc1(x))
            x = torch.relu(self.fc2(x))
            return 0.004 * torch.sigmoid(self.fc3(x))
    return _ForceNet()


def state_input(st: Dict[str, np.ndarray], nodes: slice, dtype=None):
    """[1, 10 N] (float32 as the reference casts it, unless dtype is given):
    LPos, EPos, LVel, EVel of the cloth's nodes, flattened."""
    torch = _torch()
    x = np.concatenate([st[k][nodes].reshape(-1) for k in ("LPos", "EPos", "LVel", "EVel")])
    return torch.from_numpy(x).to(torch.float32 if dtype is None else dtype).unsqueeze(0)


def _tangent_input(tg: Dict[str, np.ndarray], k: int, nodes: slice) -> np.ndarray:
    return np.concatenate([tg[f][k, nodes].reshape(-1) for f in ("LPos", "EPos", "LVel", "EVel")])


def force_nodes(width: int, force_at: Sequence) -> List[int]:
    """Node of each (first, second) pair as the reference indexes it."""
    return [int(a) * width + int(b) for a, b in force_at]


def embed_step(net, spec: ClothSpec, goal_lpos: np.ndarray, sample: int, h: float = 1e-3,
               force_at: Sequence = ((0, 0), (4, 0), (0, 4), (4, 4)), loop: str = "reference",
               tangent_mode: int = 1, tol: float = 0.0, maxiter: int = -1, device: int = 0,
               input_dtype=None) -> Dict:
    """One training evaluation of train_embed from the spec's initial state:
    returns dict(loss, forces [F, 2], grads {parameter name: array}, final
    LPos, dloss_dforces [F, 2]) and leaves the gradients in the network's
    .grad (accumulated, as loss.backward() does). tangent_mode 1 carries the
    reference's EigenSolver backward (its autograd), 0 the exact derivative.
    input_dtype: the network input's dtype (float32, the reference's cast,
    by default)."""
    torch = _torch()
    if loop not in ("reference", "intended"):
        raise ValueError("loop must be 'reference' or 'intended'")
    if sample < 2:
        raise ValueError("sample must be at least 2")
    if loop == "reference":
        schedule = [True] + [False] * max(0, sample - 7)
    else:
        schedule = [s <= 5 for s in range(sample - 1)]
    F = sum(schedule)
    D = 2 * F
    N = spec.width * spec.length
    fn = force_nodes(spec.width, force_at)
    b0 = ClothBatch([spec], device=device)
    K = b0.n_tangents
    b0.close()
    copies = max(1, math.ceil(D / K))
    batch = ClothBatch([spec] * copies, device=device)
    batch.tangent_enable(tangent_mode)
    T = batch.total_nodes
    sl = batch.node_slice(0)
    offs = [batch.node_slice(c).start for c in range(copies)]
    inputs, preds, dins = [], [], []
    fi = 0
    for forced in schedule:
        st = batch.get_state()
        if forced:
            x_in = state_input(st, sl, input_dtype)
            pred = net(x_in)
            inputs.append(x_in)
            preds.append(pred)
            tg = batch.tangent_get_state()
            dins.append([_tangent_input(tg, d % K, batch.node_slice(d // K)) for d in range(D)])
            f = pred.detach().double().numpy()[0]
            ext = np.zeros((T, 5))
            dext = np.zeros((K, T, 5))
            for o in offs:
                for n in fn:
                    ext[o + n, 2] += f[0]
                    ext[o + n, 1] += f[1]
            for d in (2 * fi, 2 * fi + 1):
                c, k = d // K, d % K
                for n in fn:
                    dext[k, offs[c] + n, 2 if d % 2 == 0 else 1] += 1.0
            stats = batch.step_tangent(h, ext, tol=tol, maxiter=maxiter, dext_force=dext)
            fi += 1
        else:
            stats = batch.step_tangent(h, None, tol=tol, maxiter=maxiter)
        if not all(s["ok"] for s in stats):
            batch.close()
            raise RuntimeError("a step failed (non-finite system or solution)")
    st = batch.get_state()
    tg = batch.tangent_get_state()
    x = st["LPos"][sl]
    goal = np.asarray(goal_lpos, np.float64).reshape(N, 3)
    dc = goal.mean(axis=0) - x.mean(axis=0)
    loss = float(dc @ dc)
    dl_dx = np.broadcast_to(-2.0 * dc / N, (N, 3))
    a = np.array([np.sum(dl_dx * tg["LPos"][d % K, batch.node_slice(d // K)]) for d in range(D)])
    batch.close()
    # reverse over the forced steps: a later force depends on the earlier ones
    # through the network's input
    g = [None] * F
    for i in reversed(range(F)):
        gi = a[2 * i:2 * i + 2].copy()
        for j in range(i + 1, F):
            xin = inputs[j].detach().requires_grad_(True)
            out = net(xin)
            (gin,) = torch.autograd.grad(out, xin, grad_outputs=torch.from_numpy(g[j][None, :]).to(out.dtype))
            gin = gin.double().numpy()[0]
            gi += np.array([gin @ dins[j][2 * i], gin @ dins[j][2 * i + 1]])
        g[i] = gi
    surrogate = sum((preds[i][0] * torch.from_numpy(g[i]).to(preds[i].dtype)).sum() for i in range(F))
    surrogate.backward()
    grads = {name: p.grad.detach().double().numpy().copy() for name, p in net.named_parameters()}
    return dict(loss=loss, forces=np.array([p.detach().double().numpy()[0] for p in preds]), grads=grads,
                final_lpos=x.copy(), dloss_dforces=np.array(g))
