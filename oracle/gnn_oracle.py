"""CPU oracle of the learned preconditioner (test infrastructure only: the
product runs the CUDA kernels of ys_gnn.cu and never imports this file).

The learned preconditioner has no counterpart in the reference (its solve is
Eigen's Jacobi-PCG, src/Solvers.cpp:3-31), so this oracle restates the
library's own definition independently of its kernels: the system features,
the graph network (BF16 operands rounded where the tensor cores read them),
the blocks of the block lower-triangular G, the Kaporin loss
log(w^T G A G^T w / n) - (2 / n) log |det G|, and the FSAI objective (the
mean squared distance of the blocks N to those of the pattern's exact
factorised sparse approximate inverse), in float64 PyTorch on the CPU; the
parameter gradients come from torch.autograd, not from the hand-written
backward the GPU runs. Rounding to BF16 uses straight-through estimators (the value is rounded,
the derivative is the identity), which is what the GPU's BF16 operands amount
to.

Inputs: the system's coefficient slots [159, n] (ys_get_system_slots), the
batch topology (per-node cloth width / height, u, v, flags) and the packed
FP32 parameter vector.
"""
from __future__ import annotations

import numpy as np
import torch

# slot layout of one row block (the library's stencil storage)
SLOT_LL, SLOT_LE_SELF, SLOT_EL_SELF, SLOT_EE_SELF = 0, 117, 123, 129
SLOT_LE_NBR, SLOT_EL_NBR, SLOT_EE_NBR = 131, 143, 155
STENCIL = [(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1), (-2, 0), (2, 0), (0, -2), (0, 2), (-1, -1), (1, -1), (-1, 1),
           (1, 1)]
YARN_NBR = [(-1, 0), (1, 0), (0, -1), (0, 1)]  # left, right, down, up
IN, HID, MSG, OUT, LAYERS, OUT_SCALE, BLOCKS = 128, 64, 320, 192, 3, 0.1, 7
# lower offsets: self, left, down, left-down, right-down, left-2, down-2; G uses
# the first BLOCKS, the features the six couplings
PATTERN = [(0, 0), (-1, 0), (0, -1), (-1, -1), (1, -1), (-2, 0), (0, -2)]
UPPER = [(1, 0), (0, 1), (1, 1), (-1, 1), (2, 0), (0, 2)]
P_W0 = 0
P_B0 = P_W0 + HID * IN
P_L0 = P_B0 + HID
P_LSTRIDE = HID * MSG + HID
P_WH = P_L0 + LAYERS * P_LSTRIDE
P_BH = P_WH + OUT * HID
N_PARAMS = P_BH + OUT


def p_w(l):
    return P_L0 + l * P_LSTRIDE


def p_b(l):
    return p_w(l) + HID * MSG


class Topology:
    """Node order of a batch: cloth after cloth, node u + v * W."""

    def __init__(self, sizes, handles=None, pose_flags=None):
        us, vs, Ws, Hs, fixed = [], [], [], [], []
        for c, (W, H) in enumerate(sizes):
            hs = set(map(tuple, handles[c])) if handles is not None else set()
            for v in range(H):
                for u in range(W):
                    us.append(u)
                    vs.append(v)
                    Ws.append(W)
                    Hs.append(H)
                    fixed.append((u, v) in hs)
        self.u = np.array(us)
        self.v = np.array(vs)
        self.W = np.array(Ws)
        self.H = np.array(Hs)
        self.fixed = np.array(fixed)
        self.n = len(us)
        self.interior = (self.u > 0) & (self.u < self.W - 1) & (self.v > 0) & (self.v < self.H - 1)
        idx = np.arange(self.n)

        def nb(du, dv):
            ok = (self.u + du >= 0) & (self.u + du < self.W) & (self.v + dv >= 0) & (self.v + dv < self.H)
            return np.where(ok, idx + du + dv * self.W, -1)
        self.stencil = np.stack([nb(du, dv) for du, dv in STENCIL], 1)  # [n, 13]
        self.nbr = np.stack([nb(du, dv) for du, dv in YARN_NBR], 1)     # [n, 4]
        self.pat = np.stack([nb(du, dv) for du, dv in PATTERN], 1)      # [n, 7] (G: first BLOCKS)
        self.upper = np.stack([nb(du, dv) for du, dv in UPPER], 1)      # [n, 6]


def bf16(x):
    """Round to BF16 (nearest even), straight-through for the gradient."""
    return x + (x.to(torch.bfloat16).to(x.dtype) - x).detach()


def f32(x):
    return x.to(torch.float32).to(torch.float64)


def diag_blocks(slots):
    n = slots.shape[1]
    D = np.zeros((n, 5, 5))
    for r in range(3):
        for c in range(3):
            D[:, r, c] = slots[SLOT_LL + 3 * r + c]
        for k in range(2):
            D[:, r, 3 + k] = slots[SLOT_LE_SELF + 2 * r + k]
            D[:, 3 + k, r] = slots[SLOT_EL_SELF + 3 * k + r]
    D[:, 3, 3] = slots[SLOT_EE_SELF]
    D[:, 4, 4] = slots[SLOT_EE_SELF + 1]
    return D


def nbr_block(slots, d):
    """[n, 5, 5] block A(i, j) of yarn neighbour d."""
    n = slots.shape[1]
    B = np.zeros((n, 5, 5))
    s = d + 1
    k = 0 if d < 2 else 1
    for r in range(3):
        for c in range(3):
            B[:, r, c] = slots[SLOT_LL + 9 * s + 3 * r + c]
        B[:, r, 3 + k] = slots[SLOT_LE_NBR + 3 * d + r]
        B[:, 3 + k, r] = slots[SLOT_EL_NBR + 3 * d + r]
    B[:, 3 + k, 3 + k] = slots[SLOT_EE_NBR + d]
    return B


def offset_block(slots, du, dv):
    """[n, 5, 5] block A(i, i + (du, dv)): full for yarn neighbours, else the x part."""
    if (du, dv) in YARN_NBR:
        return nbr_block(slots, YARN_NBR.index((du, dv)))
    n = slots.shape[1]
    B = np.zeros((n, 5, 5))
    s = STENCIL.index((du, dv))
    for r in range(3):
        for c in range(3):
            B[:, r, c] = slots[SLOT_LL + 9 * s + 3 * r + c]
    return B


def block_factor(slots):
    """L^-1 [n, 5, 5] (FP32 values) and the factorisation flags."""
    D = diag_blocks(slots)
    S = 0.5 * (D + np.transpose(D, (0, 2, 1)))
    n = len(S)
    Linv = np.zeros((n, 5, 5))
    ok = np.ones(n, bool)
    for i in range(n):
        try:
            L = np.linalg.cholesky(S[i])
            if not np.all(np.isfinite(L)):
                raise np.linalg.LinAlgError
        except np.linalg.LinAlgError:
            ok[i] = False
            d = np.abs(np.diag(D[i]))
            L = np.diag(np.where((d > 0) & np.isfinite(d), np.sqrt(d), 1.0))
        Linv[i] = np.linalg.inv(L)
        Linv[i] = np.tril(Linv[i])
    return Linv.astype(np.float32).astype(np.float64), ok


def scaled(slots, topo, Linv, du, dv, idx):
    """E = L_i^-1 A(i, j) L_j^-T for j = idx (-1: zero), in FP32 values."""
    m = idx >= 0
    Lj = Linv[np.where(m, idx, 0)]
    E = Linv @ offset_block(slots, du, dv) @ np.transpose(Lj, (0, 2, 1))
    E[~m] = 0.0
    return E.astype(np.float32).astype(np.float64)


def features(slots, topo: Topology, Linv, ok):
    """f [n, 128] (before BF16 rounding) and the scaled couplings E [n, 6, 5, 5]
    to the six lower offsets (G uses the first BLOCKS - 1 of them)."""
    n = topo.n
    f = np.zeros((n, IN))
    E = np.zeros((n, 6, 5, 5))
    sl32 = slots.astype(np.float32).astype(np.float64)
    for b in range(1, 7):
        E[:, b - 1] = scaled(sl32, topo, Linv, *PATTERN[b], topo.pat[:, b])
        if b <= 2:
            f[:, 25 * (b - 1):25 * b] = E[:, b - 1].reshape(n, 25)
        else:
            f[:, 50 + 9 * (b - 3):59 + 9 * (b - 3)] = E[:, b - 1, :3, :3].reshape(n, 9)
    for q, (du, dv) in enumerate(UPPER):
        Eu = scaled(sl32, topo, Linv, du, dv, topo.upper[:, q])
        f[:, 86 + q] = np.sqrt((Eu ** 2).sum((1, 2)))
    f[:, 92] = (~ok).astype(float)
    f[:, 93] = topo.interior.astype(float)
    f[:, 94] = topo.fixed.astype(float)
    f[:, 95] = ((topo.u == 0) | (topo.u == topo.W - 1)).astype(float)
    f[:, 96] = ((topo.v == 0) | (topo.v == topo.H - 1)).astype(float)
    return f, E


def network(params, f, topo: Topology):
    """Outputs o [n, 128] (torch, differentiable in params)."""
    nbr = torch.as_tensor(topo.nbr)
    W0 = bf16(params[P_W0:P_B0].view(HID, IN))
    h = torch.relu(bf16(f) @ W0.T + params[P_B0:P_L0])
    for l in range(LAYERS):
        hb = bf16(h)
        zero = torch.zeros(1, HID, dtype=h.dtype)
        hz = torch.cat([hb, zero], 0)
        msg = torch.cat([hb] + [hz[torch.where(nbr[:, d] >= 0, nbr[:, d], topo.n)] for d in range(4)], 1)
        Wl = bf16(params[p_w(l):p_b(l)].view(HID, MSG))
        h = h + torch.relu(msg @ Wl.T + params[p_b(l):p_b(l) + HID])
    Wh = bf16(params[P_WH:P_BH].view(OUT, HID))
    return bf16(h) @ Wh.T + params[P_BH:P_BH + OUT]


def n_blocks(o, E, topo: Topology):
    """N [n, BLOCKS, 5, 5] over the lower pattern (zero where the source is outside)."""
    n = topo.n
    Ns = [OUT_SCALE * o[:, 0:25].reshape(n, 5, 5)]
    Et = torch.as_tensor(E)
    for b in range(1, BLOCKS):
        m = torch.as_tensor(topo.pat[:, b] >= 0, dtype=o.dtype).view(n, 1, 1)
        Ns.append(m * (OUT_SCALE * o[:, 25 * b:25 * b + 25].reshape(n, 5, 5) - Et[:, b - 1]))
    return torch.stack(Ns, 1)


def g_blocks(Nb, Linv, topo: Topology):
    """G [n, BLOCKS, 5, 5]: (I + N_0) L_i^-1 and N_b L_src^-1."""
    Lt = torch.as_tensor(Linv)
    eye = torch.eye(5, dtype=Nb.dtype)
    out = [(eye + Nb[:, 0]) @ Lt]
    for b in range(1, BLOCKS):
        j = topo.pat[:, b]
        out.append(Nb[:, b] @ Lt[torch.as_tensor(np.where(j >= 0, j, 0))])
    return torch.stack(out, 1)


def apply_gt(Gb, w, topo: Topology):
    """u = G^T w (each row's blocks scattered onto their sources)."""
    u = torch.einsum("nrc,nr->nc", Gb[:, 0], w)
    for b in range(1, BLOCKS):
        j = topo.pat[:, b]
        m = j >= 0
        contrib = torch.einsum("nrc,nr->nc", Gb[:, b], w)
        u = u.index_add(0, torch.as_tensor(j[m]), contrib[torch.as_tensor(m)])
    return u


def spmv(slots, x, topo: Topology):
    """y = A x with the stencil slots (FP32 coefficient values, as the GPU reads them)."""
    S = torch.as_tensor(slots.astype(np.float32).astype(np.float64))
    n = topo.n
    xz = torch.cat([x, torch.zeros(1, 5, dtype=x.dtype)], 0)
    yl = torch.zeros(n, 3, dtype=x.dtype)
    for s in range(13):
        j = torch.as_tensor(np.where(topo.stencil[:, s] >= 0, topo.stencil[:, s], n))
        xj = xz[j]
        for r in range(3):
            for c in range(3):
                yl[:, r] = yl[:, r] + S[SLOT_LL + 9 * s + 3 * r + c] * xj[:, c]
    ye = torch.zeros(n, 2, dtype=x.dtype)
    for r in range(3):
        for k in range(2):
            yl[:, r] = yl[:, r] + S[SLOT_LE_SELF + 2 * r + k] * x[:, 3 + k]
    for k in range(2):
        ye[:, k] = S[SLOT_EE_SELF + k] * x[:, 3 + k]
        for c in range(3):
            ye[:, k] = ye[:, k] + S[SLOT_EL_SELF + 3 * k + c] * x[:, c]
    for d in range(4):
        k = 0 if d < 2 else 1
        j = torch.as_tensor(np.where(topo.nbr[:, d] >= 0, topo.nbr[:, d], n))
        xj = xz[j]
        for r in range(3):
            yl[:, r] = yl[:, r] + S[SLOT_LE_NBR + 3 * d + r] * xj[:, 3 + k]
        ye[:, k] = ye[:, k] + S[SLOT_EE_NBR + d] * xj[:, 3 + k]
        for c in range(3):
            ye[:, k] = ye[:, k] + S[SLOT_EL_NBR + 3 * d + c] * xj[:, c]
    return torch.cat([yl, ye], 1)


def evaluate(slots, topo: Topology, params, probes):
    """dict(loss, grad [N_PARAMS], o [n, 128], G [n, 75], f, E, Linv, chol_ok)."""
    Linv, ok = block_factor(slots)
    f, E = features(slots, topo, Linv, ok)
    p = torch.as_tensor(np.asarray(params, np.float64), dtype=torch.float64).requires_grad_(True)
    o = network(p, torch.as_tensor(f), topo)
    Nb = n_blocks(o, E, topo)
    Gb = g_blocks(Nb, Linv, topo)
    w = torch.as_tensor(np.asarray(probes, np.float64))
    u = apply_gt(Gb, w, topo)
    tr = (u * spmv(slots, u, topo)).sum()
    nd = 5.0 * topo.n
    eye = torch.eye(5, dtype=torch.float64)
    logdet = torch.linalg.slogdet(eye + Nb[:, 0])[1].sum() + float(np.log(np.diagonal(Linv, 0, 1, 2)).sum())
    loss = torch.log(tr / nd) - 2.0 * logdet / nd
    loss.backward()
    return dict(loss=float(loss.detach()), grad=p.grad.numpy().copy(), o=o.detach().numpy(),
                G=Gb.detach().reshape(topo.n, 25 * BLOCKS).numpy(), f=f, E=E, Linv=Linv, chol_ok=ok)


def a_block(slots, du, dv):
    """[n, 5, 5] A(i, i + (du, dv)): the diagonal block, a yarn neighbour's
    block, the x part of another stencil offset, or zero outside the stencil."""
    if (du, dv) == (0, 0):
        return diag_blocks(slots)
    if (du, dv) in YARN_NBR or (du, dv) in STENCIL:
        return offset_block(slots, du, dv)
    return np.zeros((slots.shape[1], 5, 5))


def fsai_targets(slots, topo: Topology, Linv, blocks: int = None):
    """N* [n, BLOCKS, 5, 5]: the exact FSAI of the pattern, G*_i = chol(X_ii)^-1
    X^T with X = sym(A)[P_i, P_i]^-1 E_i, as N*_i,0 = G*_i,0 L_i - I and
    N*_i,b = G*_i,b L_src (A from the FP32 slot values; zero for absent
    sources)."""
    nblk = BLOCKS if blocks is None else blocks
    sl32 = slots.astype(np.float32).astype(np.float64)
    n = topo.n
    blocks = {}
    for b1 in range(nblk):
        for b2 in range(nblk):
            d = (PATTERN[b2][0] - PATTERN[b1][0], PATTERN[b2][1] - PATTERN[b1][1])
            if d not in blocks:
                blocks[d] = a_block(sl32, *d)
    L = np.linalg.inv(Linv)
    out = np.zeros((n, nblk, 5, 5))
    for i in range(n):
        bs = [b for b in range(nblk) if topo.pat[i, b] >= 0]
        m = len(bs)
        S = np.zeros((5 * m, 5 * m))
        for a1, b1 in enumerate(bs):
            for a2, b2 in enumerate(bs):
                d = (PATTERN[b2][0] - PATTERN[b1][0], PATTERN[b2][1] - PATTERN[b1][1])
                B = blocks[d][topo.pat[i, b1]]
                S[5 * a1:5 * a1 + 5, 5 * a2:5 * a2 + 5] += 0.5 * B
                S[5 * a2:5 * a2 + 5, 5 * a1:5 * a1 + 5] += 0.5 * B.T
        E = np.zeros((5 * m, 5))
        E[:5] = np.eye(5)
        X = np.linalg.solve(S, E)
        Lx = np.linalg.cholesky(0.5 * (X[:5] + X[:5].T))
        Gt = np.linalg.solve(Lx, X.T)
        for a, b in enumerate(bs):
            out[i, b] = Gt[:, 5 * a:5 * a + 5] @ L[topo.pat[i, b]] - (np.eye(5) if b == 0 else 0.0)
    return out


def evaluate_fsai(slots, topo: Topology, params):
    """dict(loss, grad [N_PARAMS], target [n, BLOCKS, 5, 5]) of the FSAI
    objective: mean over nodes of sum_b |N_i,b - N*_i,b|_F^2."""
    Linv, ok = block_factor(slots)
    f, E = features(slots, topo, Linv, ok)
    target = fsai_targets(slots, topo, Linv)
    p = torch.as_tensor(np.asarray(params, np.float64), dtype=torch.float64).requires_grad_(True)
    o = network(p, torch.as_tensor(f), topo)
    Nb = n_blocks(o, E, topo)
    loss = ((Nb - torch.as_tensor(target)) ** 2).sum() / topo.n
    loss.backward()
    return dict(loss=float(loss.detach()), grad=p.grad.numpy().copy(), target=target)


def slots_from_dense(A, b, W, H):
    """Stencil slots [159, W H] of one cloth from the oracle's dense system
    (3 N Lagrangian DOFs, then 2 per interior node in row order); the
    Eulerian DOFs of boundary nodes become identity rows with a zero
    right-hand side, as the library stores them. Returns (slots, A5, b5) with
    A5 [5 N, 5 N] and b5 [5 N] in node-block order."""
    N = W * H
    idx = np.full(A.shape[0], -1)
    for n in range(N):
        idx[3 * n:3 * n + 3] = 5 * n + np.arange(3)
    for v in range(1, H - 1):
        for u in range(1, W - 1):
            e = 3 * N + 2 * ((u - 1) + (v - 1) * (W - 2))
            idx[e:e + 2] = 5 * (u + v * W) + np.arange(3, 5)
    A5 = np.zeros((5 * N, 5 * N))
    A5[np.ix_(idx, idx)] = A
    used = np.zeros(5 * N, bool)
    used[idx] = True
    A5[~used, ~used] = 1.0
    b5 = np.zeros(5 * N)
    b5[idx] = b
    S = np.zeros((159, N))
    blk = lambda i, j: A5[5 * i:5 * i + 5, 5 * j:5 * j + 5]
    for n in range(N):
        u, v = n % W, n // W
        D = blk(n, n)
        for s_, (du, dv) in enumerate(STENCIL):
            if 0 <= u + du < W and 0 <= v + dv < H:
                S[SLOT_LL + 9 * s_:SLOT_LL + 9 * s_ + 9, n] = blk(n, n + du + dv * W)[:3, :3].reshape(9)
        S[SLOT_LE_SELF:SLOT_LE_SELF + 6, n] = D[:3, 3:].reshape(6)
        S[SLOT_EL_SELF:SLOT_EL_SELF + 6, n] = D[3:, :3].reshape(6)
        S[SLOT_EE_SELF:SLOT_EE_SELF + 2, n] = np.diag(D[3:, 3:])
        for d, (du, dv) in enumerate(YARN_NBR):
            if 0 <= u + du < W and 0 <= v + dv < H:
                B = blk(n, n + du + dv * W)
                k = 3 if d < 2 else 4
                S[SLOT_LE_NBR + 3 * d:SLOT_LE_NBR + 3 * d + 3, n] = B[:3, k]
                S[SLOT_EL_NBR + 3 * d:SLOT_EL_NBR + 3 * d + 3, n] = B[k, :3]
                S[SLOT_EE_NBR + d, n] = B[k, k]
    return S, A5, b5


def dense_g(Nb, Linv, topo: Topology, blocks: int):
    """Dense G [5 n, 5 n] from blocks N [n, blocks, 5, 5] in the network's
    parametrisation over the first `blocks` pattern offsets."""
    n = topo.n
    G = np.zeros((5 * n, 5 * n))
    for i in range(n):
        for b in range(blocks):
            j = topo.pat[i, b]
            if j >= 0:
                G[5 * i:5 * i + 5, 5 * j:5 * j + 5] = (Nb[i, b] + (np.eye(5) if b == 0 else 0.0)) @ Linv[j]
    return G


def pcg_iterations(A, b, G, tol=1e-10, maxiter=500):
    """Plain preconditioned CG with M^-1 = G^T G: iterations to |r| < tol |b|."""
    x = np.zeros_like(b)
    r = b.copy()
    z = G.T @ (G @ r)
    p = z.copy()
    rz = r @ z
    bb = np.linalg.norm(b)
    for it in range(1, maxiter + 1):
        q = A @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if np.linalg.norm(r) < tol * bb:
            return it
        z = G.T @ (G @ r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return maxiter


def init_params(seed: int) -> np.ndarray:
    """A random parameter vector with a non-zero head (for gradient checks)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    p[P_W0:P_B0] = rng.uniform(-1, 1, HID * IN) * np.sqrt(6 / (HID + IN))
    p[P_B0:P_L0] = 0.05 * rng.standard_normal(HID)
    for l in range(LAYERS):
        p[p_w(l):p_b(l)] = rng.uniform(-1, 1, HID * MSG) * 0.5 * np.sqrt(6 / (HID + MSG))
        p[p_b(l):p_b(l) + HID] = 0.05 * rng.standard_normal(HID)
    p[P_WH:P_BH] = rng.uniform(-1, 1, OUT * HID) * 0.3 * np.sqrt(6 / (OUT + HID))
    p[P_BH:P_BH + OUT] = 0.05 * rng.standard_normal(OUT)
    return p


def rademacher(seed: int, n: int) -> np.ndarray:
    """The GPU's probe generator: splitmix64 finaliser of seed + golden * (idx + 1),
    idx = c * n + node, sign from the low bit -> [n, 5]."""
    M = (1 << 64) - 1
    out = np.zeros((5, n))
    for c in range(5):
        for i in range(n):
            z = (seed + 0x9E3779B97F4A7C15 * (c * n + i + 1)) & M
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
            z ^= z >> 31
            out[c, i] = 1.0 if z & 1 else -1.0
    return out.T.copy()
