"""The learned preconditioner's CPU oracle (oracle/gnn_oracle.py), checked on
its own: its autograd gradient against central finite differences (BF16
rounding switched off, so the loss is smooth), G block lower triangular with
M^-1 = G^T G symmetric positive definite and log |det G| the sum over its
diagonal blocks, the untrained network's analytic inverse, and the probe
generator's Rademacher signs."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
from oracle import gnn_oracle as go  # noqa: E402


def synthetic_system(topo, seed):
    """Slots of a diagonally dominant system on the batch's stencil."""
    rng = np.random.default_rng(seed)
    n = topo.n
    s = np.zeros((159, n))
    for st in range(13):
        m = topo.stencil[:, st] >= 0
        for k in range(9):
            s[go.SLOT_LL + 9 * st + k] = np.where(m, 0.05 * rng.standard_normal(n), 0.0)
    for r in range(3):
        s[go.SLOT_LL + 3 * r + r] = 2.0 + rng.random(n)
    s[go.SLOT_LE_SELF:go.SLOT_EE_SELF] = 0.05 * rng.standard_normal((12, n))
    s[go.SLOT_EE_SELF:go.SLOT_EE_SELF + 2] = 1.5 + rng.random((2, n))
    for d in range(4):
        m = topo.nbr[:, d] >= 0
        s[go.SLOT_LE_NBR + 3 * d:go.SLOT_LE_NBR + 3 * d + 3] = np.where(m, 0.05 * rng.standard_normal((3, n)), 0)
        s[go.SLOT_EL_NBR + 3 * d:go.SLOT_EL_NBR + 3 * d + 3] = np.where(m, 0.05 * rng.standard_normal((3, n)), 0)
        s[go.SLOT_EE_NBR + d] = np.where(m, -0.3 * rng.random(n), 0)
    return s


@pytest.fixture()
def smooth(monkeypatch):
    monkeypatch.setattr(go, "bf16", lambda x: x)


def test_oracle_gradient_matches_finite_differences(smooth):
    topo = go.Topology([(4, 4), (5, 3)], handles=[[(0, 0)], [(0, 0), (4, 0)]])
    slots = synthetic_system(topo, 1)
    p0 = go.init_params(3).astype(np.float64)
    w = go.rademacher(7, topo.n)
    r = go.evaluate(slots, topo, p0, w)
    rng = np.random.default_rng(5)
    for _ in range(4):
        d = rng.standard_normal(go.N_PARAMS)
        eps = 1e-6
        lp = go.evaluate(slots, topo, p0 + eps * d, w)["loss"]
        lm = go.evaluate(slots, topo, p0 - eps * d, w)["loss"]
        fd = (lp - lm) / (2 * eps)
        an = float(r["grad"] @ d)
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


def dense_g(r, topo):
    n = topo.n
    G = np.zeros((5 * n, 5 * n))
    Gb = r["G"].reshape(n, go.BLOCKS, 5, 5)
    for i in range(n):
        for b in range(go.BLOCKS):
            j = topo.pat[i, b]
            if j >= 0:
                G[5 * i:5 * i + 5, 5 * j:5 * j + 5] = Gb[i, b]
    return G


def test_preconditioner_is_block_lower_triangular_and_spd():
    topo = go.Topology([(5, 5)], handles=[[(0, 0), (4, 0)]])
    slots = synthetic_system(topo, 2)
    r = go.evaluate(slots, topo, go.init_params(4), go.rademacher(3, topo.n))
    G = dense_g(r, topo)
    n = topo.n
    for i in range(n):
        assert not G[5 * i:5 * i + 5, 5 * i + 5:].any()  # nothing right of the diagonal block
    M = G.T @ G
    assert np.allclose(M, M.T)
    assert np.linalg.eigvalsh(M).min() > 0.0
    ld = np.linalg.slogdet(G)[1]
    blocks = sum(np.linalg.slogdet(G[5 * i:5 * i + 5, 5 * i:5 * i + 5])[1] for i in range(n))
    assert abs(ld - blocks) < 1e-8 * max(1.0, abs(ld))


def test_untrained_head_gives_the_analytic_inverse():
    """Head weights and bias zero: G = (I - E_lower) L^-1 blockwise."""
    topo = go.Topology([(4, 5)], handles=[[(0, 0)]])
    slots = synthetic_system(topo, 3)
    p = go.init_params(5)
    p[go.P_WH:] = 0.0
    r = go.evaluate(slots, topo, p, go.rademacher(1, topo.n))
    assert np.abs(r["o"]).max() == 0.0
    Gb = r["G"].reshape(topo.n, go.BLOCKS, 5, 5)
    for i in range(topo.n):
        assert np.allclose(Gb[i, 0], r["Linv"][i])
        for b in range(1, go.BLOCKS):
            j = topo.pat[i, b]
            if j >= 0:
                assert np.allclose(Gb[i, b], -r["E"][i, b - 1] @ r["Linv"][j])


def test_rademacher_signs_are_balanced():
    w = go.rademacher(11, 400)
    assert set(np.unique(w)) == {-1.0, 1.0}
    assert abs(w.mean()) < 0.1


def test_fsai_target_is_the_pattern_inverse_with_unit_diagonal_blocks():
    """The exact FSAI target: G* (from N*) has the pattern, (G* S G*^T)_ii = I
    on every diagonal block (S the symmetric part of A), and the network's
    parametrisation of the target reproduces G* (N* = 0 for absent sources)."""
    topo = go.Topology([(5, 4), (3, 3)], handles=[[(0, 0)], [(0, 0)]])
    slots = synthetic_system(topo, 4)
    Linv, ok = go.block_factor(slots)
    Nt = go.fsai_targets(slots, topo, Linv)
    n = topo.n
    G = np.zeros((5 * n, 5 * n))
    for i in range(n):
        for b in range(go.BLOCKS):
            j = topo.pat[i, b]
            if j < 0:
                assert np.all(Nt[i, b] == 0.0)
                continue
            Nb = Nt[i, b] + (np.eye(5) if b == 0 else 0.0)
            G[5 * i:5 * i + 5, 5 * j:5 * j + 5] = Nb @ Linv[j]
    # dense A from the slots (FP32 values, as the target reads them)
    e = np.eye(5 * n)
    A = np.stack([go.spmv(slots, torch_t(e[:, k].reshape(n, 5)), topo).numpy().reshape(-1) for k in range(5 * n)], 1)
    S = 0.5 * (A + A.T)
    M = G @ S @ G.T
    for i in range(n):
        assert np.allclose(M[5 * i:5 * i + 5, 5 * i:5 * i + 5], np.eye(5), atol=1e-9)


def torch_t(x):
    import torch
    return torch.as_tensor(x, dtype=torch.float64)


def test_fsai_objective_gradient_matches_finite_differences(smooth):
    topo = go.Topology([(4, 4)], handles=[[(0, 0)]])
    slots = synthetic_system(topo, 5)
    p0 = go.init_params(6)
    r = go.evaluate_fsai(slots, topo, p0)
    rng = np.random.default_rng(2)
    for _ in range(3):
        d = rng.standard_normal(go.N_PARAMS)
        d /= np.linalg.norm(d)
        eps = 1e-4
        lp = go.evaluate_fsai(slots, topo, p0 + eps * d)["loss"]
        lm = go.evaluate_fsai(slots, topo, p0 - eps * d)["loss"]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - r["grad"] @ d) <= 1e-6 * max(1.0, abs(fd)), (fd, r["grad"] @ d)


def test_seven_block_pattern_leaves_iterations_to_learn():
    """Why G has seven blocks: on a system the oracle assembles (a 10 x 10
    plain cloth after 4 steps), the exact FSAI -- the Kaporin minimiser a
    network on the pattern can at best reach -- needs at most one PCG
    iteration fewer than the untrained first-order form on the 3-block
    pattern (9 -> 8), but at least two fewer on the 7-block pattern (9 -> 6)."""
    from oracle import oracle as O
    rng = np.random.default_rng(7)
    base = np.array([1e-3, 1e3, 1e-5])
    lines = lambda n: base * (1 + 0.2 * (2 * rng.random((n, 3)) - 1))
    W = 10
    spec = O.ClothSpec(width=W, length=W, warp=lines(W), weft=lines(W), pose=0, weave=0, wind_vel=(0, 0.5, 0),
                       wind_density=1.0, wind_drag=0.5, handles=[(0, 0), (W - 1, 0)])
    c = O.OracleCloth(spec)
    for _ in range(4):
        c.step(1e-3, cg_tol=1e-10)
    A, b = c.system(1e-3)
    slots, A5, b5 = go.slots_from_dense(A, b, W, W)
    topo = go.Topology([(W, W)], handles=[[(0, 0), (W - 1, 0)]])
    Linv, ok = go.block_factor(slots)
    _, E = go.features(slots, topo, Linv, ok)
    its = {}
    for nb in (3, 7):
        first = np.zeros((topo.n, nb, 5, 5))
        for bb in range(1, nb):
            first[:, bb] = -E[:, bb - 1] * (topo.pat[:, bb] >= 0)[:, None, None]
        exact = go.fsai_targets(slots, topo, Linv, blocks=nb)
        its[nb] = [go.pcg_iterations(A5, b5, go.dense_g(N, Linv, topo, nb)) for N in (first, exact)]
    assert its[3][1] >= its[3][0] - 1, its
    assert its[7][1] <= its[7][0] - 2, its
