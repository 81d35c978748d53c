"""Learned preconditioner on the GPU: the tcgen05 GEMM against torch, the
network's outputs, G blocks, both training objectives (the exact-FSAI
regression and the Kaporin number) and their hand-written gradients against
the CPU oracle (torch float64 autograd), training and what it gains over the
untrained network, the learned solve against Jacobi-PCG at the same FP64
residual, and the learned step as one CUDA graph (fallback included)."""
import os
import sys

import numpy as np
import pytest

from pkg import gpu_available, ys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
from oracle import gnn_oracle as go  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def to_bf16_bits(x):
    import torch
    return torch.as_tensor(x, dtype=torch.float32).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)


@pytest.mark.parametrize("N", [64, 128, 192])
def test_tc_gemm_matches_torch(N):
    import ctypes
    import torch
    rng = np.random.default_rng(N)
    M, K = 300, 192
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    Ab, Bb = to_bf16_bits(A), to_bf16_bits(B)
    C = np.zeros((M, N), np.float32)
    N_ = ys._native
    N_.check(N_.load().ys_tc_gemm_bf16(0, ctypes.c_void_p(Ab.ctypes.data), ctypes.c_void_p(Bb.ctypes.data),
                                       ctypes.c_void_p(C.ctypes.data), M, N, K), "ys_tc_gemm_bf16")
    At = torch.as_tensor(Ab.view(np.int16)).view(torch.bfloat16).double()
    Bt = torch.as_tensor(Bb.view(np.int16)).view(torch.bfloat16).double()
    ref = (At @ Bt.T).numpy()
    assert np.abs(C - ref).max() <= 1e-4 * np.abs(ref).max()


def stepped_batch(seed, n_cloths, lo, hi, steps=4):
    rng = np.random.default_rng(seed)
    specs = ys.training_specs(rng, n_cloths, lo, hi)
    b = ys.ClothBatch(specs)
    for _ in range(steps):
        assert all(s["ok"] for s in b.step(1e-3, tol=1e-10))
    return b, specs


def topo_of(specs):
    return go.Topology([(s.width, s.length) for s in specs], handles=[s.handles for s in specs])


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_network_and_gradient_match_oracle():
    """Kaporin objective: outputs and G blocks within BF16 tolerance (2e-2
    relative), the loss within 2e-3 absolute (a logarithm near 0); the
    hand-written gradient within 5e-2 relative of the oracle's autograd
    gradient, cosine >= 0.998."""
    b, specs = stepped_batch(11, 3, 5, 9)
    params = go.init_params(3)
    net = ys.LearnedPreconditioner(params=params)
    net.set_objective("kaporin")
    n = b.total_nodes
    w = go.rademacher(9, n)
    gpu = net.loss_grad(b, probes=w)
    seeded = net.loss_grad(b, seed=9)
    assert abs(seeded["loss"] - gpu["loss"]) <= 1e-9
    slots, _ = b.system_slots()
    ora = go.evaluate(slots, topo_of(specs), params, w)
    assert rel(gpu["outputs"], ora["o"]) < 2e-2
    assert rel(gpu["G"], ora["G"]) < 2e-2
    assert abs(gpu["loss"] - ora["loss"]) <= 2e-3
    g, o = gpu["grad"].astype(np.float64), ora["grad"]
    assert rel(g, o) < 5e-2
    assert g @ o / (np.linalg.norm(g) * np.linalg.norm(o)) >= 0.998
    # every parameter group receives its share of the gradient
    for lo, hi in [(go.P_W0, go.P_B0), (go.p_w(0), go.p_b(0)), (go.p_w(2), go.p_b(2)), (go.P_WH, go.P_BH)]:
        assert rel(g[lo:hi], o[lo:hi]) < 8e-2
    net.close()
    b.close()


def test_fsai_objective_and_gradient_match_oracle():
    """FSAI objective: the exact-FSAI targets the GPU computes per node (FP32
    local Cholesky) and the loss within 2e-2 relative of the oracle's
    (float64), the hand-written gradient within 5e-2 relative of the
    oracle's autograd gradient, cosine >= 0.998."""
    b, specs = stepped_batch(13, 3, 5, 9)
    params = go.init_params(4)
    net = ys.LearnedPreconditioner(params=params)
    gpu = net.loss_grad(b)
    slots, _ = b.system_slots()
    ora = go.evaluate_fsai(slots, topo_of(specs), params)
    assert abs(gpu["loss"] - ora["loss"]) <= 2e-2 * abs(ora["loss"])
    g, o = gpu["grad"].astype(np.float64), ora["grad"]
    assert rel(g, o) < 5e-2
    assert g @ o / (np.linalg.norm(g) * np.linalg.norm(o)) >= 0.998
    for lo, hi in [(go.P_W0, go.P_B0), (go.p_w(0), go.p_b(0)), (go.p_w(2), go.p_b(2)), (go.P_WH, go.P_BH)]:
        assert rel(g[lo:hi], o[lo:hi]) < 8e-2
    net.close()
    b.close()


def test_training_lowers_the_loss():
    net = ys.LearnedPreconditioner(seed=1)
    b, _ = stepped_batch(12, 16, 5, 20, steps=1)
    losses = []
    for k in range(40):
        b.step(1e-3, tol=1e-10)
        losses.append(net.train_step(b, seed=k + 1, lr=2e-3))
    assert np.isfinite(losses).all()
    # compare the same system before and after
    before = net.loss_grad(b, seed=99)["loss"]
    for k in range(40):
        net.train_step(b, seed=200 + k, lr=2e-3)
    after = net.loss_grad(b, seed=99)["loss"]
    assert after < before
    b.close()
    net.close()


def trained_net():
    if os.path.exists(ys.precond.PARAMS_FILE):
        return ys.LearnedPreconditioner.pretrained()
    net = ys.LearnedPreconditioner(seed=0)
    ys.train_preconditioner(net, systems=64 * 120, cloths_per_batch=64, steps_per_batch=40, lr=2e-3, seed=0)
    return net


def test_learned_solve_same_residual_fewer_iterations():
    """Held-out cloths: the learned solve meets the same |b - A x| <= 1e-10 |b|
    rule as Jacobi-PCG (checked on the true residual), the states agree to the
    solve's accuracy, and it needs fewer iterations."""
    net = trained_net()
    rng = np.random.default_rng(777)
    specs = ys.training_specs(rng, 12, 10, 40)
    runs = {}
    for kind in ("jacobi", "learned"):
        b = ys.ClothBatch(specs)
        if kind == "learned":
            b.set_preconditioner("learned", net)
        its, states = [], []
        for _ in range(6):
            st = b.step(1e-3, tol=1e-10)
            assert all(s["ok"] and s["cg_error"] <= 1e-10 for s in st)
            its.append([s["cg_iterations"] for s in st])
            states.append(b.get_state())
        if kind == "learned":
            assert b.precond_info()["fallbacks"] == 0
            # the check: true residual of a fresh learned solve
            b.assemble(1e-3)
            stats = b.solve(tol=1e-10)
            x = b.solution()
            ax = b.apply(x)
            slots, rhs = b.system_slots()
            for c in range(b.n_cloths):
                sl = b.node_slice(c)
                r = rhs.T[sl] - ax[sl]
                assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(rhs.T[sl]), c
        runs[kind] = (np.array(its), states)
        b.close()
    ij, il = runs["jacobi"][0], runs["learned"][0]
    assert il.mean() < ij.mean()
    for sj, sl in zip(runs["jacobi"][1], runs["learned"][1]):
        for k in ("LPos", "LVel"):
            assert np.linalg.norm(sl[k] - sj[k]) <= 1e-7 * np.linalg.norm(sj[k]) + 1e-15, k
    net.close()


def test_broken_network_falls_back_to_jacobi():
    net = ys.LearnedPreconditioner(params=np.full(ys.precond.param_count(), np.nan, np.float32))
    rng = np.random.default_rng(5)
    specs = ys.training_specs(rng, 3, 6, 12)
    ref = ys.ClothBatch(specs)
    b = ys.ClothBatch(specs)
    b.set_preconditioner("learned", net)
    for _ in range(3):
        assert all(s["ok"] for s in ref.step(1e-3, tol=1e-10))
        assert all(s["ok"] for s in b.step(1e-3, tol=1e-10))
    assert b.precond_info()["fallbacks"] == 3
    a, c = ref.get_state(), b.get_state()
    for k in a:
        assert np.array_equal(a[k], c[k]), k
    b.close()
    ref.close()
    net.close()


def test_graphed_learned_step_equals_launch_by_launch():
    """The learned-preconditioner step as one CUDA graph launch per step (the
    network evaluated every third solve, in the graph that holds it) gives the
    states and iteration counts of the launch-by-launch learned step, bit for
    bit, across a change of h."""
    net = trained_net()
    specs = ys.training_specs(np.random.default_rng(11), 6, 8, 30)
    a, c = ys.ClothBatch(specs), ys.ClothBatch(specs)
    for x in (a, c):
        x.set_preconditioner("learned", net)
        x.precond_refresh(3)
    c.use_graphs(True)
    for k in range(7):
        h = 1e-3 if k != 4 else 5e-4
        sa, sc = a.step(h, tol=1e-10), c.step(h, tol=1e-10)
        assert all(s["ok"] for s in sc)
        assert [s["cg_iterations"] for s in sa] == [s["cg_iterations"] for s in sc]
    sa, sc = a.get_state(), c.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sc[k]), k
    assert a.precond_info() == c.precond_info() == dict(learned_solves=7, fallbacks=0)
    a.close()
    c.close()
    net.close()


def test_graphed_learned_step_with_a_broken_network_falls_back_to_jacobi():
    """In the graph, a network of NaN weights breaks the learned solve down; the
    graph's verdict kernel holds the update back and the step is solved again by
    Jacobi-PCG: states equal the Jacobi step's bit for bit."""
    net = ys.LearnedPreconditioner(params=np.full(ys.precond.param_count(), np.nan, np.float32))
    specs = ys.training_specs(np.random.default_rng(5), 3, 6, 12)
    ref, b = ys.ClothBatch(specs), ys.ClothBatch(specs)
    b.set_preconditioner("learned", net)
    b.use_graphs(True)
    for _ in range(3):
        assert all(s["ok"] for s in ref.step(1e-3, tol=1e-10))
        assert all(s["ok"] for s in b.step(1e-3, tol=1e-10))
    assert b.precond_info()["fallbacks"] == 3
    x, y = ref.get_state(), b.get_state()
    for k in x:
        assert np.array_equal(x[k], y[k]), k
    b.close()
    ref.close()
    net.close()


def test_training_lowers_the_kaporin_number_on_held_out_systems():
    """Training on the Kaporin objective (without model selection) lowers the
    Kaporin condition number of G A G^T on systems it never saw (same
    systems, same probes; the loss differs from log kappa / n only by the
    systems' own log det A / n)."""
    b, _ = stepped_batch(4242, 24, 10, 45, steps=6)
    untrained = ys.LearnedPreconditioner(seed=0)
    trained = ys.LearnedPreconditioner(seed=0)
    untrained.set_objective("kaporin")
    ys.train_preconditioner(trained, systems=64 * 60, cloths_per_batch=64, steps_per_batch=30, lr=1e-3, seed=3,
                            select=False, objective="kaporin")
    lt = trained.loss_grad(b, seed=5)["loss"]
    lu = untrained.loss_grad(b, seed=5)["loss"]
    assert lt < lu
    b.close()
    trained.close()
    untrained.close()


def test_trained_network_converges_faster_than_the_untrained_one():
    """What training gains: on held-out systems the shipped network (trained
    on the FSAI objective) reaches a residual at least three times smaller
    than the untrained network (the analytic first-order inverse) after 5
    learned PCG iterations, and needs fewer iterations to 1e-10."""
    b, _ = stepped_batch(999, 16, 10, 40, steps=5)
    shipped = trained_net()
    untrained = ys.LearnedPreconditioner(seed=0)
    rs = ys.precond.validation_residual(shipped, b)
    ru = ys.precond.validation_residual(untrained, b)
    assert rs <= ru - 0.5, (rs, ru)
    its = {}
    for name, net in (("trained", shipped), ("untrained", untrained)):
        b.assemble(1e-3)
        b.set_preconditioner("learned", net)
        st = b.solve(tol=1e-10)
        assert all(x["ok"] and x["cg_error"] <= 1e-10 for x in st)
        its[name] = np.mean([x["cg_iterations"] for x in st])
    b.set_preconditioner("jacobi")
    assert its["trained"] < its["untrained"], its
    b.close()
    shipped.close()
    untrained.close()
