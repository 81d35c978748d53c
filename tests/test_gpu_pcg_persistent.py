"""The persistent per-cloth PCG (ys_set_pcg_schedule, csrc/ys_pcg_cluster.cu)
against the phase PCG (three launches per iteration): the same Jacobi-PCG
(Eigen's ConjugateGradient, src/Solvers.cpp:3-31) with the same arithmetic
and summation order, so states, iteration counts and residuals agree bit for
bit, for every cluster shape, launch by launch and as a graph, in the
forward step, the forward-mode tangent solves (A and A^T) and the reverse
adjoint's solve.
"""
import numpy as np
import pytest

from pkg import gpu_available, ys

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _specs(sides, seed):
    rng = np.random.default_rng(seed)
    base = np.array([1e-3, 1e3, 1e-5])
    out = []
    for i, s in enumerate(sides):
        W, H = int(s[0]), int(s[1])
        j = lambda n: base * (1.0 + 0.2 * (2.0 * rng.random((n, 3)) - 1.0))  # noqa: E731
        out.append(ys.ClothSpec(width=W, length=H, warp=j(H), weft=j(W), height=0.05, L=1e-3, R=1e-4,
                                pose=i % 2, weave=i % 3, mu=0.3 * (1 + 0.1 * rng.random()),
                                S=1e-4 * (1 + 0.1 * rng.random()), wind_vel=(0.0, 0.3 + 0.2 * rng.random(), 0.0),
                                wind_density=1.0, wind_drag=0.5, handles=[(0, 0), (W - 1, 0)]))
    return out


SMALL = [(5, 5), (3, 7), (11, 9), (8, 8), (10, 12)]              # <= 128 nodes
MIXED = [(50, 50), (5, 5), (17, 23), (33, 40), (12, 12), (47, 31), (7, 19)]  # up to 2,500 nodes


def _run(sides, shape, graphed, steps=6, seed=3):
    b = ys.ClothBatch(_specs(sides, seed))
    if shape is not None:
        b.set_pcg_schedule(True, *shape)
    b.use_graphs(graphed)
    rng = np.random.default_rng(seed + 1)
    ext = 1e-4 * rng.standard_normal((b.total_nodes, 5))
    out = []
    for k, h in enumerate([1e-3] * 4 + [5e-4] * (steps - 4)):
        stats = b.step(h, ext if k % 2 else None, tol=1e-10, check_every=4)
        assert all(s["ok"] for s in stats)
        out.append((b.get_state(), [(s["cg_iterations"], s["cg_error"]) for s in stats]))
    b.close()
    return out


def _same(a, c):
    for (sa, ia), (sc, ic) in zip(a, c):
        assert ia == ic
        for k in sa:
            assert np.array_equal(sa[k], sc[k]), k


@pytest.mark.parametrize("sides,shape", [(SMALL, (128, 1)), (SMALL, (256, 1)), (SMALL, (128, 2)),
                                         (MIXED, (512, 8)), (MIXED, (1024, 4)), (MIXED, (256, 16)),
                                         (MIXED, (1024, 8))])
def test_persistent_equals_phases(sides, shape):
    ref = _run(sides, None, False)
    _same(ref, _run(sides, shape, False))


@pytest.mark.parametrize("sides,shape", [(SMALL, (128, 1)), (MIXED, (512, 8))])
def test_persistent_graphed_equals_phases(sides, shape):
    _same(_run(sides, None, True), _run(sides, shape, True))


def test_shape_that_does_not_hold_the_largest_cloth_is_refused():
    b = ys.ClothBatch(_specs(MIXED, 0))
    with pytest.raises(ys.YarnSimError):
        b.set_pcg_schedule(True, 512, 4)  # 2,048 < 2,500 nodes
    with pytest.raises(ys.YarnSimError):
        b.set_pcg_schedule(True, 384, 8)  # not a supported CTA size
    b.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_tangent_solves_equal(mode):
    """The tangent step's solves (A dq = rhs exactly; A^T in reference mode)."""
    outs = []
    for shape in (None, (128, 4)):
        b = ys.ClothBatch(_specs([(9, 11), (14, 6)], 5))
        if shape:
            b.set_pcg_schedule(True, *shape)
        b.tangent_enable(mode)
        K = b.n_tangents
        rng = np.random.default_rng(2)
        nl = sum(w + h for w, h in [(9, 11), (14, 6)])
        b.tangent_seed(rng.standard_normal((K, nl)) * 1e-4, rng.standard_normal((K, nl)) * 1e2,
                       rng.standard_normal((K, nl)) * 1e-6, rng.standard_normal((K, 2)) * 1e-5,
                       rng.standard_normal((K, 2)) * 1e-2)
        res = []
        for _ in range(3):
            st = b.step_tangent(1e-3, tol=1e-12, maxiter=100000)
            assert all(s["ok"] for s in st)
            res.append((b.get_state(), b.tangent_get_state()))
        b.close()
        outs.append(res)
    for (sa, ta), (sc, tc) in zip(*outs):
        for k in sa:
            assert np.array_equal(sa[k], sc[k]), k
        for k in ta:
            assert np.array_equal(ta[k], tc[k]), k


@pytest.mark.parametrize("mode", ["exact", "reference"])
def test_adjoint_solve_equal(mode):
    outs = []
    for shape in (None, (128, 2)):
        b = ys.ClothBatch(_specs([(12, 13)], 7))
        if shape:
            b.set_pcg_schedule(True, *shape)
        N = b.total_nodes
        rng = np.random.default_rng(4)
        g = dict(LPos=rng.standard_normal((N, 3)), LVel=rng.standard_normal((N, 3)),
                 EPos=rng.standard_normal((N, 2)), EVel=rng.standard_normal((N, 2)),
                 EPosBar=rng.standard_normal((N, 2)))
        adj = ys.Adjoint(b, mode)
        gs, gp, ge = adj.step_back(1e-3, g, None, tol=1e-12, maxiter=100000, want_ext=True)
        outs.append((gs, gp, ge))
        adj.close()
        b.close()
    (a, pa, ea), (c, pc, ec) = outs
    for k in a:
        assert np.array_equal(a[k], c[k]), k
    for k in pa:
        assert np.array_equal(pa[k], pc[k]), k
    assert np.array_equal(ea, ec)


def test_autotune_offers_the_persistent_schedule():
    b = ys.ClothBatch(_specs(SMALL, 1))
    s0 = b.get_state()
    sc = b.autotune(1e-3, steps=2)
    assert sc["pcg"] in ("phases", "persistent") and sc["ms_per_step"] > 0
    s1 = b.get_state()
    for k in s0:
        assert np.array_equal(s0[k], s1[k]), k
    b.close()


@pytest.mark.parametrize("threads", [64, 256])
def test_producer_block_size_does_not_change_results(threads):
    """The record producers and the gather at another block size
    (ys_set_producer_threads): the same bits."""
    def run(t):
        b = ys.ClothBatch(_specs(MIXED, 9))
        if t:
            b.set_producer_threads(t)
        out = []
        for _ in range(3):
            assert all(s["ok"] for s in b.step(1e-3, tol=1e-10))
            out.append(b.get_state())
        b.close()
        return out
    for a, c in zip(run(None), run(threads)):
        for k in a:
            assert np.array_equal(a[k], c[k]), k
