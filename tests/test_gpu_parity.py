"""GPU parity: the CUDA path through the C ABI against the reference-built
fixtures and the CPU oracle.

Tolerances: assembled A and b at a given state <= 1e-11 relative (same
arithmetic, different summation order); states along a trajectory <= 1e-8
relative per step (the solve is run to Eigen's default tolerance on both
sides, so round-off is amplified only by the conditioning of A).
"""
import numpy as np
import pytest

import goldens
from layout import ref_to_node5
from pkg import gpu_available, spec_from_golden, ys

pytestmark = pytest.mark.gpu

SYSTEM_TOL = 1e-11
STATE_TOL = 1e-8


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def batch_for(g):
    b = ys.ClothBatch([spec_from_golden(g)])
    st = goldens.init_state(g)
    if st is not None:
        b.set_state(**st)
    return b


def ext5(g, total=None):
    ext = g.get("ext_force")
    return None if ext is None else np.ascontiguousarray(ref_to_node5(ext, int(g["width"]), int(g["length"])))


@pytest.mark.parametrize("name", goldens.names())
def test_system_matches_reference(name):
    g = goldens.load(name)
    b = batch_for(g)
    for s in (int(x) for x in g["dumps"]):
        b.set_state(**goldens.state(g, s))
        b.assemble(float(g["h"]), ext5(g))
        A, rhs = b.export_system(0)
        dim = A.shape[0]
        assert goldens.rel(A, g["d%d_A" % s].reshape(dim, dim)) <= SYSTEM_TOL, s
        assert goldens.rel(rhs, g["d%d_b" % s].ravel()) <= SYSTEM_TOL, s
    b.close()


@pytest.mark.parametrize("name", goldens.names())
def test_trajectory_matches_reference(name):
    g = goldens.load(name)
    b = batch_for(g)
    for s in range(int(g["steps"])):
        stats = b.step(float(g["h"]), ext5(g))
        assert stats[0]["ok"]
        ref = goldens.state(g, s + 1)
        st = b.get_state()
        for k in ("LPos", "LVel", "EPos", "EVel", "EPosBar"):
            assert goldens.rel(st[k], ref[k]) <= STATE_TOL, (s + 1, k, goldens.rel(st[k], ref[k]))
    b.close()


def test_batched_uneven_cloths_match_single_runs():
    """All fixtures stepped together in one batch: per-cloth segmented
    reductions must give each cloth exactly its own solve."""
    names = [n for n in goldens.names() if "ext_force" not in goldens.load(n)]
    gs = [goldens.load(n) for n in names]
    batch = ys.ClothBatch([spec_from_golden(g) for g in gs])
    T = batch.total_nodes
    full = {k: np.zeros((T, 3 if k.startswith("L") else 2)) for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")}
    cur = batch.get_state()
    for c, g in enumerate(gs):
        st = goldens.init_state(g) or goldens.state(g, 0)
        for k in full:
            full[k][batch.node_slice(c)] = st[k]
    batch.set_state(**full)
    steps = min(int(g["steps"]) for g in gs)
    for s in range(steps):
        stats = batch.step(1e-3)
        assert all(x["ok"] for x in stats)
        st = batch.get_state()
        for c, g in enumerate(gs):
            ref = goldens.state(g, s + 1)
            for k in ("LPos", "LVel", "EPos", "EVel"):
                assert goldens.rel(st[k][batch.node_slice(c)], ref[k]) <= STATE_TOL, (names[c], s + 1, k)
    batch.close()


def test_bitwise_deterministic():
    g = goldens.load("twill6_upright_wind_pert")
    out = []
    for _ in range(2):
        b = batch_for(g)
        for _ in range(3):
            b.step(1e-3)
        out.append(b.get_state())
        b.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


def test_apply_system_matches_dense_product():
    g = goldens.load("satin7x5_flat_pert")
    b = batch_for(g)
    b.assemble(1e-3)
    A, _ = b.export_system(0)
    W, H = int(g["width"]), int(g["length"])
    rng = np.random.default_rng(3)
    x5 = rng.standard_normal((W * H, 5))
    for v in range(H):
        for u in range(W):
            if u in (0, W - 1) or v in (0, H - 1):
                x5[u + v * W, 3:] = 0.0
    y5 = b.apply(x5)
    from layout import node5_to_ref
    yr = A @ node5_to_ref(x5, W, H)
    assert goldens.rel(node5_to_ref(y5, W, H), yr) <= 1e-13
    b.close()


def test_large_cloth_against_oracle():
    """A 50x50 twill cloth (the largest side of the batched workload) against
    the CPU oracle for a few steps."""
    from oracle.oracle import ClothSpec as OSpec, OracleCloth
    rng = np.random.default_rng(11)
    W = H = 50
    base = np.array([1e-3, 1e3, 1e-5])
    kw = dict(width=W, length=H, warp=base * (1 + 0.2 * (2 * rng.random((H, 3)) - 1)),
              weft=base * (1 + 0.2 * (2 * rng.random((W, 3)) - 1)), weave=1, pose=1, handles=[(0, 0), (W - 1, 0)],
              wind_vel=(0.1, 0.4, 0.0), wind_density=1.0, wind_drag=0.5)
    b = ys.ClothBatch([ys.ClothSpec(**kw)])
    oc = OracleCloth(OSpec(**kw))
    for _ in range(3):
        assert b.step(1e-3)[0]["ok"]
        assert oc.step(1e-3)["status"] == 0
    st, ref = b.get_state(), oc.get_state()
    for k in ("LPos", "LVel", "EPos", "EVel"):
        assert goldens.rel(st[k], ref[k]) <= STATE_TOL, k
    b.close()


def test_nonfinite_cloth_is_reported_and_left_unchanged():
    """SimStep returns false on a non-finite system (src/TrainHelper.cpp:22-48);
    the other cloths of the batch still step."""
    gs = [goldens.load("plain5_flat_rest"), goldens.load("satin7x5_flat_pert")]
    batch = ys.ClothBatch([spec_from_golden(g) for g in gs])
    st = batch.get_state()
    st["LVel"][batch.node_slice(0).start + 7, 1] = np.nan
    batch.set_state(**st)
    before = batch.get_state()
    stats = batch.step(1e-3)
    assert not stats[0]["ok"] and stats[1]["ok"]
    after = batch.get_state()
    sl = batch.node_slice(0)
    assert np.array_equal(np.nan_to_num(after["LPos"][sl]), np.nan_to_num(before["LPos"][sl]))
    assert not np.array_equal(after["LPos"][batch.node_slice(1)], before["LPos"][batch.node_slice(1)])
    batch.close()


def test_reference_style_driver_loop():
    """SimHomo-style loop (src/Simulate.h:34-101) through the reference-named API."""
    g = goldens.load("plain5_flat_rest")
    yarn = ys.Yarn(R=1e-4, rho=1e-3, Y=1e3, B=1e-5)
    cloth = ys.Cloth(5, 5, 0.05, 1e-3, 1e-4, [yarn], 1.0, 1000.0, 1000.0, 0.3, 1e-4, 1e4, ys.WovenPattern.Plain,
                     ys.InitPose.Flat)
    cloth.spec.warp, cloth.spec.weft = g["warp"], g["weft"]
    cloth.set_handles([(0, 0), (4, 0)])
    env = ys.Environment(cloth, (0.0, 0.0, 9.8), ys.Wind())
    phy = ys.PhysicsCloth(env)
    for s in range(5):
        assert ys.SimStep(cloth, phy, 1e-3)
    st = cloth.get_ClothState()
    assert goldens.rel(st.LPos, g["s5_LPos"]) <= STATE_TOL


def test_graphed_step_equals_launch_by_launch():
    """ys_use_graphs: the whole step as one CUDA graph (conditional while node
    over the PCG) gives the launch-by-launch step's states bit for bit, with
    and without an external force and after h changes (graph rebuilt)."""
    gs = [goldens.load("twill6_upright_wind_pert"), goldens.load("plain5_extforce")]
    outs = []
    for graphed in (False, True):
        b = ys.ClothBatch([spec_from_golden(g) for g in gs])
        full = b.get_state()
        ext = np.zeros((b.total_nodes, 5))
        for c, g in enumerate(gs):
            st = goldens.init_state(g) or goldens.state(g, 0)
            for k in full:
                full[k][b.node_slice(c)] = st[k]
            e = ext5(g)
            if e is not None:
                ext[b.node_slice(c)] = e
        ext[b.node_slice(0), 2] = 1e-4
        b.set_state(**full)
        b.use_graphs(graphed)
        st = []
        for k, h in enumerate([1e-3] * 4 + [5e-4] * 3):
            stats = b.step(h, ext if k % 2 else None, check_every=4)
            assert all(s["ok"] for s in stats)
            st.append((b.get_state(), [s["cg_iterations"] for s in stats]))
        b.close()
        outs.append(st)
    for (a, ia), (c, ic) in zip(*outs):
        assert ia == ic
        for k in a:
            assert np.array_equal(a[k], c[k]), k


def test_autotune_restores_state_and_keeps_results():
    """ys_autotune leaves the state as it found it, and the schedule it picks
    gives the same states as the default schedule, bit for bit."""
    gs = [goldens.load(n) for n in ("twill6_upright_wind_pert", "plain6_stiff_upright_wind")]
    runs = []
    for tune in (False, True):
        b = ys.ClothBatch([spec_from_golden(g) for g in gs])
        s0 = b.get_state()
        if tune:
            sc = b.autotune(1e-3, steps=2)
            assert sc["check_every"] in (2, 4, 8, 16, 32) and sc["ms_per_step"] > 0
            s1 = b.get_state()
            for k in s0:
                assert np.array_equal(s0[k], s1[k]), k
        out = []
        for _ in range(4):
            assert all(s["ok"] for s in b.step(1e-3))
            out.append(b.get_state())
        b.close()
        runs.append(out)
    for a, c in zip(*runs):
        for k in a:
            assert np.array_equal(a[k], c[k]), k
