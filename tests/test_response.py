"""Impact-zone collision response (Collision::collision_response,
src/Collision.cpp:73-156) and the backward of its projections
(src/Collision.cpp:478-682) against the CPU restatement
oracle/response_oracle.py.

- CPU: the product's response loop and projection solver (csrc/ys_zones.h),
  driven by the test-only emulator's detection, give the oracle's rounds,
  zones and received impacts, its positions to 1e-12 m and velocities to
  1e-9 m/s; every projection meets its optimality conditions to 1e-9 of the
  thickness; the backward matches the oracle's restatement of the
  reference's derivative to 1e-9 relative, and that derivative matches
  central differences of the projection.
- GPU: ys_collider_respond and ys_collider_respond_backward give the same
  results through the C ABI.
Parity with the reference's own numbers is unpinned: its projections run an
augmented Lagrangian over Alglib, which is not part of the reference tree.
"""
import numpy as np
import pytest

import response_cases as RC
from oracle import response_oracle as RO
from pkg import gpu_available, ys

SCENES = {
    "drop20": lambda: RC.drop_scene(20, depth=1e-3),
    "drop24_deep": lambda: RC.drop_scene(24, depth=1.6e-3, levels=4, seed=3),
    "fold10": lambda: RC.fixture_scene("collide_fold10"),
    "sphere12": lambda: RC.fixture_scene("collide_sphere12"),
}
DAMP = 0.1


def _faces(s):
    return RC.topology(s["W"], s["H"])[0]


def _oracle(s, damp=DAMP, mass=None):
    return RO.respond(s["x"], _faces(s), RC.emu_detector(s), s["thickness"], s["h"], damp, obs_x=s["obs_x"],
                      v=s["v"], mass=mass)


def _rows(accepted):
    return np.array([[t, *nd, tt, *w, *n] for (t, nd, tt, w, n) in accepted]).reshape(-1, 13)


def _canon(rows):
    """Each received impact as its constraint: type, nodes in ascending order
    and the coefficient w_k n of each (an edge-edge impact found with its
    edges in the other roles is the same constraint; which of the two comes
    first in time can flip with the last bit of the positions)."""
    out = []
    for r in rows:
        nodes = r[1:5].astype(int)
        coef = r[6:10, None] * r[None, 10:13]
        o = np.argsort(nodes)
        out.append((int(r[0]), tuple(nodes[o]), coef[o].reshape(-1)))
    return out


def _check_against_oracle(res, x, v, n_rounds, n_zones, received):
    assert res["converged"]
    assert n_rounds == res["rounds"] and n_zones == res["zones"]
    mine, theirs = _canon(received), _canon(_rows(res["accepted"]))
    assert len(mine) == len(theirs)
    for a, b in zip(mine, theirs):
        assert a[:2] == b[:2]
        # the GPU's narrow phase contracts to FMA: weights and normals agree to
        # ~1e-12, their products to 1e-10
        assert np.abs(a[2] - b[2]).max() <= 1e-10
    assert np.abs(x - res["x"]).max() <= 1e-12
    assert np.abs(v - res["v"]).max() <= 1e-9


def test_ldp_meets_optimality_and_matches_scipy():
    rng = np.random.default_rng(0)
    for k, n in ((1, 3), (4, 6), (12, 9), (30, 12), (8, 30)):
        G = rng.normal(size=(k, n))
        h = G @ rng.normal(size=n) - rng.random(k) * (rng.random(k) < 0.5)  # feasible, some tight
        u, lam, st = RC.emu_ldp(G, h)
        uo, lo, ok = RO.ldp(G, h)
        assert ok and st == 0
        slack = G @ u - h
        assert slack.min() >= -1e-12 and lam.min() >= 0.0
        assert np.abs(lam * slack).max() <= 1e-12 * max(1.0, lam.max())
        assert np.abs(u - G.T @ lam).max() <= 1e-12 * max(1.0, np.abs(u).max())
        assert np.abs(u - uo).max() <= 1e-10 * max(1.0, np.abs(uo).max())
    # duplicated and opposite constraints
    G = np.array([[1.0, 0.0], [1.0, 0.0], [2.0, 0.0], [0.0, 1.0]])
    u, lam, st = RC.emu_ldp(G, np.array([1.0, 1.0, 2.0, -1.0]))
    assert st == 0 and np.allclose(u, [1.0, 0.0], atol=1e-14)
    u, lam, st = RC.emu_ldp(np.array([[1.0], [-1.0]]), np.array([1.0, 1.0]))  # x >= 1 and x <= -1
    assert st == 1 and not np.any(u)


@pytest.mark.parametrize("name", sorted(SCENES))
def test_emulated_response_matches_oracle(name):
    s = SCENES[name]()
    res = _oracle(s)
    got = RC.emu_respond(s, damp=DAMP)
    info = got["info"]
    assert info[1] == 1 and info[2] == int(res["changed"]) and info[4] == 0
    assert info[5] == len(res["accepted"]) and info[6] == len(res["tape"])
    _check_against_oracle(res, got["x"], got["v"], info[0], info[3], got["impacts"])
    for rec in res["tape"]:
        assert RO.kkt_residual(rec, s["thickness"], s["obs_x"], res["accepted"], s["x"]) <= 1e-9
    assert res["changed"] and res["rounds"] >= 1


def test_response_separates_the_cloth_from_the_sphere():
    s = RC.drop_scene(20, depth=1e-3)
    got = RC.emu_respond(s)
    r = np.linalg.norm(s["obs_x"], axis=1).max()
    before = np.linalg.norm(s["x"], axis=1) - r
    after = np.linalg.norm(got["x"], axis=1) - r
    assert before.min() < -5e-4 and after.min() > -1e-4  # the polyhedron lies inside the sphere
    moved = np.abs(got["x"] - s["x"]).max(axis=1) > 0
    assert np.allclose(got["v"][~moved], s["v"][~moved], rtol=0, atol=0)


def test_response_with_masses_matches_oracle():
    s = RC.drop_scene(16, depth=1.2e-3, seed=5)
    mass = 1.0 + np.random.default_rng(1).random(s["W"] * s["H"])
    res = _oracle(s, mass=mass)
    got = RC.emu_respond(s, mass=mass)
    _check_against_oracle(res, got["x"], got["v"], got["info"][0], got["info"][3], got["impacts"])


@pytest.mark.parametrize("name", ["drop20", "fold10"])
def test_emulated_backward_matches_oracle(name):
    s = SCENES[name]()
    res = _oracle(s)
    got = RC.emu_respond(s)
    rng = np.random.default_rng(7)
    gx, gv = rng.normal(size=s["x"].shape), rng.normal(size=s["x"].shape)
    g, gw, gn, _ = RC.emu_respond_backward(gx, gv, got["info"][5])
    og, ogv, ogw, ogn = RO.respond_backward(res, s["obs_x"], s["thickness"], s["h"], DAMP, gx, gv)
    _check_backward(g, gw, gn, got["impacts"], og, ogw, ogn, res)


def _check_backward(g, gw, gn, received, og, ogw, ogn, res):
    scale = lambda a: max(1.0, np.abs(a).max())
    assert np.abs(g - og).max() <= 1e-9 * scale(og)
    # weights and normals: impacts received with the same node roles (an
    # edge-edge impact may arrive with its edges swapped, see _canon)
    same = np.all(received[:, 1:5] == _rows(res["accepted"])[:, 1:5], axis=1)
    assert same.mean() >= 0.9
    assert np.abs(gw[same] - ogw[same]).max() <= 1e-9 * scale(ogw)
    assert np.abs(gn[same] - ogn[same]).max() <= 1e-9 * scale(ogn)


def test_projection_derivative_matches_central_differences():
    """The reference's derivative of one projection (as restated) against
    central differences of the projection in its anchor, weights and normals,
    on the zones of the first round of a drop (their active sets are stable
    under the perturbation)."""
    s = RC.drop_scene(14, depth=1.2e-3, seed=2)
    res = RO.respond(s["x"], _faces(s), RC.emu_detector(s), s["thickness"], s["h"], DAMP, obs_x=s["obs_x"],
                     v=s["v"], max_iter=1)
    rng = np.random.default_rng(3)
    checked = 0
    for rec in res["tape"][:6]:
        nodes, imps = rec["nodes"], rec["imps"]
        gz = rng.normal(size=3 * len(nodes))
        gin, grads = RO.projection_backward(rec, res["accepted"], s["obs_x"], s["thickness"], gz)

        def loss(xold_zone, acc):
            x = np.array(s["x"], np.float64).copy()
            xold = x.copy()
            xold[nodes] = xold_zone.reshape(-1, 3)
            r = RO.project(nodes, imps, acc, x, xold, s["obs_x"], s["thickness"], None)
            return float(np.dot(gz, r["xout"]))
        x0 = np.array(s["x"])[nodes].reshape(-1)
        eps = 1e-8
        fd = np.zeros_like(x0)
        for i in range(len(x0)):
            e = np.zeros_like(x0)
            e[i] = eps
            fd[i] = (loss(x0 + e, res["accepted"]) - loss(x0 - e, res["accepted"])) / (2 * eps)
        assert np.abs(fd - gin).max() <= 1e-6 * max(1.0, np.abs(gin).max())
        for idx in imps:
            for part, k in (("w", 4), ("n", 3)):
                for q in range(k):
                    acc_p, acc_m = list(res["accepted"]), list(res["accepted"])
                    t, nd, tt, w, n = acc_p[idx]
                    arr = np.array(w if part == "w" else n, np.float64)
                    ap, am = arr.copy(), arr.copy()
                    ap[q] += eps
                    am[q] -= eps
                    if part == "w":
                        acc_p[idx], acc_m[idx] = (t, nd, tt, tuple(ap), n), (t, nd, tt, tuple(am), n)
                    else:
                        acc_p[idx], acc_m[idx] = (t, nd, tt, w, tuple(ap)), (t, nd, tt, w, tuple(am))
                    fdq = (loss(x0, acc_p) - loss(x0, acc_m)) / (2 * eps)
                    an = grads[idx][0][q] if part == "w" else grads[idx][1][q]
                    assert abs(fdq - an) <= 1e-5 * max(1.0, abs(an)), (part, q, fdq, an)
        checked += 1
    assert checked >= 3


# ---------------------------------------------------------------- GPU
def _collider(s):
    of = s["obs_faces"]
    c = ys.Collider(s["W"], s["H"], obstacle_faces=of if len(of) else None, n_obstacle_nodes=len(s["obs_x"]),
                    thickness=s["thickness"])
    ox = s["obs_x"] if len(s["obs_x"]) else None
    c.set_positions(s["x"], s["x_prev"], ox, ox)
    return c


def _received_rows(imp):
    return np.column_stack([imp["type"], imp["nodes"], imp["t"], imp["w"], imp["n"]]).astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SCENES))
def test_gpu_response_matches_oracle(name):
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = SCENES[name]()
    res = _oracle(s)
    c = _collider(s)
    out = c.respond(v=s["v"], h=s["h"], damp=DAMP)
    assert out["changed"] == res["changed"] and out["infeasible"] == 0
    assert out["impacts"] == len(res["accepted"]) and out["projections"] == len(res["tape"])
    _check_against_oracle(res, out["x"], out["v"], out["rounds"], out["zones"], _received_rows(c.response_impacts()))
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["drop20", "fold10"])
def test_gpu_backward_matches_oracle(name):
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = SCENES[name]()
    res = _oracle(s)
    c = _collider(s)
    c.respond(v=s["v"], h=s["h"], damp=DAMP)
    rng = np.random.default_rng(7)
    gx, gv = rng.normal(size=s["x"].shape), rng.normal(size=s["x"].shape)
    got = c.respond_backward(gx, gv)
    og, ogv, ogw, ogn = RO.respond_backward(res, s["obs_x"], s["thickness"], s["h"], DAMP, gx, gv)
    assert np.array_equal(got["v"], ogv)
    _check_backward(got["x"], got["w"], got["n"], _received_rows(c.response_impacts()), og, ogw, ogn, res)
    c.close()


@pytest.mark.gpu
def test_gpu_response_errors():
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = SCENES["drop20"]()
    c = ys.Collider(s["W"], s["H"], obstacle_faces=s["obs_faces"], n_obstacle_nodes=len(s["obs_x"]))
    with pytest.raises(ys.YarnSimError):
        c.respond(v=s["v"])  # before set_positions
    with pytest.raises(ys.YarnSimError):
        c.respond_backward(np.zeros((s["W"] * s["H"], 3)))  # before a response
    c.set_positions(s["x"], s["x_prev"], s["obs_x"], s["obs_x"])
    with pytest.raises(ys.YarnSimError):
        c.respond(v=s["v"], h=0.0)
    with pytest.raises(ys.YarnSimError):
        c.respond(v=s["v"], mass=np.zeros(s["W"] * s["H"]))
    out = c.respond(v=s["v"], max_iter=1, check=False)  # one round cannot confirm convergence
    assert not out["converged"] and out["rounds"] == 1
    with pytest.raises(ys.YarnSimError):
        c.set_positions(s["x"], s["x_prev"], s["obs_x"], s["obs_x"])
        c.respond(v=s["v"], max_iter=1)
    c.close()


@pytest.mark.gpu
def test_simstep_with_collision_matches_step_then_oracle_response():
    """SimStep(cloth, phy, collision, h) (src/TrainHelper.cpp:99-158): the
    step, collision_response(0.1) and cloth.update() give the plain step's
    state followed by the oracle's response."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    yarn = ys.Yarn(R=1e-4, rho=1e-3, Y=1e3, B=1e-5)

    def make():
        cloth = ys.Cloth(10, 10, 0.05, 1e-3, 1e-4, [yarn], 1.0, 1000.0, 1000.0, 0.3, 1e-4, 1e4,
                         ys.WovenPattern.Plain, ys.InitPose.Flat)
        cloth.set_handles([(0, 0), (9, 0)])
        phy = ys.PhysicsCloth(ys.Environment(cloth, (0.0, 0.0, 9.8), ys.Wind()))
        st = phy.batch.get_state()
        st["LVel"][:, 2] = 3.0  # into the sphere above
        # off the plane: on an exactly planar cloth the self-collision cubics
        # of coplanar edges vanish and their roots are rounding noise (in the
        # reference too), which the GPU's FMA and the CPU round differently
        st["LPos"][:, 2] += np.random.default_rng(0).normal(0.0, 1e-5, len(st["LPos"]))
        phy.batch.set_state(**st)
        return cloth, phy, st
    cloth, phy, st0 = make()
    r = 0.02
    ox, of = RC.icosphere(r, 3)
    ox = ox + st0["LPos"].mean(axis=0) + np.array([0.0, 0.0, 2e-3 + r])
    col = ys.Collision(cloth, ox, of, thickness=5e-4, h=1e-3)
    assert ys.SimStep(cloth, phy, col, 1e-3)
    got = phy.batch.get_state()
    assert col.last["changed"] and col.last["converged"]
    cloth2, phy2, _ = make()
    assert ys.SimStep(cloth2, phy2, 1e-3)
    plain = phy2.batch.get_state()
    s = dict(W=10, H=10, x=plain["LPos"], x_prev=st0["LPos"], obs_x=ox, obs_faces=of, thickness=5e-4, h=1e-3,
             v=plain["LVel"])
    res = _oracle(s)
    assert res["changed"]
    assert np.abs(got["LPos"] - res["x"]).max() <= 1e-12
    assert np.abs(got["LVel"] - res["v"]).max() <= 1e-9
    fixed = np.zeros(100, bool)
    fixed[[0, 9]] = True
    assert np.array_equal(got["LPosFix"][~fixed], got["LPos"][~fixed])
    assert np.array_equal(got["LPosFix"][fixed], plain["LPosFix"][fixed])
    assert np.array_equal(got["EPos"], plain["EPos"])
    col.close()


def test_scene_topology_is_the_collider_mesh():
    F, E = RC.topology(6, 5)
    faces, edges = ys.cloth_mesh_topology(6, 5)
    assert np.array_equal(F, faces) and np.array_equal(E, edges)


@pytest.mark.parametrize("name", ["drop20", "drop24_deep"])
def test_full_backward_matches_central_differences(name):
    """The first round of the response (max_iter = 1: one detection, one
    projection per zone) as a map of the step's end and start positions: the
    backward with the impact chain and the root's exact derivative against
    central differences of L = g . x_out + gv . v_out, both on the product's
    code (emulator). One round keeps each zone's anchor and its positions the
    same, where the reference's attribution of anchor gradients is exact."""
    s = SCENES[name]()
    base = RC.emu_respond(s, max_iter=1)
    rng = np.random.default_rng(11)
    gx, gv = rng.normal(size=s["x"].shape), rng.normal(size=s["x"].shape)
    g, gw, gn, gp = RC.emu_respond_backward(gx, gv, base["info"][5], flags=3)

    def loss(x, xp):
        out = RC.emu_respond(dict(s, x=x, x_prev=xp), max_iter=1)
        assert out["info"][5] == base["info"][5]  # the same impacts
        return float(np.sum(gx * out["x"]) + np.sum(gv * out["v"]))
    moved = np.where(np.abs(base["x"] - s["x"]).max(axis=1) > 0)[0]
    eps = 1e-9
    checked = 0
    for nd in moved[:5]:
        for c in range(3):
            for which in ("x", "x_prev"):
                xp_, xm_ = np.array(s["x"], float), np.array(s["x"], float)
                pp_, pm_ = np.array(s["x_prev"], float), np.array(s["x_prev"], float)
                (xp_ if which == "x" else pp_)[nd, c] += eps
                (xm_ if which == "x" else pm_)[nd, c] -= eps
                fd = (loss(xp_, pp_) - loss(xm_, pm_)) / (2 * eps)
                an = (g if which == "x" else gp)[nd, c]
                assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (which, nd, c, fd, an)
                checked += 1
    assert checked >= 15
    # the reference's root derivative differs only where the roots move
    g1, _, _, gp1 = RC.emu_respond_backward(gx, gv, base["info"][5], flags=1)
    assert np.abs(g1 - g).max() > 0.0 or np.abs(gp1 - gp).max() > 0.0


@pytest.mark.gpu
def test_gpu_full_backward_matches_emulated():
    """ys_collider_respond_backward with the impact chain (both root
    derivatives) equals the product's host code on the emulator's detection."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = SCENES["drop20"]()
    emu = RC.emu_respond(s)
    c = _collider(s)
    out = c.respond(v=s["v"], h=s["h"], damp=DAMP)
    assert out["impacts"] == emu["info"][5]
    rng = np.random.default_rng(5)
    gx, gv = rng.normal(size=s["x"].shape), rng.normal(size=s["x"].shape)
    for flags in (1, 3):
        got = c.respond_backward(gx, gv, impacts=True, exact_root=bool(flags & 2))
        g, gw, gn, gp = RC.emu_respond_backward(gx, gv, emu["info"][5], flags=flags)
        assert np.abs(got["x"] - g).max() <= 1e-8 * max(1.0, np.abs(g).max())
        assert np.abs(got["x_prev"] - gp).max() <= 1e-8 * max(1.0, np.abs(gp).max())
    c.close()


def test_tangled_layers_resolve_by_reverting_zones():
    """The 50 x 50 sphere detection fixture is tangled beyond what a step's
    detection separates: some zones gather constraints with nearly opposite
    normals whose exact projection lies far away. Those zones go back to
    their positions at the start of the step (reverted), and the response
    converges in a few rounds."""
    import time
    s = RC.fixture_scene("collide_sphere50")
    t0 = time.time()
    got = RC.emu_respond(s)
    assert got["info"][1] == 1 and got["info"][7] == 0  # converged, no overflow
    assert got["info"][8] > 0  # reverted zones
    rev = [i for i in range(len(got["x"])) if np.array_equal(got["x"][i], s["x_prev"][i])
           and not np.array_equal(s["x"][i], s["x_prev"][i])]
    assert rev, "no node back at its start position"
    assert time.time() - t0 < 60.0


def test_zone_cap_stops_the_response():
    """A zone that gathers more impacts than the zone limit (set to 8 here)
    stops the response (no convergence, zone_overflow) instead of projecting
    it (the reference would run its 100 rounds and exit)."""
    s = RC.fixture_scene("collide_sphere50")
    L = RC._lib()
    L.emu_set_max_zone_impacts(8)
    try:
        got = RC.emu_respond(s)
    finally:
        L.emu_set_max_zone_impacts(-1)
    assert got["info"][7] == 1 and got["info"][1] == 0


@pytest.mark.gpu
def test_gpu_tangled_layers_and_zone_cap():
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = RC.fixture_scene("collide_sphere50")
    c = _collider(s)
    out = c.respond(v=s["v"], h=s["h"], damp=DAMP)
    emu = RC.emu_respond(s, damp=DAMP)
    assert out["converged"] and not out["zone_overflow"] and out["reverted"] == emu["info"][8]
    c.set_positions(s["x"], s["x_prev"], s["obs_x"], s["obs_x"])
    c.set_max_zone_impacts(8)
    out = c.respond(v=s["v"], h=s["h"], damp=DAMP, check=False)
    assert out["zone_overflow"] and not out["converged"]
    c.set_positions(s["x"], s["x_prev"], s["obs_x"], s["obs_x"])
    with pytest.raises(ys.YarnSimError) as e:
        c.respond(v=s["v"], h=s["h"], damp=DAMP)
    assert e.value.status == 4
    c.close()


def test_zone_projection_matches_a_general_qp_solver():
    """The zone projection (least-distance programme through NNLS) against
    scipy's SLSQP on the primal problem min 1/2 sum a |x - x_old|^2 subject
    to w n . x >= thickness, for random zones with shared nodes."""
    from scipy.optimize import minimize
    rng = np.random.default_rng(4)
    for trial in range(12):
        m, k = int(rng.integers(2, 7)), int(rng.integers(1, 6))
        xold = rng.normal(size=(m, 3)) * 1e-3
        a = 0.5 + rng.random(m)
        G = np.zeros((k, 3 * m))
        h = np.zeros(k)
        for j in range(k):
            nodes = rng.choice(m, size=min(m, 3), replace=False)
            n = rng.normal(size=3)
            n /= np.linalg.norm(n)
            w = rng.normal(size=len(nodes))
            for q, nd in enumerate(nodes):
                G[j, 3 * nd:3 * nd + 3] += w[q] * n
            h[j] = 5e-4 - G[j] @ xold.reshape(-1) + 1e-3 * rng.random()  # violated at x_old
        # our solver in y = sqrt(a) x: min |u| s.t. (G / sqrt(a)) u >= h
        isa = np.repeat(1.0 / np.sqrt(a), 3)
        u, lam, st = RC.emu_ldp(G * isa[None, :], h)
        if st == 1:
            continue
        x_ours = xold.reshape(-1) + u * isa
        res = minimize(lambda x: 0.5 * np.sum(np.repeat(a, 3) * (x - xold.reshape(-1)) ** 2), xold.reshape(-1),
                       jac=lambda x: np.repeat(a, 3) * (x - xold.reshape(-1)),
                       constraints=[dict(type="ineq", fun=lambda x: G @ x - (h + G @ xold.reshape(-1)),
                                         jac=lambda x: G)],
                       method="SLSQP", options=dict(ftol=1e-16, maxiter=500))
        assert res.success, res.message
        assert np.abs(res.x - x_ours).max() <= 1e-8 * max(1.0, np.abs(x_ours).max()) + 1e-10


def test_large_zone_solver_matches_the_exact_one():
    """Hildreth's iterations (ldp_sparse, the solver of zones above 64
    impacts) against the exact least-distance solver on random zones of
    contact-like rows (4 node blocks each, shared nodes, some constraints
    inactive): u and the multipliers to 1e-9 relative."""
    rng = np.random.default_rng(8)
    for trial in range(6):
        m, k = int(rng.integers(20, 60)), int(rng.integers(30, 90))
        n = 3 * m
        cols = np.full((k, 4), -1, np.int32)
        coef = np.zeros((k, 4, 3))
        G = np.zeros((k, n))
        for j in range(k):
            nodes = rng.choice(m, size=int(rng.integers(1, 5)), replace=False)
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            w = rng.random(len(nodes))
            w = w / w.sum() * (1 if rng.random() < 0.5 else -1)
            for q, (nd, wq) in enumerate(zip(nodes, w)):
                cols[j, q] = nd
                coef[j, q] = wq * nrm
                G[j, 3 * nd:3 * nd + 3] += wq * nrm
        h = rng.normal(size=k) * 1e-4
        u_e, lam_e, st_e = RC.emu_ldp(G, h)
        if st_e != 0:
            continue
        u_s, lam_s, st_s = RC.emu_ldp_sparse(cols, coef, h, n)
        assert st_s == 0
        assert np.abs(u_s - u_e).max() <= 1e-9 * max(np.abs(u_e).max(), 1e-300), trial
        assert np.abs(lam_s - lam_e).max() <= 1e-7 * max(np.abs(lam_e).max(), 1e-300), trial
        assert (G @ u_s - h).min() >= -1e-12 * np.abs(h).max()
