"""The reference's learnable modules besides YarnSimNetHeter:

- YarnSimNetHomo (src/YarnSimNetHomo.h:4-111): forward() from a reference
  fixture's state gives the fixture's next state (1e-8), with the material
  set through constraint_para of the inverted values; the rollout's gradient
  w.r.t. the four raw parameters in forward mode equals the reverse
  adjoint's (1e-8) and central differences (exact mode, 1e-6, or ten times
  the difference quotient's own error estimated from two step sizes);
- YarnSimNetControl (src/YarnSimNet.h:132-245): forward(state, idx) is the
  step with the setting's lift and drag forces at nodes a * width + b; the
  gradient w.r.t. the twelve forces over a schedule of settings against
  central differences (1e-6);
- YarnSimNetColli (src/YarnSimNetColli.h:4-116): forward() is SimStep with
  collision (src/TrainHelper.cpp:99-149) against the merged table and
  ground; over a rollout in which the cloth's lower edge reaches the ground,
  the gradient w.r.t. raw rho, Y, B through the adjoint and the response's
  backward against central differences (exact mode, 1e-5).
"""
import numpy as np
import pytest

import goldens
from pkg import gpu_available, spec_from_golden, ys

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


RANGES = dict(rho=(0.003, 0.0001), Y=(2e6, 10.0), B=(1e-3, 1e-7), S=(2000.0, 1e-6))


def _homo_net(g, mode="reference"):
    warp = np.asarray(g["warp"], float).reshape(-1, 3)
    rho, Y, B = warp[0]
    raw = {n: ys.invert_constraint_para(v, *RANGES[n]) for n, v in
           dict(rho=rho, Y=Y, B=B, S=float(g["S"])).items()}
    return ys.YarnSimNetHomo(int(g["width"]), int(g["length"]), float(g["R"]), float(g["L"]), raw, RANGES,
                             [tuple(int(a) for a in r) for r in np.asarray(g["handles"]).reshape(-1, 2)],
                             h=float(g["h"]), mu=float(g["mu"]), kf=float(g["kf"]), df=float(g["df"]),
                             kc=float(g["kc"]), handle_stiffness=float(g["handle_stiffness"]),
                             gravity=float(np.asarray(g["G"])[2]),
                             wind_vel=tuple(float(x) for x in g["wind_vel"]),
                             wind_density=float(g["wind_density"]), wind_drag=float(g["wind_drag"]),
                             woven_pattern=int(g["weave"]), height=float(g["height"]), mode=mode)


def test_homo_forward_matches_reference_fixture():
    g = goldens.load("plain6_stiff_upright_wind")
    warp = np.asarray(g["warp"], float).reshape(-1, 3)
    assert np.all(warp == warp[0])  # one yarn type
    net = _homo_net(g)
    for s in (0, 5, 10):
        st, ok = net(goldens.state(g, s))
        assert ok
        ref = goldens.state(g, s + 1)
        for k in ("LPos", "LVel", "EPos", "EVel", "EPosBar"):
            assert goldens.rel(st[k], ref[k]) <= 1e-8, (s, k, goldens.rel(st[k], ref[k]))


def _loss(tx, te):
    return (tx * tx).sum() * 1e3 + (te * te).sum() * 1e3


def test_homo_gradient_forward_reverse_and_differences():
    import torch
    g = goldens.load("plain6_stiff_upright_wind")
    state0 = goldens.state(g, 3)
    steps = 4
    net = _homo_net(g, mode="exact")
    tx, te = net.rollout(state0, steps)
    _loss(tx, te).backward()
    gf = torch.cat([getattr(net, n).grad for n in ("rho", "Y", "B", "S")]).numpy().copy()
    net.zero_grad()
    tx, te = net.rollout_adjoint(state0, steps, checkpoint_every=2)
    _loss(tx, te).backward()
    gr = torch.cat([getattr(net, n).grad for n in ("rho", "Y", "B", "S")]).numpy().copy()
    assert np.abs(gf - gr).max() <= 1e-8 * np.abs(gf).max(), (gf, gr)
    for i, n in enumerate(("rho", "Y", "B", "S")):
        p = getattr(net, n)
        x0 = float(p.data[0])
        fds = []
        for eps in (1e-6, 2e-6):
            vals = []
            for sgn in (1, -1):
                p.data[0] = x0 + sgn * eps
                with torch.no_grad():
                    tx, te = net.rollout(state0, steps)
                    vals.append(float(_loss(tx, te)))
            fds.append((vals[0] - vals[1]) / (2 * eps))
        p.data[0] = x0
        fd = fds[0]
        noise = abs(fds[0] - fds[1]) / max(abs(fd), 1e-300)  # the quotient's own error, estimated
        err = abs(fd - gf[i]) / max(abs(fd), 1e-300)
        assert err <= max(1e-6, 10 * noise), (n, fd, gf[i], err, noise)


def _control_net(mode="exact"):
    mat = dict(rho=1e-3, Y=1e3, B=1e-5, S=1e-4, mu=0.3)
    rng = np.random.default_rng(3)
    forces = [(2e-5 * rng.standard_normal(), 2e-5 * rng.standard_normal()) for _ in range(6)]
    return ys.YarnSimNetControl(7, 6, 1e-4, 1e-3, mat, forces, [(0, 0), (0, 6), (5, 3)], h=1e-3, mode=mode)


def test_control_forward_is_the_step_with_the_setting_forces():
    net = _control_net()
    b = ys.ClothBatch([net.spec()])
    s0 = b.get_state()
    for idx in (0, 3, 6):
        st, ok = net(s0, idx)
        assert ok
        b.set_state(**s0)
        e = None
        if idx < 6:
            f = net.forces().detach().numpy()
            e = np.zeros((b.total_nodes, 5))
            for (a, c) in [(0, 0), (0, 6), (5, 3)]:
                e[a * 7 + c, 2] += f[idx, 0]
                e[a * 7 + c, 1] += f[idx, 1]
        assert b.step(1e-3, e)[0]["ok"]
        ref = b.get_state()
        for k in ref:
            assert np.array_equal(st[k], ref[k]), (idx, k)
    b.close()


def test_control_gradient_matches_differences():
    import torch
    net = _control_net()
    b = ys.ClothBatch([net.spec()])
    s0 = b.get_state()
    b.close()
    schedule = [0, 0, 1, 2, 6, 3, 4, 5, 5, 6]
    tx, te = net.rollout(s0, schedule, checkpoint_every=3)
    (tx[-1].mean(0) ** 2).sum().backward()
    names = ["lift_force_" + n for n in ys.learn.FORCE_NAMES] + ["drag_force_" + n for n in ys.learn.FORCE_NAMES]
    grads = {n: float(getattr(net, n).grad[0]) for n in names}
    scale = max(abs(v) for v in grads.values())
    for n in names:
        p = getattr(net, n)
        x0 = float(p.data[0])
        eps = 1e-7
        vals = []
        for sgn in (1, -1):
            p.data[0] = x0 + sgn * eps
            with torch.no_grad():
                tx, te = net.rollout(s0, schedule, checkpoint_every=3)
                vals.append(float((tx[-1].mean(0) ** 2).sum()))
        p.data[0] = x0
        fd = (vals[0] - vals[1]) / (2 * eps)
        assert abs(fd - grads[n]) <= 1e-6 * abs(fd) + 1e-9 * scale, (n, fd, grads[n])


def _ground_and_table(z_ground, z_table):
    ground = np.array([[-0.02, -0.02, z_ground], [0.03, -0.02, z_ground], [0.03, 0.02, z_ground],
                       [-0.02, 0.02, z_ground]])
    table = np.array([[0.05, -0.01, z_table], [0.07, -0.01, z_table], [0.07, 0.01, z_table],
                      [0.05, 0.01, z_table]])
    x = np.concatenate([ground, table])
    f = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7]], dtype=np.int32)
    return x, f


def _colli_net(mode, z_ground):
    x, f = _ground_and_table(z_ground, 0.02)
    raw = {n: ys.invert_constraint_para(v, *RANGES[n]) for n, v in dict(rho=1e-3, Y=1e3, B=1e-5).items()}
    return ys.YarnSimNetColli(6, 5, 0.01, 1e-4, 1e-3, raw, RANGES, [(0, 0), (5, 0)], x, f, h=1e-3, S=1e-4,
                              mu=0.3, mode=mode)


def test_colli_forward_is_simstep_with_collision():
    net = _colli_net("reference", 0.006 - 0.0006)
    cloth = ys.Cloth(6, 5, 0.01, 1e-3, 1e-4, [ys.Yarn(1e-4, *[float(v) for v in net.theta()[:3]])], 1.0,
                     1000.0, 1000.0, 0.3, 1e-4, 1e4, ys.WovenPattern.Plain, ys.InitPose.Upright)
    cloth.set_handles([(0, 0), (5, 0)])
    env = ys.Environment(cloth, (0.0, 0.0, 9.8), ys.Wind())
    phy = ys.PhysicsCloth(env)
    col = ys.Collision(cloth, net.obstacle_x, net.obstacle_faces, thickness=5e-4, h=1e-3)
    st = phy.batch.get_state()
    moved = False
    for _ in range(12):
        mine, ok = net(st)
        assert ok
        assert ys.SimStep(cloth, phy, col, 1e-3)
        ref = phy.batch.get_state()
        for k in ref:
            assert np.array_equal(mine[k], ref[k]), k
        moved = moved or bool(col.last and col.last["changed"])
        st = ref
    assert moved  # the lower edge reached the ground
    col.close()


def test_colli_gradient_matches_differences():
    import torch
    net = _colli_net("exact", 0.006 - 0.0006)
    b = ys.ClothBatch([net.spec()])
    s0 = b.get_state()
    b.close()
    steps = 12

    def loss(tx, te):
        return (tx[-1, :, 2] ** 2).sum() * 1e4 + (tx[-1, :, 0] ** 2).sum() * 1e4

    tx, te = net.rollout(s0, steps, checkpoint_every=5)
    assert float(tx[-1, :, 2].min()) < 0.006  # below the initial lower edge: in contact
    loss(tx, te).backward()
    gr = {n: float(getattr(net, n).grad[0]) for n in ("rho", "Y", "B")}
    for n in ("rho", "Y", "B"):
        p = getattr(net, n)
        x0 = float(p.data[0])
        eps = 1e-6
        vals = []
        for sgn in (1, -1):
            p.data[0] = x0 + sgn * eps
            with torch.no_grad():
                tx, te = net.rollout(s0, steps, checkpoint_every=5)
                vals.append(float(loss(tx, te)))
        p.data[0] = x0
        fd = (vals[0] - vals[1]) / (2 * eps)
        assert abs(fd - gr[n]) <= 1e-5 * abs(fd) + 1e-10, (n, fd, gr[n])
