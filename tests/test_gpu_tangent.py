"""GPU forward-mode sensitivities (ys_step_tangent through the C ABI).

- against the host emulation of the same kernels (tests/emu) on the same
  seeds: both run the templated element code over Dual<K>; they differ only
  in the order of the PCG reductions, so with the solves run to 1e-14 the
  tangents agree to 1e-8 relative;
- against Richardson-extrapolated central differences of the GPU step itself
  on a 17x17 cloth with two yarn materials: 1e-5 relative for the parameter
  directions, 1e-4 for the random perturbations of every node's position and
  velocity (these move every crossing through the steep sliding-friction
  switch, sigmoid(1e4 (|F| - mu c)), where the difference quotient is least
  accurate);
- a cloth's tangents in a batch of uneven cloths equal its tangents alone.
"""
import numpy as np
import pytest

import goldens
from emu_py import EmuCloth
from pkg import gpu_available, ys
from test_emu_tangent import NDIR, _directions, group

pytestmark = pytest.mark.gpu

TOL = 1e-14


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _K():
    return int(ys._native.load().ys_tangent_count())


def _gpu_tangents(kw, state, d, h, steps):
    """Tangents of the K directions in d after `steps` steps (and the final state)."""
    b = ys.ClothBatch([ys.ClothSpec(**kw)])
    b.set_state(**state)
    b.tangent_enable()
    b.tangent_seed(d["drho"], d["dY"], d["dB"], d["dS"][:, None], d["dmu"][:, None])
    b.tangent_set_state(dlpos=d["dX"], dlvel=d["dV"])
    for _ in range(steps):
        st = b.step_tangent(h, tol=TOL, maxiter=100000)
        assert st[0]["ok"]
    out = b.tangent_get_state(), b.get_state()
    b.close()
    return out


@pytest.mark.parametrize("name,start", [("plain6_stiff_upright_wind", 10), ("twill6_upright_wind_pert", None)])
def test_gpu_tangents_match_emulation(name, start):
    g = goldens.load(name)
    kw = goldens.spec_kwargs(g)
    h = float(g["h"])
    state = goldens.state(g, start) if start is not None else goldens.init_state(g)
    N = kw["width"] * kw["length"]
    dall, _ = _directions(kw, N, seed=2)
    K = _K()
    for gi in range(NDIR // K):
        d = group(dall, gi, K)
        T, _ = _gpu_tangents(kw, state, d, h, 3)
        em = EmuCloth(**kw)
        em.set_state(state)
        em.tangent_init()
        em.tangent_seed(d["drho"], d["dY"], d["dB"], d["dS"], d["dmu"])
        em.tangent_set_state(dlpos=d["dX"], dlvel=d["dV"])
        for _ in range(3):
            assert em.step_tangent(h, tol=TOL) == 0
        E = em.tangent_get_state()
        for key in ("LPos", "LVel", "EPos", "EVel", "EPosBar"):
            for k in range(K):
                ref = E[key][k]
                if not np.any(ref):
                    assert not np.any(T[key][k]), (key, gi * K + k)
                    continue
                err = goldens.rel(T[key][k], ref)
                assert err <= 1e-8, (name, key, gi * K + k, err)


def _hetero17(weave):
    rng = np.random.default_rng(17 + weave)
    y1 = np.array([2e-3, 5e5, 1.4e-4]) * (1 + 0.1 * rng.random(3))
    y2 = np.array([2.5e-3, 1.7e5, 1.1e-4]) * (1 + 0.1 * rng.random(3))
    W = H = 17
    warp = np.array([y1 if j % 2 == 0 else y2 for j in range(H)])
    weft = np.array([y1 if i % 2 == 0 else y2 for i in range(W)])
    return dict(width=W, length=H, warp=warp, weft=weft, weave=weave, pose=0, S=1000.0, mu=0.5, R=5e-4, L=1e-3,
                height=0.05, handles=[(0, 0), (W - 1, 0)], wind_vel=(0.0, 1.0, 0.0), wind_density=1.0,
                wind_drag=0.5)


@pytest.mark.parametrize("weave", [0, 1, 2])
def test_gpu_tangents_match_finite_differences(weave):
    kw = _hetero17(weave)
    h, warm, steps = 1e-3, 8, 3
    b0 = ys.ClothBatch([ys.ClothSpec(**kw)])
    for _ in range(warm):  # leave the exactly straight start, where bending is not differentiable
        assert b0.step(h, tol=TOL, maxiter=100000)[0]["ok"]
    state = b0.get_state()
    b0.close()
    N = 17 * 17
    d, lines = _directions(kw, N, seed=3)
    K = _K()
    T, fin = {}, None
    for gi in range(NDIR // K):
        Tg, fin = _gpu_tangents(kw, state, group(d, gi, K), h, steps)
        for key, v in Tg.items():
            T.setdefault(key, []).extend(list(v))
    scale = {k: np.abs(v).max() for k, v in fin.items()}

    def rollout(k, eps):
        L2 = lines.copy()
        L2[:, 0] += eps * d["drho"][k]
        L2[:, 1] += eps * d["dY"][k]
        L2[:, 2] += eps * d["dB"][k]
        kw2 = dict(kw, warp=L2[:17], weft=L2[17:], S=kw["S"] + eps * d["dS"][k], mu=kw["mu"] + eps * d["dmu"][k])
        b = ys.ClothBatch([ys.ClothSpec(**kw2)])
        st = dict(state)
        st["LPos"] = state["LPos"] + eps * d["dX"][k]
        st["LVel"] = state["LVel"] + eps * d["dV"][k]
        b.set_state(**st)
        for _ in range(steps):
            assert b.step(h, tol=TOL, maxiter=100000)[0]["ok"]
        out = b.get_state()
        b.close()
        return out

    eps = 1e-4
    for k in range(NDIR):
        a, c, a2, c2 = rollout(k, eps), rollout(k, -eps), rollout(k, eps / 2), rollout(k, -eps / 2)
        keys = ("EPosBar",) if k == 4 else ("LPos", "LVel")
        for key in keys:
            fd = (4 * (a2[key] - c2[key]) / eps - (a[key] - c[key]) / (2 * eps)) / 3
            if np.abs(fd).max() < 1e-7 * scale[key]:
                continue
            err = np.abs(T[key][k] - fd).max() / np.abs(fd).max()
            assert err <= (1e-4 if k in (5, 6) else 1e-5), (weave, k, key, err)


def test_batched_tangents_equal_single():
    kws = [_hetero17(1), dict(_hetero17(2), width=9, length=12, warp=_hetero17(2)["warp"][:12],
                              weft=_hetero17(2)["weft"][:9], handles=[(0, 0), (8, 0)])]
    h = 1e-3
    singles = []
    ds = []
    K = _K()
    for i, kw in enumerate(kws):
        N = kw["width"] * kw["length"]
        d, _ = _directions(kw, N, seed=10 + i)
        d = group(d, 0, K)
        ds.append(d)
        singles.append(_gpu_tangents(kw, ys.ClothBatch([ys.ClothSpec(**kw)]).get_state(), d, h, 3)[0])
    b = ys.ClothBatch([ys.ClothSpec(**kw) for kw in kws])
    b.tangent_enable()
    b.tangent_seed(np.concatenate([d["drho"] for d in ds], axis=1), np.concatenate([d["dY"] for d in ds], axis=1),
                   np.concatenate([d["dB"] for d in ds], axis=1), np.stack([d["dS"] for d in ds], axis=1),
                   np.stack([d["dmu"] for d in ds], axis=1))
    b.tangent_set_state(dlpos=np.concatenate([d["dX"] for d in ds], axis=1),
                        dlvel=np.concatenate([d["dV"] for d in ds], axis=1))
    for _ in range(3):
        assert all(s["ok"] for s in b.step_tangent(h, tol=TOL, maxiter=100000))
    T = b.tangent_get_state()
    off = 0
    for kw, single in zip(kws, singles):
        N = kw["width"] * kw["length"]
        for key in single:
            assert np.array_equal(T[key][:, off:off + N], single[key]), key
        off += N
    b.close()


# ---------------------------------------------------------------- learning
def _grad_setup(name):
    import torch
    g = goldens.load(name)
    tmpl = dict(width=int(g["width"]), length=int(g["length"]), height=float(g["height"]), L=float(g["L"]),
                R=float(g["R"]), pose=int(g["pose"]), weave=int(g["weave"]), kc=float(g["kc"]), kf=float(g["kf"]),
                df=float(g["df"]), handle_stiffness=float(g["handle_stiffness"]),
                G=tuple(float(x) for x in g["G"]), wind_vel=tuple(float(x) for x in g["wind_vel"]),
                wind_density=float(g["wind_density"]), wind_drag=float(g["wind_drag"]),
                handles=[tuple(int(a) for a in r) for r in g["handles"]])
    state0 = {k: g["init_" + k] for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")}
    steps = int(g["steps"])
    gt_x = torch.tensor(np.stack([g["target%d_LPos" % s] for s in range(1, steps + 1)]))
    gt_e = torch.tensor(np.stack([g["target%d_EPos" % s] for s in range(1, steps + 1)]))
    return g, tmpl, state0, steps, gt_x, gt_e


@pytest.mark.parametrize("name", goldens.grad_names())
def test_reference_gradient_matches_libtorch(name):
    """ys.rollout(mode="reference") + the training loss: the gradient the
    reference's own loss.backward() computes, 1e-7 relative per parameter."""
    import torch
    g, tmpl, state0, steps, gt_x, gt_e = _grad_setup(name)
    if not np.all(np.isfinite(g["grad"])):
        pytest.skip("the reference's LibTorch gradient is not finite for this window")
    theta = torch.tensor(g["params"], dtype=torch.float64, requires_grad=True)
    tx, te = ys.rollout(theta, tmpl, state0, steps, 1e-3, "reference", tol=1e-14)
    loss = ys.position_loss(tx, te, gt_x, gt_e)
    loss.backward()
    assert abs(loss.item() - float(g["loss"][0])) <= 1e-6 * abs(float(g["loss"][0]))
    err = np.abs(theta.grad.numpy() - g["grad"]) / np.abs(g["grad"])
    assert err.max() <= 1e-7, err


def test_exact_gradient_matches_finite_differences():
    """ys.rollout(mode="exact"): the loss gradient against Richardson central
    differences of the GPU rollout, 1e-5 relative per parameter; 1e-3 for mu,
    whose effect on this loss is about 1e-6 of the loss, the limit of what the
    difference quotient resolves."""
    import torch
    g, tmpl, state0, steps, gt_x, gt_e = _grad_setup("grad_plain6_upright")
    th0 = np.array(g["params"], float)
    theta = torch.tensor(th0, requires_grad=True)
    tx, te = ys.rollout(theta, tmpl, state0, steps, 1e-3, "exact", tol=1e-14)
    loss = ys.position_loss(tx, te, gt_x, gt_e)
    loss.backward()
    grad = theta.grad.numpy()

    def L(th):
        with torch.no_grad():
            a, b = ys.rollout(torch.tensor(th), tmpl, state0, steps, 1e-3, "exact", tol=1e-14)
            return ys.position_loss(a, b, gt_x, gt_e).item()

    for p in range(8):
        eps = 1e-4 * th0[p]
        d = np.zeros(8)
        d[p] = eps
        d1 = (L(th0 + d) - L(th0 - d)) / (2 * eps)
        d2 = (L(th0 + d / 2) - L(th0 - d / 2)) / eps
        fd = (4 * d2 - d1) / 3
        if abs(fd) * th0[p] < 1e-8 * loss.item():
            continue  # below the resolution of the loss
        tol = 1e-3 if ys.PARAM_NAMES[p] == "mu" else 1e-5
        assert abs(grad[p] - fd) <= tol * abs(fd), (ys.PARAM_NAMES[p], grad[p], fd)


def test_yarnsimnet_heter_rollout_gradient():
    """YarnSimNetHeter's raw parameters through constraint_para (the ranges of
    src/TrainHeter.h:80-105): grad = dL/dtheta * dtheta/draw."""
    import torch
    g, tmpl, state0, steps, gt_x, gt_e = _grad_setup("grad_plain6_upright")
    ranges = dict(rho_1=(0.003, 0.001), rho_2=(0.003, 0.001), Y_1=(800000.0, 0.0), Y_2=(300000.0, 0.0),
                  B_1=(0.00018, 0.00005), B_2=(0.00018, 0.00005), S=(1200.0, 0.0), mu=(1.0, 0.0))
    init = dict(zip(("rho_1", "Y_1", "B_1", "rho_2", "Y_2", "B_2", "S", "mu"), g["params"]))
    raw = {k: ys.invert_constraint_para(v, *ranges[k]) for k, v in init.items()}
    net = ys.YarnSimNetHeter(tmpl["width"], tmpl["length"], tmpl["R"], tmpl["L"], raw, ranges, tmpl["handles"],
                             wind_vel=tmpl["wind_vel"], wind_density=tmpl["wind_density"],
                             wind_drag=tmpl["wind_drag"], height=tmpl["height"], mode="reference")
    assert np.allclose(net.theta().detach().numpy(), g["params"], rtol=1e-12)
    tx, te = net.rollout(state0, steps, tol=1e-14)
    ys.position_loss(tx, te, gt_x, gt_e).backward()
    order = ("rho_1", "Y_1", "B_1", "rho_2", "Y_2", "B_2", "S", "mu")
    for p, n in enumerate(order):
        up, lo = ranges[n]
        s = 1.0 / (1.0 + np.exp(-raw[n]))
        expect = g["grad"][p] * (up - lo) * s * (1 - s)
        got = getattr(net, n).grad.item()
        assert abs(got - expect) <= 1e-7 * abs(expect), (n, got, expect)
