"""The heterogeneous benchmark configuration's gradient at its own scale: a
17 x 17 two-yarn blend (plain, twill, satin) over a 20-step window from the
state the reference's own run reached at step 200, loss = the training loss
of src/TrainHeter.h:194-222 against a trajectory of a second seeded
parameter set (tests/golden/make_grad_golden.py config1, the reference's
LibTorch autograd in the harness).

- reference mode: the reverse-mode adjoint (checkpoint every 5 steps)
  reproduces the reference's LibTorch gradient, 1e-6 relative per parameter
  (a parameter whose gradient is below 1e-10 of the largest -- mu here,
  about 1e-20: the friction does not act in these windows -- to 1e-10 of the
  largest). On the plain weave the reference's own gradient is NaN in every
  component (its LibTorch backward through this window); that case is
  checked in exact mode only (central differences below);
- exact mode: the reverse-mode adjoint equals the forward-mode tangents'
  gradient to 1e-10 relative (two independent derivative computations of
  the same discrete step; the same floor at 1e-4 of the largest component);
- exact mode against central differences with a relative step of 1e-6 and
  the solves run to 1e-14: 1e-6 relative per parameter, or -- for a
  parameter whose effect on the loss sits below what a difference quotient
  resolves -- within ten times the quotient's own noise, estimated from the
  change between steps 1e-6 and 2e-6 (the numbers are in the assertion
  message).
"""
import numpy as np
import pytest

import goldens
from pkg import gpu_available, ys

pytestmark = pytest.mark.gpu

NAMES = [n for n in goldens.grad_names() if n.startswith("grad_config1_")]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")
    if not NAMES:
        pytest.skip("config-1 gradient fixtures not generated")


def _setup(name):
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


def _adjoint_grad(name, mode):
    import torch
    g, tmpl, state0, steps, gt_x, gt_e = _setup(name)
    theta = torch.tensor(g["params"], dtype=torch.float64, requires_grad=True)
    tx, te = ys.rollout_adjoint(theta, tmpl, state0, steps, 1e-3, mode, tol=1e-14, checkpoint_every=5)
    loss = ys.position_loss(tx, te, gt_x, gt_e)
    loss.backward()
    return g, loss.item(), theta.grad.numpy().copy()


@pytest.mark.parametrize("name", NAMES)
def test_reference_mode_adjoint_matches_libtorch(name):
    g0 = goldens.load(name)
    if not np.all(np.isfinite(g0["grad"])):
        pytest.skip("the reference's LibTorch gradient is not finite for this window")
    g, loss, grad = _adjoint_grad(name, "reference")
    assert np.all(np.isfinite(grad))
    assert abs(loss - float(g["loss"][0])) <= 1e-6 * abs(float(g["loss"][0]))
    ref = np.asarray(g["grad"], float)
    scale = np.maximum(np.abs(ref), 1e-4 * np.abs(ref).max())
    err = np.abs(grad - ref) / scale
    assert err.max() <= 1e-6, dict(zip(ys.PARAM_NAMES, err))


@pytest.mark.parametrize("name", NAMES)
def test_exact_adjoint_matches_forward_tangents(name):
    import torch
    g, tmpl, state0, steps, gt_x, gt_e = _setup(name)
    _, _, grad_adj = _adjoint_grad(name, "exact")
    theta = torch.tensor(g["params"], dtype=torch.float64, requires_grad=True)
    tx, te = ys.rollout(theta, tmpl, state0, steps, 1e-3, "exact", tol=1e-14)
    ys.position_loss(tx, te, gt_x, gt_e).backward()
    grad_fwd = theta.grad.numpy()
    err = np.abs(grad_adj - grad_fwd) / np.maximum(np.abs(grad_fwd), 1e-4 * np.abs(grad_fwd).max())
    assert err.max() <= 1e-10, dict(zip(ys.PARAM_NAMES, err))


def _losses(tmpl, state0, steps, thetas, gt_x, gt_e):
    """Training loss of each parameter set, all rollouts in one batch."""
    specs = [ys.two_yarn_spec(tmpl, th) for th in thetas]
    b = ys.ClothBatch(specs)
    n = specs[0].num_nodes
    b.set_state(**{k: np.concatenate([np.asarray(state0[k])] * len(specs)) for k in state0})
    xs, es = [], []
    for _ in range(steps):
        st = b.step(1e-3, tol=1e-14, maxiter=100000)
        assert all(s["ok"] for s in st)
        cur = b.get_state()
        xs.append(cur["LPos"].reshape(len(specs), n, 3))
        es.append(cur["EPos"].reshape(len(specs), n, 2))
    b.close()
    X, E = np.stack(xs, 1), np.stack(es, 1)
    gx, ge = gt_x.numpy()[None], gt_e.numpy()[None]
    dl, de = X - gx, E - ge
    return ((dl * dl).sum(-1).mean(-1).sum(-1) + (de * de).sum(-1).mean(-1).sum(-1)) / max(steps - 1, 1)


@pytest.mark.parametrize("name", NAMES[:1])
def test_exact_adjoint_matches_central_differences(name):
    g, tmpl, state0, steps, gt_x, gt_e = _setup(name)
    _, loss, grad = _adjoint_grad(name, "exact")
    th0 = np.array(g["params"], float)
    thetas = []
    for p in range(8):
        for rel in (1e-6, 2e-6):
            for sgn in (1, -1):
                th = th0.copy()
                th[p] *= 1 + sgn * rel
                thetas.append(th)
    L = _losses(tmpl, state0, steps, thetas, gt_x, gt_e).reshape(8, 2, 2)
    report = {}
    for p in range(8):
        d1 = (L[p, 0, 0] - L[p, 0, 1]) / (2e-6 * th0[p])
        d2 = (L[p, 1, 0] - L[p, 1, 1]) / (4e-6 * th0[p])
        noise = abs(d1 - d2) / max(abs(d1), 1e-300)
        err = abs(grad[p] - d1) / max(abs(d1), 1e-300)
        report[ys.PARAM_NAMES[p]] = (err, noise)
        assert err <= max(1e-6, 10 * noise), (ys.PARAM_NAMES[p], grad[p], d1, err, noise, report)
