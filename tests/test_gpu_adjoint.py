"""Reverse-mode step (ys_adjoint_step through the C ABI) and the checkpointed
reverse rollout, against the forward-mode tangents of the same step
(ys_step_tangent), which are themselves checked against finite differences
and the reference's LibTorch gradient (tests/test_gpu_tangent.py).

The check is the adjoint identity: for a direction d (state, per-line
materials, S, mu, external force) with forward tangent J d, and any g,
    g . (J d) = (J^T g) . d.
Both sides are computed independently on the GPU with the solves run to
1e-14, in both gradient definitions (exact: the derivative of the discrete
step; reference: what the reference's loss.backward() computes). Tolerance
1e-9 relative to the sum of the magnitudes of the terms.
"""
import numpy as np
import pytest

import goldens
from pkg import gpu_available, spec_from_golden, ys

pytestmark = pytest.mark.gpu

TOL = 1e-14
REL = 1e-9
COMPS = dict(LPos=3, LVel=3, EPos=2, EVel=2, EPosBar=2)
MODES = {"exact": 0, "reference": 1}


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _case(name, step):
    g = goldens.load(name)
    spec = spec_from_golden(g)
    st = goldens.state(g, step) if step is not None else goldens.init_state(g)
    return spec, st


def _random_direction(spec, rng, ext):
    N, nl = spec.num_nodes, spec.width + spec.length
    lines = np.concatenate([np.asarray(spec.warp, float).reshape(spec.length, 3),
                            np.asarray(spec.weft, float).reshape(spec.width, 3)])
    d = dict(LPos=1e-5 * rng.standard_normal((N, 3)), LVel=1e-3 * rng.standard_normal((N, 3)),
             EPos=1e-6 * rng.standard_normal((N, 2)), EVel=1e-4 * rng.standard_normal((N, 2)),
             EPosBar=1e-6 * rng.standard_normal((N, 2)),
             rho=lines[:, 0] * rng.standard_normal(nl), Y=lines[:, 1] * rng.standard_normal(nl),
             B=lines[:, 2] * rng.standard_normal(nl), S=spec.S * rng.standard_normal(1),
             mu=spec.mu * rng.standard_normal(1))
    d["ext"] = 1e-4 * rng.standard_normal((N, 5)) if ext else None
    return d


def _forward_tangent(spec, state, d, mode, h, steps, ext_force=None):
    """Tangents of the state after each of `steps` steps along direction d."""
    b = ys.ClothBatch([spec])
    b.set_state(**state)
    b.tangent_enable(MODES[mode])
    K = b.n_tangents
    pad = lambda a: np.concatenate([a[None], np.zeros((K - 1,) + a.shape)])  # noqa: E731
    b.tangent_seed(pad(d["rho"]), pad(d["Y"]), pad(d["B"]), pad(d["S"]), pad(d["mu"]))
    b.tangent_set_state(dlpos=pad(d["LPos"]), dlvel=pad(d["LVel"]), depos=pad(d["EPos"]),
                        deposbar=pad(d["EPosBar"]), devel=pad(d["EVel"]))
    out = []
    for s in range(steps):
        dext = pad(d["ext"]) if (d["ext"] is not None and s == 0) else None
        if dext is None and ext_force is not None:
            dext = np.zeros((K, spec.num_nodes, 5))
        st = b.step_tangent(h, ext_force, tol=TOL, maxiter=100000, kact=1, dext_force=dext)
        assert st[0]["ok"]
        t = b.tangent_get_state()
        out.append({k: t[k][0] for k in COMPS})
    b.close()
    return out


def _dot(a, b):
    return float(np.sum(np.asarray(a) * np.asarray(b)))


@pytest.mark.parametrize("mode", ["exact", "reference"])
@pytest.mark.parametrize("name,step", [("plain6_stiff_upright_wind", 10), ("twill6_upright_wind_pert", None),
                                       ("satin7x5_flat_pert", None)])
def test_one_step_adjoint_identity(name, step, mode):
    spec, state = _case(name, step)
    h = 1e-3
    rng = np.random.default_rng(1)
    ext = 1e-3 * rng.standard_normal((spec.num_nodes, 5))
    d = _random_direction(spec, rng, ext=True)
    tan = _forward_tangent(spec, state, d, mode, h, 1, ext_force=ext)[0]
    g = {k: rng.standard_normal((spec.num_nodes, c)) for k, c in COMPS.items()}
    lhs_terms = [_dot(g[k], tan[k]) for k in COMPS]
    b = ys.ClothBatch([spec])
    b.set_state(**state)
    adj = ys.Adjoint(b, mode)
    gs, gp, ge = adj.step_back(h, g, ext, tol=TOL, maxiter=100000, want_ext=True)
    after = b.get_state()
    for k in state:
        assert np.array_equal(after[k], np.asarray(state[k])), k  # the batch's state is left as it was
    rhs_terms = [_dot(gs[k], d[k]) for k in COMPS] + [_dot(gp[k], d[k]) for k in ("rho", "Y", "B", "S", "mu")]
    rhs_terms.append(_dot(ge, d["ext"]))
    lhs, rhs = sum(lhs_terms), sum(rhs_terms)
    scale = sum(abs(x) for x in rhs_terms) + sum(abs(x) for x in lhs_terms)
    assert abs(lhs - rhs) <= REL * scale, (lhs, rhs, scale)
    adj.close()
    b.close()


@pytest.mark.parametrize("mode", ["exact", "reference"])
def test_each_input_separately(mode):
    """The identity per input group (state fields, each material, S, mu):
    a wrong column of one group cannot hide behind the others."""
    spec, state = _case("twill6_upright_wind_pert", None)
    h = 1e-3
    rng = np.random.default_rng(4)
    g = {k: rng.standard_normal((spec.num_nodes, c)) for k, c in COMPS.items()}
    b = ys.ClothBatch([spec])
    b.set_state(**state)
    adj = ys.Adjoint(b, mode)
    gs, gp, _ = adj.step_back(h, g, tol=TOL, maxiter=100000)
    adj.close()
    b.close()
    full = _random_direction(spec, rng, ext=False)
    for group in list(COMPS) + ["rho", "Y", "B", "S", "mu"]:
        d = {k: (v if k == group else (None if v is None else np.zeros_like(v))) for k, v in full.items()}
        tan = _forward_tangent(spec, state, d, mode, h, 1)[0]
        lhs = sum(_dot(g[k], tan[k]) for k in COMPS)
        rhs = _dot(gs[group], d[group]) if group in COMPS else _dot(gp[group], d[group])
        # the scale of the sum's terms, not of its result: mu's effect on this
        # step is 1e-14 and its products with g cancel to a small fraction
        scale = sum(float(np.abs(g[k] * tan[k]).sum()) for k in COMPS)
        assert abs(lhs - rhs) <= REL * scale, (group, lhs, rhs, scale)


def test_pass_count_and_batch_do_not_change_the_adjoint():
    """Fewer copies (more passes per step) and a batch of uneven cloths give
    the same adjoint bit for bit: every direction's derivatives depend only on
    its own seeds and its own cloth."""
    specs = [spec_from_golden(goldens.load(n)) for n in ("twill6_upright_wind_pert", "satin7x5_flat_pert")]
    states = [goldens.init_state(goldens.load(n)) for n in ("twill6_upright_wind_pert", "satin7x5_flat_pert")]
    h = 1e-3
    rng = np.random.default_rng(2)
    res = []
    for copies in (128, 9):
        b = ys.ClothBatch([specs[0]])
        b.set_state(**states[0])
        adj = ys.Adjoint(b, "exact", copies=copies)
        g = {k: np.random.default_rng(3).standard_normal((specs[0].num_nodes, c)) for k, c in COMPS.items()}
        res.append(adj.step_back(h, g, tol=TOL, maxiter=100000))
        adj.close()
        b.close()
    for k in COMPS:
        assert np.array_equal(res[0][0][k], res[1][0][k]), k
    for k in ("rho", "Y", "B", "S", "mu"):
        assert np.array_equal(res[0][1][k], res[1][1][k]), k
    # both cloths in one batch
    b = ys.ClothBatch(specs)
    st = {k: np.concatenate([np.asarray(s[k]) for s in states]) for k in states[0]}
    b.set_state(**st)
    adj = ys.Adjoint(b, "exact")
    g1 = {k: np.random.default_rng(3).standard_normal((specs[0].num_nodes, c)) for k, c in COMPS.items()}
    g2 = {k: rng.standard_normal((specs[1].num_nodes, c)) for k, c in COMPS.items()}
    gb = {k: np.concatenate([g1[k], g2[k]]) for k in COMPS}
    gs, gp, _ = adj.step_back(h, gb, tol=TOL, maxiter=100000)
    adj.close()
    b.close()
    sl = slice(0, specs[0].num_nodes)
    for k in COMPS:
        assert goldens.rel(gs[k][sl], res[0][0][k]) <= 1e-13, k
    nl0 = specs[0].width + specs[0].length
    for k in ("rho", "Y", "B"):
        assert goldens.rel(gp[k][:nl0], res[0][1][k]) <= 1e-13, k


@pytest.mark.parametrize("mode", ["exact", "reference"])
def test_checkpointed_rollout_matches_forward_tangents(mode):
    """Eight steps, a checkpoint every 3 (segments of 3, 3, 2): the reverse
    sweep's gradient of a loss on every step's state equals the forward
    tangents' contraction with the same loss gradient."""
    spec, state = _case("plain6_stiff_upright_wind", 10)
    h, steps = 1e-3, 8
    rng = np.random.default_rng(6)
    d = _random_direction(spec, rng, ext=False)
    tans = _forward_tangent(spec, state, d, mode, h, steps)
    g_traj = {k: rng.standard_normal((steps, spec.num_nodes, c)) for k, c in COMPS.items()}
    lhs = sum(_dot(g_traj[k][s], tans[s][k]) for s in range(steps) for k in COMPS)
    b = ys.ClothBatch([spec])
    ro = ys.CheckpointedRollout(b, state, steps, h, mode=mode, checkpoint_every=3, tol=TOL)
    ro.forward()
    assert sorted(ro.checkpoints) == [0, 3, 6]
    g = ro.backward(g_traj)
    b.close()
    terms = [_dot(g["state0"][k], d[k]) for k in COMPS] + [_dot(g[k], d[k]) for k in ("rho", "Y", "B", "S", "mu")]
    rhs = sum(terms)
    assert abs(lhs - rhs) <= 1e-8 * sum(abs(t) for t in terms), (lhs, rhs)
