"""Forward-mode sensitivities of the step (the product's element / gather
code over Dual<8>, compiled for the host by the test-only emulator) against
central finite differences of the same emulated step.

Eight directions, carried ys_tangent_count() at a time: rho, Y and B of
every yarn line (relative perturbations), S and mu of the cloth, one line's
rho alone, and random perturbations of the initial positions and velocities. Finite differences
are Richardson-extrapolated central differences of states after a few steps,
with PCG solved to 1e-14. The states start from deformed configurations: at
an exactly straight yarn the bending term switches off (sin(theta) = 0,
src/PhysicsCloth.cpp:579-822), a point where the step is not differentiable.

Tolerance: positions and velocities 1e-5 relative (max-norm) in every
direction with a measurable effect; the friction coefficient only moves the
slide anchors (EPosBar) measurably on these cloths, so mu is checked there.
"""
import copy

import numpy as np
import pytest

import goldens
from emu_py import EmuCloth

NDIR = 8
TOL = 1e-14
REL = 1e-5


def _directions(kw, N, seed):
    W, H = kw["width"], kw["length"]
    lines = np.concatenate([np.asarray(kw["warp"], float).reshape(H, 3), np.asarray(kw["weft"], float).reshape(W, 3)])
    nl = W + H
    K = NDIR
    d = dict(drho=np.zeros((K, nl)), dY=np.zeros((K, nl)), dB=np.zeros((K, nl)), dS=np.zeros(K), dmu=np.zeros(K),
             dX=np.zeros((K, N, 3)), dV=np.zeros((K, N, 3)))
    d["drho"][0] = lines[:, 0]
    d["dY"][1] = lines[:, 1]
    d["dB"][2] = lines[:, 2]
    d["dS"][3] = kw["S"]
    d["dmu"][4] = kw["mu"]
    rng = np.random.default_rng(seed)
    d["dX"][5] = 1e-4 * rng.standard_normal((N, 3))
    d["dV"][6] = 1e-2 * rng.standard_normal((N, 3))
    d["drho"][7, 2] = lines[2, 0]
    return d, lines


def group(d, g, K):
    """Directions g*K .. g*K+K-1 of d (the directions one tangent step carries)."""
    return {k: v[g * K:(g + 1) * K] for k, v in d.items()}


def _rollout(kw, state, d, lines, k, eps, h, steps):
    W, H = kw["width"], kw["length"]
    kw2 = copy.deepcopy(kw)
    L2 = lines.copy()
    L2[:, 0] += eps * d["drho"][k]
    L2[:, 1] += eps * d["dY"][k]
    L2[:, 2] += eps * d["dB"][k]
    kw2["warp"], kw2["weft"] = L2[:H], L2[H:]
    kw2["S"] = kw["S"] + eps * d["dS"][k]
    kw2["mu"] = kw["mu"] + eps * d["dmu"][k]
    em = EmuCloth(**kw2)
    st = {key: np.array(v, float) for key, v in state.items()}
    st["LPos"] = st["LPos"] + eps * d["dX"][k]
    st["LVel"] = st["LVel"] + eps * d["dV"][k]
    em.set_state(st)
    for _ in range(steps):
        em.assemble(h)
        em.solve(TOL, 100000)
        assert em.update() == 0
    return em.get_state()


def _fd(kw, state, d, lines, k, eps, h, steps):
    run = lambda e: _rollout(kw, state, d, lines, k, e, h, steps)
    a, b, a2, b2 = run(eps), run(-eps), run(eps / 2), run(-eps / 2)
    return {key: (4 * (a2[key] - b2[key]) / eps - (a[key] - b[key]) / (2 * eps)) / 3
            for key in ("LPos", "LVel", "EPos", "EVel", "EPosBar")}


CASES = [("plain6_stiff_upright_wind", 10, 3), ("twill6_upright_wind_pert", None, 3)]


@pytest.mark.parametrize("name,start,steps", CASES)
def test_tangents_match_finite_differences(name, start, steps):
    g = goldens.load(name)
    kw = goldens.spec_kwargs(g)
    h = float(g["h"])
    state = goldens.state(g, start) if start is not None else goldens.init_state(g)
    N = kw["width"] * kw["length"]
    d, lines = _directions(kw, N, seed=1)
    em0 = EmuCloth(**kw)
    K = em0.K
    for gi in range(NDIR // K):
        dg = group(d, gi, K)
        em = EmuCloth(**kw)
        em.set_state(state)
        em.tangent_init()
        em.tangent_seed(dg["drho"], dg["dY"], dg["dB"], dg["dS"], dg["dmu"])
        em.tangent_set_state(dlpos=dg["dX"], dlvel=dg["dV"])
        for _ in range(steps):
            assert em.step_tangent(h, tol=TOL) == 0
        T = em.tangent_get_state()
        scale = {key: np.abs(v).max() for key, v in em.get_state().items()}
        for kk in range(K):
            k = gi * K + kk
            fd = _fd(kw, state, d, lines, k, 1e-4, h, steps)
            keys = ("EPosBar",) if k == 4 else ("LPos", "LVel")
            for key in keys:
                ref = fd[key]
                if np.abs(ref).max() < 1e-7 * scale[key]:
                    continue  # no measurable effect of this direction on this quantity
                err = np.abs(T[key][kk] - ref).max() / np.abs(ref).max()
                assert err <= REL, (name, k, key, err)


def test_zero_seeds_give_zero_tangents():
    g = goldens.load("satin7x5_flat_pert")
    kw = goldens.spec_kwargs(g)
    em = EmuCloth(**kw)
    em.set_state(goldens.init_state(g))
    em.tangent_init()
    for _ in range(2):
        assert em.step_tangent(float(g["h"])) == 0
    for key, v in em.tangent_get_state().items():
        assert not np.any(v), key


@pytest.mark.parametrize("name", ["grad_plain6_upright", "grad_twill6_upright"])
def test_reference_mode_matches_libtorch_gradient(name):
    """The reference-mode tangents (M, D, A held constant, transposed solves,
    Shear_F's detached angle factor) reproduce the gradient the reference's
    own loss.backward() computes (tests/golden/make_grad_golden.py)."""
    g = np.load(goldens.os.path.join(goldens.GOLDEN_DIR, name + ".npz"))
    W, H = int(g["width"]), int(g["length"])
    N, steps, th = W * H, int(g["steps"]), g["params"]
    warp = np.array([th[0:3] if j % 2 == 0 else th[3:6] for j in range(H)])
    weft = np.array([th[0:3] if i % 2 == 0 else th[3:6] for i in range(W)])
    kw = dict(width=W, length=H, warp=warp, weft=weft, weave=int(g["weave"]), pose=int(g["pose"]), R=float(g["R"]),
              L=float(g["L"]), height=float(g["height"]), S=th[6], mu=th[7],
              handles=[tuple(int(a) for a in x) for x in g["handles"]], wind_vel=tuple(float(x) for x in g["wind_vel"]),
              wind_density=float(g["wind_density"]), wind_drag=float(g["wind_drag"]))
    init = {k: g["init_" + k] for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")}
    parity = np.array([j % 2 for j in range(H)] + [i % 2 for i in range(W)])
    K = EmuCloth(**kw).K
    grad = np.zeros(8)
    for g0 in range(0, 8, K):
        em = EmuCloth(**kw)
        em.set_state(init)
        em.tangent_init(1)
        seeds = [np.zeros((K, W + H)) for _ in range(3)] + [np.zeros(K), np.zeros(K)]
        for kk in range(K):
            p = g0 + kk
            if p < 6:
                seeds[p % 3][kk] = (parity == p // 3)
            else:
                seeds[3 if p == 6 else 4][kk] = 1.0
        em.tangent_seed(*seeds)
        for s in range(1, steps + 1):
            assert em.step_tangent(1e-3, tol=1e-14) == 0
            st, T = em.get_state(), em.tangent_get_state()
            dx = st["LPos"] - g["target%d_LPos" % s]
            de = st["EPos"] - g["target%d_EPos" % s]
            for kk in range(K):
                grad[g0 + kk] += 2.0 / N * (np.sum(dx * T["LPos"][kk]) + np.sum(de * T["EPos"][kk])) / max(steps - 1, 1)
    err = np.abs(grad - g["grad"]) / np.abs(g["grad"])
    assert err.max() <= 1e-9, err
