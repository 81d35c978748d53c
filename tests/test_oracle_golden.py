"""The CPU oracle (oracle/yarn_oracle.c) against fixtures produced by the
reference's own physics sources (tests/golden/make_golden.py).

These pin the oracle before it is trusted as the checker of the GPU path.
"""
import numpy as np
import pytest

import goldens
from oracle.oracle import ClothSpec, OracleCloth

# assembled pieces at one given state: same arithmetic, different summation
# order -> round-off level
SYSTEM_TOL = 1e-11
# per-step state along a trajectory (solve to Eigen's default tolerance on
# both sides; round-off is amplified by the condition number of A)
STATE_TOL = 1e-8


def make(g):
    oc = OracleCloth(ClothSpec(**goldens.spec_kwargs(g)))
    st = goldens.init_state(g)
    if st is not None:
        oc.set_state(st)
    return oc


@pytest.mark.parametrize("name", goldens.names())
def test_initial_state_and_normals(name):
    g = goldens.load(name)
    oc = make(g)
    s0 = goldens.state(g, 0)
    st = oc.get_state()
    for k in ("LPos", "LVel", "EPos", "EVel", "EPosBar"):
        assert goldens.rel(st[k], s0[k]) <= 1e-15, k
    assert goldens.rel(oc.normals(), g["s0_normal"]) <= 1e-12


@pytest.mark.parametrize("name", goldens.names())
def test_system_pieces_at_reference_states(name):
    """FillMV + system formation at each dumped step, from the reference's
    own state at that step (src/PhysicsCloth.cpp:46-156,
    src/TrainHelper.cpp:19-20)."""
    g = goldens.load(name)
    oc = make(g)
    ext = g.get("ext_force")
    for s in g["dumps"]:
        s = int(s)
        st = goldens.state(g, s)
        oc.set_state(st)
        oc.fill()
        d = oc.dense()
        dim = oc.dim
        for ours, ref in (("M", "M"), ("K", "FPos"), ("D", "FVel"), ("V", "Vel")):
            assert goldens.rel(d[ours], g["d%d_%s" % (s, ref)].reshape(d[ours].shape)) <= SYSTEM_TOL, (s, ours)
        F = d["F"] + (ext if ext is not None else 0.0)
        assert goldens.rel(F, g["d%d_F" % s].ravel()) <= SYSTEM_TOL, (s, "F")
        A, b = oc.system(float(g["h"]), ext)
        assert goldens.rel(A, g["d%d_A" % s].reshape(dim, dim)) <= SYSTEM_TOL, (s, "A")
        assert goldens.rel(b, g["d%d_b" % s].ravel()) <= SYSTEM_TOL, (s, "b")
        slide_ref = g["d%d_slide" % s].ravel()
        assert np.abs(d["slide"][:slide_ref.size] - slide_ref).max() <= 1e-9, (s, "slide")


@pytest.mark.parametrize("name", goldens.names())
def test_trajectory(name):
    """Full SimStep loop (src/TrainHelper.cpp:15-54) against the reference's
    per-step states."""
    g = goldens.load(name)
    oc = make(g)
    ext = g.get("ext_force")
    h = float(g["h"])
    for s in range(int(g["steps"])):
        info = oc.step(h, ext)
        assert info["status"] == 0
        ref = goldens.state(g, s + 1)
        st = oc.get_state()
        for k in ("LPos", "LVel", "EPos", "EVel", "EPosBar"):
            assert goldens.rel(st[k], ref[k]) <= STATE_TOL, (s + 1, k, goldens.rel(st[k], ref[k]))


def test_dense_pcg_matches_direct_solve():
    rng = np.random.default_rng(0)
    n = 40
    Q = rng.standard_normal((n, n))
    A = Q @ Q.T + n * np.eye(n)
    b = rng.standard_normal(n)
    from oracle.oracle import dense_pcg
    x, it, err = dense_pcg(A, b, tol=1e-14)
    assert err <= 1e-14
    assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-10, atol=1e-12)
