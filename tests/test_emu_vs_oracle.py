"""The product's element / node functions (csrc/ys_items.cuh), compiled for
the host by the test-only emulator in tests/emu, against the reference
fixtures. This checks the GPU path's arithmetic on a machine without a GPU;
the same comparisons run on the device in tests/test_gpu_parity.py."""
import numpy as np
import pytest

import goldens
from emu_py import EmuCloth
from layout import ref_to_node5

SYSTEM_TOL = 1e-11
STATE_TOL = 1e-8


def make(g):
    em = EmuCloth(**goldens.spec_kwargs(g))
    st = goldens.init_state(g)
    if st is not None:
        em.set_state(st)
    return em


def ext5(g):
    ext = g.get("ext_force")
    return None if ext is None else ref_to_node5(ext, int(g["width"]), int(g["length"]))


@pytest.mark.parametrize("name", goldens.names())
def test_emulated_system_matches_reference(name):
    g = goldens.load(name)
    em = make(g)
    for s in (int(x) for x in g["dumps"]):
        em.set_state(goldens.state(g, s))
        em.assemble(float(g["h"]), ext5(g))
        if s == 0:
            assert goldens.rel(em.normals(), g["s0_normal"]) <= 1e-12
        A, b = em.system()
        dim = A.shape[0]
        assert goldens.rel(A, g["d%d_A" % s].reshape(dim, dim)) <= SYSTEM_TOL, s
        assert goldens.rel(b, g["d%d_b" % s].ravel()) <= SYSTEM_TOL, s


@pytest.mark.parametrize("name", goldens.names())
def test_emulated_trajectory_matches_reference(name):
    g = goldens.load(name)
    em = make(g)
    for s in range(int(g["steps"])):
        info = em.step(float(g["h"]), ext5(g))
        assert info["status"] == 0
        ref = goldens.state(g, s + 1)
        st = em.get_state()
        for k in ("LPos", "LVel", "EPos", "EVel", "EPosBar"):
            assert goldens.rel(st[k], ref[k]) <= STATE_TOL, (s + 1, k, goldens.rel(st[k], ref[k]))


@pytest.mark.parametrize("weave", [0, 1, 2])
@pytest.mark.parametrize("S", [1e6, 1e8])
def test_shear_dominated_system_matches_oracle(weave, S):
    """Shear (with jamming) made the dominant stiffness, on a perturbed state,
    so its Hessian is resolved far below the system tolerance."""
    from oracle.oracle import ClothSpec, OracleCloth
    rng = np.random.default_rng(weave * 7 + int(np.log10(S)))
    W, H = 7, 6
    base = np.array([1e-3, 1e3, 1e-5])
    kw = dict(width=W, length=H, warp=np.tile(base, (H, 1)), weft=np.tile(base, (W, 1)), weave=weave, pose=1,
              S=S, handles=[(0, 0), (W - 1, 0)])
    oc = OracleCloth(ClothSpec(**kw))
    em = EmuCloth(**kw)
    st = oc.get_state()
    N = W * H
    st["LPos"] = st["LPos"] + 1.5e-4 * rng.standard_normal((N, 3))
    st["LVel"] = 1e-2 * rng.standard_normal((N, 3))
    oc.set_state(st)
    em.set_state(st)
    oc.fill()
    A_ref, b_ref = oc.system(1e-3)
    em.assemble(1e-3)
    A, b = em.system()
    shear_scale = np.abs(A_ref[:3 * N, :3 * N]).max()
    assert shear_scale > 1e-2  # shear dominates the node-node blocks
    assert goldens.rel(A, A_ref) <= 1e-12
    assert goldens.rel(b, b_ref) <= 1e-12
