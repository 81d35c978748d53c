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
