"""Parity at the benchmark configurations' own scale, against fixtures made
by the reference's own physics sources (tests/golden/make_config_golden.py):

- config0_plain5_flat: the 5 x 5 plain cloth, 200 steps, every step;
- config1_{plain,twill,satin}17: the 17 x 17 two-yarn blend in the three
  weave patterns (the reference's own blend rule), 500 steps, every 10th
  step.

Two measures, both at 1e-8 per kept step (the solve runs to Eigen's default
tolerance on both sides, so only round-off, amplified by the conditioning of
A and by 500 steps, separates them):
- field-max relative: max |a - b| / max |b| over the whole field (LPos,
  LVel, EPos, EVel, EPosBar), as the older fixtures are checked;
- per component: |a - b| / max(|b|, 1e-3 max |b|), every component against
  its own size, with a floor at a thousandth of the field's largest entry
  for components that are zero up to round-off.

The CPU oracle is checked on the same fixtures (CPU tests), the GPU path
through the C ABI (GPU tests), each cloth alone and all four in one batch.
"""
import numpy as np
import pytest

import goldens
from pkg import gpu_available, spec_from_golden, ys

FIELD_TOL = 1e-8
COMP_TOL = 1e-8
KEYS = ("LPos", "LVel", "EPos", "EVel", "EPosBar")


def _check(st, g, s, where):
    ref = goldens.state(g, s)
    for k in KEYS:
        e1 = goldens.rel(st[k], ref[k])
        e2 = goldens.rel_comp(st[k], ref[k])
        assert e1 <= FIELD_TOL, (where, s, k, "field", e1)
        assert e2 <= COMP_TOL, (where, s, k, "component", e2)


@pytest.mark.parametrize("name", goldens.config_names())
def test_oracle_matches_reference_at_config_scale(name):
    from oracle.oracle import ClothSpec, OracleCloth
    g = goldens.load(name)
    assert float(g["status"][0]) == 0.0
    oc = OracleCloth(ClothSpec(**goldens.spec_kwargs(g)))
    kept = set(int(s) for s in g["kept"])
    _check(oc.get_state(), g, 0, name)
    assert goldens.rel(oc.normals(), g["s0_normal"]) <= 1e-12
    for s in range(int(g["steps"])):
        assert oc.step(float(g["h"]))["status"] == 0
        if s + 1 in kept:
            _check(oc.get_state(), g, s + 1, name)


def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


@pytest.mark.gpu
@pytest.mark.parametrize("name", goldens.config_names())
def test_gpu_matches_reference_at_config_scale(name):
    _need_gpu()
    g = goldens.load(name)
    b = ys.ClothBatch([spec_from_golden(g)])
    kept = set(int(s) for s in g["kept"])
    _check(b.get_state(), g, 0, name)
    for s in range(int(g["steps"])):
        assert b.step(float(g["h"]))[0]["ok"]
        if s + 1 in kept:
            _check(b.get_state(), g, s + 1, name)
    b.close()


@pytest.mark.gpu
def test_gpu_config_fixtures_in_one_batch():
    """The four configurations stepped together: each cloth's states equal
    its own fixture (per-cloth solves and stopping tests)."""
    _need_gpu()
    names = goldens.config_names()
    gs = [goldens.load(n) for n in names]
    b = ys.ClothBatch([spec_from_golden(g) for g in gs])
    steps = max(int(g["steps"]) for g in gs)
    for s in range(steps):
        active = [int(g["steps"]) > s for g in gs]
        if not all(active):
            break
        stats = b.step(1e-3)
        assert all(x["ok"] for x in stats)
        st = b.get_state()
        for c, g in enumerate(gs):
            if s + 1 in set(int(x) for x in g["kept"]):
                _check({k: st[k][b.node_slice(c)] for k in KEYS}, g, s + 1, names[c])
    b.close()
