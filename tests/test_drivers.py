"""The reference's simulation drivers on the package API (drivers.py) against
the reference's own runs of the same set-ups (the harness builds the cloth
as each driver does; tests/golden/make_golden.py, make_config_golden.py):

- sim_homo: SimHomo's material, wind and handles (src/Simulate.h:10-106) on a
  6 x 6 cloth, the plain6_stiff_upright_wind fixture (12 steps);
- sim_heter: SimHeter's cotton / polyester blend in wind
  (src/Simulate.h:332-452), 10 x 10, 30 steps;
- sim_control: SimControl's free cloth lifted and dragged at its corners for
  six steps (src/Simulate.h:218-330), 5 x 5, 30 steps;
- sim_collision (SimCollision, src/Simulate.h:108-216) against a ground
  plane: no node ends a step below the plane by more than the thickness;
- the collision benchmark scene (DropOnSphere) on a smaller cloth: it falls
  onto the sphere, every response converges, no node ends inside the sphere
  by more than the thickness.

States at 1e-8 relative per step (field-max), as the other trajectory
fixtures; the HDF5 file a driver writes reads back to the states it
returned.
"""
import os

import numpy as np
import pytest

import goldens
from pkg import gpu_available, ys

pytestmark = pytest.mark.gpu
TOL = 1e-8
KEYS = ("LPos", "LVel", "EPos", "EVel", "EPosBar")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _check(out, g, steps):
    for s in range(steps + 1):
        ref = goldens.state(g, s)
        for k in KEYS:
            assert goldens.rel(out[k][s], ref[k]) <= TOL, (s, k, goldens.rel(out[k][s], ref[k]))


def test_sim_homo_matches_reference(tmp_path):
    g = goldens.load("plain6_stiff_upright_wind")
    p = str(tmp_path / "homo.h5")
    out = ys.sim_homo(width=6, length=6, steps=12, height=float(g["height"]), h5_path=p)
    _check(out, g, 12)
    back = ys.h5.data_loader(p, 0, 13)
    for k in KEYS:
        assert np.array_equal(back[k], out[k]), k
    size, phy = ys.h5.cloth_property_loader(p)
    assert (size["width"], size["length"]) == (6, 6) and phy["Y"] == 500000.0


def test_sim_heter_matches_reference():
    g = goldens.load("driver_simheter10")
    out = ys.sim_heter(width=10, length=10, steps=30, height=float(g["height"]))
    _check(out, g, 30)


def test_sim_control_matches_reference():
    g = goldens.load("driver_simcontrol5")
    out = ys.sim_control(width=5, length=5, steps=30, height=float(g["height"]))
    _check(out, g, 30)


def test_sim_collision_against_a_ground_plane():
    # a ground of two triangles 1 mm under the bottom row of an upright 5 x 5
    # cloth that hangs 25 mm high: the cloth swings in the wind above it
    z = 0.025 - 4e-3 - 1e-3
    vx = np.array([[-0.02, -0.02, z], [0.03, -0.02, z], [-0.02, 0.03, z], [0.03, 0.03, z]])
    vf = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    out = ys.sim_collision(vx, vf, steps=20)
    assert out["LPos"].shape[0] == 21
    assert np.isfinite(out["LPos"]).all()
    assert out["LPos"][:, :, 2].min() >= z - 0.0005


def test_drop_on_sphere_first_contact():
    """A 20 x 20 cloth dropped 3 mm onto a 1 cm sphere (h = 5e-4): it reaches
    the sphere and rests on it without passing through."""
    sc = ys.DropOnSphere(width=20, radius=0.01, levels=3, drop=0.003, h=5e-4)
    try:
        log = sc.run(120)
        assert all(x["ok"] for x in log)
        assert all(x["converged"] and not x["zone_overflow"] for x in log)
        assert any(x["impacts"] > 0 for x in log), "no contact"
        x = sc.state()["LPos"]
        r = np.linalg.norm(x - sc.center, axis=1)
        assert r.min() >= 0.01 - sc.thickness - 1e-4
    finally:
        sc.close()
