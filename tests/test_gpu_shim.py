"""The C++ binding (include/yarnsim_torch.h) run on the GPU: a LibTorch
program (tests/cpp/shim_driver.cpp, built here) steps cloths through
yarnsim::GpuCloth -- the SimHomo loop of src/Simulate.h:78-101 with SimStep
replaced, the reference's ClothState tensors in and out -- and takes the
training loss's gradient through yarnsim::AdjointRollout, a
torch::autograd::Function whose backward is the checkpointed reverse
adjoint. Checked against fixtures of the reference's own runs:

- SimHomo's set-up (plain6_stiff_upright_wind, 12 steps): 1e-8 relative per
  step; the 17 x 17 twill blend of the heterogeneous configuration from the
  reference's own state at every 40th step: one step at 1e-8, ten steps at
  1e-7 (the window bounds of tests/test_config_parity.py: over 500 steps the
  trajectories separate by amplified round-off);
- the reference's LibTorch gradient of the training loss
  (grad_plain6_upright, and the 17 x 17 window when generated), reference
  mode: 1e-7 relative per parameter (1e-6 at 17 x 17).
"""
import importlib.util
import os
import subprocess

import numpy as np
import pytest

import goldens
from pkg import ROOT, gpu_available

pytestmark = pytest.mark.gpu

_spec = importlib.util.spec_from_file_location("cpp_build", os.path.join(ROOT, "tests", "cpp", "build.py"))
cpp_build = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(cpp_build)

KEYS = ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not gpu_available():
        pytest.skip("no CUDA device")
    out = str(tmp_path_factory.mktemp("shim") / "shim_driver")
    try:
        return cpp_build.driver(out)
    except subprocess.CalledProcessError as e:
        pytest.fail("building the C++ driver failed:\n" + e.stderr[-3000:])


def _write_case(tmp, g, init, steps, extra):
    W, H = int(g["width"]), int(g["length"])
    N = W * H
    np.asarray(g["warp"], "<f8").reshape(H, 3).tofile(os.path.join(tmp, "warp"))
    np.asarray(g["weft"], "<f8").reshape(W, 3).tofile(os.path.join(tmp, "weft"))
    np.concatenate([np.asarray(init[k], "<f8").reshape(-1) for k in KEYS]).tofile(os.path.join(tmp, "init"))
    cfg = dict(width=W, length=H, height=float(g["height"]), L=float(g["L"]), R=float(g["R"]), pose=int(g["pose"]),
               weave=int(g["weave"]), kc=float(g["kc"]), kf=float(g["kf"]), df=float(g["df"]),
               mu=float(g.get("mu", 0.0)), S=float(g.get("S", 0.0)), handle_stiffness=float(g["handle_stiffness"]),
               G=",".join(repr(float(x)) for x in g["G"]), wind_vel=",".join(repr(float(x)) for x in g["wind_vel"]),
               wind_density=float(g["wind_density"]), wind_drag=float(g["wind_drag"]),
               handles=",".join(str(int(x)) for x in np.asarray(g["handles"]).reshape(-1)),
               warp=os.path.join(tmp, "warp"), weft=os.path.join(tmp, "weft"), init=os.path.join(tmp, "init"),
               steps=steps, h=float(g["h"]), out=os.path.join(tmp, "out"))
    cfg.update(extra)
    path = os.path.join(tmp, "cfg")
    with open(path, "w") as f:
        for k, v in cfg.items():
            f.write("%s=%s\n" % (k, v))
    return path, N


def _run(driver, cfg):
    r = subprocess.run([driver, cfg], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]


def _rows(out, N):
    for row in out:
        yield dict(LPos=row[:3 * N].reshape(N, 3), LVel=row[6 * N:9 * N].reshape(N, 3),
                   EPos=row[9 * N:11 * N].reshape(N, 2), EPosBar=row[11 * N:13 * N].reshape(N, 2),
                   EVel=row[13 * N:15 * N].reshape(N, 2))


def test_cpp_simstep_loop_matches_reference(driver, tmp_path):
    name, steps = "plain6_stiff_upright_wind", 12
    g = goldens.load(name)
    init = goldens.init_state(g) or goldens.state(g, 0)
    cfg, N = _write_case(str(tmp_path), g, init, steps, dict(mode="traj"))
    _run(driver, cfg)
    out = np.fromfile(str(tmp_path / "out"), "<f8").reshape(steps, 15 * N)
    kept = [int(s) for s in g["kept"]] if "kept" in g else list(range(steps + 1))
    for s, st in enumerate(_rows(out, N), start=1):
        if s not in kept:
            continue
        ref = goldens.state(g, s)
        for k in st:
            assert goldens.rel(st[k], ref[k]) <= 1e-8, (name, s, k, goldens.rel(st[k], ref[k]))


def test_cpp_simstep_windows_match_reference_at_config_scale(driver, tmp_path):
    name = "config1_twill17"
    if not os.path.exists(os.path.join(goldens.GOLDEN_DIR, name + ".npz")):
        pytest.skip("fixture not generated")
    g = goldens.load(name)
    kept = set(int(s) for s in g["kept"])
    for a in range(0, int(g["steps"]), 40):
        d = tmp_path / ("w%d" % a)
        d.mkdir()
        cfg, N = _write_case(str(d), g, goldens.state(g, a), 10, dict(mode="traj"))
        _run(driver, cfg)
        out = np.fromfile(str(d / "out"), "<f8").reshape(10, 15 * N)
        for j, st in enumerate(_rows(out, N), start=1):
            if a + j not in kept or j not in (1, 10):
                continue
            tol = 1e-8 if j == 1 else 1e-7
            ref = goldens.state(g, a + j)
            for k in st:
                assert goldens.rel(st[k], ref[k]) <= tol, (name, a, j, k, goldens.rel(st[k], ref[k]))


@pytest.mark.parametrize("name", ["grad_plain6_upright", "grad_config1_twill17"])
def test_cpp_autograd_matches_reference_gradient(driver, tmp_path, name):
    path = os.path.join(goldens.GOLDEN_DIR, name + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    g = goldens.load(name)
    steps = int(g["steps"])
    W, H = int(g["width"]), int(g["length"])
    g = dict(g)
    g["warp"] = np.zeros((H, 3))  # the two yarn types come from theta
    g["weft"] = np.zeros((W, 3))
    init = {k: g["init_" + k] for k in KEYS}
    N = W * H
    tg = np.concatenate([np.stack([g["target%d_LPos" % s] for s in range(1, steps + 1)]).reshape(-1),
                         np.stack([g["target%d_EPos" % s] for s in range(1, steps + 1)]).reshape(-1)])
    tg.astype("<f8").tofile(str(tmp_path / "targets"))
    cfg, _ = _write_case(str(tmp_path), g, init, steps,
                         dict(mode="grad", theta=",".join(repr(float(x)) for x in g["params"]),
                              targets=str(tmp_path / "targets"), adjoint=1, k=5, mu=0.0, S=0.0, tol=1e-14))
    _run(driver, cfg)
    out = np.fromfile(str(tmp_path / "out"), "<f8")
    loss, grad = out[0], out[1:9]
    assert abs(loss - float(g["loss"][0])) <= 1e-6 * abs(float(g["loss"][0]))
    tol = 1e-7 if W <= 6 else 1e-6
    err = np.abs(grad - g["grad"]) / np.abs(g["grad"])
    assert err.max() <= tol, err
