"""Generates tests/golden/grad_*.npz: the gradient the reference's own
parameter learning computes, from the reference itself.

oracle/_ref/ref_harness (the reference's physics sources built by
oracle/ref/build_ref.sh) runs in mode=grad: a cloth with two yarn types
(rho, Y, B each), S and mu as LibTorch leaves, a ground-truth rollout with a
second parameter set from the same initial state, the training loss of
src/TrainHeter.h:194-231,
    sum_s (mean_N |x_s - x^_s|^2 + mean_N |e_s - e^_s|^2) / max(steps - 1, 1),
and loss.backward() through SimStep and EigenSolver's backward. Each fixture
holds the configuration, the initial state, the ground-truth targets, the
learned-parameter trajectory, the loss and
d loss / d (rho0, Y0, B0, rho1, Y1, B1, S, mu).

Needs the reference sources (REF_SRC, or where oracle/ref/refpath.py finds them); run from the repo
root:  python tests/golden/make_grad_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import HARNESS, ROOT, perturbed_state, read_records  # noqa: E402

# the parameter values of src/TrainHeter.h:47-78: the training start and the
# ground truth, in the order rho0, Y0, B0, rho1, Y1, B1, S, mu
INIT = [0.00225, 335000.0, 0.000125, 0.00245, 145000.0, 0.0001, 600.0, 0.7]
TRUTH = [0.002, 500000.0, 0.00014, 0.0025, 170000.0, 0.00011, 1000.0, 0.5]

def _config1_case(weave, seed):
    """The 17 x 17 blend of the benchmark's heterogeneous configuration: the
    learned parameters start from the fixture's own two yarn types, S and mu
    (make_config_golden.py), the ground truth is a second seeded set within
    +-30 % of it; a 20-step window from the fixture's state at step 200."""
    g = np.load(os.path.join(HERE, "config1_%s17.npz" % weave))
    warp = g["warp"]
    start = [*warp[0], *warp[1], float(g["S"]), float(g["mu"])]
    rng = np.random.default_rng(seed)
    truth = [x * (1.0 + 0.3 * (2.0 * rng.random() - 1.0)) for x in start]
    return dict(name="grad_config1_%s17" % weave, W=17, H=17, weave=weave, pose=0, R=float(g["R"]), steps=20,
                start=("config1_%s17" % weave, 200), wind=((0.0, 0.0, 0.0), 0.0, 0.0), handles=[(0, 0), (16, 0)],
                params=start, truth=truth)


CONFIG1 = ("plain", "twill", "satin")

CASES = [
    dict(name="grad_plain6_upright", W=6, H=6, weave="plain", pose=0, R=5e-4, steps=4,
         start=("plain6_stiff_upright_wind", 10), wind=((0.0, 5.0, 0.0), 2.0, 0.5), handles=[(0, 0), (5, 0)]),
    dict(name="grad_twill6_upright", W=6, H=6, weave="twill", pose=0, R=5e-4, steps=3,
         start=("plain6_stiff_upright_wind", 10), wind=((0.2, 3.0, 0.0), 1.0, 0.5), handles=[(0, 0), (5, 0)]),
]


def run_case(cs, tmp):
    W, H, L, height = cs["W"], cs["H"], 1e-3, 0.05
    if "start" in cs:
        g = np.load(os.path.join(HERE, cs["start"][0] + ".npz"))
        s = cs["start"][1]
        init = {k: g["s%d_%s" % (s, k)] for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")}
    else:
        init = perturbed_state(np.random.default_rng(cs["seed"]), W, H, L, cs["pose"], height, cs["pert"])
    flat = np.concatenate([np.asarray(init[k]).ravel() for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")])
    ipath = os.path.join(tmp, cs["name"] + ".init")
    flat.astype("<f8").tofile(ipath)
    wind = cs["wind"]
    cfg = dict(mode="grad", width=W, length=H, pose="flat" if cs["pose"] == 1 else "upright", weave=cs["weave"], L=L,
               R=cs["R"], height=height, kc=1.0, kf=1000.0, df=1000.0, handle_stiffness=1e4, G="0,0,9.8", h=1e-3,
               handles=",".join("%d,%d" % hp for hp in cs["handles"]), steps=cs["steps"],
               wind_vel="%r,%r,%r" % wind[0], wind_density=wind[1], wind_drag=wind[2], init_state=ipath,
               params=",".join(repr(float(x)) for x in cs.get("params", INIT)),
               gt_params=",".join(repr(float(x)) for x in cs.get("truth", TRUTH)),
               out=os.path.join(tmp, cs["name"] + ".bin"))
    cpath = os.path.join(tmp, cs["name"] + ".cfg")
    with open(cpath, "w") as f:
        for k, v in cfg.items():
            f.write("%s=%s\n" % (k, v))
    subprocess.run([HARNESS, cpath], check=True, capture_output=True)
    rec = read_records(cfg["out"])
    out = dict(width=W, length=H, weave=["plain", "twill", "satin"].index(cs["weave"]), pose=cs["pose"], L=L,
               R=cs["R"], height=height, kc=1.0, kf=1000.0, df=1000.0, handle_stiffness=1e4, G=np.array([0, 0, 9.8]),
               h=1e-3, handles=np.array(cs["handles"], dtype=np.int32).reshape(-1, 2), steps=cs["steps"],
               wind_vel=np.array(wind[0]), wind_density=wind[1], wind_drag=wind[2],
               params=np.array(cs.get("params", INIT)), gt_params=np.array(cs.get("truth", TRUTH)))
    for k, v in init.items():
        out["init_" + k] = np.asarray(v)
    for k, v in rec.items():
        out[k.replace(".", "_")] = v
    np.savez_compressed(os.path.join(HERE, cs["name"] + ".npz"), **out)
    return rec


def main(argv):
    """No arguments: the small cases; "config1": the three 17 x 17 windows
    (minutes each, run in parallel)."""
    if not os.path.exists(HARNESS):
        subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    cases = [_config1_case(w, 201 + i) for i, w in enumerate(CONFIG1)] if "config1" in argv else CASES
    from concurrent.futures import ThreadPoolExecutor
    with tempfile.TemporaryDirectory() as tmp, ThreadPoolExecutor(len(cases)) as ex:
        for cs, rec in zip(cases, ex.map(lambda c: run_case(c, tmp), cases)):
            print(cs["name"], "loss", rec["loss"][0], "grad", rec["grad"])


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
