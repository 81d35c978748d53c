"""Generates tests/golden/embed_plain5*.npz: one evaluation of the reference's
control learning (train_embed, src/TrainEmbed.h:84-176) from the reference
itself, with its loop as written and (``_intended``) with the forced steps
0..5 its comment describes.

oracle/_ref/ref_harness (mode=embed) builds the reference's ForceNet
(src/ForceNet.h) with torch::manual_seed(seed), runs train_embed's loop (with
its `if (s = force_stop_frame)`), SimStep with the predicted lift and drag at
the four corners, the mass-centre loss against a goal and loss.backward().
The fixture holds the configuration, the goal, the network's parameters,
the predicted forces, the loss, every parameter's gradient and the final
positions. The goal is the last step of the trajectory file the reference
ships (tests/golden/h5_wind_yarn12_plain5.npz).

Needs the reference sources (REF_SRC, or where oracle/ref/refpath.py finds them); run from the repo
root:  python tests/golden/make_embed_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import HARNESS, read_records  # noqa: E402

CFG = dict(width=5, length=5, height=5.0, L=1e-3, R=5e-4, rho=0.002, Y=5e5, B=1.4e-4, kc=1.0, kf=1000.0, df=1000.0,
           mu=0.5, S=1000.0, handle_stiffness=1e4, G="0,0,9.8", wind_vel="0,5,0", wind_density=2.0, wind_drag=0.5,
           h=1e-3, sample=12, seed=7, force_at="0,0,4,0,0,4,4,4")


def run(tmp, goal, cfg_extra, name):
    gp = os.path.join(tmp, "goal.bin")
    np.ascontiguousarray(goal, "<f8").tofile(gp)
    cfg = dict(CFG, mode="embed", goal=gp, out=os.path.join(tmp, name + ".bin"), **cfg_extra)
    cp = os.path.join(tmp, name + ".cfg")
    with open(cp, "w") as f:
        for k, v in cfg.items():
            f.write("%s=%s\n" % (k, v))
    subprocess.run([HARNESS, cp], check=True, capture_output=True)
    return read_records(cfg["out"])


def main():
    goal = np.load(os.path.join(HERE, "h5_wind_yarn12_plain5.npz"))["last_LPos"]
    for name, extra in (("embed_plain5", {}), ("embed_plain5_intended", {"loop": "intended"})):
        with tempfile.TemporaryDirectory() as tmp:
            rec = run(tmp, goal, extra, name)
        out = {"cfg_" + k: np.array(v) for k, v in dict(CFG, **extra).items()}
        out["goal"] = goal
        for k, v in rec.items():
            out[k.replace(".", "__")] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("%s: loss %.6e, forces %s, status %s" % (name, rec["loss"][0], rec["forces"], rec["status"]))


if __name__ == "__main__":
    main()
