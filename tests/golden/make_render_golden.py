"""Generates tests/golden/render_*.npz: the reference's own OBJ output
(RenderCloth, src/Render.cpp, in its three forms: triangle mesh with texture
coordinates and vertex normals, quad mesh, yarn splines) of the final state of
a short run, together with that run's states (the fixture is also a
trajectory fixture).

oracle/_ref/ref_harness (built by oracle/ref/build_ref.sh with src/Render.cpp)
renders with render=PREFIX. Run from the repo root:
python tests/golden/make_render_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import HARNESS, LIT, ROOT, run_case  # noqa: E402

CASES = [
    dict(name="render_twill6_upright_wind", W=6, H=6, weave="twill", pose=0, mat=LIT, spread=0.2, pert=1e-5,
         wind=((0.3, 1.0, 0.2), 2.0, 0.5), handles=[(0, 0), (5, 0)], steps=3, dumps=[0], seed=11, render=True),
    dict(name="render_satin7x5_flat", W=7, H=5, weave="satin", pose=1, mat=LIT, spread=0.2, pert=1e-5,
         wind=None, handles=[(0, 0), (6, 0)], steps=2, dumps=[0], seed=12, render=True),
]


def main():
    if not os.path.exists(HARNESS):
        subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        for cs in CASES:
            rec = run_case(cs, tmp)
            print(cs["name"], "status", rec["status"][0])


if __name__ == "__main__":
    sys.exit(main())
