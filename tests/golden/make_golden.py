"""Generates the golden fixtures in tests/golden/*.npz from the reference itself.

The reference's own physics sources (src/Cloth.cpp, src/PhysicsCloth.cpp,
src/MatrixMp.cpp, src/Mesh.cpp, src/Geometry.cpp) are compiled unmodified into
oracle/_ref/ref_harness by oracle/ref/build_ref.sh (serial build, Eigen CG
restated in oracle/ref/shim/eigen_cg.cpp). This script writes a config per
case, runs the harness, and stores its per-step states and the dense system
pieces at selected steps.

Needs the reference sources (REF_SRC, or where oracle/ref/refpath.py finds them); run from the repo
root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# material of the 5x5 benchmark cloth, passed straight to the reference's own
# parameters: Yarn(R, rho, Y, B), S, mu
LIT = dict(rho=1e-3, Y=1e3, B=1e-5, S=1e-4, mu=0.3, R=1e-4)
# the reference's own SimHomo material (src/Simulate.h:16-28)
STIFF = dict(rho=2e-3, Y=5e5, B=1.4e-4, S=1000.0, mu=0.5, R=5e-4)


def read_records(path):
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    o = 0
    while o < len(buf):
        (nl,) = struct.unpack_from("<i", buf, o); o += 4
        name = buf[o:o + nl].decode(); o += nl
        (nd,) = struct.unpack_from("<i", buf, o); o += 4
        dims = struct.unpack_from("<%dq" % nd, buf, o); o += 8 * nd
        n = int(np.prod(dims)) if nd else 1
        out[name] = np.frombuffer(buf, dtype="<f8", count=n, offset=o).reshape(dims).copy(); o += 8 * n
    return out


def line_params(rng, n, base, spread):
    """Per-yarn-line (rho, Y, B) drawn uniformly within +-spread of base."""
    a = np.empty((n, 3))
    for j, k in enumerate(("rho", "Y", "B")):
        a[:, j] = base[k] * (1.0 + spread * (2.0 * rng.random(n) - 1.0))
    return a


def perturbed_state(rng, W, H, L, pose, height, pert):
    N = W * H
    st = {}
    lp = np.zeros((N, 3)); ep = np.zeros((N, 2))
    for v in range(H):
        for u in range(W):
            i = u + v * W
            lp[i] = (u * L, v * L, height) if pose == 1 else (u * L, 0.0, height - v * L)
            ep[i] = (u * L, v * L)
    interior = np.zeros(N, bool)
    for v in range(1, H - 1):
        for u in range(1, W - 1):
            interior[u + v * W] = True
    st["LPosFix"] = lp.copy()
    st["LPos"] = lp + pert * rng.standard_normal((N, 3))
    st["LVel"] = 1e-2 * rng.standard_normal((N, 3))
    st["EPos"] = ep + np.where(interior[:, None], 0.3 * pert * rng.standard_normal((N, 2)), 0.0)
    st["EPosBar"] = st["EPos"] + np.where(interior[:, None], 0.1 * pert * rng.standard_normal((N, 2)), 0.0)
    st["EVel"] = np.where(interior[:, None], 1e-3 * rng.standard_normal((N, 2)), 0.0)
    return st


CASES = [
    # name, W, H, weave, pose, material, spread, perturb, wind, handles, steps, dumps, ext
    dict(name="plain5_flat_rest", W=5, H=5, weave="plain", pose=1, mat=LIT, spread=0.2, pert=0.0,
         wind=None, handles=[(0, 0), (4, 0)], steps=40, dumps=[0, 10, 39], seed=1),
    dict(name="twill6_upright_wind_pert", W=6, H=6, weave="twill", pose=0, mat=LIT, spread=0.2, pert=1e-5,
         wind=((0.3, 1.0, 0.2), 2.0, 0.5), handles=[(0, 0), (5, 0)], steps=4, dumps=[0, 1, 3], seed=2),
    dict(name="satin7x5_flat_pert", W=7, H=5, weave="satin", pose=1, mat=LIT, spread=0.2, pert=1e-5,
         wind=((0.0, 0.5, -0.3), 1.0, 0.8), handles=[(0, 0), (6, 0)], steps=4, dumps=[0, 2], seed=3),
    dict(name="plain6_stiff_upright_wind", W=6, H=6, weave="plain", pose=0, mat=STIFF, spread=0.0, pert=0.0,
         wind=((0.0, 5.0, 0.0), 2.0, 0.5), handles=[(0, 0), (5, 0)], steps=12, dumps=[0, 6, 11], seed=4),
    dict(name="plain5_extforce", W=5, H=5, weave="plain", pose=1, mat=LIT, spread=0.0, pert=0.0,
         wind=None, handles=[], steps=6, dumps=[0, 5], seed=5, ext=True),
]


def run_case(cs, tmp):
    rng = np.random.default_rng(cs["seed"])
    W, H, mat = cs["W"], cs["H"], cs["mat"]
    warp = line_params(rng, H, mat, cs["spread"])
    weft = line_params(rng, W, mat, cs["spread"])
    L, height = 1e-3, 0.05
    pose = cs["pose"]
    cfg = dict(width=W, length=H, pose="flat" if pose == 1 else "upright", weave=cs["weave"], L=L, R=mat["R"],
               height=height, yarn0="%r,%r,%r" % (mat["rho"], mat["Y"], mat["B"]), mu=mat["mu"], S=mat["S"],
               kc=1.0, kf=1000.0, df=1000.0, handle_stiffness=1e4, G="0,0,9.8", h=1e-3,
               handles=",".join("%d,%d" % hp for hp in cs["handles"]), steps=cs["steps"],
               dump_steps=",".join(map(str, cs["dumps"])),
               warp_lines=";".join(",".join(repr(float(x)) for x in r) for r in warp),
               weft_lines=";".join(",".join(repr(float(x)) for x in r) for r in weft),
               out=os.path.join(tmp, cs["name"] + ".bin"))
    wind = cs.get("wind")
    if wind:
        cfg["wind_vel"] = "%r,%r,%r" % wind[0]
        cfg["wind_density"], cfg["wind_drag"] = wind[1], wind[2]
    init = None
    if cs["pert"] > 0:
        init = perturbed_state(rng, W, H, L, pose, height, cs["pert"])
        flat = np.concatenate([init[k].ravel() for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")])
        p = os.path.join(tmp, cs["name"] + ".init")
        flat.astype("<f8").tofile(p)
        cfg["init_state"] = p
    ext = None
    if cs.get("ext"):
        dim = 3 * W * H + 2 * (W - 2) * (H - 2)
        ext = np.zeros(dim)
        # lift and drag at the four corners, as in SimControl (src/Simulate.h:265-285)
        for (u, v) in [(0, 0), (W - 1, 0), (0, H - 1), (W - 1, H - 1)]:
            n = u + v * W
            ext[3 * n + 1] = 0.002
            ext[3 * n + 2] = 0.002
        cfg["ext_force"] = ",".join(repr(float(x)) for x in ext)
    if cs.get("render"):
        cfg["render"] = os.path.join(tmp, cs["name"])
    cpath = os.path.join(tmp, cs["name"] + ".cfg")
    with open(cpath, "w") as f:
        for k, v in cfg.items():
            f.write("%s=%s\n" % (k, v))
    subprocess.run([HARNESS, cpath], check=True, capture_output=True)
    rec = read_records(cfg["out"])
    out = dict(width=W, length=H, weave=["plain", "twill", "satin"].index(cs["weave"]), pose=pose, L=L,
               R=mat["R"], height=height, mu=mat["mu"], S=mat["S"], kc=1.0, kf=1000.0, df=1000.0,
               handle_stiffness=1e4, G=np.array([0, 0, 9.8]), h=1e-3, warp=warp, weft=weft,
               handles=np.array(cs["handles"], dtype=np.int32).reshape(-1, 2), steps=cs["steps"],
               dumps=np.array(cs["dumps"]))
    if wind:
        out.update(wind_vel=np.array(wind[0]), wind_density=wind[1], wind_drag=wind[2])
    else:
        out.update(wind_vel=np.zeros(3), wind_density=0.0, wind_drag=0.0)
    if init is not None:
        for k, v in init.items():
            out["init_" + k] = v
    if ext is not None:
        out["ext_force"] = ext
    for k, v in rec.items():
        out[k.replace(".", "_")] = v
    if cs.get("render"):
        for kind in ("tri", "rect", "yarn"):
            with open(os.path.join(tmp, "%s_%s.obj" % (cs["name"], kind))) as f:
                out["obj_" + kind] = np.array(f.read())
    np.savez_compressed(os.path.join(HERE, cs["name"] + ".npz"), **out)
    return rec


def main():
    if not os.path.exists(HARNESS):
        subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        for cs in CASES:
            rec = run_case(cs, tmp)
            print(cs["name"], "status", rec["status"][0], "records", len(rec))


if __name__ == "__main__":
    sys.exit(main())
