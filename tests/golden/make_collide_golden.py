"""Generates tests/golden/collide_*.npz: broad-phase pair lists and
narrow-phase impacts of the reference's collision detection.

oracle/_ref/ref_harness (mode=collide) builds the reference's own BVH
(src/BVH.cpp via AccelStruct, src/CollisionUtil.cpp) over the cloth mesh of a
W x H cloth and over an obstacle mesh, traverses it as
Collision::for_overlapping_faces does and runs the narrow phase of
comp_face_impacts (restated: src/Collision.cpp needs Alglib). Inputs are
synthetic: a cloth folded over itself whose two layers pass through each
other during the step, and a cloth moving into a sphere (an icosphere built
here). Each fixture holds the inputs, the pair list in emission order and
the impacts.

Needs the reference sources (REF_SRC, or where oracle/ref/refpath.py finds them); run from the repo
root:  python tests/golden/make_collide_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import HARNESS, ROOT, read_records  # noqa: E402


def icosphere(center, radius, levels):
    """Vertices [V][3] and faces [F][3] of a subdivided icosahedron."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(p, float) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(levels):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                p = v[a] + v[b]
                v.append(p / np.linalg.norm(p))
                mid[k] = len(v) - 1
            return mid[k]

        nf = []
        for (a, b, c) in f:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.array(center) + radius * np.array(v), np.array(f, dtype=np.int64)


def folded(W, H, L, gap_prev, gap_now, seed):
    """A cloth folded at row H/2 into two horizontal layers; the upper layer
    moves from gap_prev above the lower one to gap_now (negative: through)."""
    rng = np.random.default_rng(seed)
    x = np.zeros((W * H, 3)); xp = np.zeros((W * H, 3))
    half = H // 2
    for v in range(H):
        for u in range(W):
            n = u + v * W
            if v < half:
                y, zp, z = v * L, 0.0, 0.0
            else:
                y, zp, z = (H - 1 - v) * L + 0.3 * L, gap_prev, gap_now
            jit = 1e-5 * rng.standard_normal(3)
            xp[n] = (u * L + jit[0], y + jit[1], zp + jit[2])
            x[n] = (u * L + jit[0] + 2e-5 * rng.standard_normal(), y + jit[1], z + jit[2])
    return x, xp


def draped(W, H, L, center, radius, seed):
    """A flat cloth centred over a sphere moving down into it."""
    rng = np.random.default_rng(seed)
    x = np.zeros((W * H, 3)); xp = np.zeros((W * H, 3))
    for v in range(H):
        for u in range(W):
            n = u + v * W
            px = center[0] + (u - (W - 1) / 2) * L
            py = center[1] + (v - (H - 1) / 2) * L
            r2 = (px - center[0]) ** 2 + (py - center[1]) ** 2
            top = center[2] + np.sqrt(max(radius ** 2 - r2, 0.0))
            xp[n] = (px, py, top + 0.8e-3 + 1e-5 * rng.standard_normal())
            x[n] = (px, py, top - 0.6e-3 + 1e-5 * rng.standard_normal())
    return x, xp


CASES = [
    dict(name="collide_fold10", W=10, H=10, L=1e-3, thickness=5e-4, state=lambda: folded(10, 10, 1e-3, 2e-3, -1e-3, 1)),
    dict(name="collide_fold16_near", W=16, H=16, L=1e-3, thickness=5e-4,
         state=lambda: folded(16, 16, 1e-3, 1.5e-3, 0.4e-3, 2)),
    dict(name="collide_sphere12", W=12, H=12, L=1e-3, thickness=5e-4,
         state=lambda: draped(12, 12, 1e-3, (0.0, 0.0, 0.0), 0.02, 3),
         sphere=((0.0, 0.0, 0.0), 0.02, 2)),
    # the collision benchmark's size: a 50 x 50 cloth on a 3 cm sphere of 1280 faces
    dict(name="collide_sphere50", W=50, H=50, L=1e-3, thickness=5e-4,
         state=lambda: draped(50, 50, 1e-3, (0.0, 0.0, 0.0), 0.03, 5),
         sphere=((0.0, 0.0, 0.0), 0.03, 3)),
]


def run_case(cs, tmp):
    x, xp = cs["state"]()
    W, H = cs["W"], cs["H"]
    sp = os.path.join(tmp, cs["name"] + ".state")
    np.concatenate([x.ravel(), xp.ravel()]).astype("<f8").tofile(sp)
    cfg = dict(mode="collide", width=W, length=H, L=cs["L"], R=1e-4, thickness=cs["thickness"], ccd=1,
               cloth_state=sp, out=os.path.join(tmp, cs["name"] + ".bin"))
    out = dict(width=W, length=H, L=cs["L"], thickness=cs["thickness"], x=x, x_prev=xp)
    if "sphere" in cs or "mesh" in cs:
        vo, fo = cs["mesh"] if "mesh" in cs else icosphere(*cs["sphere"])
        op = os.path.join(tmp, cs["name"] + ".obs")
        np.concatenate([[len(vo)], vo.ravel(), vo.ravel(), [len(fo)], fo.ravel().astype(float)]).astype("<f8").tofile(op)
        cfg["obstacle"] = op
        out.update(obs_x=vo, obs_x_prev=vo.copy(), obs_faces=fo)
    cpath = os.path.join(tmp, cs["name"] + ".cfg")
    with open(cpath, "w") as f:
        for k, v in cfg.items():
            f.write("%s=%s\n" % (k, v))
    subprocess.run([HARNESS, cpath], check=True, capture_output=True)
    rec = read_records(cfg["out"])
    out["pairs"] = rec["pairs"].astype(np.int64) if rec["pairs"].size else np.zeros((0, 3), np.int64)
    out["impacts"] = rec["impacts"] if rec["impacts"].size else np.zeros((0, 15))
    np.savez_compressed(os.path.join(HERE, cs["name"] + ".npz"), **out)
    return out


def frame_cases(path):
    """Cases from frames recorded on the GPU by record_drop_frames.py (the
    collision benchmark scene): one fixture per frame, collide_drop50_s<step>."""
    f = np.load(path)
    out = []
    for s in f["frames"]:
        s = int(s)
        x, xp = f["x_%d" % s].copy(), f["x_prev_%d" % s].copy()
        out.append(dict(name="collide_drop50_s%d" % s, W=int(f["width"]), H=int(f["length"]), L=1e-3,
                        thickness=float(f["thickness"]), state=(lambda x=x, xp=xp: (x, xp)),
                        mesh=(f["obs_x"].copy(), f["obs_faces"].astype(np.int64))))
    return out


def main(argv=()):
    """No arguments: the synthetic cases; "frames <npz>": fixtures from
    frames of the collision benchmark scene."""
    if not os.path.exists(HARNESS):
        subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    cases = frame_cases(argv[1]) if len(argv) > 1 and argv[0] == "frames" else CASES
    with tempfile.TemporaryDirectory() as tmp:
        for cs in cases:
            o = run_case(cs, tmp)
            print(cs["name"], "pairs", len(o["pairs"]), "impacts", len(o["impacts"]),
                  "VF", int((o["impacts"][:, 0] == 0).sum()) if len(o["impacts"]) else 0)


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
