"""Generates the benchmark-scale reference fixtures tests/golden/config*.npz
from the reference itself (oracle/_ref/ref_harness, the reference's own
physics sources in a serial build; see make_golden.py).

- config0_plain5_flat: the 5 x 5 plain-weave cloth of the plain method,
  flat, two top corners pinned, per-yarn-line rho, Y, B and per-cloth S, mu
  drawn uniformly within +-20 % of (1e-3, 1e3, 1e-5, 1e-4, 0.3), gravity,
  h = 1e-3, 200 steps; every step's state is kept.
- config1_{plain,twill,satin}17: the 17 x 17 heterogeneous blend in the
  three weave patterns: two yarn types assigned by the reference's own blend
  rule (warp line v and weft line u take yarn v % 2 and u % 2,
  src/Cloth.cpp:195-268), type 0 within +-20 % of the values above, type 1 =
  type 0 times factors drawn uniformly in [1.5, 3] per parameter, upright,
  two top corners pinned, h = 1e-3, 500 steps; every 10th state is kept,
  and the state one step after every 20th.
- driver_simheter10, driver_simcontrol5: the set-ups of the reference's
  SimHeter and SimControl drivers (src/Simulate.h:218-452), 30 steps each,
  every step kept (they pin the package's drivers, drivers.py).

The harness writes every step; the fixtures keep LPos, LVel, EPos, EVel and
EPosBar at the kept steps (the dense systems of a 17 x 17 cloth, 14 MB each,
are not stored).

Run from the repo root with the reference sources present (REF_SRC):
    python tests/golden/make_config_golden.py [case ...]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import HARNESS, LIT, ROOT, read_records  # noqa: E402

KEYS = ("LPos", "LVel", "EPos", "EVel", "EPosBar", "LPosFix")


def material(rng):
    """One yarn type's (rho, Y, B) and the cloth's (S, mu), +-20 % of LIT."""
    f = 1.0 + 0.2 * (2.0 * rng.random(5) - 1.0)
    yarn = np.array([LIT["rho"], LIT["Y"], LIT["B"]]) * f[:3]
    return yarn, LIT["S"] * f[3], LIT["mu"] * f[4]


def config0(rng):
    W = H = 5
    f = lambda n, k: LIT[k] * (1.0 + 0.2 * (2.0 * rng.random(n) - 1.0))  # noqa: E731
    warp = np.stack([f(H, "rho"), f(H, "Y"), f(H, "B")], axis=1)
    weft = np.stack([f(W, "rho"), f(W, "Y"), f(W, "B")], axis=1)
    S = LIT["S"] * (1.0 + 0.2 * (2.0 * rng.random() - 1.0))
    mu = LIT["mu"] * (1.0 + 0.2 * (2.0 * rng.random() - 1.0))
    return dict(W=W, H=H, weave="plain", pose=1, warp=warp, weft=weft, S=S, mu=mu, yarns=None,
                handles=[(0, 0), (W - 1, 0)], steps=200, keep_every=1)


def config1(rng, weave):
    W = H = 17
    y0, S, mu = material(rng)
    y1 = y0 * (1.5 + 1.5 * rng.random(3))
    warp = np.array([(y0, y1)[v % 2] for v in range(H)])
    weft = np.array([(y0, y1)[u % 2] for u in range(W)])
    return dict(W=W, H=H, weave=weave, pose=0, warp=warp, weft=weft, S=S, mu=mu, yarns=(y0, y1),
                handles=[(0, 0), (W - 1, 0)], steps=500, keep_every=10, pairs_every=20)


def driver_heter():
    """SimHeter's set-up (src/Simulate.h:332-452): cotton / polyester blend,
    R = 0.5 mm, S = 1000, mu = 0.5, upright in wind (0, 5, 0), 10 x 10, two
    top corners pinned; 30 steps."""
    W = H = 10
    y0, y1 = np.array([0.002, 500000.0, 0.00014]), np.array([0.0025, 170000.0, 0.00011])
    return dict(W=W, H=H, weave="plain", pose=0, warp=np.array([(y0, y1)[v % 2] for v in range(H)]),
                weft=np.array([(y0, y1)[u % 2] for u in range(W)]), S=1000.0, mu=0.5, yarns=(y0, y1),
                handles=[(0, 0), (W - 1, 0)], steps=30, keep_every=1, R=0.0005,
                wind=((0.0, 5.0, 0.0), 2.0, 0.5))


def driver_control():
    """SimControl's set-up (src/Simulate.h:218-330): a free flat 5 x 5 cloth,
    Y = 5e4, B = 1e-5, R = 0.5 mm, S = 1000, mu = 0.5, lifted and dragged at
    its corners (0.002 N) for steps 0..5; 30 steps."""
    W = H = 5
    y0 = np.array([0.002, 50000.0, 0.00001])
    ext = np.zeros(3 * W * H + 2 * (W - 2) * (H - 2))
    for n in (0, W - 1, W * (H - 1), W * H - 1):
        ext[3 * n + 1] = 0.002
        ext[3 * n + 2] = 0.002
    return dict(W=W, H=H, weave="plain", pose=1, warp=np.tile(y0, (H, 1)), weft=np.tile(y0, (W, 1)), S=1000.0,
                mu=0.5, yarns=(y0,), handles=[], steps=30, keep_every=1, R=0.0005,
                wind=((0.0, 0.0, 0.0), 2.0, 0.5), ext=ext, ext_steps=6)


def cases():
    out = {"config0_plain5_flat": config0(np.random.default_rng(100))}
    for i, weave in enumerate(("plain", "twill", "satin")):
        out["config1_%s17" % weave] = config1(np.random.default_rng(101 + i), weave)
    out["driver_simheter10"] = driver_heter()
    out["driver_simcontrol5"] = driver_control()
    return out


def run_case(name, cs, tmp):
    W, H = cs["W"], cs["H"]
    L, R, height = 1e-3, cs.get("R", LIT["R"]), 0.05
    cfg = dict(width=W, length=H, pose="flat" if cs["pose"] == 1 else "upright", weave=cs["weave"], L=L, R=R,
               height=height, mu=repr(float(cs["mu"])), S=repr(float(cs["S"])), kc=1.0, kf=1000.0, df=1000.0,
               handle_stiffness=1e4, G="0,0,9.8", h=1e-3, handles=",".join("%d,%d" % hp for hp in cs["handles"]),
               steps=cs["steps"], dump_steps="", out=os.path.join(tmp, name + ".bin"))
    wind = cs.get("wind")
    if wind:
        cfg["wind_vel"] = "%r,%r,%r" % wind[0]
        cfg["wind_density"], cfg["wind_drag"] = wind[1], wind[2]
    if cs.get("ext") is not None:
        cfg["ext_force"] = ",".join(repr(float(x)) for x in cs["ext"])
        cfg["ext_steps"] = cs["ext_steps"]
    if cs["yarns"] is not None:
        # the reference's own constructor with one yarn or a two-yarn blend
        for i, y in enumerate(cs["yarns"]):
            cfg["yarn%d" % i] = ",".join(repr(float(x)) for x in y)
    else:
        cfg["yarn0"] = ",".join(repr(float(x)) for x in cs["warp"][0])
        cfg["warp_lines"] = ";".join(",".join(repr(float(x)) for x in r) for r in cs["warp"])
        cfg["weft_lines"] = ";".join(",".join(repr(float(x)) for x in r) for r in cs["weft"])
    cpath = os.path.join(tmp, name + ".cfg")
    with open(cpath, "w") as f:
        for k, v in cfg.items():
            f.write("%s=%s\n" % (k, v))
    subprocess.run([HARNESS, cpath], check=True, capture_output=True)
    rec = read_records(cfg["out"])
    # every keep_every-th state, and the state after each pairs_every-th one
    # (one step from the reference's own state: the per-step parity check)
    pe = cs.get("pairs_every", 0)
    kept = sorted(set(s for s in range(cs["steps"] + 1) if s % cs["keep_every"] == 0) |
                  set(s + 1 for s in range(cs["steps"]) if pe and s % pe == 0))
    out = dict(width=W, length=H, weave=["plain", "twill", "satin"].index(cs["weave"]), pose=cs["pose"], L=L, R=R,
               height=height, mu=cs["mu"], S=cs["S"], kc=1.0, kf=1000.0, df=1000.0, handle_stiffness=1e4,
               G=np.array([0, 0, 9.8]), h=1e-3, warp=cs["warp"], weft=cs["weft"],
               handles=np.array(cs["handles"], dtype=np.int32).reshape(-1, 2), steps=cs["steps"],
               kept=np.array(kept), status=rec["status"])
    if wind:
        out.update(wind_vel=np.array(wind[0]), wind_density=wind[1], wind_drag=wind[2])
    else:
        out.update(wind_vel=np.zeros(3), wind_density=0.0, wind_drag=0.0)
    if cs.get("ext") is not None:
        out.update(ext_force=cs["ext"], ext_steps=cs["ext_steps"])
    for s in kept:
        for k in KEYS:
            out["s%d_%s" % (s, k)] = rec["s%d.%s" % (s, k)]
    out["s0_normal"] = rec["s0.normal"]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return name, float(rec["status"][0]), len(kept)


def main(argv):
    if not os.path.exists(HARNESS):
        subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh")], check=True)
    todo = cases()
    if argv:
        todo = {k: v for k, v in todo.items() if k in argv}
    with tempfile.TemporaryDirectory() as tmp, ThreadPoolExecutor(len(todo)) as ex:
        for name, status, n in ex.map(lambda kv: run_case(kv[0], kv[1], tmp), todo.items()):
            print(name, "status", status, "kept states", n)


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
