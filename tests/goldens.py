"""Helpers to load the reference-generated fixtures in tests/golden/."""
import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    """Trajectory / system fixtures (tests/golden/make_golden.py)."""
    return sorted(n for n in (os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))
                  if not n.startswith(("grad_", "collide_", "h5_", "embed_", "config", "driver_")))


def grad_names():
    """Reference-gradient fixtures (tests/golden/make_grad_golden.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "grad_*.npz")))


def load(name):
    return dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))


def spec_kwargs(g):
    """Construction parameters of a fixture, as keyword arguments."""
    return dict(width=int(g["width"]), length=int(g["length"]), warp=g["warp"], weft=g["weft"],
                height=float(g["height"]), L=float(g["L"]), R=float(g["R"]), pose=int(g["pose"]),
                weave=int(g["weave"]), kc=float(g["kc"]), kf=float(g["kf"]), df=float(g["df"]),
                mu=float(g["mu"]), S=float(g["S"]), handle_stiffness=float(g["handle_stiffness"]),
                G=tuple(float(x) for x in g["G"]), wind_vel=tuple(float(x) for x in g["wind_vel"]),
                wind_density=float(g["wind_density"]), wind_drag=float(g["wind_drag"]),
                handles=[tuple(int(a) for a in r) for r in g["handles"].reshape(-1, 2)])


def init_state(g):
    if "init_LPos" not in g:
        return None
    return {k: g["init_" + k] for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")}


def state(g, step):
    return {k: g["s%d_%s" % (step, k)] for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")}


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def config_names():
    """Benchmark-scale reference fixtures (tests/golden/make_config_golden.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "config*.npz")))


def rel_comp(a, b, floor=1e-3):
    """Largest per-component relative error |a - b| / max(|b|, floor * max|b|):
    every component is held to the tolerance against its own size, except
    components smaller than `floor` times the field's largest, which are held
    against that floor (a component that is zero up to round-off has no
    meaningful relative error of its own)."""
    a = np.asarray(a); b = np.asarray(b)
    scale = np.maximum(np.abs(b), floor * max(np.abs(b).max(), 1e-300))
    return float((np.abs(a - b) / scale).max())
