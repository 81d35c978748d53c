"""StepStats, the per-cloth result sequence step() and solve() return: over a
ys_cloth_stats array filled as the C ABI fills it, entries read as the dicts
the API documents, slices and equality behave like a list of those dicts, and
the whole-batch aggregates agree with the entries. No GPU needed."""
import importlib

import numpy as np

from pkg import NAME, ys

N = importlib.import_module(NAME + "._native")
cloth = importlib.import_module(NAME + ".cloth")


def _filled(n, seed=0):
    rng = np.random.default_rng(seed)
    arr = (N.ClothStats * n)()
    for i in range(n):
        arr[i].ok = int(rng.random() > 0.1)
        arr[i].cg_iterations = int(rng.integers(0, 40))
        arr[i].cg_error = float(rng.random() * 1e-10)
        arr[i].hit_maxiter = int(rng.random() > 0.9)
    return arr


def _dicts(arr):
    return [dict(ok=bool(s.ok), cg_iterations=s.cg_iterations, cg_error=s.cg_error, hit_maxiter=bool(s.hit_maxiter))
            for s in arr]


def test_entries_slices_and_equality():
    arr = _filled(37)
    st = cloth.StepStats(arr)
    ref = _dicts(arr)
    assert len(st) == 37
    assert [st[i] for i in range(37)] == ref
    assert st[-1] == ref[-1] and st[3:9] == ref[3:9]
    assert list(st) == ref and st == ref
    for d in st:
        assert set(d) == {"ok", "cg_iterations", "cg_error", "hit_maxiter"}
        assert isinstance(d["ok"], bool) and isinstance(d["cg_iterations"], int)


def test_aggregates():
    arr = _filled(256, seed=3)
    st = cloth.StepStats(arr)
    ref = _dicts(arr)
    assert st.all_ok == all(d["ok"] for d in ref)
    assert st.max_iterations == max(d["cg_iterations"] for d in ref)
    assert st.max_error == max(d["cg_error"] for d in ref)
    assert st.iterations.tolist() == [d["cg_iterations"] for d in ref]
    for i in range(256):
        arr[i].ok = 1
    assert cloth.StepStats(arr).all_ok


def test_exported_from_the_package():
    assert ys.StepStats is cloth.StepStats
