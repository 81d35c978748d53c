"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, and
exports every entry point that include/yarnsim.h declares. No compute call is
made (there may be no GPU)."""
import ctypes
import os
import re

from pkg import ROOT, ys


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "yarnsim.h")).read()
    return sorted(set(re.findall(r"\b(ys_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_entry_points():
    names = declared_symbols()
    for n in ("ys_batch_create", "ys_step", "ys_assemble", "ys_solve", "ys_export_system", "ys_set_state",
              "ys_get_state"):
        assert n in names


def test_library_builds_and_exports_every_declared_symbol():
    path = ys.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_targets_sm_103a():
    from importlib import import_module
    bl = import_module(ys.__name__ + ".buildlib")
    assert "arch=compute_103a,code=sm_103a" in " ".join(bl.ARCH)


def test_binding_covers_header():
    from importlib import import_module
    nat = import_module(ys.__name__ + "._native")
    assert sorted(nat.EXPORTED) == declared_symbols()
