"""The C++ binding (include/yarnsim_torch.h) on the CPU: its test driver
compiles against LibTorch, and its reference binding (YarnSimGpu on the
reference's own Cloth and Environment) compiles and links against the
reference's headers and objects and libyarnsim.so. Running either needs a
GPU (tests/test_gpu_shim.py)."""
import os
import subprocess

import pytest

from pkg import ROOT, ys

import importlib.util

_spec = importlib.util.spec_from_file_location("cpp_build", os.path.join(ROOT, "tests", "cpp", "build.py"))
cpp_build = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(cpp_build)


def test_driver_compiles(tmp_path):
    ys.build()
    try:
        cpp_build.driver(str(tmp_path / "shim_driver"))
    except subprocess.CalledProcessError as e:
        pytest.fail(e.stderr[-3000:])
    assert os.path.exists(tmp_path / "shim_driver")


def test_reference_binding_compiles_and_links(tmp_path):
    from oracle.ref.refpath import ref_src
    src = ref_src()
    objs = os.path.join(ROOT, "oracle", "_ref", "obj")
    if src is None or not os.path.isdir(objs):
        pytest.skip("the reference sources or their oracle build are not here")
    ys.build()
    try:
        cpp_build.reference_binding(str(tmp_path / "reference_binding"), src)
    except subprocess.CalledProcessError as e:
        pytest.fail(e.stderr[-3000:])
    assert os.path.exists(tmp_path / "reference_binding")
