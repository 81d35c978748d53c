"""Compile recipes of the C++ binding's test programs (test infrastructure).

driver(out): tests/cpp/shim_driver.cpp against include/ and the installed
LibTorch, linked with libyarnsim.so (runs on a GPU).
reference_binding(out, ref_src): tests/cpp/reference_binding.cpp against
the reference's own headers (the oracle build's shims), linked with its
objects from oracle/_ref/obj and libyarnsim.so (compile and link check).
"""
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PKG = os.path.join(ROOT, "fine-grained-differentiable-physics-a-yarn-level-model-for-fabrics_gb300")
LIB_DIR = os.path.join(PKG, "_lib")


def _torch_flags():
    import torch
    tdir = os.path.dirname(torch.__file__)
    inc = [os.path.join(tdir, "include"), os.path.join(tdir, "include", "torch", "csrc", "api", "include")]
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    cflags = ["-std=c++17", "-O1", "-D_GLIBCXX_USE_CXX11_ABI=%d" % abi] + sum([["-isystem", p] for p in inc], [])
    lib = os.path.join(tdir, "lib")
    lflags = ["-L", lib, "-Wl,-rpath," + lib, "-ltorch", "-ltorch_cpu", "-lc10",
              "-L", LIB_DIR, "-Wl,-rpath," + LIB_DIR, "-lyarnsim", "-lpthread"]
    return cflags, lflags


def driver(out):
    cflags, lflags = _torch_flags()
    cmd = ["g++"] + cflags + ["-I", os.path.join(ROOT, "include"), os.path.join(HERE, "shim_driver.cpp"),
                              "-o", out] + lflags
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def reference_binding(out, ref_src):
    cflags, lflags = _torch_flags()
    shim = os.path.join(ROOT, "oracle", "ref", "shim")
    objs = [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))
            if os.path.basename(o) != "ref_harness.o"]
    cmd = (["g++"] + cflags + ["-w", "-include", os.path.join(shim, "prelude.h"), "-I", shim, "-I", ref_src,
                              "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "reference_binding.cpp"),
                              "-o", out] + objs + lflags + ["-lgomp"])
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out
