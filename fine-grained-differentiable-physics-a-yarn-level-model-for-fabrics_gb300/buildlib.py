"""Builds the CUDA library (_lib/libyarnsim.so) for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into one shared
library with a plain C ABI (include/yarnsim.h).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libyarnsim.so")
SOURCES = ["ys_tangent.cu", "ys_kernels.cu", "ys_api.cu", "ys_collide.cu", "ys_gnn.cu", "ys_adjoint.cu",
           "ys_pcg_cluster.cu"]
HEADERS = ["ys_common.cuh", "ys_dual.cuh", "ys_physics.cuh", "ys_items.cuh", "ys_elem_kernels.cuh", "ys_kernels.cuh", "ys_collide.cuh", "ys_bvh.h",
           "ys_gnn.cuh", "ys_tc.cuh", "ys_zones.h", "ys_pool.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC"]
# the collision tests keep IEEE products and sums separate, as the reference's
# CPU arithmetic does: a contracted cross product of two equal vectors is its
# rounding error instead of zero, and the CCD cubic of a static face against a
# moving vertex (exactly linear) then grows spurious roots
PER_FILE = {"ys_collide.cu": ["-fmad=false"]}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libyarnsim.so")
    return p


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(ROOT, "include", "yarnsim.h"),
                                                                 os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if needed) and return the path of libyarnsim.so."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(LIB_DIR, src.replace(".cu", ".o"))
        cmd = [cc] + ARCH + FLAGS + PER_FILE.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s" % r.stderr[-4000:])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
