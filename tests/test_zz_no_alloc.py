"""ys_apply_system_noalloc through the C ABI against ys_apply_system.

The variant computes the same row products from a static per-device scratch
copy of x, so its result must equal ys_apply_system's (the tolerance below
allows only last-bit differences; the arithmetic is the same). Two calls in a
row check that nothing left in the scratch by one call leaks into the next.
This file is named to be collected after every other test file, so it also
runs after the rest of the suite has used the device.
"""
import ctypes

import numpy as np
import pytest

import goldens
from pkg import gpu_available, spec_from_golden, ys

pytestmark = pytest.mark.gpu

N = ys._native
REL_TOL = 1e-14
MAX_NODES = 65536


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _apply_both(b, x):
    """(y from ys_apply_system, y from ys_apply_system_noalloc), x a CUDA tensor [nodes, 5]."""
    import torch
    L = N.load()
    y_ref = torch.full_like(x, float("nan"))
    y_new = torch.full_like(x, float("nan"))
    torch.cuda.synchronize()
    N.check(L.ys_apply_system(b._h, _ptr(x), _ptr(y_ref), N.YS_ON_DEVICE), "ys_apply_system")
    N.check(L.ys_apply_system_noalloc(b._h, _ptr(x), _ptr(y_new)), "ys_apply_system_noalloc")
    b.synchronize()
    return y_ref.cpu().numpy(), y_new.cpu().numpy()


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _random_x(n, seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    return torch.randn((n, 5), generator=g, dtype=torch.float64).cuda()


def test_two_calls_in_a_row_match_apply_system():
    specs = [spec_from_golden(goldens.load(n)) for n in ("satin7x5_flat_pert", "twill6_upright_wind_pert")]
    b = ys.ClothBatch(specs)
    b.assemble(1e-3)
    n = b.total_nodes
    for seed in (1, 2):
        y_ref, y_new = _apply_both(b, _random_x(n, seed))
        assert np.isfinite(y_new).all()
        assert _rel(y_new, y_ref) <= REL_TOL, seed
    b.close()


def test_large_batch_two_calls_match_apply_system():
    rng = np.random.default_rng(5)
    base = np.array([1e-3, 1e3, 1e-5])
    specs = []
    for c in range(26):  # 26 * 50 * 50 = 65,000 nodes, just under the scratch limit
        W = H = 50
        specs.append(ys.ClothSpec(width=W, length=H, weave=c % 3, pose=1, handles=[(0, 0), (W - 1, 0)],
                                  warp=base * (1 + 0.2 * (2 * rng.random((H, 3)) - 1)),
                                  weft=base * (1 + 0.2 * (2 * rng.random((W, 3)) - 1)),
                                  wind_vel=(0.1, 0.3, 0.0), wind_density=1.0, wind_drag=0.5))
    b = ys.ClothBatch(specs)
    assert b.total_nodes <= MAX_NODES
    b.assemble(1e-3)
    for seed in (3, 4):
        y_ref, y_new = _apply_both(b, _random_x(b.total_nodes, seed))
        assert np.isfinite(y_new).all()
        assert _rel(y_new, y_ref) <= REL_TOL, seed
    b.close()


def test_rejects_batches_beyond_scratch_limit():
    import torch
    W = H = 50
    base = np.array([1e-3, 1e3, 1e-5])
    specs = [ys.ClothSpec(width=W, length=H, warp=np.tile(base, (H, 1)), weft=np.tile(base, (W, 1)), pose=1,
                          handles=[(0, 0), (W - 1, 0)]) for _ in range(27)]
    b = ys.ClothBatch(specs)
    assert b.total_nodes > MAX_NODES
    b.assemble(1e-3)
    x = torch.zeros((b.total_nodes, 5), dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    st = N.load().ys_apply_system_noalloc(b._h, _ptr(x), _ptr(y))
    assert st == N.YS_ERR_ARG
    assert "scratch limit" in N.last_error()
    b.close()


def test_rejects_host_arrays():
    """A host array in place of x or y is refused before anything launches."""
    import torch
    specs = [spec_from_golden(goldens.load("satin7x5_flat_pert"))]
    b = ys.ClothBatch(specs)
    b.assemble(1e-3)
    L = N.load()
    n = b.total_nodes
    x_dev = torch.zeros((n, 5), dtype=torch.float64, device="cuda")
    y_dev = torch.zeros_like(x_dev)
    x_host = np.zeros((n, 5))
    y_host = np.zeros((n, 5))
    hp = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    before = b.profile_read(reset=False)["total_launches"]
    assert L.ys_apply_system_noalloc(b._h, hp(x_host), _ptr(y_dev)) == N.YS_ERR_ARG
    assert "x is not" in N.last_error()
    assert L.ys_apply_system_noalloc(b._h, _ptr(x_dev), hp(y_host)) == N.YS_ERR_ARG
    assert "y is not" in N.last_error()
    assert b.profile_read(reset=False)["total_launches"] == before
    b.close()
