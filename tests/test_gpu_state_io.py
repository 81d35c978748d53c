"""State and external-force transfer through the C ABI from host memory of
both kinds: pageable arrays go through the handle's device stage, page-locked
ones (a pinned tensor's storage) are read and written by the transposition
kernels themselves. Both must move the same bits, for a ragged batch whose
node count is no multiple of the kernels' 256-node blocks.
"""
import numpy as np
import pytest
import torch

from pkg import gpu_available, ys

pytestmark = pytest.mark.gpu

KEYS = ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _batch(seed=5):
    rng = np.random.default_rng(seed)
    base = np.array([1e-3, 1e3, 1e-5])
    specs = []
    for i, (W, H) in enumerate([(17, 23), (5, 5), (33, 12), (9, 31)]):
        j = lambda n: base * (1.0 + 0.2 * (2.0 * rng.random((n, 3)) - 1.0))  # noqa: E731
        specs.append(ys.ClothSpec(width=W, length=H, warp=j(H), weft=j(W), height=0.05, L=1e-3, R=1e-4,
                                  pose=i % 2, weave=i % 3, wind_vel=(0.0, 0.4, 0.0), wind_density=1.0,
                                  wind_drag=0.5, handles=[(0, 0), (W - 1, 0)]))
    return ys.ClothBatch(specs)


def _pinned(shape):
    return torch.zeros(shape, dtype=torch.float64).pin_memory().numpy()


def _empty(T, pinned):
    mk = _pinned if pinned else np.zeros
    return {k: mk((T, 3 if k.startswith("L") else 2)) for k in KEYS}


def test_pinned_and_pageable_state_round_trip():
    b = _batch()
    T = b.total_nodes
    assert T % 256 != 0
    for _ in range(2):
        assert all(s["ok"] for s in b.step(1e-3, tol=1e-10))
    pageable = b.get_state(out=_empty(T, False))
    pinned = b.get_state(out=_empty(T, True))
    for k in KEYS:
        assert np.array_equal(pageable[k], pinned[k]), k
    # a perturbed state uploaded from pinned memory reads back unchanged
    rng = np.random.default_rng(0)
    src = _empty(T, True)
    for k in KEYS:
        src[k][:] = pageable[k] + 1e-6 * rng.standard_normal(pageable[k].shape)
    b.set_state(**src)
    back = b.get_state(out=_empty(T, False))
    for k in KEYS:
        assert np.array_equal(back[k], src[k]), k
    b.close()


def test_pinned_and_pageable_external_force_step_alike():
    outs = []
    for pinned in (False, True):
        b = _batch()
        T = b.total_nodes
        rng = np.random.default_rng(1)
        ext = (_pinned if pinned else np.zeros)((T, 5))
        ext[:] = 1e-4 * rng.standard_normal((T, 5))
        for _ in range(3):
            assert all(s["ok"] for s in b.step(1e-3, ext, tol=1e-10))
        outs.append(b.get_state(out=_empty(T, pinned)))
        b.close()
    for k in KEYS:
        assert np.array_equal(outs[0][k], outs[1][k]), k
