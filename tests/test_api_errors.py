"""Argument errors of the C ABI: every entry point returns a status instead of
aborting (the reference throws or exits), and batch creation rejects bad
descriptions before it touches the device, so these run on CPU too."""
import numpy as np
import pytest

from pkg import gpu_available, ys


def spec(**kw):
    base = dict(width=5, length=5, warp=np.tile([1e-3, 1e3, 1e-5], (5, 1)), weft=np.tile([1e-3, 1e3, 1e-5], (5, 1)),
                handles=[(0, 0), (4, 0)])
    base.update(kw)
    return ys.ClothSpec(**base)


@pytest.mark.parametrize("bad", [
    dict(width=2, warp=np.tile([1e-3, 1e3, 1e-5], (5, 1)), weft=np.tile([1e-3, 1e3, 1e-5], (2, 1))),
    dict(L=1e-4, R=1e-4),
    dict(weave=3),
    dict(pose=2),
    dict(handles=[(5, 0)]),
    dict(handles=[(0, -1)]),
], ids=["narrow", "R_not_below_L", "weave", "pose", "handle_u", "handle_v"])
def test_bad_cloth_descriptions_are_argument_errors(bad):
    with pytest.raises(ys.YarnSimError) as e:
        ys.ClothBatch([spec(**bad)])
    assert e.value.status == 1


def test_empty_batch_is_an_argument_error():
    with pytest.raises(ys.YarnSimError) as e:
        ys.ClothBatch([])
    assert e.value.status == 1


@pytest.mark.gpu
def test_call_order_and_step_size_errors():
    if not gpu_available():
        pytest.skip("no CUDA device")
    b = ys.ClothBatch([spec()])
    with pytest.raises(ys.YarnSimError) as e:
        b.solve()
    assert e.value.status == 1
    with pytest.raises(ys.YarnSimError):
        b.step(0.0)
    with pytest.raises(ys.YarnSimError):
        b.step(-1e-3)
    assert all(s["ok"] for s in b.step(1e-3))  # still usable
    b.close()
