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


@pytest.mark.gpu
def test_tangent_and_control_argument_errors():
    if not gpu_available():
        pytest.skip("no CUDA device")
    b = ys.ClothBatch([spec()])
    with pytest.raises(ys.YarnSimError):
        b.step_tangent(1e-3, dext_force=np.zeros((b.n_tangents, b.total_nodes, 5)))  # before tangent_enable
    b.tangent_enable(0)
    with pytest.raises(ValueError):
        b.step_tangent(1e-3, dext_force=np.zeros((1, b.total_nodes, 5)))  # wrong shape
    with pytest.raises(ys.YarnSimError):
        b.step_tangent(1e-3, kact=b.n_tangents + 1)
    st = b.step_tangent(1e-3, np.zeros((b.total_nodes, 5)), dext_force=np.zeros((b.n_tangents, b.total_nodes, 5)))
    assert st[0]["ok"]
    b.close()
    with pytest.raises(ValueError):
        ys.control.embed_step(ys.control.ForceNet(250), spec(), np.zeros((25, 3)), 5, loop="other")


@pytest.mark.gpu
def test_response_calls_before_a_response_are_argument_errors():
    if not gpu_available():
        pytest.skip("no CUDA device")
    c = ys.Collider(4, 4)
    with pytest.raises(ys.YarnSimError) as e:
        c.respond_backward(np.zeros((16, 3)))  # no response yet
    assert e.value.status == 1
    with pytest.raises(ys.YarnSimError):
        c.set_max_zone_impacts(0)
    c.set_max_zone_impacts(1000)
    with pytest.raises(ys.YarnSimError):
        c.response_impacts()
    c.close()
