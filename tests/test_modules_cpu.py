"""Host-side parts of the learnable modules (no GPU): parameter registration,
constraint_para mappings and the control module's force layout (the
reference's lift / drag positions, src/YarnSimNet.h:186-196)."""
import numpy as np

from pkg import ys

RANGES = dict(rho=(0.003, 0.0001), Y=(2e6, 10.0), B=(1e-3, 1e-7), S=(2000.0, 1e-6))


def test_homo_parameters_and_theta():
    vals = dict(rho=1e-3, Y=1e3, B=1e-5, S=1e-4)
    raw = {n: ys.invert_constraint_para(v, *RANGES[n]) for n, v in vals.items()}
    net = ys.YarnSimNetHomo(5, 4, 1e-4, 1e-3, raw, RANGES, [(0, 0), (4, 0)], mu=0.3)
    assert sorted(n for n, _ in net.named_parameters()) == ["B", "S", "Y", "rho"]
    th = net.theta().detach().numpy()
    assert th.shape == (8,)
    np.testing.assert_allclose(th[:3], [1e-3, 1e3, 1e-5], rtol=1e-12)
    np.testing.assert_array_equal(th[:3], th[3:6])  # one yarn type: both parities equal
    np.testing.assert_allclose(th[6:], [1e-4, 0.3], rtol=1e-12)
    sp = net.spec()
    assert sp.width == 5 and sp.length == 4 and sp.pose == ys.InitPose.Upright and sp.height == 0.0
    assert np.all(np.asarray(sp.warp) == np.asarray(sp.warp)[0])


def test_homo_gradient_reaches_the_raw_parameters():
    import torch
    raw = {n: ys.invert_constraint_para(v, *RANGES[n]) for n, v in dict(rho=1e-3, Y=1e3, B=1e-5, S=1e-4).items()}
    net = ys.YarnSimNetHomo(5, 4, 1e-4, 1e-3, raw, RANGES, [(0, 0), (4, 0)])
    th = net.theta()
    (th * torch.arange(1.0, 9.0, dtype=torch.float64)).sum().backward()
    # d/d raw = (sum of the two parities' weights) x sigmoid'(raw) x (upper - lower)
    for i, n in enumerate(("rho", "Y", "B")):
        up, lo = RANGES[n]
        s = torch.sigmoid(torch.tensor(raw[n], dtype=torch.float64))
        want = float(((i + 1) + (i + 4)) * s * (1 - s) * (up - lo))
        np.testing.assert_allclose(float(getattr(net, n).grad[0]), want, rtol=1e-12)


def test_control_parameters_and_force_layout():
    mat = dict(rho=1e-3, Y=1e3, B=1e-5, S=1e-4, mu=0.3)
    forces = [(0.1 * (i + 1), -0.01 * (i + 1)) for i in range(6)]
    net = ys.YarnSimNetControl(7, 6, 1e-4, 1e-3, mat, forces, [(0, 0), (0, 6), (5, 3)])
    names = sorted(n for n, _ in net.named_parameters())
    assert len(names) == 12 and "lift_force_one" in names and "drag_force_six" in names
    sp = net.spec()
    assert sp.handles == [] and sp.height == 5.0 and sp.pose == ys.InitPose.Upright
    assert net.ext_force(6) is None
    for idx in range(6):
        e = net.ext_force(idx)
        nz = np.argwhere(e != 0)
        # node a * width + b: z (lift) and y (drag) components only
        assert set(map(tuple, nz)) == {(0, 1), (0, 2), (6, 1), (6, 2), (38, 1), (38, 2)}
        assert np.all(e[[0, 6, 38], 2] == forces[idx][0]) and np.all(e[[0, 6, 38], 1] == forces[idx][1])


def test_colli_parameters():
    x = np.zeros((3, 3))
    f = np.array([[0, 1, 2]], dtype=np.int32)
    raw = {n: 0.0 for n in ("rho", "Y", "B")}
    net = ys.YarnSimNetColli(6, 5, 0.01, 1e-4, 1e-3, raw, RANGES, [(0, 0), (5, 0)], x, f)
    assert sorted(n for n, _ in net.named_parameters()) == ["B", "Y", "rho"]
    th = net.theta().detach().numpy()
    np.testing.assert_allclose(th[0], 0.5 * (RANGES["rho"][0] + RANGES["rho"][1]), rtol=1e-12)
    assert th[6] == 1000.0 and th[7] == 0.5 and net.thickness == 0.0005
