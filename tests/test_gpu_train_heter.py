"""train_heter_full (src/TrainHeter.h:11-306) on a trajectory file SimHeter
wrote (drivers.sim_heter, the reference's HDF5 layout): started at the
parameters that made the data the loss is at round-off; started away from
them, the gradient it steps along matches central differences of its own
loss (exact mode, 1e-5 relative, or ten times the difference quotient's own
error estimated from two step sizes); the training record is written as
SaveTrainProc writes it (src/Saver.cpp:93-150)."""
import numpy as np
import pytest

from pkg import gpu_available, ys

pytestmark = pytest.mark.gpu

TRUE = dict(rho_1=0.002, rho_2=0.0025, Y_1=500000.0, Y_2=170000.0, B_1=0.00014, B_2=0.00011, S=1000.0, mu=0.5)


@pytest.fixture(scope="module")
def data(tmp_path_factory):
    if not gpu_available():
        pytest.skip("no CUDA device")
    path = str(tmp_path_factory.mktemp("heter") / "heter.h5")
    ys.drivers.sim_heter(width=6, length=6, steps=20, yarns=((0.002, 500000.0, 0.00014), (0.0025, 170000.0, 0.00011)),
                         S=1000.0, h5_path=path)
    return path


def test_true_parameters_give_round_off_loss_and_the_record_is_written(data, tmp_path):
    out = str(tmp_path / "train.h5")
    hist = ys.drivers.train_heter_full(data, epoch=1, batch=1, sample=5, steps=20, all_steps=True, init=TRUE,
                                       save_path=out, lr={k: 0.0 for k in TRUE})
    assert len(hist["loss"]) == 4  # samples // batch iterations
    assert max(hist["loss"]) <= 1e-20, hist["loss"]
    f = ys.h5.read(out)
    assert f["/Loss"].shape == (4, 1)
    for n in ("rho1", "rho2", "Y1", "Y2", "B1", "B2", "S", "mu"):
        assert f["/" + n].shape == (4, 1)
    np.testing.assert_allclose(f["/rho1"][:, 0], TRUE["rho_1"], rtol=1e-12)


def test_gradient_matches_central_differences(data):
    init = dict(TRUE, rho_1=0.0021, Y_2=160000.0, B_1=0.00013, S=1100.0)
    kw = dict(epoch=1, iters=1, batch=1, sample=6, steps=20, all_steps=False, mode="exact",
              lr={k: 0.0 for k in TRUE})
    base = ys.drivers.train_heter_full(data, init=init, **kw)
    assert base["loss"][0] > 1e-12
    import torch
    for n in ("rho_1", "Y_2", "B_1", "S"):
        lo, up = ys.drivers.HETER_RANGES[n][1], ys.drivers.HETER_RANGES[n][0]
        raw = ys.invert_constraint_para(init[n], up, lo)
        fds = []
        for eps in (1e-4, 2e-4):
            vals = []
            for sgn in (1, -1):
                v = ys.constraint_para(torch.tensor([raw + sgn * eps], dtype=torch.float64), up, lo).item()
                vals.append(ys.drivers.train_heter_full(data, init=dict(init, **{n: v}), **kw)["loss"][0])
            fds.append((vals[0] - vals[1]) / (2 * eps))
        fd = fds[0]
        # the quotient's own error (truncation and the loss's round-off), from two step sizes
        noise = abs(fds[0] - fds[1]) / abs(fd)
        g = base["grad"][n][0]
        assert abs(g - fd) <= max(1e-5, 10 * noise) * abs(fd), (n, g, fd, noise)
