"""Control learning through the simulator (ForceNet, src/ForceNet.h; one
evaluation of train_embed, src/TrainEmbed.h:84-176) against the reference's
own LibTorch run (tests/golden/make_embed_golden.py), and the external-force
tangents (ys_step_tangent_ext) against central differences.
"""
import os

import numpy as np
import pytest

import goldens
from pkg import gpu_available, ys

torch = pytest.importorskip("torch")
GOLDEN = os.path.join(goldens.GOLDEN_DIR, "embed_plain5.npz")


def _golden():
    return dict(np.load(GOLDEN))


def _spec(g):
    c = lambda k: float(g["cfg_" + k])
    yarn = ys.Yarn(R=c("R"), rho=c("rho"), Y=c("Y"), B=c("B"))
    spec = ys.ClothSpec.from_yarns(int(g["cfg_width"]), int(g["cfg_length"]), c("height"), c("L"), c("R"), [yarn],
                                   c("kc"), c("kf"), c("df"), c("mu"), c("S"), c("handle_stiffness"),
                                   ys.WovenPattern.Plain, ys.InitPose.Upright)
    spec.G = tuple(float(x) for x in str(g["cfg_G"]).split(","))
    spec.wind_vel = tuple(float(x) for x in str(g["cfg_wind_vel"]).split(","))
    spec.wind_density, spec.wind_drag = c("wind_density"), c("wind_drag")
    return spec


def _net(g):
    net = ys.control.ForceNet(10 * int(g["cfg_width"]) * int(g["cfg_length"]), 2)
    with torch.no_grad():
        for name, p in net.named_parameters():
            p.copy_(torch.from_numpy(g["param__" + name.replace(".", "__")]).to(p.dtype))
    return net


def test_force_layout_follows_the_reference_index():
    # (first, second) -> first * width + second: the four corners of a square cloth
    assert ys.control.force_nodes(5, [(0, 0), (4, 0), (0, 4), (4, 4)]) == [0, 20, 4, 24]


def test_network_matches_the_reference_forward():
    g = _golden()
    net = _net(g)
    assert sum(p.numel() for p in net.parameters()) == 250 * 125 + 125 + 125 * 60 + 60 + 60 * 2 + 2
    x = torch.zeros(1, 250)
    out = net(x)
    assert out.shape == (1, 2) and float(out.min()) > 0.0 and float(out.max()) < 0.004


@pytest.mark.gpu
@pytest.mark.parametrize("loop", ["reference", "intended"])
def test_embed_step_matches_the_reference_gradient(loop):
    """Loss, predicted forces and the gradient of every ForceNet parameter of
    one train_embed evaluation, with the tangents in the reference's
    EigenSolver-backward mode, against the reference's own autograd: its loop
    as written (one forced step) and forcing steps 0..5, where each force
    also depends on the earlier ones through the network's input."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    g = dict(np.load(GOLDEN if loop == "reference" else GOLDEN.replace(".npz", "_intended.npz")))
    net = _net(g)
    out = ys.control.embed_step(net, _spec(g), g["goal"], int(g["cfg_sample"]), h=float(g["cfg_h"]),
                                loop=loop, tangent_mode=ys._native.YS_TANGENT_REFERENCE)
    assert np.allclose(out["forces"].reshape(-1), g["forces"], rtol=1e-6, atol=0)
    # the loss is a small difference of mass centres (5e-5 after eleven steps)
    assert abs(out["loss"] - g["loss"][0]) <= 1e-7 * g["loss"][0]
    # later forces come from float32 casts of the state, whose last bits can
    # differ between two FP64 simulators; 1e-12 m for the one-force loop
    assert np.abs(out["final_lpos"] - g["final__LPos"]).max() <= (1e-12 if loop == "reference" else 1e-9)
    for name, grad in out["grads"].items():
        ref = g["grad__" + name.replace(".", "__")]
        scale = max(np.abs(ref).max(), 1e-30)
        assert np.abs(grad - ref).max() <= 1e-4 * scale, name


@pytest.mark.gpu
@pytest.mark.parametrize("loop", ["reference", "intended"])
def test_force_gradient_matches_central_differences(loop):
    """d loss / d forces from the exact external-force tangents (and, for
    the intended loop, the chain through the network's inputs) against
    central differences of the loss in a constant-output network's forces."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    g = _golden()
    spec = _spec(g)

    class Const(torch.nn.Module):
        def __init__(self, f):
            super().__init__()
            self.f = torch.nn.Parameter(torch.tensor([f], dtype=torch.float64))
            self.w = torch.nn.Parameter(torch.zeros(1, 250, dtype=torch.float64))

        def forward(self, x):
            return self.f + 1e-3 * (x.double() * self.w).sum() * torch.ones(1, 2, dtype=torch.float64)

    f0 = [0.002, 0.0015]
    rng = np.random.default_rng(0)
    w0 = 1e-2 * rng.normal(size=(1, 250))

    def run(f):
        net = Const(f)
        with torch.no_grad():
            net.w.copy_(torch.from_numpy(w0))
        return ys.control.embed_step(net, spec, g["goal"], 9, loop=loop, tangent_mode=ys._native.YS_TANGENT_EXACT,
                                     input_dtype=torch.float64, tol=1e-14, maxiter=100000), net
    out, net = run(f0)
    an = net.f.grad.numpy()[0]
    eps = 1e-6
    for j in range(2):
        fp, fm = list(f0), list(f0)
        fp[j] += eps
        fm[j] -= eps
        fd = (run(fp)[0]["loss"] - run(fm)[0]["loss"]) / (2 * eps)
        # the tangent-vs-difference bar of the parameter gradients (sliding
        # friction makes the step only piecewise smooth)
        assert abs(fd - an[j]) <= 1e-4 * max(abs(an[j]), 1e-12), (j, fd, an[j])
