"""Per-node control forces through the reverse-mode adjoint
(drivers.CentroidControl on ys_adjoint_step): the collision benchmark's
control problem, the cloth's centroid after the controlled window driven
toward a seeded target 10-30 cm away (the mass-centre loss of
src/TrainControl.h:192-203 on a per-node force at every step).

- the gradient with respect to every node's force at every step, taken in
  one reverse sweep with checkpoints, against central differences of the
  GPU rollout along random force directions: 1e-6 relative;
- the benchmark scene itself (50 x 50 cloth, 100 steps of h = 5e-4,
  7,500 force components per step): Adam on the forces lowers the loss, and
  the controlled window has no impacts with the sphere (the rollout has no
  collision response; the large forces can fold the cloth's lighter edges
  onto itself, which CentroidControl.collide reports).
"""
import numpy as np
import pytest

from pkg import gpu_available, ys

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def test_force_gradient_matches_central_differences():
    sc = ys.DropOnSphere(width=12, radius=0.01, levels=2, drop=0.05, h=5e-4)
    try:
        ctl = ys.drivers.CentroidControl(sc, steps=10, seed=3, checkpoint_every=4)
        rng = np.random.default_rng(0)
        f0 = 2e-6 * rng.standard_normal(ctl.forces.shape)
        L0, g, _ = ctl.gradient(f0)
        for trial in range(3):
            d = rng.standard_normal(ctl.forces.shape)
            d /= np.linalg.norm(d)
            eps = 1e-6
            lp = ctl.loss_and_traj(f0 + eps * d)[0]
            lm = ctl.loss_and_traj(f0 - eps * d)[0]
            fd = (lp - lm) / (2 * eps)
            ad = float((g * d).sum())
            assert abs(ad - fd) <= 1e-6 * abs(fd), (trial, ad, fd)
    finally:
        sc.close()


def test_drop50_control_lowers_the_loss():
    sc = ys.DropOnSphere(width=50, radius=0.03, levels=3, drop=0.05, h=5e-4)
    try:
        ctl = ys.drivers.CentroidControl(sc, steps=100, seed=7, checkpoint_every=20)
        d0 = np.linalg.norm(ctl.state0["LPos"].mean(axis=0) - ctl.target)
        assert 0.1 <= d0 <= 0.3 + 1e-3
        hist = ctl.optimise(iterations=5, lr=2e-5)
        assert hist[-1] < 0.5 * hist[0], hist
        assert all(b < a for a, b in zip(hist, hist[1:])), hist
        _, traj, _ = ctl.loss_and_traj()
        assert ctl.collide(traj)["sphere"] == 0
    finally:
        sc.close()
