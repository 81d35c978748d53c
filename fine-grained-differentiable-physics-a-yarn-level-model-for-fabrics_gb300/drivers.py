"""The reference's simulation drivers (src/Simulate.h) on the package API.

Each driver builds the cloth the way the reference does (Cloth, Environment,
PhysicsCloth, set_handles) and runs its loop of SimStep (src/TrainHelper.cpp
:15-149) on the GPU path. Instead of the fixed output paths of the reference
(./data/*.h5, ./objs/Cloth%04d.obj) the caller passes h5_path and obj_dir
(None: not written); every driver returns the per-step states as arrays
[steps + 1, nodes, 3|2] (the initial state first), the layout data_loader
reads back. `height` defaults to the reference's 5 m.

- sim_homo       SimHomo       src/Simulate.h:10-106
- sim_collision  SimCollision  src/Simulate.h:108-216 (obstacle meshes as
                 arguments: the reference's ./obs/wall.obj and ground.obj are
                 not in its repository)
- sim_control    SimControl    src/Simulate.h:218-330
- sim_heter      SimHeter      src/Simulate.h:332-452
- DropOnSphere   the collision benchmark scene: a flat cloth dropped onto an
                 icosphere with self-collision (the reference's collision
                 step, SimStep with a Collision)
- train_heter_full  train_heter_full  src/TrainHeter.h:11-306 (parameter
                 learning from a SimHeter trajectory file)
"""
from __future__ import annotations

import os
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import h5 as _h5
from .cloth import Cloth, Environment, InitPose, PhysicsCloth, SimStep, Wind, WovenPattern, Yarn
from .collide import Collision, icosphere
from .render import RenderCloth, RenderType

FULL = ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")

# the reference drivers' material (src/Simulate.h:16-32, 132-148)
HOMO = dict(L=0.001, R=0.0005, rho=0.002, Y=500000.0, B=0.00014, kc=1.0, mu=0.5, df=1000.0, kf=1000.0, S=1000.0,
            handle_stiffness=1e4, G=(0.0, 0.0, 9.8))
# the benchmark configurations' material (the reference's Yarn(R, rho, Y, B)
# arguments with R = 0.1 mm, S and mu per cloth)
BENCH = dict(HOMO, R=0.0001, rho=0.001, Y=1000.0, B=1e-5, S=1e-4, mu=0.3)


def _record(states: Dict[str, List[np.ndarray]], cloth: Cloth):
    st = cloth.get_ClothState().as_dict()
    for k in FULL:
        states[k].append(np.array(st[k]))


def _finish(states, cloth: Cloth, h5_path: Optional[str], physical: Dict):
    out = {k: np.array(v) for k, v in states.items()}
    if h5_path:
        _h5.save_trajectory(h5_path, cloth.width, cloth.length, physical, out)
    return out


def _physical_homo(env: Environment, p: Dict, pattern: int) -> Dict:
    """The H5Physical record SaveClothHomoYarn writes (src/Saver.cpp:184-300)."""
    w = env.wind
    return dict(Gravity=float(env.G[2]), rho=p["rho"], R=p["R"], L=p["L"], Y=p["Y"], B=p["B"], kc=p["kc"],
                kf=p["kf"], df=p["df"], mu=p["mu"], S=p["S"], handle_stiff=p["handle_stiffness"],
                wind_velocity_x=float(w.WindVelocity[0]), wind_velocity_y=float(w.WindVelocity[1]),
                wind_velocity_z=float(w.WindVelocity[2]), wind_density=float(w.WindDensity),
                wind_drag=float(w.WindDrag), woven_pattern=int(pattern))


def _obj(cloth, obj_dir, i):
    if obj_dir:
        os.makedirs(obj_dir, exist_ok=True)
        RenderCloth(cloth, os.path.join(obj_dir, "Cloth%04d.obj" % i), RenderType.MeshTriangle)


def _run(cloth, phy, steps, h, obj_dir, ext=None, force_steps=None, collision=None):
    states = {k: [] for k in FULL}
    _record(states, cloth)
    for i in range(steps):
        if collision is not None:
            ok = SimStep(cloth, phy, collision, h)
        else:
            f = ext if (ext is not None and (force_steps is None or i < force_steps)) else None
            ok = SimStep(cloth, phy, h, f)
        if not ok:
            break
        _record(states, cloth)
        _obj(cloth, obj_dir, i)
    return states


def sim_homo(width: int = 10, length: int = 10, steps: int = 100, h: float = 0.001, handles=None,
             wind=Wind((0.0, 5.0, 0.0), 2.0, 0.5), params: Optional[Dict] = None, h5_path: Optional[str] = None,
             obj_dir: Optional[str] = None, height: float = 5.0, device: int = 0) -> Dict[str, np.ndarray]:
    """SimHomo: a homogeneous plain cloth hanging from its two top corners in
    wind (10 x 10, 100 steps, the reference's material)."""
    p = dict(HOMO, **(params or {}))
    yarn = Yarn(p["R"], p["rho"], p["Y"], p["B"])
    cloth = Cloth(width, length, height, p["L"], p["R"], [yarn], p["kc"], p["kf"], p["df"], p["mu"], p["S"],
                  p["handle_stiffness"], WovenPattern.Plain, InitPose.Upright)
    env = Environment(cloth, p["G"], wind)
    cloth.set_handles(handles if handles is not None else [(0, 0), (width - 1, 0)])
    phy = PhysicsCloth(env, device=device)
    states = _run(cloth, phy, steps, h, obj_dir)
    return _finish(states, cloth, h5_path, _physical_homo(env, p, WovenPattern.Plain))


def sim_heter(width: int = 10, length: int = 10, steps: int = 100, h: float = 0.001, handles=None,
              yarns: Sequence[Tuple[float, float, float]] = ((0.002, 500000.0, 0.00014), (0.0025, 170000.0, 0.00011)),
              S: float = 1000.0, wind=Wind((0.0, 5.0, 0.0), 2.0, 0.5), pattern: int = WovenPattern.Plain,
              h5_path: Optional[str] = None, obj_dir: Optional[str] = None, height: float = 5.0,
              device: int = 0) -> Dict[str, np.ndarray]:
    """SimHeter: a two-yarn blend (cotton / polyester by default) hanging in
    wind; yarn lines alternate by parity (src/Cloth.cpp:195-268)."""
    p = dict(HOMO)
    ys_ = [Yarn(p["R"], *y) for y in yarns]
    cloth = Cloth(width, length, height, p["L"], p["R"], ys_, p["kc"], p["kf"], p["df"], p["mu"], S,
                  p["handle_stiffness"], pattern, InitPose.Upright)
    env = Environment(cloth, p["G"], wind)
    cloth.set_handles(handles if handles is not None else [(0, 0), (width - 1, 0)])
    phy = PhysicsCloth(env, device=device)
    states = _run(cloth, phy, steps, h, obj_dir)
    w = env.wind
    physical = dict(Gravity=float(env.G[2]), Yarn1_rho=yarns[0][0], Yarn2_rho=yarns[1][0], R=p["R"], L=p["L"],
                    Yarn1_Y=yarns[0][1], Yarn2_Y=yarns[1][1], Yarn1_B=yarns[0][2], Yarn2_B=yarns[1][2], kc=p["kc"],
                    kf=p["kf"], df=p["df"], mu=p["mu"], S=S, handle_stiff=p["handle_stiffness"],
                    wind_velocity_x=float(w.WindVelocity[0]), wind_velocity_y=float(w.WindVelocity[1]),
                    wind_velocity_z=float(w.WindVelocity[2]), wind_density=float(w.WindDensity),
                    wind_drag=float(w.WindDrag), woven_pattern=int(pattern))
    return _finish(states, cloth, h5_path, physical)


def control_force(width: int, length: int, up: float = 0.002, forward: float = 0.002) -> np.ndarray:
    """SimControl's external force: lift (z) and drag (y) at the four corners
    (the reference's DOF indices 1, 2, 13, 14, 61, 62, 73, 74 of a 5 x 5
    cloth), in node layout [nodes, 5]."""
    f = np.zeros((width * length, 5))
    for n in (0, width - 1, width * (length - 1), width * length - 1):
        f[n, 1] = forward
        f[n, 2] = up
    return f


def sim_control(width: int = 5, length: int = 5, steps: int = 100, h: float = 0.001, force_steps: int = 6,
                ext_force: Optional[np.ndarray] = None, h5_path: Optional[str] = None, obj_dir: Optional[str] = None,
                height: float = 5.0, device: int = 0) -> Dict[str, np.ndarray]:
    """SimControl: a free flat cloth (Y = 5e4, B = 1e-5) lifted and dragged at
    its corners for the first `force_steps` steps (the reference zeroes the
    force once i > 5)."""
    p = dict(HOMO, Y=50000.0, B=0.00001)
    yarn = Yarn(p["R"], p["rho"], p["Y"], p["B"])
    cloth = Cloth(width, length, height, p["L"], p["R"], [yarn], p["kc"], p["kf"], p["df"], p["mu"], p["S"],
                  p["handle_stiffness"], WovenPattern.Plain, InitPose.Flat)
    env = Environment(cloth, p["G"], Wind((0.0, 0.0, 0.0), 2.0, 0.5))
    cloth.set_handles([])
    phy = PhysicsCloth(env, device=device)
    f = control_force(width, length) if ext_force is None else np.ascontiguousarray(ext_force, np.float64)
    states = _run(cloth, phy, steps, h, obj_dir, ext=f, force_steps=force_steps)
    return _finish(states, cloth, h5_path, _physical_homo(env, p, WovenPattern.Plain))


def sim_collision(obstacle_x: np.ndarray, obstacle_faces: np.ndarray, width: int = 5, length: int = 5,
                  steps: int = 20, h: float = 0.001, height: float = 0.025, thickness: float = 0.0005,
                  handles=None, wind=Wind((0.0, 5.0, 0.0), 2.0, 0.5), h5_path: Optional[str] = None,
                  obj_dir: Optional[str] = None, device: int = 0) -> Dict[str, np.ndarray]:
    """SimCollision: an upright cloth hanging in wind against obstacle
    meshes, each step followed by the impact-zone response
    (collision_response(0.1)). The reference loads its table and ground from
    ./obs/wall.obj and ./obs/ground.obj; here the merged obstacle mesh is
    passed in (vertices [V, 3], faces [F, 3])."""
    p = dict(HOMO)
    yarn = Yarn(p["R"], p["rho"], p["Y"], p["B"])
    cloth = Cloth(width, length, height, p["L"], p["R"], [yarn], p["kc"], p["kf"], p["df"], p["mu"], p["S"],
                  p["handle_stiffness"], WovenPattern.Plain, InitPose.Upright)
    env = Environment(cloth, p["G"], wind)
    cloth.set_handles(handles if handles is not None else [(0, 0), (width - 1, 0)])
    phy = PhysicsCloth(env, device=device)
    col = Collision(cloth, obstacle_x, obstacle_faces, thickness=thickness, h=h, device=device)
    try:
        states = _run(cloth, phy, steps, h, obj_dir, collision=col)
    finally:
        col.close()
    return _finish(states, cloth, h5_path, _physical_homo(env, p, WovenPattern.Plain))


class DropOnSphere:
    """The collision benchmark scene: a width x width plain cloth lying flat
    `drop` metres above the top of a fixed icosphere (radius, `levels`
    subdivisions: 20 * 4^levels faces; 3 gives 1,280), centred over it, free
    (no handles), falling under gravity with self-collision and cloth-sphere
    collision every step (SimStep with a Collision, src/TrainHelper.cpp:
    99-149: step, then collision_response(damp)), step size h. Material: the
    benchmark configurations' (BENCH: R = 0.1 mm), collision thickness = the
    yarn radius unless given.

    damp is the velocity update after a projection, v += damp (x - x_before)
    / h. The reference's SimStep passes 0.1: a node projected out of the
    obstacle keeps 90 % of its approach speed, the next step drives it back
    in, and a free-falling cloth landing on a sphere folds onto itself within
    about 20 steps of contact (the fold's zones then move nodes by
    millimetres per projection and speeds grow without bound). With 1.0 the
    projection is inelastic (the velocity follows the projected position)
    and the cloth drapes; that is the default here.

    run(steps) advances the scene and times each step's parts; `frames`
    records (x_prev, x) -- the detection's input -- at chosen steps.

    tune=True times the step schedules once from the initial state
    (ClothBatch.autotune, state restored; every schedule gives the same
    bits) and keeps the fastest: for one cloth this is usually the
    persistent PCG, one launch per solve."""

    def __init__(self, width: int = 50, radius: float = 0.03, levels: int = 3, drop: float = 0.05,
                 h: float = 5e-4, thickness: Optional[float] = None, params: Optional[Dict] = None, device: int = 0,
                 ext_force=None, damp: float = 1.0, tune: bool = True):
        p = dict(BENCH, **(params or {}))
        self.p, self.h, self.width, self.damp = p, float(h), int(width), float(damp)
        self.thickness = p["R"] if thickness is None else float(thickness)
        half = 0.5 * (width - 1) * p["L"]
        self.center = np.array([half, half, 0.0])
        self.radius = float(radius)
        self.sphere_x, self.sphere_f = icosphere(radius, levels, self.center)
        yarn = Yarn(p["R"], p["rho"], p["Y"], p["B"])
        self.cloth = Cloth(width, width, radius + drop, p["L"], p["R"], [yarn], p["kc"], p["kf"], p["df"], p["mu"],
                           p["S"], p["handle_stiffness"], WovenPattern.Plain, InitPose.Flat)
        self.env = Environment(self.cloth, p["G"], Wind())
        self.cloth.set_handles([])
        self.phy = PhysicsCloth(self.env, device=device)
        self.col = Collision(self.cloth, self.sphere_x, self.sphere_f, thickness=self.thickness, h=self.h,
                             device=device)
        self.ext = ext_force
        self.schedule = self.phy.batch.autotune(self.h, steps=3) if tune else None
        self.steps_done = 0
        self.frames = {}
        self.log = []

    def close(self):
        self.col.close()

    def step(self, record_frame: bool = False) -> Dict:
        """One SimStep with collision; returns its timings and response
        counters."""
        b = self.phy.batch
        t0 = time.perf_counter()
        before = b.get_state()
        stats = b.step(self.h, self.ext)
        ok = bool(stats[0]["ok"])
        st = b.get_state()
        t1 = time.perf_counter()
        info = dict(step=self.steps_done, ok=ok, cg_iterations=stats[0]["cg_iterations"])
        if ok:
            if record_frame:
                self.frames[self.steps_done] = (before["LPos"].copy(), st["LPos"].copy())
            changed = self.col.collision_response(self.damp, st["LPos"], before["LPos"], st["LVel"])
            r = self.col.last
            t2 = time.perf_counter()
            if changed:
                # no handles: every node's fixed position follows it
                b.set_state(LPos=r["x"], LPosFix=r["x"].copy(), LVel=r["v"], EPos=st["EPos"],
                            EPosBar=st["EPosBar"], EVel=st["EVel"])
            t3 = time.perf_counter()
            info.update(changed=bool(changed), rounds=r["rounds"], zones=r["zones"], impacts=int(r["impacts"]),
                        converged=bool(r["converged"]), zone_overflow=bool(r["zone_overflow"]),
                        step_ms=1e3 * (t1 - t0), collision_ms=1e3 * (t2 - t1), writeback_ms=1e3 * (t3 - t2))
        self.steps_done += 1
        self.log.append(info)
        return info

    def run(self, steps: int, frames: Sequence[int] = ()) -> List[Dict]:
        fr = set(int(s) for s in frames)
        out = []
        for _ in range(steps):
            info = self.step(record_frame=self.steps_done in fr)
            out.append(info)
            if not info["ok"]:
                break
        return out

    def state(self) -> Dict[str, np.ndarray]:
        return self.phy.batch.get_state()


def centroid_target(seed: int, start: np.ndarray, lo: float = 0.10, hi: float = 0.30) -> np.ndarray:
    """A seeded target point lo..hi metres from `start` (a centroid), in a
    random direction of the upper half-space (z >= 0), so a cloth above an
    obstacle is steered away from it."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=3)
    d[2] = abs(d[2])
    d /= np.linalg.norm(d)
    return np.asarray(start, float) + (lo + (hi - lo) * rng.random()) * d


class CentroidControl:
    """The control problem of the collision benchmark: per-node external
    forces f_s [nodes, 3] at every step s < steps (the state of a cloth's
    SimStep with ext_force, src/TrainHelper.cpp:56-97) minimising
        L = |centroid(LPos after the last step) - target|^2,
    the mass-centre loss of the reference's control learning
    (src/TrainControl.h:192-203) on a per-node force instead of a network.
    gradient() runs the rollout forward (checkpoints every `checkpoint_every`
    steps) and backward through ys_adjoint_step, giving dL/df for all
    nodes x steps at once; optimise() takes Adam steps on the forces.

    The scene is DropOnSphere's cloth before it reaches the sphere (it
    falls 50 mm; contact comes at step 201 of h = 5e-4), so the controlled
    window has no impacts; collide() checks that with the scene's detection."""

    def __init__(self, scene: "DropOnSphere", steps: int = 100, target: Optional[np.ndarray] = None, seed: int = 0,
                 checkpoint_every: int = 20, mode: str = "exact", copies: int = 128):
        from .learn import CheckpointedRollout  # noqa: F401 (import check)
        self.scene, self.steps, self.k, self.mode, self.copies = scene, int(steps), int(checkpoint_every), mode, copies
        b = scene.phy.batch
        self.state0 = b.get_state()
        self.n = b.total_nodes
        c0 = self.state0["LPos"].mean(axis=0)
        self.target = centroid_target(seed, c0) if target is None else np.asarray(target, float)
        self.forces = np.zeros((self.steps, self.n, 3))

    def _ext(self, forces):
        out = []
        for s in range(self.steps):
            e = np.zeros((self.n, 5))
            e[:, :3] = forces[s]
            out.append(e)
        return out

    def loss_and_traj(self, forces=None):
        from .learn import CheckpointedRollout
        f = self.forces if forces is None else forces
        ro = CheckpointedRollout(self.scene.phy.batch, self.state0, self.steps, self.scene.h, self._ext(f),
                                 self.mode, self.k, copies=self.copies)
        traj = ro.forward()
        c = traj["LPos"][-1].mean(axis=0)
        return float(((c - self.target) ** 2).sum()), traj, ro

    def gradient(self, forces=None):
        """(L, dL/df [steps, nodes, 3], trajectory)."""
        L, traj, ro = self.loss_and_traj(forces)
        c = traj["LPos"][-1].mean(axis=0)
        g = {k: np.zeros_like(v) for k, v in traj.items()}
        g["LPos"][-1] = np.broadcast_to(2.0 * (c - self.target) / self.n, g["LPos"][-1].shape)
        out = ro.backward(g, want_ext=True)
        self.scene.phy.batch.set_state(**self.state0)
        return L, out["ext"][:, :, :3], traj

    def optimise(self, iterations: int = 20, lr: float = 2e-5) -> List[float]:
        """Adam on the forces (lr in newtons); returns the loss before each
        iteration and after the last."""
        m = np.zeros_like(self.forces)
        v = np.zeros_like(self.forces)
        hist = []
        for it in range(1, iterations + 1):
            L, g, _ = self.gradient()
            hist.append(L)
            m = 0.9 * m + 0.1 * g
            v = 0.999 * v + 0.001 * g * g
            mh, vh = m / (1 - 0.9 ** it), v / (1 - 0.999 ** it)
            self.forces -= lr * mh / (np.sqrt(vh) + 1e-30)
        hist.append(self.loss_and_traj()[0])
        self.scene.phy.batch.set_state(**self.state0)
        return hist

    def collide(self, traj) -> Dict[str, int]:
        """Impacts the scene's detection finds along the trajectory: with the
        sphere, and of the cloth with itself. The controlled rollout has no
        collision response: the cloth starts 5 cm above the sphere, and the
        forces that move its centroid 10-30 cm in 50 ms (about 100 m/s^2, more
        than the benchmark yarns' stretch stiffness carries) can fold its
        lighter edges onto it."""
        col = self.scene.col.collider
        out = dict(sphere=0, self=0)
        prev = self.state0["LPos"]
        ox = self.scene.sphere_x
        for x in traj["LPos"]:
            col.set_positions(x, prev, ox, ox)
            if len(col.pairs()):
                nodes = col.impacts()["nodes"]
                obs = (nodes < 0).any(axis=1)
                out["sphere"] += int(obs.sum())
                out["self"] += int((~obs).sum())
            prev = x
        return out


# ------------------------------------------------------------ training driver
# train_heter_full's starting values and ranges (src/TrainHeter.h:50-100;
# ranges are (upper, lower) pairs as the reference passes them)
HETER_INIT = dict(rho_1=0.00225, rho_2=0.00245, Y_1=335000.0, Y_2=145000.0, B_1=0.000125, B_2=0.0001, S=600.0,
                  mu=0.7)
HETER_RANGES = dict(rho_1=(0.003, 0.001), rho_2=(0.003, 0.001), Y_1=(800000.0, 0.0), Y_2=(300000.0, 0.0),
                    B_1=(0.00018, 0.00005), B_2=(0.00018, 0.00005), S=(1200.0, 0.0), mu=(1.0, 0.0))
# per-parameter SGD learning rates (src/TrainHeter.h:131-150)
HETER_LR = dict(rho_1=0.1, rho_2=1e-4, Y_1=12e16, Y_2=7e16, B_1=0.219, B_2=0.145, S=19e10, mu=14e9)


def train_heter_full(data_path: str, epoch: int = 1, iters: int = 1, batch: int = 1, sample: int = 10,
                     steps: Optional[int] = None, all_steps: bool = True, random: bool = False,
                     save_path: Optional[str] = None, init: Optional[Dict[str, float]] = None,
                     ranges: Optional[Dict[str, Tuple[float, float]]] = None, lr: Optional[Dict[str, float]] = None,
                     handles=None, h: float = 1e-3, mode: str = "reference", seed: int = 0,
                     wordy: bool = False) -> Dict:
    """train_heter_full (src/TrainHeter.h:11-306): learns the eight
    parameters of a two-yarn cloth (rho, Y, B of each yarn type, S, mu,
    through constraint_para) from a trajectory file SimHeter wrote
    (data_path, the reference's HDF5 layout). Per iteration: `batch` samples
    of `sample` consecutive states (sequential, or drawn at random), each
    rolled out for sample - 1 steps from its first state on the GPU with the
    forward-mode Jacobian; loss = sum over steps of mean |x - x^|^2 + mean
    |e - e^|^2, divided by (successful steps - 1); SGD with the reference's
    per-parameter learning rates, skipped when a gradient is not finite.
    samples = steps // sample; iterations = (iters if random else samples //
    batch) when all_steps, else iters. handles default to the two top
    corners (the reference hard-codes (0, 0), (16, 0) for its 17 x 17
    cloth). Returns dict(loss=[...], params={name: [...]}, grad={name:
    [...]}) per training step (constrained parameters after the step; the
    raw parameters' gradients) and, with save_path, writes loss and
    parameters as SaveTrainProc does (datasets Loss, rho1, rho2, Y1, Y2, B1,
    B2, S, mu; src/Saver.cpp:93-150)."""
    import torch
    from .learn import YarnSimNetHeter, constraint_para, invert_constraint_para, rollout_with_jacobian

    size, phy = _h5.cloth_property_loader_heter(data_path)
    W, L = int(size["width"]), int(size["length"])
    if steps is None:
        steps = int(len(_h5.read(data_path)["/Steps/Position/Node 0 0/LPOS"]))
    samples = steps // sample
    iteration = (iters if random else samples // batch) if all_steps else iters
    ranges = dict(HETER_RANGES, **(ranges or {}))
    init = dict(HETER_INIT, **(init or {}))
    lr = dict(HETER_LR, **(lr or {}))
    raw = {k: invert_constraint_para(v, *ranges[k]) for k, v in init.items()}
    handles = handles if handles is not None else [(0, 0), (W - 1, 0)]
    net = YarnSimNetHeter(W, L, float(phy["R"]), float(phy["L"]), raw, ranges, handles, h=h, kf=float(phy["kf"]),
                          df=float(phy["df"]), kc=float(phy["kc"]), handle_stiffness=float(phy["handle_stiff"]),
                          gravity=float(phy["Gravity"]),
                          wind_vel=(phy["wind_velocity_x"], phy["wind_velocity_y"], phy["wind_velocity_z"]),
                          wind_density=float(phy["wind_density"]), wind_drag=float(phy["wind_drag"]),
                          woven_pattern=int(phy["woven_pattern"]), mode=mode)
    names = ("rho_1", "rho_2", "Y_1", "Y_2", "B_1", "B_2", "S", "mu")
    opt = torch.optim.SGD([{"params": [getattr(net, n)], "lr": lr[n]} for n in names], lr=1e5)
    rng = np.random.default_rng(seed)
    hist = {"loss": [], "params": {n: [] for n in names}, "grad": {n: [] for n in names}}
    for epc in range(epoch):
        for it in range(iteration):
            opt.zero_grad()
            theta = net.theta()
            th = theta.detach().cpu().numpy()
            gtheta = np.zeros(8)
            loss, success = 0.0, 0
            for bch in range(batch):
                choice = int(rng.integers(0, samples)) if random else it * batch + bch
                data = _h5.data_loader(data_path, choice * sample, choice * sample + sample)
                state0 = {k: data[k][0] for k in FULL}
                tx, te, Jx, Je, stats = rollout_with_jacobian(net.template, th, state0, sample - 1, h, mode)
                n_ok = next((s for s, st in enumerate(stats) if not st[0]["ok"]), sample - 1)
                for s in range(n_ok):
                    dx = tx[s] - data["LPos"][s + 1]
                    de = te[s] - data["EPos"][s + 1]
                    loss += float((dx * dx).sum(-1).mean() + (de * de).sum(-1).mean())
                    gtheta += np.einsum("nc,ncp->p", 2.0 * dx / len(dx), Jx[s])
                    gtheta += np.einsum("nc,ncp->p", 2.0 * de / len(de), Je[s])
                success += n_ok
            div = max(success - 1, 1)
            loss /= div
            theta.backward(torch.as_tensor(gtheta / div, dtype=theta.dtype))
            for n in names:
                hist["grad"][n].append(float(getattr(net, n).grad[0]))
            if all(torch.isfinite(getattr(net, n).grad).all() for n in names):
                opt.step()
            hist["loss"].append(loss)
            for n in names:
                hist["params"][n].append(float(constraint_para(getattr(net, n), *ranges[n])))
            if wordy:
                print("epoch %d batch %d loss %.6e" % (epc, it, loss))
    if save_path:
        T = len(hist["loss"])
        ds = {"/Loss": np.array(hist["loss"]).reshape(T, 1)}
        for n in names:
            ds["/" + n.replace("_", "")] = np.array(hist["params"][n]).reshape(T, 1)
        _h5.write(save_path, ds)
    return hist
