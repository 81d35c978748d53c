#!/usr/bin/env python
"""Batched yarn-level cloth stepping on GB300: one JSON line.

Workload (the batched-cloth benchmark): 256 plain-weave cloths with side
lengths drawn uniformly from 5..50 crossings (seeded), hanging from their two
top corners, per-yarn-line material drawn within +-20% of rho = 1e-3 kg/m,
Y = 1e3, B = 1e-5 (the reference's Yarn(R, rho, Y, B) arguments, R = 0.1 mm,
L = 1 mm), S = 1e-4 and mu = 0.3 within +-20% per cloth, gravity 9.8, seeded
sinusoidal wind (pressure amplitude 0..2 N/m^2 -> speed sqrt(p / rho_air),
period 0.2..1 s), h = 1e-3 s, FP64 Jacobi-PCG to relative residual 1e-10.
A step advances every cloth of the batch by h. Inputs are synthetic.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores (the C
restatement in oracle/, as the reference's own LibTorch build does not run on
the GPU host) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

H = 1e-3
TOL = 1e-10
N_CLOTHS = 256
WIND_RHO = 1.0
WIND_DRAG = 0.5


# ---------------------------------------------------------------- workload
def workload(seed: int, n_cloths: int = N_CLOTHS):
    """Seeded cloth descriptions (dicts of ClothSpec fields) and wind table."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(5, 51, size=n_cloths)
    base = np.array([1e-3, 1e3, 1e-5])
    specs, wind = [], []
    for s in sides:
        W = Hh = int(s)
        j = lambda n: base * (1.0 + 0.2 * (2.0 * rng.random((n, 3)) - 1.0))
        specs.append(dict(width=W, length=Hh, warp=j(Hh), weft=j(W), height=0.05, L=1e-3, R=1e-4, pose=0, weave=0,
                          kc=1.0, kf=1000.0, df=1000.0, mu=0.3 * (1 + 0.2 * (2 * rng.random() - 1)),
                          S=1e-4 * (1 + 0.2 * (2 * rng.random() - 1)), handle_stiffness=1e4, G=(0.0, 0.0, 9.8),
                          wind_vel=(0.0, 0.0, 0.0), wind_density=WIND_RHO, wind_drag=WIND_DRAG,
                          handles=[(0, 0), (W - 1, 0)]))
        wind.append((2.0 * rng.random(), 0.2 + 0.8 * rng.random(), 2 * math.pi * rng.random()))
    return specs, np.array(wind)


def rank_seed(seed: int, rank: int) -> int:
    """Each rank steps its own independent batch: the data path shards by
    cloth with no exchange (weak scaling)."""
    return seed + 1000 * rank


def max_over_ranks(value: float, dist, device: str) -> float:
    """The job's time is its slowest rank's (the only collective besides the
    barriers)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def wind_at(wind, step):
    """[n, 3] wind velocity at time step*h: along +y (normal to the hanging cloth)."""
    t = step * H
    amp = np.sqrt(wind[:, 0] / WIND_RHO)
    v = np.zeros((len(wind), 3))
    v[:, 1] = amp * np.sin(2 * math.pi * t / wind[:, 1] + wind[:, 2])
    return v


# ---------------------------------------------------------------- helpers
class NvmlSampler:
    """SM clock, its maximum and the active clock-event reasons, read through
    NVML (read-only queries) by a thread every `period` seconds."""
    CLOCK_SM = 1  # nvmlClockType_t NVML_CLOCK_SM
    REASONS = ((0x8, "hw_slowdown"), (0x40, "hw_thermal_slowdown"), (0x20, "sw_thermal_slowdown"),
               (0x4, "sw_power_cap"))

    def __init__(self, index=0, period=0.002):
        import ctypes
        self.c = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.lib = lib
        self.h = ctypes.c_void_p()
        bus = None
        try:
            import torch
            p = torch.cuda.get_device_properties(index)
            bus = "%08x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        except Exception:
            bus = None
        rc = lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h)) if bus else 1
        if rc != 0 and lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle for device %d" % index)
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(self.h, self.CLOCK_SM, ctypes.byref(mx)) != 0:
            raise RuntimeError("nvmlDeviceGetMaxClockInfo failed")
        self.max_mhz = float(mx.value)
        self.period = period
        self.sm, self.bits = [], 0
        self.stop = threading.Event()

    def _sample(self):
        c = self.c
        clk, r = c.c_uint(), c.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, self.CLOCK_SM, c.byref(clk)) == 0:
            self.sm.append(float(clk.value))
        if self.reasons_fn(self.h, c.byref(r)) == 0:
            self.bits |= r.value

    def _run(self):
        while not self.stop.is_set():
            self._sample()
            time.sleep(self.period)

    def __enter__(self):
        self._sample()
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=5)
        self._sample()

    def summary(self):
        return {"sm_mhz": statistics.median(self.sm) if self.sm else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(n for b, n in self.REASONS if self.bits & b), "samples": len(self.sm),
                "source": "nvml, every %g ms" % (self.period * 1e3)}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.nvml = None

    def __enter__(self):
        # NVML polled every 2 ms when libnvidia-ml loads: a timed region of a
        # fraction of a second still gets dozens of samples
        try:
            self.nvml = NvmlSampler(self.index).__enter__()
            return self
        except Exception:
            self.nvml = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.nvml is not None:
            self.nvml.__exit__(*a)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            return self.nvml.summary()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def measure_fp64_peak(torch):
    """cuBLAS DGEMM throughput (TFLOP/s): the FP64 ceiling of this GPU."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for _ in range(3):
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


# FP64 flops per node of one assembly launch, counted by ncu on the first
# 128 cloths of this workload (seed 0, 122,504 nodes; bench.py --cloths 128
# --schedule launch): 2 x DFMA + DADD + DMUL thread instructions of the
# launch (sm__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum)
# divided by the batch's nodes. The counts depend on the state only through
# branch outcomes and on the sizes through the share of boundary nodes, so
# they carry over to the 256-cloth batch to within a few per cent.
ASSEMBLY_FP64_FLOPS_PER_NODE = {"geom": 624.5, "edges": 3379.5, "bends": 2142.3, "faces": 379.4,
                                "gather": 1467.0, "shear": 3489.6, "finalize": 801.5}
# DRAM bytes (read + write) of the persistent solve per pass over the rows
# (not captured: the tuner does not pick the persistent PCG for this batch)
PERSIST_DRAM_BYTES_PER_ROW_PASS = None


def schedule_name(c):
    """'graph|launch/phases-every-E/producers-P' or 'graph|launch/persistent-TxC/producers-P'."""
    g = "graph" if c["graphs"] else "launch"
    if c["pcg"] == "persistent":
        return "%s/persistent-%dx%d/producers-%d" % (g, c["pcg_threads"], c["pcg_cluster"], c["producer_threads"])
    return "%s/phases-every-%d/producers-%d" % (g, c["check_every"], c["producer_threads"])


def assembly_roof(prof, n, steps, fp64_peak):
    """The assembly kernels against the FP64 ceiling: flops per node (counted
    by ncu) x nodes / their event time per step."""
    kinds = ("geom", "edges", "bends", "faces", "gather", "shear", "finalize")
    ms = sum(prof["ms"].get(k, 0.0) for k in kinds) / steps
    out = {"kernels": list(kinds), "ms_per_step": ms, "bound": "fp64", "unit": "TFLOP/s",
           "peak": fp64_peak, "peak_source": "cuBLAS DGEMM measured in this run"}
    if ASSEMBLY_FP64_FLOPS_PER_NODE and ms > 0:
        fl = sum(ASSEMBLY_FP64_FLOPS_PER_NODE.values()) * n
        out.update(flops_per_node=ASSEMBLY_FP64_FLOPS_PER_NODE, achieved=fl / (ms * 1e-3) / 1e12)
        out["frac"] = out["achieved"] / fp64_peak
    return out


# ---------------------------------------------------------------- CPU arm
def _cpu_worker(args):
    specs, idx, warm, steps, seed = args
    from oracle.oracle import ClothSpec, OracleCloth
    _, wind = workload(seed)
    cloths = [OracleCloth(ClothSpec(**specs[i])) for i in idx]
    t0 = 0.0
    for s in range(warm + steps):
        if s == warm:
            t0 = time.perf_counter()
        wv = wind_at(wind, s)
        for c, i in zip(cloths, idx):
            c.set_wind(wv[i])
            c.step(H, cg_tol=TOL)
    return time.perf_counter() - t0


def cpu_sample(specs, seed, target_nodes, steps, cores, warm=0):
    """Times the oracle on a bounded sample of the workload's cloths; returns
    (batch steps/s extrapolated to the full batch, description)."""
    import multiprocessing as mp
    from oracle.oracle import build as build_oracle
    build_oracle()
    order = np.random.default_rng(seed + 99).permutation(len(specs))
    idx, nodes = [], 0
    for i in order:
        if nodes >= target_nodes:
            break
        idx.append(int(i))
        nodes += specs[i]["width"] * specs[i]["length"]
    total = sum(s["width"] * s["length"] for s in specs)
    # balance the sample over the workers by node count
    shards = [[] for _ in range(cores)]
    load = [0] * cores
    for i in sorted(idx, key=lambda i: -specs[i]["width"] * specs[i]["length"]):
        k = int(np.argmin(load))
        shards[k].append(i)
        load[k] += specs[i]["width"] * specs[i]["length"]
    shards = [s for s in shards if s]
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(shards)) as pool:
        times = pool.map(_cpu_worker, [(specs, s, warm, steps, seed) for s in shards])
    wall = max(times)  # each worker times its own stepping loop (process start-up excluded)
    per_step = wall / steps
    value = (nodes / total) / per_step
    desc = "%d of %d cloths (%d of %d nodes), %d step(s) after %d untimed, %d processes; slowest worker's loop time" % (
        len(idx), len(specs), nodes, total, steps, warm, len(shards))
    return value, desc, wall


def precond_compare(ys, dev, repeats=6):
    """Solve time and iterations of the learned preconditioner against
    Jacobi-PCG on the same assembled systems, both to the same 1e-10 relative
    residual: one 100 x 100 cloth and 64 cloths of 40 x 40 (plain weave,
    material within +-20 %, hanging from two corners), after a few steps."""
    import time
    net = ys.LearnedPreconditioner.pretrained(device=dev)
    out = {}
    for name, sizes in [("cloth_100x100", [100]), ("batch_64x40x40", [40] * 64)]:
        rng = np.random.default_rng(3)
        base = np.array([1e-3, 1e3, 1e-5])
        j = lambda m: base * (1.0 + 0.2 * (2.0 * rng.random((m, 3)) - 1.0))
        b = ys.ClothBatch([ys.ClothSpec(width=W, length=W, warp=j(W), weft=j(W), height=0.05, L=1e-3, R=1e-4,
                                        pose=0, weave=0, mu=0.3, S=1e-4, G=(0, 0, 9.8),
                                        handles=[(0, 0), (W - 1, 0)]) for W in sizes], device=dev)
        for _ in range(4):
            b.step(H, tol=TOL)
        res = {"jacobi": [], "learned": []}
        for _ in range(repeats):
            b.assemble(H)
            for kind in ("jacobi", "learned"):
                b.set_preconditioner(kind, net if kind == "learned" else None)
                b.synchronize()
                t0 = time.perf_counter()
                st = b.solve(tol=TOL)
                b.synchronize()
                ms = (time.perf_counter() - t0) * 1e3
                assert all(x["ok"] and x["cg_error"] <= TOL for x in st)
                res[kind].append((max(x["cg_iterations"] for x in st), ms))
            b.set_preconditioner("jacobi")
            b.step(H, tol=TOL)
        steps = {}
        b.use_graphs(True)  # both arms: one CUDA graph launch per step
        for kind, every in (("jacobi", 1), ("learned_refresh4", 4), ("learned_refresh8", 8)):
            b.set_preconditioner("learned" if kind != "jacobi" else "jacobi", net if kind != "jacobi" else None)
            b.precond_refresh(every)
            for _ in range(2):  # captures the graphs
                b.step(H, tol=TOL)
            ts = []
            for _ in range(8):  # a multiple of the refresh interval: the network's cost is in the mean
                b.synchronize()
                t0 = time.perf_counter()
                b.step(H, tol=TOL)
                b.synchronize()
                ts.append((time.perf_counter() - t0) * 1e3)
            steps[kind] = float(np.mean(ts))
        fb = b.precond_info()["fallbacks"]
        b.close()
        out[name] = {
            "nodes": int(sum(W * W for W in sizes)),
            "jacobi": {"max_iterations": float(np.mean([r[0] for r in res["jacobi"]])),
                       "solve_ms": float(np.median([r[1] for r in res["jacobi"]]))},
            "learned": {"max_iterations": float(np.mean([r[0] for r in res["learned"]])),
                        "solve_ms_with_inference": float(np.median([r[1] for r in res["learned"]])),
                        "fallbacks": fb},
            "step_ms": steps,
            "step_schedule": "one CUDA graph per step, both preconditioners; mean of 8 steps after 2",
            "residual": "both |r| <= 1e-10 |b| (FP64)"}
    net.close()
    return out


def collision_compare(ys, dev, repeats=5):
    """Collision detection and impact-zone response on the GPU collider,
    timed end to end through the Python API with host arrays (tree build on
    the host, uploads, kernels, downloads, the host zone solver): a W x W
    cloth (1 mm spacing) moving 3 mm in one step onto a sphere (radius 30 mm,
    20 480 faces) so its middle passes the top by 1 mm."""
    import time
    out = {}
    for W in (64, 128):
        ox, of = ys.collide.icosphere(0.03, 5)
        u, v = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
        xp = np.zeros((W * W, 3))
        xp[:, 0] = (u.reshape(-1) - (W - 1) / 2) * 1e-3
        xp[:, 1] = (v.reshape(-1) - (W - 1) / 2) * 1e-3
        xp[:, 2] = 0.03 + 2e-3
        x = xp.copy()
        x[:, 2] -= 3e-3
        x += np.random.default_rng(0).normal(0.0, 1e-5, x.shape)
        vel = (x - xp) / H
        c = ys.Collider(W, W, obstacle_faces=of, n_obstacle_nodes=len(ox), thickness=5e-4, device=dev)
        det, resp, back = [], [], []
        for _ in range(repeats):
            t0 = time.perf_counter()
            c.set_positions(x, xp, ox, ox)
            P = c.pairs()
            I = c.impacts()
            det.append((time.perf_counter() - t0) * 1e3)
            t0 = time.perf_counter()
            c.set_positions(x, xp, ox, ox)
            r = c.respond(v=vel, h=H, damp=0.1)
            resp.append((time.perf_counter() - t0) * 1e3)
            t0 = time.perf_counter()
            c.respond_backward(np.ones_like(x), np.ones_like(x))
            back.append((time.perf_counter() - t0) * 1e3)
        c.close()
        out["drop_%dx%d" % (W, W)] = {
            "cloth_faces": 2 * (W - 1) ** 2, "obstacle_faces": int(len(of)), "pairs": int(len(P)),
            "impacts_round0": int(len(I["t"])), "rounds": r["rounds"], "zones": r["zones"],
            "received_impacts": int(r["impacts"]), "converged": r["converged"],
            "detect_ms": float(np.median(det)), "respond_ms": float(np.median(resp)),
            "respond_backward_ms": float(np.median(back))}
    return out


def schedule_compare(ys, dev):
    """One hanging cloth of side 5, 17 and 50 (the configurations' sizes;
    the batched workload's material): the tuner's best phase-PCG and best
    persistent-PCG step times (ms), each over 5 steps from the same state."""
    specs, _ = workload(7, 1)
    out = {}
    for W in (5, 17, 50):
        sp = dict(specs[0], width=W, length=W, warp=specs[0]["warp"][:1].repeat(W, 0),
                  weft=specs[0]["weft"][:1].repeat(W, 0), handles=[(0, 0), (W - 1, 0)])
        b = ys.ClothBatch([ys.ClothSpec(**sp)], device=dev)
        sc = b.autotune(H, tol=TOL, steps=5)
        b.close()
        best = {}
        for c in sc["candidates"]:
            k = c["pcg"]
            if k not in best or c["ms_per_step"] < best[k]["ms_per_step"]:
                best[k] = c
        out["%dx%d" % (W, W)] = {k: {"ms_per_step": v["ms_per_step"], "schedule": schedule_name(v)}
                                 for k, v in best.items()}
    return out


def drop_scene(ys, dev, steps=1000):
    """The collision benchmark scene end to end (DropOnSphere): a 50 x 50
    plain cloth (1 mm spacing, the batched workload's material, R = 0.1 mm,
    collision thickness = R) lying 5 cm above a fixed sphere of radius 3 cm
    (an icosphere of 1,280 faces), free, self-collision and cloth-sphere
    collision every step, h = 5e-4, `steps` steps in FP64 through the public
    API with host arrays: the step (assembly, PCG, update, state download),
    the collision response (detection rounds on the GPU, zones and
    projections on the host) and the write-back of moved nodes."""
    sc = ys.DropOnSphere(width=50, radius=0.03, levels=3, drop=0.05, h=5e-4, device=dev)
    t0 = time.perf_counter()
    log = sc.run(steps)
    wall = time.perf_counter() - t0
    x = sc.state()["LPos"]
    r = np.linalg.norm(x - sc.center, axis=1)
    sc.close()
    ok = [e for e in log if e["ok"]]
    contact = [e["step"] for e in ok if e["impacts"] > 0]
    med = lambda k: float(np.median([e[k] for e in ok])) if ok else None  # noqa: E731
    return {
        "cloth": "50x50 plain, flat, free, R = 0.1 mm; sphere r = 30 mm, 1280 faces; drop 50 mm; h = 5e-4; "
                 "thickness 0.1 mm; inelastic projections (damp 1)",
        "steps": len(log), "all_ok": len(ok) == len(log), "all_converged": all(e["converged"] for e in ok),
        "zone_overflow": any(e["zone_overflow"] for e in ok), "first_contact_step": contact[0] if contact else None,
        "steps_with_impacts": len(contact), "max_rounds": max(e["rounds"] for e in ok) if ok else None,
        "max_zones": max(e["zones"] for e in ok) if ok else None,
        "received_impacts": int(sum(e["impacts"] for e in ok)),
        "ms_per_step": 1e3 * wall / max(len(log), 1),
        "step_schedule": schedule_name(sc.schedule) if sc.schedule else None,
        "median_ms": {"step": med("step_ms"), "collision": med("collision_ms"), "writeback": med("writeback_ms")},
        "contact_median_ms": {"collision": float(np.median([e["collision_ms"] for e in ok if e["impacts"] > 0]))
                              if contact else None},
        "min_distance_to_centre_mm": float(r.min() * 1e3)}


# ---------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cloths", type=int, default=N_CLOTHS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precond", action="store_true", help="skip the learned-vs-Jacobi solve comparison")
    ap.add_argument("--no-collision", action="store_true", help="skip the collision detection / response timing")
    ap.add_argument("--drop-steps", type=int, default=1000,
                    help="steps of the 50x50 drop-onto-sphere scene (0: skip it)")
    ap.add_argument("--profile", action="store_true", help="print the per-kernel table to stderr")
    ap.add_argument("--precond-only", action="store_true",
                    help="run only the learned-vs-Jacobi comparison and print its JSON (a profiling target)")
    ap.add_argument("--schedule", default="auto", choices=["auto", "graph", "launch", "persistent"],
                    help="auto: ys_autotune picks graph or launch-by-launch steps and the PCG schedule; "
                         "graph: one CUDA graph launch per step (conditional PCG loop); launch: kernel by kernel; "
                         "persistent: kernel by kernel with the persistent PCG (512-thread CTAs, the smallest "
                         "cluster that holds the largest cloth)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    seed = rank_seed(args.seed, rank)  # each rank steps its own batch (weak scaling)
    specs, wind = workload(seed, args.cloths)
    total_nodes = sum(s["width"] * s["length"] for s in specs)
    config = {"workload": "batched hanging plain-weave cloths, sides U{5..50}, seeded material and wind",
              "cloths_per_gpu": args.cloths, "nodes_per_gpu": int(total_nodes), "h": H, "pcg_rtol": TOL,
              "precision": "fp64", "seed": args.seed,
              "l2": "working set (A alone %.0f MB) exceeds the 129 MB L2; no flush between steps" %
                    (159 * 8 * total_nodes / 1e6)}
    metric = "batch steps/s (%d cloths advanced by h per step)" % args.cloths

    if args.impl == "reference":
        if rank != 0:
            return 0
        cores = os.cpu_count() or 1
        steps = max(1, args.steps)
        value, desc, wall = cpu_sample(specs, seed, target_nodes=total_nodes, steps=steps, cores=cores,
                                       warm=max(0, args.warmup))
        line = {"impl": "reference", "metric": metric, "value": value, "unit": "steps/s", "n_gpus": 0,
                "steps": steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port",
                                 "sample": desc},
                "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    import importlib
    ys = importlib.import_module("fine-grained-differentiable-physics-a-yarn-level-model-for-fabrics_gb300")
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    dev = local_rank
    torch.cuda.set_device(dev)
    if args.precond_only:
        print(json.dumps({"precond": precond_compare(ys, dev)}))
        return 0

    batch = ys.ClothBatch([ys.ClothSpec(**s) for s in specs], device=dev)
    if args.schedule == "auto":
        batch.set_winds(wind_at(wind, 0))
        sched = batch.autotune(H, tol=TOL, steps=3)
        config["schedule"] = {"chosen_by": "ys_autotune", "graph": sched["graphs"],
                              "check_every": sched["check_every"], "pcg": sched["pcg"]}
        config["schedule"]["producer_threads"] = sched["producer_threads"]
        if sched["pcg"] == "persistent":
            config["schedule"].update(pcg_threads=sched["pcg_threads"], pcg_cluster=sched["pcg_cluster"])
        config["schedule"]["timed_ms_per_step"] = {schedule_name(c): round(c["ms_per_step"], 4)
                                                   for c in sched["candidates"]}
    elif args.schedule == "persistent":
        big = max(s["width"] * s["length"] for s in specs)
        cl = 1
        while 512 * cl < big:
            cl *= 2
        batch.set_pcg_schedule(True, 512, cl)
        config["schedule"] = {"chosen_by": "flag", "graph": False, "pcg": "persistent", "pcg_threads": 512,
                              "pcg_cluster": cl}
    else:
        batch.use_graphs(args.schedule == "graph")
        config["schedule"] = {"chosen_by": "flag", "graph": args.schedule == "graph", "check_every": 16,
                              "pcg": "phases"}

    def barrier():
        if dist is not None:
            dist.barrier()

    step_no = 0
    iters = []

    def do_step():
        nonlocal step_no
        batch.set_winds(wind_at(wind, step_no))
        st = batch.step(H, tol=TOL)
        step_no += 1
        return st

    for _ in range(args.warmup):
        st = do_step()
    assert all(s["ok"] for s in st), "warm-up step failed"
    torch.cuda.synchronize()
    batch.profile_read(reset=True)

    # ---- timed region: device-resident state
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record()
        for _ in range(args.steps):
            st = do_step()
            iters.append(st.max_iterations)
        e1.record()
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = batch.profile_read(reset=True)["total_launches"]
    ok = st.all_ok
    if dist is not None:
        ms = max_over_ranks(ms, dist, "cuda")
    ms_per_step = ms / args.steps
    value = world * args.steps / (ms / 1e3)

    # ---- end to end through the public API with host buffers
    host = {k: torch.zeros((total_nodes, 3 if k.startswith("L") else 2), dtype=torch.float64).pin_memory()
            for k in ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")}
    hn = {k: v.numpy() for k, v in host.items()}
    batch.get_state(out=hn)
    e2e_steps = max(3, args.steps // 2)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.set_state(**hn)
        do_step()
        batch.get_state(out=hn)
    torch.cuda.synchronize()
    barrier()
    e2e_s = time.perf_counter() - t0
    if dist is not None:
        e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    state_bytes = total_nodes * 15 * 8
    e2e = {"value": world * e2e_steps / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": state_bytes + 24 * args.cloths,
           "d2h_bytes_per_step": state_bytes}

    # ---- per-kernel profile (a second pass of the same steps, events per launch)
    sizes = np.array([s["width"] * s["length"] for s in specs])
    node_iters = 0  # rows the SpMV launches processed: a cloth runs iters + 1 of them
    batch.profile(True)
    prof_steps = max(3, args.steps // 4)
    for _ in range(prof_steps):
        st = do_step()
        node_iters += int(sum(n * (x["cg_iterations"] + (0 if x["hit_maxiter"] else 1)) for n, x in zip(sizes, st)))
    batch.profile(False)
    prof = batch.profile_read(reset=True)
    tot_ms = sum(prof["ms"].values())
    share = {k: v / tot_ms for k, v in prof["ms"].items() if v > 0}
    dominant = max(prof["ms"], key=lambda k: prof["ms"][k])
    # algorithmic bytes / flops per launch of the main kernels
    n = total_nodes
    alg = {
        # 159 coefficients + own p read + q write per node
        "spmv": dict(bytes=n * (159 * 8 + 5 * 8 + 5 * 8), flops=n * (2 * 159 + 10)),
        # x, p, r, q, dinv read; x, r written
        "axpy": dict(bytes=n * (5 * 5 * 8 + 2 * 5 * 8), flops=n * 5 * 8),
        "dir": dict(bytes=n * (3 * 5 * 8 + 5 * 8), flops=n * 5 * 3),
        # the persistent solve per iteration: the 159 coefficients stream from
        # HBM, the vectors stay on chip (b, Dinv read and x written once per
        # solve, counted per pass over the rows below); the phase kernels' flops
        "pcg_persist": dict(bytes=n * 159 * 8, flops=n * (2 * 159 + 10 + 5 * 8 + 5 * 3)),
    }
    precond = None
    if rank == 0 and not args.no_precond:
        # the learned preconditioner on this workload itself, after the runs
        # above, in the schedule they used (the state keeps advancing)
        net = ys.LearnedPreconditioner.pretrained(device=dev)
        on_workload = {}
        for kind in ("jacobi", "learned_refresh4", "learned_refresh8"):
            if kind != "jacobi":
                batch.set_preconditioner("learned", net)
                batch.precond_refresh(int(kind[-1]))
            for _ in range(2):
                do_step()
            ts, its = [], []
            for _ in range(8):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                st = do_step()
                torch.cuda.synchronize()
                ts.append((time.perf_counter() - t0) * 1e3)
                assert all(x["ok"] and x["cg_error"] <= TOL for x in st)
                its.append(max(x["cg_iterations"] for x in st))
            # mean over 8 steps: the network's evaluations (every 4 or 8 steps) are in it
            on_workload[kind] = {"step_ms": float(np.mean(ts)), "max_iterations": float(np.mean(its))}
        on_workload["fallbacks"] = batch.precond_info()["fallbacks"]
        batch.set_preconditioner("jacobi")
        net.close()
        precond = precond_compare(ys, dev)
        precond["bench_workload"] = on_workload
    collision = None
    if rank == 0 and not args.no_collision:
        collision = collision_compare(ys, dev)
    sched_cmp = None
    if rank == 0 and args.schedule == "auto":
        sched_cmp = schedule_compare(ys, dev)
    drop = None
    if rank == 0 and args.drop_steps > 0:
        drop = drop_scene(ys, dev, args.drop_steps)
    hbm_peak, peak_kind = peaks()
    fp64_peak = measure_fp64_peak(torch)

    def roof(kname):
        # cloths leave the PCG as they converge, so a launch processes only the
        # rows of the cloths still iterating: rates use the rows counted
        if prof["launches"].get(kname, 0) == 0 or kname not in alg:
            return None
        secs = prof["ms"][kname] * 1e-3
        a = alg[kname]
        frac_rows = node_iters / float(n)  # full-batch SpMV equivalents
        return dict(gbs=a["bytes"] * frac_rows / secs / 1e9, tflops=a["flops"] * frac_rows / secs / 1e12,
                    us=secs / frac_rows * 1e6, launches=prof["launches"][kname], row_passes=frac_rows)

    roofline = None
    persist = roof("pcg_persist")
    spmv = roof("spmv")
    if persist:
        # DRAM bytes per row pass: ncu's dram__bytes_read + write of one persistent solve
        # launch over every node of a 64-cloth batch, divided by its row passes
        tr = PERSIST_DRAM_BYTES_PER_ROW_PASS
        roofline = {"kernel": "k_pcg_cluster (persistent per-cloth Jacobi-PCG, %d x %d threads per cloth)" %
                              (config["schedule"].get("pcg_cluster", 0), config["schedule"].get("pcg_threads", 0)),
                    "bound": "hbm", "achieved": persist["gbs"], "peak": hbm_peak, "unit": "GB/s",
                    "frac": persist["gbs"] / hbm_peak, "peak_source": peak_kind,
                    "traffic": tr * n if tr else None,
                    "traffic_source": "ncu capture at 102,400 nodes (64 x 40 x 40), per row pass, scaled per node"
                                      if tr else None,
                    "fp64": {"achieved_tflops": persist["tflops"], "dgemm_tflops": fp64_peak,
                             "frac": persist["tflops"] / fp64_peak},
                    "us_per_full_batch_pass": persist["us"], "full_batch_passes": persist["row_passes"],
                    "launches": persist["launches"],
                    "dominant_kernel_by_time": dominant, "time_share": share}
    elif spmv:
        roofline = {"kernel": "k_pcg_spmv (stencil SpMV, 159 FP64 coefficients per node)", "bound": "hbm",
                    "achieved": spmv["gbs"], "peak": hbm_peak, "unit": "GB/s", "frac": spmv["gbs"] / hbm_peak,
                    "peak_source": peak_kind,
                    # DRAM bytes of one full-batch SpMV pass: ncu's dram__bytes_read + write of a
                    # launch over every node of a 128-cloth batch (1355 B per node), times the nodes
                    "traffic": 1355.0 * n, "traffic_source": "ncu capture at 122,512 nodes, scaled per node",
                    "fp64": {"achieved_tflops": spmv["tflops"], "dgemm_tflops": fp64_peak,
                             "frac": spmv["tflops"] / fp64_peak},
                    "us_per_full_batch_pass": spmv["us"], "full_batch_passes": spmv["row_passes"],
                    "launches": spmv["launches"],
                    "dominant_kernel_by_time": dominant, "time_share": share}
    if roofline is not None:
        roofline["pcg_ms_per_step"] = sum(prof["ms"].get(k, 0.0) for k in
                                          ("pcg_setup", "spmv", "axpy", "dir", "pcg_persist")) / prof_steps
        roofline["assembly"] = assembly_roof(prof, n, prof_steps, fp64_peak)

    line = {"metric": metric, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "cloth_steps_per_s": value * args.cloths, "pcg_iterations_per_step": statistics.mean(iters),
            "all_cloths_ok": ok, "gpu_launches": int(launches), "e2e": e2e, "roofline": roofline,
            "clocks": clk.summary()}
    if precond is not None:
        line["precond"] = precond
    if collision is not None:
        line["collision"] = collision
    if drop is not None:
        line["collision_drop50"] = drop
    if sched_cmp is not None:
        line["single_cloth_pcg_schedules"] = sched_cmp

    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        v, desc, wall = cpu_sample(specs, seed, target_nodes=total_nodes, steps=1, cores=cores)
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": cores, "kind": "port", "sample": desc}
    if args.profile and rank == 0:
        for k in prof["ms"]:
            if prof["launches"][k]:
                print("%-10s %8.3f ms  %6d launches  %5.1f%%" % (k, prof["ms"][k], prof["launches"][k],
                                                               100 * prof["ms"][k] / tot_ms), file=sys.stderr)
    batch.close()
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
