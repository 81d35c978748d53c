"""The multi-rank path of bench.py on CPU: two gloo ranks each build their own
seeded shard (no data exchange), the timing reduction takes the slowest rank,
two ranks stepping their shards (with the host build of the step's element
code, tests/emu) reach the states one process reaches stepping the same
shards, and the reference arm's other ranks exit without work."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    specs, wind = bench.workload(bench.rank_seed(0, rank), 16)
    nodes = sum(s["width"] * s["length"] for s in specs)
    t = bench.max_over_ranks(1.0 + rank, dist, "cpu")
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), np.array([nodes, t, wind[0, 0]]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_take_the_slowest(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0, r1 = (np.load(str(tmp_path / ("rank%d.npy" % r))) for r in (0, 1))
    assert r0[1] == r1[1] == 2.0          # max over ranks seen by both
    assert (r0[0], r0[2]) != (r1[0], r1[2])  # independent shards


def _shard_digest(rank, steps=2):
    """Per-cloth sums of the state after `steps` steps of rank's shard."""
    import bench
    from emu_py import EmuCloth
    specs, _ = bench.workload(bench.rank_seed(0, rank), 2)
    out = []
    for sp in specs:
        c = EmuCloth(**sp)
        for _ in range(steps):
            assert c.step(1e-3, tol=1e-10)["status"] == 0
        st = c.get_state()
        out.append([float(st[k].sum()) for k in ("LPos", "LVel", "EPos", "EVel", "EPosBar")])
    return np.array(out)


def _rank_step(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    mine = torch.as_tensor(_shard_digest(rank))
    got = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(got, mine)  # the test's own comparison; the sharded step exchanges nothing
    if rank == 0:
        np.save(os.path.join(out_dir, "digests.npy"), torch.stack(got).numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_step_their_shards_like_one_process(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_step, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = np.load(str(tmp_path / "digests.npy"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    ref = np.stack([_shard_digest(r) for r in (0, 1)])
    assert np.array_equal(got, ref)
    assert not np.array_equal(ref[0], ref[1])  # different shards


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
