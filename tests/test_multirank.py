"""The multi-GPU path of the benchmark on CPU ranks (gloo, world size 2).

A single TTV does not shard ("replicas only"): every rank runs the whole
workload with no data-path collective; the only exchange is the max of the
timed region over ranks.  The reference arm runs on rank 0 alone."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.aggregate(10.0 * (rank + 1), 1e9, 4, world, dist)
    out.put((rank, ms, value))
    dist.destroy_process_group()


def test_max_over_ranks_and_weak_scaling_value():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time; value counts both ranks' bytes
    for rank, ms, value in res:
        assert ms == 20.0
        assert abs(value - 2 * 1e9 * 4 / 0.020 / 1e9) < 1e-9


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
