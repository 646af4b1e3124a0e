"""The multi-GPU path's host logic, with world-size-2 gloo ranks on the CPU.

ROIs are independent, so N GPUs fit N shards with no collective on the data
path (weak scaling): each rank draws its own ROIs (its own seed), times its
steps, and the job's time is the slowest rank's, one MAX all-reduce.  Rank 0
alone prints the JSON line; the reference arm runs on rank 0 only and the
other ranks exit 0 without output."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    from gaussmle_gb300 import simulate
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, _ = bench.dist_init()
        dt = bench.max_over_ranks(0.5 + r, w, "cpu")       # ranks took 0.5 s and 1.5 s
        rate = bench.job_rate(1000, 10, w, dt)
        shard = simulate.xynb11_poisson(n=64, seed=bench.rank_seed(1000, r))
        q.put((r, w, dt, rate, float(shard.data.sum()), float(shard.truth[:, 0].sum())))
    finally:
        dist.destroy_process_group()


def test_two_ranks_time_and_shard():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, dt0, rate0, d0, x0), (r1, w1, dt1, rate1, d1, x1) = res
    assert (r0, r1) == (0, 1) and w0 == w1 == 2
    assert dt0 == dt1 == 1.5                      # the slowest rank's time
    assert rate0 == rate1 == pytest.approx(1000 * 10 * 2 / 1.5)
    assert d0 != d1 and x0 != x1                  # each rank fits its own ROIs


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1",
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1"], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
