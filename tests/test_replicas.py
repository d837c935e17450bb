"""Multi-GPU = independent replicas: seeds, the max-over-ranks time and the whole-job rate.

The SpMM path has no exchange step, so N GPUs run N replicas with no data-path collective.
These tests run the cross-rank logic as two `gloo` ranks on the CPU.
"""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import numpy as np
    import torch.distributed as dist
    sys.path[:0] = [ROOT, os.path.join(ROOT, "sparse-register-tiling_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from spreg.replicas import max_over_ranks, shard_seed, whole_job_rate
        ms = max_over_ranks(10.0 * (rank + 1))  # rank 1 is the slow one
        rate = whole_job_rate(1e9, 4, world, ms)
        args = bench.argparse.Namespace(replicas=2, m=32, k=64, n=8, sparsity=0.8)
        As, _ = bench.make_inputs(args, rank)
        digest = [float(np.abs(A).sum()) for A in As]
        seeds = [shard_seed(rank, r) for r in range(3)]
        out = [None] * world
        dist.all_gather_object(out, {"ms": ms, "rate": rate, "digest": digest, "seeds": seeds})
        if rank == 0:
            q.put(out)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_the_slowest_and_hold_distinct_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r["ms"] for r in res] == [20.0, 20.0]
    assert res[0]["rate"] == pytest.approx(2 * 4 * 1e9 / 0.020)
    assert not set(res[0]["seeds"]) & set(res[1]["seeds"])
    assert not set(res[0]["digest"]) & set(res[1]["digest"])  # the ranks' weights differ


def test_single_process_and_argument_checks():
    sys.path[:0] = [os.path.join(ROOT, "sparse-register-tiling_gb300")]
    from spreg.replicas import max_over_ranks, shard_seed, whole_job_rate
    assert max_over_ranks(3.5) == 3.5
    assert whole_job_rate(100.0, 10, 1, 1000.0) == pytest.approx(1000.0)
    with pytest.raises(ValueError):
        whole_job_rate(1.0, 0, 1, 1.0)
    with pytest.raises(ValueError):
        shard_seed(0, 1000)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
