"""Replicas only: bench.py's multi-rank plumbing on CPU (gloo, world size 2).

The path does not shard: with N GPUs each rank advances its own replica, and the
ranks meet only in a barrier and in max/sum reductions of timings and particle
counts.  These tests run that plumbing as two CPU processes over gloo: whole-job
throughput = particles on all ranks x steps / slowest rank's time.  The
reference arm runs on rank 0 only; the other ranks exit without work.
"""
import os
import socket
import sys

import pytest

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.init("gloo")
    d.barrier()
    ms = 100.0 + 50.0 * rank            # rank 1 is the slower replica
    particles = 1000.0 * (rank + 1)
    ms_max = d.max(ms)
    n_total = d.sum(particles)
    steps = 4
    value = n_total * steps / (ms_max / 1e3)
    # the reference arm: rank 0 runs it, the others return 0 at once
    args = type("A", (), {"steps": 1, "warmup": 0, "weights": 0, "gpus": world})()
    rc_other = bench.run_reference(args, None) if rank != 0 else 0
    d.barrier()
    d.close()
    q.put((rank, ms_max, n_total, value, rc_other))


def test_replica_reductions_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    for rank, ms_max, n_total, value, rc_other in out:
        assert ms_max == 150.0
        assert n_total == 3000.0
        assert value == pytest.approx(3000.0 * 4 / 0.150)
        assert rc_other == 0


def test_single_rank_dist_is_a_no_op():
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    if d.world != 1:
        pytest.skip("launched under a multi-rank launcher")
    d.init("gloo")
    assert not d.pg and d.max(2.5) == 2.5 and d.sum(3.0) == 3.0
    d.barrier()
    d.close()


def test_record_push_count():
    """The push roofline counts 8 more bytes per particle for each push that reads
    the sort's records: one per sort in the timed steps, default shape only."""
    sys.path.insert(0, ROOT)
    import bench
    lanes = 4
    shape = {"lane_particles": 4, "deposit": lanes}
    assert bench.record_pushes("fp32", shape, 20, 20, lanes) == 1
    assert bench.record_pushes("fp32", shape, 41, 20, lanes) == 3
    assert bench.record_pushes("fp32", shape, 5, 1, lanes) == 5
    assert bench.record_pushes("fp32", shape, 20, 0, lanes) == 0
    assert bench.record_pushes("fp64", shape, 20, 20, lanes) == 0
    assert bench.record_pushes("fp32", dict(shape, lane_particles=2), 20, 20, lanes) == 0
    assert bench.record_pushes("fp32", dict(shape, deposit=0), 20, 20, lanes) == 0
