"""Multi-GPU runs are frame-level replicas: each rank reconstructs its own
frames and the ranks meet only at the timing barrier and the max-over-ranks
reduction.  That host logic runs here on two gloo ranks on the CPU (the
pool's boxes have one GPU each)."""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (r + 1) * 10 ms for its frames: the job took the slowest
        ms = bench.max_over_ranks(10.0 * (rank + 1), world, "cpu")
        dist.barrier()
        out.put((rank, ms, bench.job_throughput(1000, world, ms)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [20.0, 20.0]
    # 2 ranks x 1000 particles in 20 ms
    assert got[0][2] == pytest.approx(100_000.0)


def test_single_rank_is_a_no_op():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.job_throughput(500, 1, 10.0) == pytest.approx(50_000.0)


def test_roofline_kernel_is_chosen_on_the_frame_stream():
    """With diffuse generation on, the diffuse stage's time is a span beside the surface
    stages, so the roofline's kernel is the longest stage of the frame's own stream."""
    sys.path.insert(0, ROOT)
    import bench
    stage = {"grid": 0.2, "anisotropy": 0.95, "band": 0.92, "field": 2.78, "marching_cubes": 0.86, "diffuse": 4.56}
    alg = {k: 1.0 for k in stage}
    assert bench.dominant_stage(stage, alg, diffuse=True) == "field"
    assert bench.dominant_stage(dict(stage, field=0.5), alg, diffuse=True) == "anisotropy"
    # surface only: every stage is on the frame's stream
    assert bench.dominant_stage(dict(stage, diffuse=9.0), alg, diffuse=False) == "diffuse"
