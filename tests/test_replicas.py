"""Multi-GPU form of the path: replicas (each rank owns a cache and renders
its own views; no exchange), timed by the slowest rank.  The host side of that
-- barrier, max over ranks, per-rank views -- runs here as two gloo ranks on
CPU (no GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "gpu-out-of-core-volume-data_gb300"))
    import torch.distributed as dist

    import bench
    import gcgb300 as gc

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bench.rank_barrier()
        walls = bench.max_over_ranks([1.0 + rank, 10.0 - rank])
        cfg = bench.CONFIGS["c2"]
        views = [tuple(round(v, 5) for v in bench.path_camera(gc.look_at, cfg, f, rank)) for f in range(3)]
        out.put((rank, walls, views))
    finally:
        dist.destroy_process_group()


def test_replicas_time_by_slowest_rank_and_render_different_views():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r, walls, views = q.get(timeout=120)
        res[r] = (walls, views)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the element-wise maximum (the slowest rank per entry)
    assert res[0][0] == res[1][0] == [2.0, 10.0]
    # each replica renders its own views of the path
    assert res[0][1] != res[1][1]
