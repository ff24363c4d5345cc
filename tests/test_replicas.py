"""Multi-GPU form of the path: replicas (each rank owns a cache and renders
its own views; no exchange), timed by the slowest rank.  The host side of that
-- barrier, max over ranks, per-rank views -- runs here as two gloo ranks on
CPU (no GPU)."""
import os
import socket

import numpy as np
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


def shared_worker(rank, world, port, shm, out):
    import sys

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "gpu-out-of-core-volume-data_gb300"))
    os.environ.update(WORLD_SIZE=str(world), LOCAL_RANK=str(rank), RANK=str(rank), MASTER_PORT=str(port))
    import numpy as np
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=world - 1 - rank, world_size=world)
    try:
        bench.SHM_DIR = shm
        calls = []

        def fill(t):  # the store builder: runs on local rank 0 only
            calls.append(1)
            t.copy_(torch.arange(t.numel(), dtype=torch.int64).remainder(251).to(torch.uint8))
            return np.arange(7, dtype=np.uint64) * 3

        store, bins = bench.node_shared_store(torch, "k", 1 << 20, fill)
        out.put((rank, len(calls), int(store.numel()), int(store.to(torch.int64).sum()),
                 [int(b) for b in bins], sorted(os.listdir(shm))))
    finally:
        dist.destroy_process_group()


def test_replicas_share_one_host_store(tmp_path):
    """Replicas on one node map one host brick store: local rank 0 builds it
    into a shared file, the other rank maps the same bytes (and bins), and the
    file's name is gone once both hold their mapping."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=shared_worker, args=(r, 2, port, str(tmp_path), q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r = q.get(timeout=120)
        res[r[0]] = r[1:]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = int((np.arange(1 << 20) % 251).sum())
    assert res[0] == (1, 1 << 20, want, [0, 3, 6, 9, 12, 15, 18], [])
    assert res[1] == (0, 1 << 20, want, [0, 3, 6, 9, 12, 15, 18], [])
