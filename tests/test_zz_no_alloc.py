"""The allocation-free miss list (gc_miss_list_noalloc) against the miss list
the cache builds inside gc_cache_update, through the C ABI.

gc_miss_list_noalloc serves callers that cannot allocate device memory when
they need the list -- a frame recorded into a CUDA graph, a loop with a hard
deadline, a host that owns all device memory -- by keeping its scan scratch in
a fixed device array.  This file is collected last so that a run stopping at
its first failure has already run every other test; it also passes alone.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_REQ = 4096


def request_buffer(rng, layout, mx, my, mz, ts, n_req, stale):
    req = np.zeros(mx * my * mz, np.uint32)
    # older timestamps that must not be listed
    req[rng.integers(0, req.size - 1, stale)] = rng.integers(1, max(2, ts), stale, dtype=np.uint32) % max(1, ts)
    for _ in range(n_req):
        l = int(rng.integers(0, layout.nb_levels))
        nb = layout.nb_bricks[l]
        off = sum(layout.nb_bricks[k][0] for k in range(l))
        x, y, z = (int(rng.integers(0, nb[a])) for a in range(3))
        req[off + x + y * mx + z * mx * my] = ts
    return req


def test_no_alloc_miss_list_equals_cache_update(gc, torch_cuda):
    torch = torch_cuda
    vol = gc.volume_desc((2048, 2048, 2048), 16, 1, 2, 1)  # 6.4 M page-directory entries
    layout = gc.compute_layout(vol)
    cm = gc.CacheManager(vol, layout, (64, 64, 64), max_requests=MAX_REQ, sync_loader=True)
    cm.set_source_callback(lambda *a: gc.BRICK_UNKNOWN)  # scans only, no installs
    mx, my, mz = cm.info.mrpd_dims
    n = mx * my * mz
    rng = np.random.default_rng(2024)
    out_list = torch.zeros(MAX_REQ * 4, dtype=torch.int32, device="cuda")
    out_total = torch.zeros(1, dtype=torch.int32, device="cuda")
    for call, n_req in enumerate((9000, 2500)):  # two calls in a row: the shared scratch is reused
        ts = cm.timestamp()
        req = request_buffer(rng, layout, mx, my, mz, ts, n_req, 5000)
        # existing entry point: the scan inside the cache update
        cm.load_buffer(gc.DUMP_REQUESTS, req)
        cm.update()
        total_ref, list_ref = cm.last_misses()
        # the allocation-free entry point on the same buffer
        d_req = torch.from_numpy(req.view(np.int32)).cuda()
        out_list.fill_(-1)
        out_total.fill_(-1)
        gc.miss_list_noalloc(d_req.data_ptr(), n, ts, layout, MAX_REQ, out_list.data_ptr(), out_total.data_ptr())
        torch.cuda.synchronize()
        total = int(out_total.item())
        got = out_list.cpu().numpy().view(np.uint32).reshape(-1, 4)[: min(total, MAX_REQ)]
        assert total == total_ref > 0, (call, total, total_ref)
        assert np.array_equal(got, list_ref), call
    # sizes beyond the fixed scratch are rejected, not scanned
    with pytest.raises(gc.GcError, match="too large"):
        gc.miss_list_noalloc(out_list.data_ptr(), 2048 * 4096 + 2, 1, layout, MAX_REQ, out_list.data_ptr(),
                             out_total.data_ptr())
    cm.close()


def test_no_alloc_scan_reports_an_expired_wait(gc, torch_cuda, monkeypatch):
    """Every look-back wait of the scan is bounded.  The test hook
    GC_TEST_NOALLOC_SILENT_TILE makes one scan tile publish nothing -- a flag
    that nothing sets -- so that the next tile's wait runs out: the call must
    then report GC_MISS_LIST_FAILED in out_total (not hang, not fault), and the
    next call without the hook must give the right list again (the scratch
    keeps no stale error)."""
    torch = torch_cuda
    vol = gc.volume_desc((256, 256, 256), 16, 1, 1, 1)  # 14,079 entries: 4 scan tiles
    layout = gc.compute_layout(vol)
    cm = gc.CacheManager(vol, layout, (8, 8, 8), max_requests=50, sync_loader=True)
    cm.set_source_callback(lambda *a: gc.BRICK_UNKNOWN)
    mx, my, mz = cm.info.mrpd_dims
    n = mx * my * mz
    rng = np.random.default_rng(7)
    ts = cm.timestamp()
    req = request_buffer(rng, layout, mx, my, mz, ts, 300, 100)
    cm.load_buffer(gc.DUMP_REQUESTS, req)
    cm.update()
    total_ref, list_ref = cm.last_misses()
    d_req = torch.from_numpy(req.view(np.int32)).cuda()
    out_list = torch.zeros(50 * 4, dtype=torch.int32, device="cuda")
    out_total = torch.zeros(1, dtype=torch.int32, device="cuda")
    monkeypatch.setenv("GC_TEST_NOALLOC_SILENT_TILE", "1")
    gc.miss_list_noalloc(d_req.data_ptr(), n, ts, layout, 50, out_list.data_ptr(), out_total.data_ptr())
    torch.cuda.synchronize()
    assert int(out_total.item()) & 0xFFFFFFFF == gc.MISS_LIST_FAILED
    monkeypatch.delenv("GC_TEST_NOALLOC_SILENT_TILE")
    gc.miss_list_noalloc(d_req.data_ptr(), n, ts, layout, 50, out_list.data_ptr(), out_total.data_ptr())
    torch.cuda.synchronize()
    total = int(out_total.item())
    assert total == total_ref > 50
    assert np.array_equal(out_list.cpu().numpy().view(np.uint32).reshape(-1, 4), list_ref)
    cm.close()
