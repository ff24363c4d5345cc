"""Bit-exact cache state: LRU order, page directory, pool, miss lists and
completude of the CUDA update path against the oracle's restatement of
CacheManager::update, replaying recorded usage/request buffers."""
import ctypes

import numpy as np
import pytest

import scenario

pytestmark = pytest.mark.gpu


def random_frame(rng, ts, usage, req, nslots, layout, mx, my, p_used, n_req):
    used = rng.random(nslots) < p_used
    usage[used] = ts
    for _ in range(n_req):
        l = int(rng.integers(0, layout.nb_levels))
        nb = layout.nb_bricks[l]
        off = sum(layout.nb_bricks[k][0] for k in range(l))
        x, y, z = (int(rng.integers(0, nb[a])) for a in range(3))
        req[off + x + y * mx + z * mx * my] = ts


def compare_state(gc, cm, oc, tag):
    lru = np.zeros(oc.nslots, dtype=oc.lru().dtype)
    cm.dump(gc.DUMP_LRU, lru)
    assert np.array_equal(lru, oc.lru()), f"{tag}: LRU differs"
    mrpd = np.zeros((oc.nentries, 4), np.uint32)
    cm.dump(gc.DUMP_MRPD, mrpd)
    assert np.array_equal(mrpd, oc.mrpd()), f"{tag}: page directory differs"
    pool = np.zeros(oc.pool_bytes, np.uint8)
    cm.dump(gc.DUMP_POOL, pool)
    assert np.array_equal(pool, oc.pool()), f"{tag}: pool differs"
    assert cm.completude() == pytest.approx(oc.completude(), abs=0)


def device_reads_pageable(torch):
    """cudaDevAttrPageableMemoryAccess of device 0 (Grace-Blackwell: 1)."""
    import ctypes as C

    rt = None
    for name in ("libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            pass
    assert rt is not None, "CUDA runtime library not found"
    v = C.c_int(0)
    assert rt.cudaDeviceGetAttribute(C.byref(v), 88, 0) == 0  # cudaDevAttrPageableMemoryAccess
    return bool(v.value)


# upload routes: "pageable" = numpy store (gathered by a kernel where the
# device reads pageable memory, else staged), "pinned" = page-locked store
# (always gathered), "staged" = GC_CACHE_STAGED_UPLOAD (host copies + one
# cudaMemcpyAsync)
@pytest.mark.parametrize("maxreq,route", [(50, "pageable"), (700, "pageable"), (700, "pinned"), (50, "staged"),
                                          (300, "files")])
def test_update_replay_with_installs(gc, orc, torch_cuda, maxreq, route, tmp_path):
    size = (256, 256, 256)
    vol = gc.volume_desc(size, 16, 1, 1, 1)
    layout = gc.compute_layout(vol)
    o = scenario.orc_volume(orc, (256, 256, 256), 1, 1, 8)
    store, offs = scenario.orc_store(orc, gc, o.reshape(-1).view(np.uint8), vol, layout)
    cm = gc.CacheManager(vol, layout, (10, 10, 10), max_requests=maxreq, sync_loader=True,
                         staged_upload=route == "staged")
    if route == "files":  # the reference's LZ4 brick files, read by the loader's threads
        if not gc.lz4_available():
            pytest.skip("liblz4 is not installed")
        gc.write_brick_files(tmp_path, vol, layout, store, offs)
        cm.set_source_files(tmp_path, threads=4)
        expect_direct = False
    else:
        src = torch_cuda.from_numpy(store).pin_memory() if route == "pinned" else store
        cm.set_source_host(src, offs)
        expect_direct = route == "pinned" or (route == "pageable" and device_reads_pageable(torch_cuda))
    assert cm.stats().upload_direct == int(expect_direct)
    oc = orc.Cache(cm.desc)
    oc.set_source(store, offs)
    mx, my, _ = oc.mrpd_dims
    rng = np.random.default_rng(maxreq)
    usage = np.zeros(oc.nslots, np.uint32)
    req = np.zeros(oc.nentries, np.uint32)
    for f in range(14):
        ts = f + 1
        assert cm.timestamp() == ts == oc.timestamp
        random_frame(rng, ts, usage, req, oc.nslots, layout, mx, my, 0.3, 900)
        cm.load_buffer(gc.DUMP_USAGE, usage)
        cm.load_buffer(gc.DUMP_REQUESTS, req)
        oc.usage()[:] = usage
        oc.requests()[:] = req
        c1, c2 = cm.update(), oc.update()
        assert c1 == c2
        compare_state(gc, cm, oc, f"frame {f}")
    st = cm.stats()
    assert st.bricks_installed > 0 and st.device_error == 0


def test_store_size_is_checked(gc, orc, torch_cuda):
    """Every level of the brick store must lie inside the bytes given: the
    upload kernel reads the store directly, so a short store is rejected up
    front instead of being read past its end."""
    size = (64, 64, 64)
    vol = gc.volume_desc(size, 16, 1, 1, 1)
    layout = gc.compute_layout(vol)
    o = scenario.orc_volume(orc, size, 1, 4, 5)
    store, offs = scenario.orc_store(orc, gc, o.reshape(-1).view(np.uint8), vol, layout)
    cm = gc.CacheManager(vol, layout, (6, 6, 6), max_requests=50, sync_loader=True)
    with pytest.raises(gc.GcError, match="does not fit"):
        cm.set_source_host(store[: store.size - 1], offs)
    cm.set_source_host(store, offs)
    cm.close()


def test_update_replay_large_geometry(gc, orc, torch_cuda):
    """2048^3 u16 geometry: 6.4 M page-directory entries, 262,144 pool slots.
    No brick data (every load is Unknown): checks the LRU partition and the
    capped, ordered miss list at full size."""
    vol = gc.volume_desc((2048, 2048, 2048), 16, 1, 2, 1)
    layout = gc.compute_layout(vol)
    cm = gc.CacheManager(vol, layout, (64, 64, 64), max_requests=4096, sync_loader=True)
    cm.set_source_callback(lambda *a: gc.BRICK_UNKNOWN)
    oc = orc.Cache(cm.desc)
    mx, my, _ = oc.mrpd_dims
    rng = np.random.default_rng(7)
    usage = np.zeros(oc.nslots, np.uint32)
    req = np.zeros(oc.nentries, np.uint32)
    for f in range(3):
        ts = f + 1
        random_frame(rng, ts, usage, req, oc.nslots, layout, mx, my, 0.4, 20000)
        cm.load_buffer(gc.DUMP_USAGE, usage)
        cm.load_buffer(gc.DUMP_REQUESTS, req)
        oc.usage()[:] = usage
        oc.requests()[:] = req
        oc_total, oc_list = oc.request_list(4096)  # the list the update below builds
        assert cm.update() == oc.update()
        lru = np.zeros(oc.nslots, dtype=oc.lru().dtype)
        cm.dump(gc.DUMP_LRU, lru)
        assert np.array_equal(lru, oc.lru())
        total, lst = cm.last_misses()
        assert total == oc_total and np.array_equal(lst, oc_list)
        # property: used slots first, each group in previous order
        cx = (lru["cx"] // 16) + (lru["cy"] // 16) * 64 + (lru["cz"] // 16) * 4096
        assert np.array_equal(np.sort(cx), np.arange(oc.nslots))
        k = int((usage == ts).sum())
        assert np.all(usage[cx[:k]] == ts) and np.all(usage[cx[k:]] != ts)
    st = cm.stats()
    assert st.load_errors > 0 and st.device_error == 0


def test_unknown_bricks_stay_unmapped(gc, orc, torch_cuda):
    """A brick source that fails for some bricks: they stay unmapped, the
    failures are counted, every other brick installs (no device fault)."""
    size = (64, 64, 64)
    vol = gc.volume_desc(size, 16, 1, 1, 1)
    layout = gc.compute_layout(vol)
    o = scenario.orc_volume(orc, size, 1, 4, 5)
    store, offs = scenario.orc_store(orc, gc, o.reshape(-1).view(np.uint8), vol, layout)
    big = 16 ** 3
    calls = []

    def loader(user, level, x, y, z, dst, nbytes):
        calls.append((level, x, y, z))
        nb = layout.nb_big_bricks[level]
        if (x + y + z) % 3 == 0 or x >= nb[0] or y >= nb[1] or z >= nb[2] or nbytes != big:
            return gc.BRICK_UNKNOWN
        i = offs[level] + ((z * nb[1] + y) * nb[0] + x) * big
        ctypes.memmove(dst, store.ctypes.data + i, big)
        return gc.BRICK_SUCCESS

    cm = gc.CacheManager(vol, layout, (6, 6, 6), max_requests=50, sync_loader=True)
    cm.set_source_callback(loader)
    mx, my, mz = cm.info.mrpd_dims
    req = np.zeros(mx * my * mz, np.uint32)
    off = 0
    for l in range(layout.nb_levels):  # every brick of every level requested at ts 1
        nb = layout.nb_bricks[l]
        for z in range(nb[2]):
            for y in range(nb[1]):
                req[off + z * mx * my + y * mx: off + z * mx * my + y * mx + nb[0]] = 1
        off += nb[0]
    cm.load_buffer(gc.DUMP_REQUESTS, req)
    assert cm.update() is False
    cm.update()  # install
    mrpd = np.zeros((mx * my * mz, 4), np.uint32)
    cm.dump(gc.DUMP_MRPD, mrpd)
    st = cm.stats()
    assert st.load_errors == sum(1 for c in calls if sum(c[1:]) % 3 == 0) > 0
    assert st.bricks_installed == len(calls) - st.load_errors
    assert int((mrpd[:, 3] == 1).sum()) == st.bricks_installed and st.device_error == 0
