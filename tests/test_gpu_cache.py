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


@pytest.mark.parametrize("size,bpc,ch,B,c,bb", [
    ((64, 64, 64), 1, 1, 16, 1, (1, 1, 1)),
    ((96, 64, 80), 2, 1, 32, 2, (2, 1, 1)),
    ((64, 48, 56), 1, 2, 16, 2, (2, 2, 2)),   # the c5 brick layout: two u8 channels, covering 2, big bricks 2^3
    ((64, 64, 32), 1, 1, 16, 0, (1, 1, 1)),
])
def test_device_source_equals_host_store(gc, torch_cuda, size, bpc, ch, B, c, bb):
    """gc_cache_set_volume_source_device: missing bricks cut on the device from
    the resident pyramid give the same frames as the brick store the
    bricker writes (gc_cache_set_source_host): every frame's image, and after
    every update the LRU order, page directory and pool bytes, bit for bit."""
    torch = torch_cuda
    vol = gc.volume_desc(size, B, c, bpc * ch, ch, bb)
    layout = gc.compute_layout(vol)
    d = scenario.gpu_volume(gc, torch, size, bpc, 31, 5, channels=ch)
    store, offs, empty = gc.pre_process(vol, layout, d, empty_threshold=30.0 * (257 if bpc == 2 else 1))
    poffs, total = gc.pyramid_offsets(layout, vol.encoded_bytes)
    pyr = torch.empty(total, dtype=torch.uint8, device="cuda")
    pyr[: d.numel() * d.element_size()].copy_(d.view(torch.uint8))
    gc.Mipmapper.process(pyr.data_ptr(), layout, poffs, vol.encoded_bytes, ch)
    torch.cuda.synchronize()
    caches = []
    for kind in ("host", "device"):
        cm = gc.CacheManager(vol, layout, (5, 5, 5), max_requests=60, sync_loader=True)
        if kind == "host":
            cm.set_source_host(store, offs, empty_keys=empty)
        else:
            cm.set_source_device(pyr.data_ptr(), poffs, empty_keys=empty, keep=pyr)
        caches.append(cm)
    W, H = 40, 32
    tf = scenario.tf2d(3) if ch == 2 else scenario.ramp_tf()
    tfh, tfw = (tf.shape[0], tf.shape[1]) if ch == 2 else (0, tf.shape[0])
    tf_dev = torch.from_numpy(tf.reshape(-1).copy()).cuda()
    bufs = [[torch.zeros(W * H * k, dtype=dt, device="cuda") for dt, k in ((torch.int32, 1), (torch.float32, 1),
                                                                          (torch.float32, 4))] for _ in caches]
    nslots = 125
    for f in range(16):
        m = scenario.orbit_camera(gc, f // 4, 8, 2.2 + 0.2 * (f // 4))
        imgs = []
        for cm, b in zip(caches, bufs):
            if f % 4 == 0:
                for x in b:
                    x.zero_()
            cm.render(gc.make_view(m, W, H, tf_dev.data_ptr(), tfw, *[x.data_ptr() for x in b], tf_height=tfh))
            torch.cuda.synchronize()
            imgs.append(b[0].cpu().numpy())
        assert np.array_equal(imgs[0], imgs[1]), f"frame {f}: image"
        assert caches[0].update() == caches[1].update(), f"frame {f}"
        for what, dtype, n in ((gc.DUMP_LRU, np.uint8, nslots * 28), (gc.DUMP_MRPD, np.uint32, caches[0].info.mrpd_dims[0]
                                                                      * caches[0].info.mrpd_dims[1]
                                                                      * caches[0].info.mrpd_dims[2] * 4),
                               (gc.DUMP_POOL, np.uint8, caches[0].info.pool_bytes)):
            a, b2 = (cm.dump(what, np.zeros(n, dtype)) for cm in caches)
            assert np.array_equal(a, b2), (f, what)
    st = [cm.stats() for cm in caches]
    assert st[1].bricks_installed == st[0].bricks_installed > 0
    assert st[1].bytes_h2d == 0 and st[1].device_error == 0
    for cm in caches:
        cm.close()
