"""Ray caster parity: the CUDA render + update loop against the oracle's FP32
restatement of RayCastDVR/RayCastMOP and CacheManager::update, frame by frame.

Tolerances (per RGBA channel, in 1/255 units):
  CUDA vs FP32 oracle : 0   (same operation sequence; cache state bit-exact)
  CUDA vs FP64 oracle : 1   (the double-precision restatement of the method)
"""
import time

import numpy as np
import pytest

import scenario

pytestmark = pytest.mark.gpu

RGBA_TOL_FP32 = 0
RGBA_TOL_FP64 = 1
FAST_OUTLIER_SHARE = 1e-3  # fast build vs FP64: pixels allowed beyond 1/255 (termination crossings)


class Scene:
    def __init__(self, gc, orc, torch, size, bpc, B, c, bb, pool, maxreq, seed=21, nblobs=6, sync=True, channels=1,
                 **cache_kw):
        self.gc, self.orc, self.torch = gc, orc, torch
        self.vol = gc.volume_desc(size, B, c, bpc * channels, channels, bb)
        self.layout = gc.compute_layout(self.vol)
        d = scenario.gpu_volume(gc, torch, size, bpc, seed, nblobs, channels=channels)
        self.store, self.offs, _ = gc.pre_process(self.vol, self.layout, d)
        o = scenario.orc_volume(orc, size, bpc, seed, nblobs, channels=channels)
        ref, roffs = scenario.orc_store(orc, gc, o.reshape(-1).view(np.uint8), self.vol, self.layout)
        assert np.array_equal(self.store.numpy(), ref)
        self.ref = ref
        self.cm = gc.CacheManager(self.vol, self.layout, pool, max_requests=maxreq, sync_loader=sync, **cache_kw)
        self.cm.set_source_host(self.store, self.offs)
        self.oc = orc.Cache(self.cm.desc)
        self.oc.set_source(ref, roffs)

    def buffers(self, W, H):
        t = self.torch
        g = (t.zeros(W * H, dtype=t.int32, device="cuda"), t.zeros(W * H, dtype=t.float32, device="cuda"),
             t.zeros(W * H * 4, dtype=t.float32, device="cuda"))
        o = (np.zeros(W * H, np.uint32), np.zeros(W * H, np.float32), np.zeros(W * H * 4, np.float32))
        return g, o

    def view(self, m, W, H, tf_dev, tfw, g, **kw):
        return self.gc.make_view(m, W, H, tf_dev.data_ptr(), tfw, g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
                                 **kw)

    def compare_cache(self, tag):
        gc, oc, cm = self.gc, self.oc, self.cm
        lru = np.zeros(oc.nslots, dtype=oc.lru().dtype)
        cm.dump(gc.DUMP_LRU, lru)
        assert np.array_equal(lru, oc.lru()), tag
        for what, ref in ((gc.DUMP_USAGE, oc.usage()), (gc.DUMP_REQUESTS, oc.requests())):
            a = np.zeros_like(ref)
            cm.dump(what, a)
            assert np.array_equal(a, ref), (tag, what)
        mrpd = np.zeros((oc.nentries, 4), np.uint32)
        cm.dump(gc.DUMP_MRPD, mrpd)
        assert np.array_equal(mrpd, oc.mrpd()), tag
        pool = np.zeros(oc.pool_bytes, np.uint8)
        cm.dump(gc.DUMP_POOL, pool)
        assert np.array_equal(pool, oc.pool()), tag


def rgba_diff(a, b):
    return np.abs(a.view(np.uint8).astype(np.int32) - b.view(np.uint8).astype(np.int32))


LOOP_CASES = {
    # size, bpc, B, c, big brick, pool, maxreq, W, H, view kwargs
    "u8_dvr_ref": ((64, 64, 64), 1, 16, 1, (1, 1, 1), (4, 4, 4), 50, 56, 48, dict()),
    "u16_mop_tri": ((48, 48, 48), 2, 8, 1, (2, 1, 1), (5, 5, 5), 64, 40, 36,
                    dict(mode=1, sampler=1, early_alpha=0.99, focal=2.4142137)),
    "u8_dvr_tri_wide": ((80, 64, 48), 1, 16, 2, (1, 1, 1), (6, 5, 5), 150, 77, 45,
                        dict(sampler=1, early_alpha=0.99)),
}


@pytest.mark.parametrize("case", sorted(LOOP_CASES))
def test_render_update_loop_matches_oracle(gc, orc, torch_cuda, case):
    size, bpc, B, c, bb, pool, maxreq, W, H, kw = LOOP_CASES[case]
    s = Scene(gc, orc, torch_cuda, size, bpc, B, c, bb, pool, maxreq)
    tf = scenario.ramp_tf() if "dvr" in case else scenario.bumps_tf(3)
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    g, o = s.buffers(W, H)
    for f in range(16):
        m = scenario.orbit_camera(gc, f // 4, 12, 2.6 + 0.3 * (f // 4))
        if f % 4 == 0:  # camera moved: restart the progressive buffers
            for x in g:
                x.zero_()
            for x in o:
                x[:] = 0
        v = s.view(m, W, H, tf_dev, 256, g, **kw)
        s.cm.render(v)
        s.oc.render(v, tf, *o)
        torch_cuda.cuda.synchronize()
        d = rgba_diff(g[0].cpu().numpy(), o[0])
        assert d.max() <= RGBA_TOL_FP32, f"frame {f}: max {d.max()} at {np.argmax(d)}"
        assert np.array_equal(g[1].cpu().numpy(), o[1]), f"frame {f}: t buffer"
        assert np.array_equal(g[2].cpu().numpy(), o[2]), f"frame {f}: colour state"
        c1, c2 = s.cm.update(), s.oc.update()
        assert c1 == c2, f"frame {f}"
        s.compare_cache(f"frame {f}")
    st = s.cm.stats()
    assert st.bricks_installed > 0 and st.device_error == 0


@pytest.mark.parametrize("mode,sampler,pt_block", [(0, 0, 0), (0, 1, 0), (1, 0, 0), (0, 1, 4)])
def test_two_channel_2d_tf_loop_matches_oracle(gc, orc, torch_cuda, mode, sampler, pt_block):
    """Two 8-bit channels (blob field + independent noise field, interleaved)
    rendered with a 2D transfer function, covering 2 and big bricks 2^3 (the
    c5 brick layout): RGBA, t buffer and colour state bit-exact vs the FP32
    oracle every frame, cache state bit-exact; also through a two-level page
    directory whose table pool holds 6 of its blocks.  (No reference
    counterpart: the reference ray caster reads one channel.)"""
    s = Scene(gc, orc, torch_cuda, (72, 64, 56), 1, 16, 2, (2, 2, 2), (6, 6, 6), 100, channels=2, seed=33,
              pt_block=pt_block, pt_slots=6 if pt_block else 0)
    tf = scenario.tf2d(5)
    th, tw = tf.shape[:2]
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    W, H = 61, 47
    g, o = s.buffers(W, H)
    for f in range(12):
        m = scenario.orbit_camera(gc, f // 4, 12, 2.7)
        if f % 4 == 0:
            for x in g:
                x.zero_()
            for x in o:
                x[:] = 0
        v = s.view(m, W, H, tf_dev, tw, g, tf_height=th, mode=mode, sampler=sampler, early_alpha=0.99)
        s.cm.render(v)
        s.oc.render(v, tf.reshape(-1), *o)
        torch_cuda.cuda.synchronize()
        d = rgba_diff(g[0].cpu().numpy(), o[0])
        assert d.max() <= RGBA_TOL_FP32, f"frame {f}: max {d.max()}"
        assert np.array_equal(g[1].cpu().numpy(), o[1]), f"frame {f}: t buffer"
        assert np.array_equal(g[2].cpu().numpy(), o[2]), f"frame {f}: colour state"
        assert s.cm.update() == s.oc.update()
        s.compare_cache(f"frame {f}")
    assert (g[0].cpu().numpy() >> 24).astype(bool).mean() > 0.05  # not an empty image


def test_batch_matches_sequential_oracle(gc, orc, torch_cuda):
    """Three views of different sizes in one persistent launch (one cache
    frame) equal the oracle rendering them one after the other."""
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 216)
    tf = scenario.ramp_tf()
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    sizes = [(64, 48), (33, 17), (96, 80)]
    bufs = [s.buffers(W, H) for W, H in sizes]
    for f in range(6):
        views = []
        for i, (W, H) in enumerate(sizes):
            m = scenario.orbit_camera(gc, i * 3 + 1, 12, 3.0)
            views.append(s.view(m, W, H, tf_dev, 256, bufs[i][0]))
        s.cm.render_batch(views)
        for i in range(len(sizes)):
            s.oc.render(views[i], tf, *bufs[i][1])
        torch_cuda.cuda.synchronize()
        for i in range(len(sizes)):
            d = rgba_diff(bufs[i][0][0].cpu().numpy(), bufs[i][1][0])
            assert d.max() <= RGBA_TOL_FP32, (f, i)
        assert s.cm.update() == s.oc.update()
        s.compare_cache(f"frame {f}")


@pytest.mark.parametrize("precision", ["exact", "fast"])
def test_converged_image_vs_fp64_oracle(gc, orc, torch_cuda, precision):
    """After convergence the FP32 CUDA image is within 1/255 of the
    double-precision restatement of the same method: every pixel for the exact
    build; for the fast build (FMA contraction, rsqrtf, hardware log2/exp2)
    all but FAST_OUTLIER_SHARE of the pixels, those where the accumulated
    alpha crosses the early-termination threshold one sample apart."""
    gc.render_precision(gc.RENDER_FAST if precision == "fast" else gc.RENDER_EXACT)
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 216)
    tf = scenario.ramp_tf()
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    W, H = 160, 128
    g, o = s.buffers(W, H)
    m = scenario.orbit_camera(gc, 3, 36, 3.2)
    for mode, sampler in ((0, 0), (0, 1), (1, 0)):
        v = s.view(m, W, H, tf_dev, 256, g, mode=mode, sampler=sampler)
        for f in range(12):
            for x in g:
                x.zero_()
            s.cm.render(v)
            conv = s.cm.update()
            if conv and f >= 1:
                break
        assert conv
        for x in g:
            x.zero_()
        s.cm.render(v)
        torch_cuda.cuda.synchronize()
        s.cm.update()
        r64 = np.zeros(W * H, np.uint32)
        scratch_u = np.zeros(s.oc.nslots, np.uint32)
        scratch_r = np.zeros(s.oc.nentries, np.uint32)
        # the oracle reads the GPU's converged page directory and pool
        s.cm.dump(gc.DUMP_MRPD, s.oc.mrpd())
        s.cm.dump(gc.DUMP_POOL, s.oc.pool())
        s.oc.render_f64(v, tf, r64, np.zeros(W * H), np.zeros(W * H * 4), scratch_u, scratch_r)
        d = rgba_diff(g[0].cpu().numpy(), r64).reshape(-1, 4).max(axis=1)
        if precision == "exact":
            assert d.max() <= RGBA_TOL_FP64, (mode, sampler, d.max())
        else:
            assert np.count_nonzero(d > RGBA_TOL_FP64) <= FAST_OUTLIER_SHARE * d.size, (mode, sampler, d.max())
        assert (g[0].cpu().numpy() >> 24).astype(bool).mean() > 0.05  # the image is not empty


def test_async_loader_converges_to_same_image(gc, orc, torch_cuda):
    """The asynchronous loader (bricks resolved on a host thread, uploaded by
    cudaMemcpyAsync on a side stream) reaches the image of the synchronous one."""
    imgs = []
    for sync in (True, False):
        s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 216, sync=sync)
        tf = scenario.ramp_tf()
        tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
        g, _ = s.buffers(96, 80)
        v = s.view(scenario.orbit_camera(gc, 2, 12, 3.0), 96, 80, tf_dev, 256, g)
        conv = False
        # the loader runs on its own thread: bound the loop by wall time, not frames
        t_end = time.time() + 20.0
        f = 0
        while time.time() < t_end:
            for x in g:
                x.zero_()
            s.cm.render(v)
            conv = s.cm.update()
            f += 1
            if conv and f > 3:
                break
            torch_cuda.cuda.synchronize()
            time.sleep(0.001)
        assert conv
        for x in g:
            x.zero_()
        s.cm.render(v)
        torch_cuda.cuda.synchronize()
        imgs.append(g[0].cpu().numpy())
        s.cm.close()
    assert np.array_equal(imgs[0], imgs[1])


def single_view_images(gc, orc, torch_cuda, specs, tf_dev):
    """Each view rendered alone to convergence through the plain frame loop."""
    single = []
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 64)
    status = torch_cuda.zeros(1, dtype=torch_cuda.int32, device="cuda")
    for (W, H), cam in specs:
        g, _ = s.buffers(W, H)
        v = s.view(scenario.orbit_camera(gc, cam, 12, 3.0), W, H, tf_dev, 256, g)
        v.status = status.data_ptr()
        for it in range(64):
            status.zero_()
            s.cm.render(v)
            s.cm.update()
            if int(status.item()) == 0:
                break
        assert int(status.item()) == 0
        single.append(g[0].cpu().numpy())
    s.cm.close()
    return single


def in_flight_marks(gc, cm, nentries):
    mrpd = np.zeros((nentries, 4), np.uint32)
    cm.dump(gc.DUMP_MRPD, mrpd)
    return int((mrpd[:, 3] == 3).sum())


@pytest.mark.parametrize("park,sync,reorder,overlap", [(0.0, True, 0, False), (0.0, False, 0, False),
                                                       (0.05, True, 0, False), (0.05, False, 4, False),
                                                       (0.0, True, 3, False), (0.0, False, 0, True),
                                                       (0.0, False, 4, True)])
def test_batch_scheduler_matches_single_views(gc, orc, torch_cuda, park, sync, reorder, overlap):
    """Continuous batching (admission by pixel budget, one persistent launch
    per tick, skipped passes for views that cannot progress, retirement on
    convergence) gives every view the image it gets when rendered alone to
    convergence, with the synchronous or the asynchronous loader, with
    arrival-order or locality-ordered admission, with views parked under
    memory pressure (a low park threshold parks views often; they resume from
    their progressive state) and with overlapped loads (bricks in flight are
    marked in the page directory; the marks are gone once the batch ends);
    the per-view status word reports convergence exactly."""
    specs = [((64, 48), 1), ((33, 17), 4), ((96, 80), 7), ((40, 40), 10), ((80, 24), 5)]
    tf_dev = torch_cuda.from_numpy(scenario.ramp_tf().reshape(-1)).cuda()
    single = single_view_images(gc, orc, torch_cuda, specs, tf_dev)

    s2 = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 64, sync=sync)
    b = gc.Batch(s2.cm, max_views=3, max_pixels=96 * 80 + 64 * 48, park_above=park, reorder_window=reorder,
                 overlap_loads=overlap)
    bufs = []
    for i, ((W, H), cam) in enumerate(specs):
        g, _ = s2.buffers(W, H)
        bufs.append(g)
        b.submit(s2.view(scenario.orbit_camera(gc, cam, 12, 3.0), W, H, tf_dev, 256, g), tag=100 + i)
    results = []
    for tick in range(4000):
        active, queued = b.tick()
        assert active <= 3
        results += b.poll()
        if len(results) == len(specs):
            break
    assert sorted(r[0] for r in results) == [100 + i for i in range(len(specs))]
    assert all(r[2] for r in results)
    torch_cuda.cuda.synchronize()
    for i in range(len(specs)):
        assert np.array_equal(bufs[i][0].cpu().numpy(), single[i]), i
    st = b.stats()
    assert st.graph_replays == st.render_ticks > 0  # every batched render replayed the graph
    if park > 0:
        assert st.parked > 0
    b.close()
    assert s2.cm.stats().device_error == 0
    assert in_flight_marks(gc, s2.cm, s2.oc.nentries) == 0


def test_overlapped_batch_argument_checks(gc, orc, torch_cuda):
    """Overlapped loads need the asynchronous loader and exclude parking."""
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 64, sync=True)
    with pytest.raises(gc.GcError, match="asynchronous loader"):
        gc.Batch(s.cm, overlap_loads=True)
    s.cm.close()
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 64, sync=False)
    with pytest.raises(gc.GcError, match="parking"):
        gc.Batch(s.cm, overlap_loads=True, park_above=0.5)
    s.cm.close()


@pytest.mark.parametrize("ticks", [1, 2, 3, 4, 6, 9])
def test_overlapped_batch_closed_mid_load(gc, orc, torch_cuda, ticks):
    """A batch with overlapped loads that ends while bricks are in flight
    installs or releases them: no page-directory entry stays marked, and the
    plain frame loop then renders a view to the image it gets alone, whichever
    of the two miss lists the batch used last."""
    specs = [((64, 48), 1), ((33, 17), 4), ((96, 80), 7)]
    tf_dev = torch_cuda.from_numpy(scenario.ramp_tf().reshape(-1)).cuda()
    single = single_view_images(gc, orc, torch_cuda, specs, tf_dev)
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 64, sync=False)
    b = gc.Batch(s.cm, max_views=2, max_pixels=1 << 16, overlap_loads=True)  # admissions while loads run
    for i, ((W, H), cam) in enumerate(specs):
        g, _ = s.buffers(W, H)
        b.submit(s.view(scenario.orbit_camera(gc, cam, 12, 3.0), W, H, tf_dev, 256, g), tag=i)
    for _ in range(ticks):
        b.tick()
    b.close()
    torch_cuda.cuda.synchronize()
    assert in_flight_marks(gc, s.cm, s.oc.nentries) == 0
    status = torch_cuda.zeros(1, dtype=torch_cuda.int32, device="cuda")
    (W, H), cam = specs[2]
    g, _ = s.buffers(W, H)
    v = s.view(scenario.orbit_camera(gc, cam, 12, 3.0), W, H, tf_dev, 256, g)
    v.status = status.data_ptr()
    for it in range(64):
        status.zero_()
        s.cm.render(v)
        s.cm.update()
        if int(status.item()) == 0:
            break
    assert int(status.item()) == 0
    assert np.array_equal(g[0].cpu().numpy(), single[2])
    assert s.cm.stats().device_error == 0


def test_coarser_level_fallback_preview(gc, orc, torch_cuda):
    """Preview mode of K_CacheManager::get: where a brick is missing a ray
    samples the first mapped coarser level instead of stopping.  With every
    brick resident it gives the normal image bit for bit; with only the
    coarse levels resident it covers more of the image than the first frame
    of the normal method and says so in status bit 1."""
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 216)
    tf_dev = torch_cuda.from_numpy(scenario.ramp_tf().reshape(-1)).cuda()
    st = torch_cuda.zeros(1, dtype=torch_cuda.int32, device="cuda")
    W, H = 80, 64

    def frame(m, fallback):
        g, _ = s.buffers(W, H)
        v = s.view(m, W, H, tf_dev, 256, g, fallback=fallback)
        v.status = st.data_ptr()
        st.zero_()
        s.cm.render(v)
        torch_cuda.cuda.synchronize()
        return g[0].cpu().numpy(), int(st.item())

    # a far view pages in the coarse levels only
    far = scenario.orbit_camera(gc, 2, 12, 9.0)
    for _ in range(12):
        _, stf = frame(far, 0)
        if s.cm.update() and stf == 0:
            break
    near = scenario.orbit_camera(gc, 2, 12, 2.2)
    img0, st0 = frame(near, 0)
    img1, st1 = frame(near, 1)
    assert st0 & 1 and st1 & 2  # normal rays stopped at missing bricks; the preview used coarse levels
    cover0, cover1 = ((img0 >> 24) > 0).mean(), ((img1 >> 24) > 0).mean()
    assert cover1 > cover0, (cover0, cover1)
    # converge the near view, then the preview equals the normal image
    for _ in range(30):
        _, stn = frame(near, 0)
        if s.cm.update() and stn == 0:
            break
    ref, stn = frame(near, 0)
    img2, st2 = frame(near, 1)
    assert stn == 0 and st2 == 0
    assert np.array_equal(ref, img2)


@pytest.mark.parametrize("mode,pt_block", [(0, 0), (1, 0), (0, 2)])
def test_coarser_level_fallback_matches_oracle(gc, orc, torch_cuda, mode, pt_block):
    """The preview mode against the oracle's restatement of the level walk of
    K_CacheManager::get (K_CacheManager.hpp:163-260): a missing brick is
    requested on the asked level only, the first mapped coarser level is
    sampled instead, an empty one ends the lookup.  Coarse levels are paged in
    by a far view, then a near view is previewed frame by frame (progressive
    buffers restarted each frame, as the mode requires): RGBA, t buffer,
    colour state and the cache state after every update equal the oracle's,
    with the one-level and the two-level page directory."""
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 60, pt_block=pt_block,
              pt_slots=64 if pt_block else 0)
    tf = scenario.ramp_tf() if mode == 0 else scenario.bumps_tf(4)
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    W, H = 72, 56
    g, o = s.buffers(W, H)
    far, near = scenario.orbit_camera(gc, 2, 12, 9.0), scenario.orbit_camera(gc, 2, 12, 2.2)
    coarse_frames = 0
    for f in range(14):
        m, fb = (far, 0) if f < 6 else (near, 1)
        for x in g:
            x.zero_()
        for x in o:
            x[:] = 0
        v = s.view(m, W, H, tf_dev, 256, g, mode=mode, fallback=fb)
        st = torch_cuda.zeros(1, dtype=torch_cuda.int32, device="cuda")
        v.status = st.data_ptr()
        s.cm.render(v)
        s.oc.render(v, tf, *o)
        torch_cuda.cuda.synchronize()
        coarse_frames += bool(int(st.item()) & 2)
        d = rgba_diff(g[0].cpu().numpy(), o[0])
        assert d.max() <= RGBA_TOL_FP32, f"frame {f}: RGBA off by {d.max()}"
        assert np.array_equal(g[1].cpu().numpy(), o[1]), f"frame {f}: t buffer"
        assert np.array_equal(g[2].cpu().numpy(), o[2]), f"frame {f}: colour state"
        assert s.cm.update() == s.oc.update(), f"frame {f}"
        s.compare_cache(f"frame {f}")
    assert coarse_frames > 0, "the near view never sampled a coarser level"


@pytest.mark.parametrize("case", ["inside", "one_pixel", "one_row", "miss", "bbox"])
def test_edge_views_match_oracle(gc, orc, torch_cuda, case):
    """Views at the edges of the method, frame by frame against the FP32
    oracle with the cache state: a camera inside the volume (rays start at
    t = 0), a 1x1 and a 97x1 image, a view that misses the volume (every pixel
    written as background), and a non-unit bounding box."""
    s = Scene(gc, orc, torch_cuda, (64, 48, 56), 1, 16, 1, (1, 1, 1), (6, 6, 6), 120)
    tf = scenario.ramp_tf()
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    W, H = {"one_pixel": (1, 1), "one_row": (97, 1)}.get(case, (45, 37))
    kw = {}
    if case == "inside":
        m = gc.look_at((0.2, 0.1, 0.3), (-0.5, 0.0, -0.6))
    elif case == "miss":
        m = gc.look_at((0.0, 0.0, 6.0), (0.0, 0.0, 12.0))  # looking away from the volume
    else:
        m = scenario.orbit_camera(gc, 1, 12, 2.8)
    if case == "bbox":
        kw = dict(bbox_min=(-1.2, -0.8, -1.0), bbox_max=(0.9, 1.1, 0.7))
    g, o = s.buffers(W, H)
    for f in range(8):
        v = s.view(m, W, H, tf_dev, 256, g, **kw)
        marched0 = s.cm.stats().rays_marched
        s.cm.render(v)
        s.oc.render(v, tf, *o)
        torch_cuda.cuda.synchronize()
        if f == 0 and case != "inside":  # a fresh frame marches exactly the rays that hit the box
            assert s.cm.stats().rays_marched - marched0 == int((o[1] > 0).sum()), case
        assert rgba_diff(g[0].cpu().numpy(), o[0]).max() <= RGBA_TOL_FP32, (case, f)
        assert np.array_equal(g[1].cpu().numpy(), o[1]) and np.array_equal(g[2].cpu().numpy(), o[2]), (case, f)
        assert s.cm.update() == s.oc.update(), (case, f)
        s.compare_cache(f"{case} frame {f}")
    if case == "miss":
        assert not (g[0].cpu().numpy() >> 24).any()
        assert s.cm.stats().rays_marched == 0
    if case == "inside":  # rays start inside the volume and advance through it
        assert (g[1].cpu().numpy() > 0).mean() > 0.5


def test_c1_orbit_matches_oracle(gc, orc, torch_cuda):
    """The c1 benchmark case at full size, as bench.py --config c1 runs it:
    256^3 u8 (seed 1, 8 blobs, sigma 10-40, amplitude 60-200, noise 20), B16,
    covering 1, 21^3 pool slots, 512^2 views on the 36-view orbit at 2.0x the
    diagonal (fov 45 deg), ramp transfer function, early termination at 0.99,
    8192 requests per cycle, every view rendered to convergence.  Every
    frame's RGBA, t buffer and colour state equal the FP32 oracle's, and the
    cache state (LRU, usage, requests, page directory, pool) equals the
    oracle's after every update."""
    import math

    import bench

    cfg = bench.CONFIGS["c1"]
    size, W, H = cfg["size"], cfg["W"], cfg["H"]
    vol = gc.volume_desc(size, cfg["B"], cfg["c"], 1, 1)
    layout = gc.compute_layout(vol)
    blobs = gc.generator_blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0],
                               cfg["amp"][1])
    d = torch_cuda.empty(size[0] * size[1] * size[2], dtype=torch_cuda.uint8, device="cuda")
    gc.generate_volume(gc.make_generator(size, 1, cfg["seed"], blobs, cfg["noise"]), d.data_ptr())
    store, offs, _ = gc.pre_process(vol, layout, d)
    ob = orc.blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0], cfg["amp"][1])
    ovol = orc.generate(size, 1, cfg["seed"], ob, cfg["nblobs"], cfg["noise"])
    ref, roffs = scenario.orc_store(orc, gc, ovol.reshape(-1).view(np.uint8), vol, layout)
    assert np.array_equal(store.numpy(), ref)
    s = Scene.__new__(Scene)
    s.gc, s.orc, s.torch, s.vol, s.layout = gc, orc, torch_cuda, vol, layout
    s.cm = gc.CacheManager(vol, layout, cfg["pool_slots"], max_requests=8192, sync_loader=True)
    s.cm.set_source_host(store, offs)
    s.oc = orc.Cache(s.cm.desc)
    s.oc.set_source(ref, roffs)
    tf = bench.tf_table(cfg["tf"])
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1).copy()).cuda()
    g, o = s.buffers(W, H)
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
    frames = 0
    for view in range(cfg["frames"]):
        m = bench.path_camera(gc.look_at, cfg, view)
        for x in g:
            x.zero_()
        for x in o:
            x[:] = 0
        v = s.view(m, W, H, tf_dev, tf.shape[0], g, focal=focal, early_alpha=cfg["early"])
        for it in range(64):
            s.cm.render(v)
            s.oc.render(v, tf, *o)
            torch_cuda.cuda.synchronize()
            tag = f"view {view} iteration {it}"
            d = rgba_diff(g[0].cpu().numpy(), o[0])
            assert d.max() <= RGBA_TOL_FP32, f"{tag}: RGBA off by {d.max()}"
            assert np.array_equal(g[1].cpu().numpy(), o[1]), f"{tag}: t buffer"
            assert np.array_equal(g[2].cpu().numpy(), o[2]), f"{tag}: colour state"
            c1, c2 = s.cm.update(), s.oc.update()
            assert c1 == c2, tag
            s.compare_cache(tag)
            frames += 1
            if c1:
                break
        assert c1, f"view {view} did not converge"
        assert (g[0].cpu().numpy() >> 24).astype(bool).mean() > 0.01  # the orbit sees the volume
    assert frames >= cfg["frames"] and s.cm.stats().device_error == 0
    s.cm.close()
