"""Brick value bins given to the cache (an extension of the reference's
cache): a missing brick whose values the transfer function cannot make
visible is stepped through instead of requested.

- the bins the device computes from the brick store equal a numpy
  restatement (min/max of each brick's voxels, covering included, as value
  bins of 64 over [0, 1], widened by one bin on either side);
- with a warm cache (no ray pauses) images are bit-identical with and
  without bins; fewer bricks are requested and loaded;
- from a cold cache, converged images stay within RESUME_TOL of the cache
  without bins.  The reference resumes a paused ray at
  origin + direction * t (RayCasters.cu:90, 107), not at the position it
  accumulated step by step, so its converged image depends, at the rounding
  level, on where each ray paused -- on the request history.  Bins change
  that history as a cold cache does against a warm one: the no-bins path
  itself differs from its own warm image by the same amount.

Tolerances: 0 (warm, bit-exact RGBA) and RESUME_TOL = 2/255 per channel
(cold, the plain loop on these seeded views: the spread the no-bins path
shows against its own warm image).  Histories can spread further (a batched
cold run showed 4/255 in one pixel), so batched views are checked warm.
"""
import numpy as np
import pytest

import scenario

pytestmark = pytest.mark.gpu


def numpy_bins(store, offs, vol, layout):
    B, bb, eb = vol.brick_size, tuple(vol.big_brick_size), vol.encoded_bytes
    dt = {1: np.uint8, 2: np.uint16}[eb]
    scale = np.float32(1.0 / 255.0) if eb == 1 else np.float32(1.0 / 65535.0)
    raw = store.numpy() if hasattr(store, "numpy") else store
    out = []
    for l in range(layout.nb_levels):
        nbig, nb = tuple(layout.nb_big_bricks[l]), tuple(layout.nb_bricks[l])
        bv = (bb[0] * B, bb[1] * B, bb[2] * B)
        n = nbig[0] * nbig[1] * nbig[2]
        a = raw[offs[l]:offs[l] + n * bv[0] * bv[1] * bv[2] * eb].view(dt)
        a = a.reshape(nbig[2], nbig[1], nbig[0], bv[2], bv[1], bv[0]).transpose(0, 3, 1, 4, 2, 5)
        full = a.reshape(nbig[2] * bv[2], nbig[1] * bv[1], nbig[0] * bv[0])
        bricks = full[:nb[2] * B, :nb[1] * B, :nb[0] * B].reshape(nb[2], B, nb[1], B, nb[0], B)
        lo = bricks.min(axis=(1, 3, 5)).astype(np.float32) * scale
        hi = bricks.max(axis=(1, 3, 5)).astype(np.float32) * scale

        def binof(x):
            return np.clip(np.floor(x * np.float32(64.0)), 0, 63).astype(np.int64)

        b0 = np.maximum(binof(lo) - 1, 0)
        b1 = np.minimum(binof(hi) + 1, 63)
        upto = np.where(b1 >= 63, np.uint64(0xFFFFFFFFFFFFFFFF),
                        (np.uint64(1) << (b1 + 1).astype(np.uint64)) - np.uint64(1))
        mask = upto & ~((np.uint64(1) << b0.astype(np.uint64)) - np.uint64(1))
        out.append(mask.reshape(-1))
    return np.concatenate(out)


def build(gc, torch, size, bpc, B, c, bb, seed=21, nblobs=6, empty_threshold=None, channels=1):
    vol = gc.volume_desc(size, B, c, bpc * channels, channels, bb)
    layout = gc.compute_layout(vol)
    d = scenario.gpu_volume(gc, torch, size, bpc, seed, nblobs, channels=channels)
    bins = []
    store, offs, empty = gc.pre_process(vol, layout, d, empty_threshold=empty_threshold, value_bins=bins)
    return vol, layout, store, offs, empty, bins[0]


@pytest.mark.parametrize("size,bpc,B,c,bb", [((64, 48, 40), 1, 16, 1, (1, 1, 1)), ((72, 56, 48), 2, 16, 2, (2, 2, 1)),
                                             ((96, 80, 64), 1, 8, 1, (2, 2, 2))])
def test_device_bins_match_numpy(gc, torch_cuda, size, bpc, B, c, bb):
    vol, layout, store, offs, _, bins = build(gc, torch_cuda, size, bpc, B, c, bb)
    ref = numpy_bins(store, offs, vol, layout)
    assert bins.shape == ref.shape
    assert np.array_equal(bins, ref)
    # a two-channel volume is never skipped
    vol2, layout2, _, _, _, bins2 = build(gc, torch_cuda, (48, 40, 36), 1, 16, 2, (2, 2, 2), channels=2)
    assert (bins2 == np.uint64(0xFFFFFFFFFFFFFFFF)).all()


def converge(cm, v, st, cap=96):
    for _ in range(cap):
        st.zero_()
        cm.render(v)
        cm.update()
        if int(st.item()) == 0:
            return True
    return False


def render_views(gc, torch, built, specs, tf, use_bins, sync=True, mode=0, warm=False, cache=(6, 6, 6), **cache_kw):
    """Each view to convergence (plain frame loop); warm: then once more from
    cleared buffers, with every brick it needs resident (no ray pauses)."""
    vol, layout, store, offs, empty, bins = built
    cm = gc.CacheManager(vol, layout, cache, max_requests=96, sync_loader=sync, **cache_kw)
    cm.set_source_host(store, offs, empty)
    if use_bins:
        cm.set_brick_bins(bins)
    tf_dev = torch.from_numpy(tf.reshape(-1)).cuda()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    imgs = []
    for (W, H), cam, dist in specs:
        g = (torch.zeros(W * H, dtype=torch.int32, device="cuda"), torch.zeros(W * H, dtype=torch.float32, device="cuda"),
             torch.zeros(W * H * 4, dtype=torch.float32, device="cuda"))
        v = gc.make_view(scenario.orbit_camera(gc, cam, 12, dist), W, H, tf_dev.data_ptr(), 256, g[0].data_ptr(),
                         g[1].data_ptr(), g[2].data_ptr(), mode=mode)
        v.status = st.data_ptr()
        assert converge(cm, v, st)
        if warm:
            for x in g:
                x.zero_()
            st.zero_()
            cm.render(v)
            cm.update()
            assert int(st.item()) == 0  # no brick was missing: no ray paused
        imgs.append(g[0].cpu().numpy())
    s = cm.stats()
    assert s.device_error == 0
    cm.close()
    return imgs, s


def rgba_diff(a, b):
    return np.abs(a.view(np.uint8).astype(np.int32) - b.view(np.uint8).astype(np.int32))


RESUME_TOL = 2
SPECS = [((64, 48), 1, 3.0), ((80, 80), 4, 2.2), ((96, 64), 7, 1.6), ((48, 48), 10, 3.4)]
IN_CORE = (8, 8, 8)  # holds every brick of the 96^3 scene


@pytest.mark.parametrize("empty_threshold", [None, 30.0])
def test_bins_warm_images_identical_fewer_loads(gc, torch_cuda, empty_threshold):
    built = build(gc, torch_cuda, (96, 96, 96), 1, 16, 1, (1, 1, 1), empty_threshold=empty_threshold)
    if empty_threshold is not None:
        assert len(built[4]) > 0  # some big bricks are empty (they are requested either way)
    tf = scenario.ramp_tf()  # alpha 0 below 40/255: low-valued bricks are invisible
    a, sa = render_views(gc, torch_cuda, built, SPECS, tf, False, warm=True, cache=IN_CORE)
    b, sb = render_views(gc, torch_cuda, built, SPECS, tf, True, warm=True, cache=IN_CORE)
    for i in range(len(SPECS)):
        assert np.array_equal(a[i], b[i]), i
    assert sb.requests_raised < sa.requests_raised
    assert sb.bricks_installed + sb.bricks_empty < sa.bricks_installed + sa.bricks_empty


def test_bins_cold_images_within_resume_rounding(gc, torch_cuda):
    built = build(gc, torch_cuda, (96, 96, 96), 1, 16, 1, (1, 1, 1))
    tf = scenario.ramp_tf()
    cold, _ = render_views(gc, torch_cuda, built, SPECS, tf, False)
    warm, _ = render_views(gc, torch_cuda, built, SPECS, tf, False, warm=True, cache=IN_CORE)
    bins, sb = render_views(gc, torch_cuda, built, SPECS, tf, True)
    for i in range(len(SPECS)):
        assert rgba_diff(cold[i], warm[i]).max() <= RESUME_TOL, i  # the reference's own spread
        assert rgba_diff(cold[i], bins[i]).max() <= RESUME_TOL, i
        assert rgba_diff(warm[i], bins[i]).max() <= RESUME_TOL, i
    assert sb.device_error == 0


def test_bins_leave_max_opacity_alone(gc, torch_cuda):
    """Maximum opacity projection takes every sample: nothing is skipped."""
    built = build(gc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1))
    tf = scenario.ramp_tf()
    a, sa = render_views(gc, torch_cuda, built, SPECS[:2], tf, False, mode=gc.MODE_MOP)
    b, sb = render_views(gc, torch_cuda, built, SPECS[:2], tf, True, mode=gc.MODE_MOP)
    for i in range(2):
        assert np.array_equal(a[i], b[i]), i
    assert sb.bricks_installed == sa.bricks_installed


@pytest.mark.parametrize("overlap", [False, True])
def test_bins_batched_views_warm_identical(gc, torch_cuda, overlap):
    """The batched form steps through the unloaded invisible bricks exactly
    like the plain path: with the visible bricks resident (a cache warmed by
    the plain loop with bins), no ray pauses and every batched view equals
    its warm image without bins bit for bit."""
    built = build(gc, torch_cuda, (96, 96, 96), 1, 16, 1, (1, 1, 1))
    tf = scenario.ramp_tf()
    ref, _ = render_views(gc, torch_cuda, built, SPECS, tf, False, warm=True, cache=IN_CORE)
    vol, layout, store, offs, empty, bins = built
    cm = gc.CacheManager(vol, layout, IN_CORE, max_requests=96, sync_loader=False)
    cm.set_source_host(store, offs, empty)
    cm.set_brick_bins(bins)
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    st = torch_cuda.zeros(1, dtype=torch_cuda.int32, device="cuda")

    def buffers(W, H):
        return tuple(torch_cuda.zeros(n, dtype=dt, device="cuda")
                     for n, dt in ((W * H, torch_cuda.int32), (W * H, torch_cuda.float32),
                                   (W * H * 4, torch_cuda.float32)))

    def view(i, g):
        (W, H), cam, dist = SPECS[i]
        return gc.make_view(scenario.orbit_camera(gc, cam, 12, dist), W, H, tf_dev.data_ptr(), 256, g[0].data_ptr(),
                            g[1].data_ptr(), g[2].data_ptr())

    for i, ((W, H), _, _) in enumerate(SPECS):  # warm the cache through the plain loop
        v = view(i, buffers(W, H))
        v.status = st.data_ptr()
        assert converge(cm, v, st)
    b = gc.Batch(cm, max_views=3, max_pixels=1 << 16, overlap_loads=overlap)
    bufs = []
    for i, ((W, H), _, _) in enumerate(SPECS):
        bufs.append(buffers(W, H))
        b.submit(view(i, bufs[-1]), tag=i)
    results = []
    for _ in range(4000):
        b.tick()
        results += b.poll()
        if len(results) == len(SPECS):
            break
    b.close()
    assert len(results) == len(SPECS) and all(r[2] for r in results)
    assert all(r[1] == 1 for r in results)  # one pass each: nothing was missing
    torch_cuda.cuda.synchronize()
    for i, g in enumerate(bufs):
        assert np.array_equal(g[0].cpu().numpy(), ref[i]), i
    assert cm.stats().device_error == 0
    cm.close()


def test_bins_count_is_checked(gc, torch_cuda):
    built = build(gc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1))
    vol, layout, store, offs, empty, bins = built
    cm = gc.CacheManager(vol, layout, (6, 6, 6), max_requests=96)
    with pytest.raises(gc.GcError, match="brick bins"):
        cm.set_brick_bins(bins[:-1])
    cm.set_brick_bins(bins)
    cm.set_brick_bins(None)  # removed
    cm.close()


def test_bins_set_and_removed_mid_run(gc, torch_cuda):
    """Bins given after bricks are resident, then taken away: the per-entry
    table is rebuilt each time (resident bricks keep their own bins) and the
    warm image stays the same bit for bit."""
    built = build(gc, torch_cuda, (96, 96, 96), 1, 16, 1, (1, 1, 1))
    vol, layout, store, offs, empty, bins = built
    tf = scenario.ramp_tf()
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    cm = gc.CacheManager(vol, layout, IN_CORE, max_requests=96)
    cm.set_source_host(store, offs, empty)
    st = torch_cuda.zeros(1, dtype=torch_cuda.int32, device="cuda")
    (W, H), cam, dist = SPECS[2]
    g = (torch_cuda.zeros(W * H, dtype=torch_cuda.int32, device="cuda"),
         torch_cuda.zeros(W * H, dtype=torch_cuda.float32, device="cuda"),
         torch_cuda.zeros(W * H * 4, dtype=torch_cuda.float32, device="cuda"))
    v = gc.make_view(scenario.orbit_camera(gc, cam, 12, dist), W, H, tf_dev.data_ptr(), 256, g[0].data_ptr(),
                     g[1].data_ptr(), g[2].data_ptr())
    v.status = st.data_ptr()

    def warm_image():
        assert converge(cm, v, st)
        for x in g:
            x.zero_()
        st.zero_()
        cm.render(v)
        cm.update()
        assert int(st.item()) == 0
        return g[0].cpu().numpy()

    ref = warm_image()
    cm.set_brick_bins(bins)
    assert np.array_equal(warm_image(), ref)
    cm.set_brick_bins(None)
    assert np.array_equal(warm_image(), ref)
    assert cm.stats().device_error == 0
    cm.close()
