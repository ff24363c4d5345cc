"""Two-level page directory on the GPU (gc_cache_desc.pt_block: the
page-table hierarchy of CacheManager.hpp:151-236 with one table cache)
against the oracle's restatement, frame by frame: images, t buffer, colour
state, converged flags, brick entries (flattened), LRU, usage, requests,
pool bytes and the table state (directory words, table blocks, table LRU,
table usage, block keys), with a roomy table pool and with pools small
enough that views evict each other's blocks.  A user kernel sampling through
the device view of a two-level cache matches the oracle too."""
import ctypes

import numpy as np
import pytest

import scenario
from test_gpu_device_view import user_lib  # noqa: F401  (fixture)
from test_gpu_render import RGBA_TOL_FP32, Scene, rgba_diff

pytestmark = pytest.mark.gpu

CASES = {
    # size, bpc, B, c, big brick, pool, maxreq, pt_block, pt_slots, W, H, tf, view kwargs
    "roomy_p4": ((64, 48, 56), 1, 8, 1, (1, 1, 1), (6, 6, 5), 40, 4, 1000, 48, 40, "ramp", dict()),
    "evicting_p2": ((96, 96, 96), 1, 8, 1, (1, 1, 1), (12, 12, 12), 100, 2, 300, 40, 32, "ramp", dict()),
    "evicting_p4_u16_mop": ((96, 96, 96), 2, 8, 1, (2, 1, 1), (12, 12, 12), 100, 4, 60, 40, 32, "bumps",
                            dict(mode=1, sampler=1, early_alpha=0.99)),
}
VIEWS = ((0, 10), (4, 10), (2, 60), (6, -40), (0, 10))


def compare_tables(s, tag):
    gc, oc, cm = s.gc, s.oc, s.cm
    for what, ref in ((gc.DUMP_PT_TOP, oc.pt_top()), (gc.DUMP_PT_POOL, oc.pt_table()), (gc.DUMP_PT_LRU, oc.pt_order()),
                      (gc.DUMP_PT_USAGE, oc.pt_usage()), (gc.DUMP_PT_KEYS, oc.pt_keys())):
        got = cm.dump(what, np.zeros_like(ref))
        assert np.array_equal(got, ref), (tag, what)


def run_views(s, torch, tf, W, H, kw, frames_per_view, check):
    tf_dev = torch.from_numpy(tf.reshape(-1).copy()).cuda()
    g, o = s.buffers(W, H)
    f = 0
    for k, (az, el) in enumerate(VIEWS):
        m = scenario.orbit_camera(s.gc, az, 8, 1.2, el)
        for x in g:
            x.zero_()
        for x in o:
            x[:] = 0
        for _ in range(frames_per_view):
            v = s.view(m, W, H, tf_dev, 256, g, **kw)
            s.cm.render(v)
            s.oc.render(v, tf, *o)
            torch.cuda.synchronize()
            d = rgba_diff(g[0].cpu().numpy(), o[0])
            assert d.max() <= RGBA_TOL_FP32, f"frame {f}: RGBA off by {d.max()}"
            assert np.array_equal(g[1].cpu().numpy(), o[1]), f"frame {f}: t buffer"
            assert np.array_equal(g[2].cpu().numpy(), o[2]), f"frame {f}: colour state"
            c1, c2 = s.cm.update(), s.oc.update()
            assert c1 == c2, f"frame {f}"
            if check:
                s.compare_cache(f"frame {f}")
                compare_tables(s, f"frame {f}")
            f += 1
            if c1:
                break
    return f


@pytest.mark.parametrize("case", sorted(CASES))
def test_two_level_loop_matches_oracle(gc, orc, torch_cuda, case):
    size, bpc, B, c, bb, pool, maxreq, P, slots, W, H, tfk, kw = CASES[case]
    s = Scene(gc, orc, torch_cuda, size, bpc, B, c, bb, pool, maxreq, pt_block=P, pt_slots=slots)
    assert s.cm.info.pt_block == P and s.cm.info.pt_slots == slots
    assert tuple(s.cm.info.pt_dims) == s.oc.pt_dims
    tf = scenario.ramp_tf() if tfk == "ramp" else scenario.bumps_tf(3)
    frames = run_views(s, torch_cuda, tf, W, H, kw, 80, True)
    assert frames > 20
    keys = s.oc.pt_keys()
    assert (keys[:, 3] != 0xFFFFFFFF).sum() > 0
    st = s.cm.stats()
    assert st.bricks_installed > 0 and st.device_error == 0


@pytest.mark.parametrize("scheduler", [0, 1])
def test_two_level_images_equal_one_level(gc, orc, torch_cuda, scheduler):
    """A roomy table pool is transparent on the GPU: both ray-caster
    schedulers render, frame by frame, what the one-level cache renders."""
    torch = torch_cuda
    size, bpc, B, c, bb, pool, maxreq = (64, 64, 64), 2, 16, 1, (1, 1, 1), (5, 5, 5), 60
    a = Scene(gc, orc, torch, size, bpc, B, c, bb, pool, maxreq)
    b = Scene(gc, orc, torch, size, bpc, B, c, bb, pool, maxreq, pt_block=2, pt_slots=4096)
    old = gc.render_tuning()
    try:
        gc.render_tuning(scheduler, 8, 128, 0)
        tf = scenario.bumps_tf(2)
        tf_dev = torch.from_numpy(tf.reshape(-1).copy()).cuda()
        W, H = 64, 48
        ga, _ = a.buffers(W, H)
        gb, _ = b.buffers(W, H)
        for f in range(18):
            m = scenario.orbit_camera(gc, f // 6, 6, 2.2)
            if f % 6 == 0:
                for x in ga + gb:
                    x.zero_()
            a.cm.render(a.view(m, W, H, tf_dev, 256, ga, sampler=1))
            b.cm.render(b.view(m, W, H, tf_dev, 256, gb, sampler=1))
            torch.cuda.synchronize()
            for x, y in zip(ga, gb):
                assert torch.equal(x, y), f"frame {f}"
            assert a.cm.update() == b.cm.update(), f"frame {f}"
    finally:
        gc.render_tuning(*old)


def test_user_kernel_two_level(gc, orc, torch_cuda, user_lib):  # noqa: F811
    """gc_sample_normalized through the device view of a two-level cache
    after an evicting run: statuses, values, usage stamps (pool and table)
    and requests equal the oracle's samples of the same state."""
    torch = torch_cuda
    s = Scene(gc, orc, torch, (96, 96, 96), 1, 8, 1, (1, 1, 1), (12, 12, 12), 100, pt_block=2, pt_slots=300)
    run_views(s, torch, scenario.ramp_tf(), 40, 32, {}, 6, False)
    s.compare_cache("after the frames")
    compare_tables(s, "after the frames")
    oc, cm = s.oc, s.cm
    v = cm.device_view()
    assert v.pt_shift == 1 and v.timestamp == cm.timestamp() == oc.timestamp
    rng = np.random.default_rng(9)
    n = 20000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.0, 0.99, (n, 3))
    pos[:, 3] = rng.integers(0, s.layout.nb_levels, n)
    d_pos = torch.from_numpy(pos).cuda()
    d_val = torch.zeros(n, dtype=torch.float32, device="cuda")
    d_st = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    assert user_lib.user_sample(ctypes.addressof(v), d_pos.data_ptr(), n, d_val.data_ptr(), d_st.data_ptr()) == 0
    want = [oc.sample_normalized(int(p[3]), float(p[0]), float(p[1]), float(p[2])) for p in pos]
    st, val = d_st.cpu().numpy(), d_val.cpu().numpy()
    want_st = np.array([w[0] for w in want])
    want_val = np.array([w[1] for w in want], np.float32)
    assert np.array_equal(st, want_st)
    mapped = st == 0
    assert mapped.any() and (st == 1).any(), "samples of resident and of missing bricks"
    assert np.array_equal(val[mapped], want_val[mapped])
    for what, ref in ((gc.DUMP_USAGE, oc.usage()), (gc.DUMP_REQUESTS, oc.requests()),
                      (gc.DUMP_PT_USAGE, oc.pt_usage())):
        got = cm.dump(what, np.zeros_like(ref))
        assert np.array_equal(got, ref), what


@pytest.mark.parametrize("sync", [True, False])
def test_two_level_batch_matches_single_views(gc, orc, torch_cuda, sync):
    """Continuous batching over a two-level cache (P = 2, a table pool for
    every block) gives every view the image it gets rendered alone through a
    one-level cache; overlapped loads are refused for a two-level cache."""
    from test_gpu_render import single_view_images

    specs = [((64, 48), 1), ((33, 17), 4), ((96, 80), 7), ((40, 40), 10), ((80, 24), 5)]
    tf_dev = torch_cuda.from_numpy(scenario.ramp_tf().reshape(-1)).cuda()
    single = single_view_images(gc, orc, torch_cuda, specs, tf_dev)
    s2 = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 64, sync=sync, pt_block=2,
               pt_slots=64)
    if not sync:
        with pytest.raises(gc.GcError, match="one-level page directory"):
            gc.Batch(s2.cm, overlap_loads=True)
    b = gc.Batch(s2.cm, max_views=3, max_pixels=96 * 80 + 64 * 48)
    bufs = []
    for i, ((W, H), cam) in enumerate(specs):
        g, _ = s2.buffers(W, H)
        bufs.append(g)
        b.submit(s2.view(scenario.orbit_camera(gc, cam, 12, 3.0), W, H, tf_dev, 256, g), tag=100 + i)
    results = []
    for _ in range(4000):
        b.tick()
        results += b.poll()
        if len(results) == len(specs):
            break
    assert sorted(r[0] for r in results) == [100 + i for i in range(len(specs))]
    assert all(r[2] for r in results)
    torch_cuda.cuda.synchronize()
    for i in range(len(specs)):
        assert np.array_equal(bufs[i][0].cpu().numpy(), single[i]), i
    b.close()
    assert s2.cm.stats().device_error == 0


def test_two_level_with_brick_bins(gc, torch_cuda):
    """Brick value bins over a two-level cache: with a table pool for every
    block the warm images equal the one-level cache's without bins; with a
    table pool that evicts (the bins of an evicted block's bricks revert to
    the user's), each view still converges within the reference's own
    resume spread of those images."""
    from test_gpu_brick_bins import IN_CORE, RESUME_TOL, SPECS, build, render_views
    from test_gpu_brick_bins import rgba_diff as bins_diff

    built = build(gc, torch_cuda, (96, 96, 96), 1, 16, 1, (1, 1, 1), empty_threshold=30.0)
    tf = scenario.ramp_tf()
    ref, _ = render_views(gc, torch_cuda, built, SPECS, tf, False, warm=True, cache=IN_CORE)
    roomy, sr = render_views(gc, torch_cuda, built, SPECS, tf, True, warm=True, cache=IN_CORE, pt_block=2,
                             pt_slots=512)
    small, ss = render_views(gc, torch_cuda, built, SPECS, tf, True, cache=IN_CORE, pt_block=2, pt_slots=16)
    for i in range(len(SPECS)):
        assert np.array_equal(ref[i], roomy[i]), i
        assert bins_diff(ref[i], small[i]).max() <= RESUME_TOL, i
    assert sr.device_error == 0 and ss.device_error == 0


def test_two_level_arguments_are_checked(gc, torch_cuda):
    """pt_block must be 0 or a power of two from 2 to 16, pt_slots at least 1."""
    vol = gc.volume_desc((64, 64, 64), 16, 1, 1, 1)
    layout = gc.compute_layout(vol)
    for blk, slots in ((3, 8), (32, 8), (1, 8)):
        with pytest.raises(gc.GcError, match="pt_block must be 0 or a power of two"):
            gc.CacheManager(vol, layout, (4, 4, 4), max_requests=16, pt_block=blk, pt_slots=slots)
    with pytest.raises(gc.GcError, match="pt_slots must be in"):
        gc.CacheManager(vol, layout, (4, 4, 4), max_requests=16, pt_block=4, pt_slots=0)
    cm = gc.CacheManager(vol, layout, (4, 4, 4), max_requests=16, pt_block=16, pt_slots=2)
    assert cm.info.pt_block == 16 and cm.info.pt_slots == 2
    cm.close()
