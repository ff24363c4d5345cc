"""Launch configurations of the ray caster (tile vs per-lane pixel scheduler,
ray-tile shape, block size, blocks per SM) change only speed: images, t and
colour state are bit-identical, and the frame loop still matches the oracle."""
import numpy as np
import pytest

import scenario
from test_gpu_render import LOOP_CASES, RGBA_TOL_FP32, Scene, rgba_diff

pytestmark = pytest.mark.gpu


@pytest.fixture
def restore_tuning(gc):
    saved = gc.render_tuning()
    yield
    gc.render_tuning(*saved)


@pytest.mark.parametrize("tuning", [(0, 8, 128, 0), (1, 16, 256, 4), (0, 4, 64, 2), (1, 32, 128, 0)])
def test_loop_matches_oracle_under_tuning(gc, orc, torch_cuda, restore_tuning, tuning):
    gc.render_tuning(*tuning)
    size, bpc, B, c, bb, pool, maxreq, W, H, kw = LOOP_CASES["u16_mop_tri"]
    s = Scene(gc, orc, torch_cuda, size, bpc, B, c, bb, pool, maxreq)
    tf = scenario.bumps_tf(3)
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    g, o = s.buffers(W, H)
    for f in range(8):
        v = s.view(scenario.orbit_camera(gc, f // 4, 12, 2.8), W, H, tf_dev, 256, g, **kw)
        if f % 4 == 0:
            for x in g:
                x.zero_()
            for x in o:
                x[:] = 0
        s.cm.render(v)
        s.oc.render(v, tf, *o)
        torch_cuda.cuda.synchronize()
        assert rgba_diff(g[0].cpu().numpy(), o[0]).max() <= RGBA_TOL_FP32, (tuning, f)
        assert np.array_equal(g[1].cpu().numpy(), o[1]) and np.array_equal(g[2].cpu().numpy(), o[2])
        assert s.cm.update() == s.oc.update()
        s.compare_cache(f"{tuning} frame {f}")


def test_autotuner_candidates_render_identically(gc, orc, torch_cuda, restore_tuning):
    s = Scene(gc, orc, torch_cuda, (64, 64, 64), 1, 16, 1, (1, 1, 1), (6, 6, 6), 216)
    tf = scenario.ramp_tf()
    tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
    sizes = [(96, 80), (37, 29), (64, 64)]
    bufs = [s.buffers(W, H)[0] for W, H in sizes]
    views = [s.view(scenario.orbit_camera(gc, i * 4 + 1, 12, 3.0), W, H, tf_dev, 256, bufs[i])
             for i, (W, H) in enumerate(sizes)]

    def clear():
        for b in bufs:
            b[1].zero_()
            b[2].zero_()

    for _ in range(40):  # converge all three views
        clear()
        s.cm.render_batch(views)
        if s.cm.update():
            break
    ref = None
    for cand in gc.AUTOTUNE_CANDIDATES:
        gc.render_tuning(*cand)
        clear()
        s.cm.render_batch(views)
        torch_cuda.cuda.synchronize()
        imgs = [np.concatenate([b[0].cpu().numpy().view(np.uint8), b[1].cpu().numpy().view(np.uint8),
                                b[2].cpu().numpy().view(np.uint8)]) for b in bufs]
        if ref is None:
            ref = imgs
        for a, r in zip(imgs, ref):
            assert np.array_equal(a, r), cand
    best, timings = gc.autotune_render(s.cm, views, clear, candidates=gc.AUTOTUNE_CANDIDATES[:6], repeats=2)
    assert gc.render_tuning() == best and len(timings) == 6


@pytest.mark.parametrize("tf_kind,sampler", [("ramp", 0), ("bumps", 1), ("ramp", 1)])
def test_empty_space_skipping_changes_nothing(gc, orc, torch_cuda, tf_kind, sampler):
    """With empty-space skipping off and on, every frame's image, t buffer,
    colour state and cache state are identical (the loop is also checked
    against the oracle with skipping on, its default, by the tests above)."""
    runs = []
    try:
        for skip in (False, True):
            gc.render_empty_skip(skip)
            s = Scene(gc, orc, torch_cuda, (64, 64, 64), 2, 16, 1, (1, 1, 1), (6, 6, 6), 216)
            tf = scenario.ramp_tf() if tf_kind == "ramp" else scenario.bumps_tf(4)
            tf_dev = torch_cuda.from_numpy(tf.reshape(-1)).cuda()
            g, _ = s.buffers(72, 56)
            frames = []
            for f in range(10):
                if f % 5 == 0:
                    for x in g:
                        x.zero_()
                v = s.view(scenario.orbit_camera(gc, f // 5 + 1, 12, 2.4), 72, 56, tf_dev, 256, g, sampler=sampler,
                           early_alpha=0.99)
                s.cm.render(v)
                s.cm.update()
                torch_cuda.cuda.synchronize()
                lru = np.zeros(s.oc.nslots, dtype=s.oc.lru().dtype)
                s.cm.dump(gc.DUMP_LRU, lru)
                frames.append([x.cpu().numpy().copy() for x in g] + [lru])
            runs.append(frames)
            s.cm.close()
    finally:
        gc.render_empty_skip(True)
    for f, frames in enumerate(zip(*runs)):
        for k in range(4):
            assert all(np.array_equal(frames[0][k], other[k]) for other in frames[1:]), (f, k)
