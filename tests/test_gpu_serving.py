"""The serving form's shared pool: one cache over several volumes (levels of
all volumes in one page directory, one pool, one LRU) renders every view to
the image a cache holding that volume alone gives, alone or in a mix of
views of all volumes, with voxel widths that differ between the volumes.

Tolerance: 0 (bit-exact RGBA) -- the shared cache runs the same page walk,
sampling and compositing per view; only where bricks live in the pool
changes.
"""
import numpy as np
import pytest

import scenario

pytestmark = pytest.mark.gpu

# (size, bytes per voxel, seed): B16, covering 1 for all (a shared pool needs
# one brick size); the u16 volume makes the voxel widths differ
VOLUMES = [((64, 64, 64), 1, 21), ((48, 40, 56), 2, 5), ((80, 64, 48), 1, 9)]


def build(gc, torch, size, bpc, seed):
    vol = gc.volume_desc(size, 16, 1, bpc, 1)
    layout = gc.compute_layout(vol)
    d = scenario.gpu_volume(gc, torch, size, bpc, seed, 6)
    store, offs, _ = gc.pre_process(vol, layout, d)
    return vol, layout, store, offs


def views_of(gc, torch, tf_dev, specs):
    out = []
    for (v, (W, H), cam, dist) in specs:
        g = (torch.zeros(W * H, dtype=torch.int32, device="cuda"), torch.zeros(W * H, dtype=torch.float32, device="cuda"),
             torch.zeros(W * H * 4, dtype=torch.float32, device="cuda"))
        view = gc.make_view(scenario.orbit_camera(gc, cam, 12, dist), W, H, tf_dev.data_ptr(), 256, g[0].data_ptr(),
                            g[1].data_ptr(), g[2].data_ptr(), volume=v)
        out.append((view, g))
    return out


def run_batch(gc, cm, views, max_views):
    b = gc.Batch(cm, max_views=max_views, max_pixels=1 << 22)
    for i, (v, _) in enumerate(views):
        b.submit(v, tag=i)
    results = []
    for _ in range(4000):
        b.tick()
        results += b.poll()
        if len(results) == len(views):
            break
    b.close()
    assert len(results) == len(views) and all(r[2] for r in results)
    return results


@pytest.mark.parametrize("sync,pt_block", [(True, 0), (False, 0), (True, 2), (False, 4)])
def test_shared_pool_views_equal_single_volume_caches(gc, torch_cuda, sync, pt_block):
    """pt_block > 0: the shared cache with a two-level page directory (one
    directory word per pt_block^3 bricks of each volume's levels, a table pool
    for every block)."""
    torch = torch_cuda
    built = [build(gc, torch, *v) for v in VOLUMES]
    tf_dev = torch.from_numpy(scenario.ramp_tf().reshape(-1)).cuda()
    specs = [(0, (64, 48), 1, 3.0), (1, (33, 17), 4, 2.6), (2, (96, 80), 7, 3.2), (1, (40, 40), 10, 3.0),
             (0, (80, 24), 5, 2.8), (2, (56, 56), 2, 2.7), (1, (72, 64), 8, 3.4)]

    # reference images: each view through a cache of its volume alone (plain loop)
    alone = {}
    for k, (vol, layout, store, offs) in enumerate(built):
        cm = gc.CacheManager(vol, layout, (8, 8, 8), max_requests=128, sync_loader=True)
        cm.set_source_host(store, offs)
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        for i, (v, g) in enumerate(views_of(gc, torch, tf_dev, specs)):
            if specs[i][0] != k:
                continue
            v.volume = 0
            v.status = st.data_ptr()
            for _ in range(64):
                st.zero_()
                cm.render(v)
                cm.update()
                if int(st.item()) == 0:
                    break
            assert int(st.item()) == 0
            alone[i] = g[0].cpu().numpy()
        cm.close()

    # one shared pool; every view served in one mix (continuous batching)
    shared = [(vol, layout) for vol, layout, _, _ in built]
    cm = gc.CacheManager(built[0][0], built[0][1], (9, 9, 9), max_requests=128, sync_loader=sync, shared=shared,
                         pt_block=pt_block, pt_slots=1024 if pt_block else 0)
    for k, (_, _, store, offs) in enumerate(built):
        cm.set_source_host(store, offs, volume=k)
    bases = [cm.volume_levels(k) for k in range(len(built))]
    assert bases[0][0] == 0 and bases[1][0] == bases[0][1] and bases[2][0] == bases[1][0] + bases[1][1]
    views = views_of(gc, torch, tf_dev, specs)
    run_batch(gc, cm, views, max_views=4)
    torch.cuda.synchronize()
    for i, (_, g) in enumerate(views):
        assert np.array_equal(g[0].cpu().numpy(), alone[i]), i
    # the same views again, one at a time through the shared cache (warm pool)
    for i, spec in enumerate(specs):
        (v, g), = views_of(gc, torch, tf_dev, [spec])
        run_batch(gc, cm, [(v, g)], max_views=1)
        torch.cuda.synchronize()
        assert np.array_equal(g[0].cpu().numpy(), alone[i]), ("alone in the shared cache", i)
    st = cm.stats()
    assert st.device_error == 0 and st.bricks_installed > 0
    cm.close()


def test_shared_cache_rejects_mismatched_bricks(gc, torch_cuda):
    a = gc.volume_desc((64, 64, 64), 16, 1, 1, 1)
    b = gc.volume_desc((64, 64, 64), 8, 1, 1, 1)
    la, lb = gc.compute_layout(a), gc.compute_layout(b)
    with pytest.raises(gc.GcError, match="same BrickSize"):
        gc.CacheManager(a, la, (8, 8, 8), max_requests=64, shared=[(a, la), (b, lb)])
