"""Two-level page directory (gc_cache_desc.pt_block, the page-table hierarchy
of CacheManager.hpp:151-236 with one table cache) in the oracle, on the CPU.

The hierarchy is defined to be transparent: while no table block in use is
evicted, brick entries, requests, usage words, LRU order and images equal
those of the one-level directory.  With a table pool too small for the
whole volume, blocks are evicted; the table state must stay consistent and
a view rendered again from a warm cache must equal the one-level image.
"""
import numpy as np
import pytest

import scenario


def make_pair(gc, orc, size, bpc, B, c, bb, pool, maxreq, pt_block, pt_slots):
    vol = gc.volume_desc(size, B, c, bpc, 1, bb)
    layout = gc.compute_layout(vol)
    o = scenario.orc_volume(orc, size, bpc, 21, 6)
    ref, roffs = scenario.orc_store(orc, gc, o.reshape(-1).view(np.uint8), vol, layout)
    caches = []
    for blk, slots in ((0, 0), (pt_block, pt_slots)):
        d = gc.CacheDesc(vol, layout, gc.u3(pool), maxreq, gc.CACHE_SYNC_LOADER, 0, blk, slots)
        oc = orc.Cache(d)
        oc.set_source(ref, roffs)
        caches.append(oc)
    return caches


def view(gc, m, W, H, **kw):
    return gc.make_view(m, W, H, 0, 256, 0, 0, 0, **kw)


def buffers(W, H):
    return np.zeros(W * H, np.uint32), np.zeros(W * H, np.float32), np.zeros(W * H * 4, np.float32)


def check_table_state(oc):
    """The table pool is consistent: each held block's directory word names
    its slot and the other words are unmapped; each mapped brick entry names
    a pool slot whose LRU record is that brick."""
    top, keys, table = oc.pt_top(), oc.pt_keys(), oc.pt_table()
    P = oc.pt_block
    held = {}
    for s in range(oc.pt_slots):
        k = keys[s]
        if k[3] == 0xFFFFFFFF:
            continue
        assert k[0] % P == 0 and k[1] % P == 0 and k[2] % P == 0
        held[s] = k
    mapped = np.nonzero(top & 1)[0]
    assert len(mapped) == len(held)
    assert sorted(int(top[w]) >> 1 for w in mapped) == sorted(held)
    lru = oc.lru()
    by_slot = {(int(r["cx"]), int(r["cy"]), int(r["cz"])): r for r in lru}
    nb = oc.desc.layout.nb_bricks
    for s, k in held.items():
        blk = table[s * P ** 3:(s + 1) * P ** 3]
        for j in np.nonzero(blk[:, 3] == 1)[0]:
            dx, dy, dz = j % P, (j // P) % P, j // (P * P)
            e = blk[j]
            r = by_slot[(int(e[0]), int(e[1]), int(e[2]))]
            lvl = int(k[3])
            assert int(r["level"]) == lvl
            got = (int(np.float32(r["vx"]) * np.float32(nb[lvl][0])), int(np.float32(r["vy"]) * np.float32(nb[lvl][1])),
                   int(np.float32(r["vz"]) * np.float32(nb[lvl][2])))
            assert got == (int(k[0]) + dx, int(k[1]) + dy, int(k[2]) + dz)


def test_two_level_directory_is_transparent(gc, orc):
    """A table pool holding every block: frame by frame the two-level cache
    renders the same images and keeps the same entries, requests, usage and
    LRU as the one-level cache (orbit with camera changes, evicting brick
    pool)."""
    one, two = make_pair(gc, orc, (64, 48, 56), 1, 8, 1, (1, 1, 1), (6, 6, 5), 40, 4, 1000)
    assert two.pt_block == 4 and two.pt_words < two.pt_slots
    tf = scenario.ramp_tf()
    W, H = 48, 40
    b1, b2 = buffers(W, H), buffers(W, H)
    for f in range(24):
        m = scenario.orbit_camera(gc, f // 6, 8, 2.4 + 0.25 * (f // 6))
        if f % 6 == 0:
            for x in b1 + b2:
                x[:] = 0
        v = view(gc, m, W, H)
        one.render(v, tf, *b1)
        two.render(v, tf, *b2)
        for a, b in zip(b1, b2):
            assert np.array_equal(a, b), f"frame {f}"
        assert one.update() == two.update(), f"frame {f}"
        assert np.array_equal(one.mrpd(), two.mrpd()), f"frame {f}"
        assert np.array_equal(one.requests(), two.requests()), f"frame {f}"
        assert np.array_equal(one.usage(), two.usage()), f"frame {f}"
        assert np.array_equal(one.lru(), two.lru()), f"frame {f}"
        check_table_state(two)
    assert (two.pt_top() & 1).sum() > 0


@pytest.mark.parametrize("pt_block,pt_slots", [(2, 300), (4, 60)])
def test_two_level_directory_evicting(gc, orc, pt_block, pt_slots):
    """A table pool that holds one view's blocks but not those of four views
    looking at different sides: the views evict each other's blocks.  The
    table state stays consistent after every update; each view converges in
    as many frames as with the one-level directory, and rendered again from
    scratch (twice) it converges in one frame, with the one-level image bit
    for bit."""
    one, two = make_pair(gc, orc, (96, 96, 96), 1, 8, 1, (1, 1, 1), (12, 12, 12), 100, pt_block, pt_slots)
    assert two.pt_slots < two.pt_words
    tf = scenario.ramp_tf()
    W, H = 40, 32
    replaced = 0
    for k, (az, el) in enumerate(((0, 10), (4, 10), (2, 60), (6, -40))):
        m = scenario.orbit_camera(gc, az, 8, 1.2, el)
        images, iters = [], []
        for oc in (one, two):
            its = []
            for p in range(3):
                b = buffers(W, H)
                for it in range(300):
                    oc.render(view(gc, m, W, H), tf, *b)
                    before = oc.pt_keys().copy() if oc is two else None
                    done = oc.update()
                    if oc is two:
                        after = oc.pt_keys()
                        replaced += int(np.sum((before[:, 3] != 0xFFFFFFFF) & np.any(before != after, axis=1)))
                        check_table_state(two)
                    if done:
                        break
                else:
                    pytest.fail(f"view {k} pass {p} did not converge")
                its.append(it)
            images.append(b)
            iters.append(its)
        assert iters[0] == iters[1], f"view {k}: frames to converge {iters}"
        assert iters[1][1:] == [0, 0], f"view {k}: a warm view needed loads {iters}"
        for a, b in zip(*images):
            assert np.array_equal(a, b), f"view {k}"
    assert replaced > 0, "no table block was evicted"


@pytest.mark.parametrize("size,B,c,P", [((64, 48, 56), 8, 1, 4), ((96, 96, 96), 16, 1, 2), ((200, 64, 33), 16, 2, 8),
                                        ((256, 256, 256), 32, 1, 16)])
def test_directory_geometry(gc, orc, size, B, c, P):
    """The directory of a two-level cache holds ceil(bricks / P) words per
    axis and level (CacheManager.hpp:160-176: realNumberOfEntries of the
    table level), levels packed along x, like the one-level directory."""
    vol = gc.volume_desc(size, B, c, 1, 1, (1, 1, 1))
    layout = gc.compute_layout(vol)
    d = gc.CacheDesc(vol, layout, gc.u3((4, 4, 4)), 16, gc.CACHE_SYNC_LOADER, 0, P, 8)
    oc = orc.Cache(d)
    nb = [tuple(layout.nb_bricks[l]) for l in range(layout.nb_levels)]
    words = [tuple(-(-n // P) for n in b) for b in nb]
    assert oc.pt_dims == (sum(w[0] for w in words), max(w[1] for w in words), max(w[2] for w in words))
    assert oc.pt_block == P and oc.pt_slots == 8
    assert oc.mrpd_dims == (sum(b[0] for b in nb), max(b[1] for b in nb), max(b[2] for b in nb))
    assert (oc.pt_top() == 0).all() and (oc.pt_keys() == 0xFFFFFFFF).all()
    assert list(oc.pt_order()) == list(range(8))
    oc.close()
