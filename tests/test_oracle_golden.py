"""The oracle pinned against outputs of the reference's own code.

Fixtures in tests/golden/ were produced by tests/golden/make_golden.py, which
compiles the reference's CPU sources (process_bricking, init_meta_data,
MetaData::write_bricks_xml) into oracle/_ref/refdriver and runs them on the
oracle's seeded synthetic volumes.
"""
import base64
import hashlib
import json
import os
import zlib

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def volume_of(orc, case):
    size, bpc, nch = tuple(case["size"]), case["bytes_per_channel"], case["channels"]
    b = orc.blobs(case["seed"], case["nblobs"], size, case["sigma"][0], case["sigma"][1], case["amp"][0],
                  case["amp"][1])
    vol = orc.generate(size, bpc, case["seed"], b, case["nblobs"], case["noise"], channels=nch, channel=0, field=0)
    for ch in range(1, nch):
        orc.generate(size, bpc, case["seed"] + ch, b, 0, case["noise"] * 4, channels=nch, channel=ch, field=1,
                     out=vol)
    return vol


@pytest.mark.parametrize("idx", range(len(load("layout.json")["layouts"])))
def test_layout_matches_reference(gc, orc, idx):
    g = load("layout.json")["layouts"][idx]
    v = gc.volume_desc(g["size"], g["B"], g["c"], g["eb"], g["nc"], g["bb"])
    for L in (gc.compute_layout(v), orc.layout(v)):
        assert L.nb_levels == len(g["levels"])
        for l, lv in enumerate(g["levels"]):
            assert list(L.initial[l]) == lv["initial"]
            assert list(L.real[l]) == lv["real"]
            assert list(L.nb_bricks[l]) == lv["nb_bricks"]
            assert list(L.nb_big_bricks[l]) == lv["nb_big_bricks"]


@pytest.mark.parametrize("name", [c["name"] for c in load("bricker.json")["cases"]])
def test_oracle_bricker_matches_reference(gc, orc, name):
    case = next(c for c in load("bricker.json")["cases"] if c["name"] == name)
    vol = volume_of(orc, case)
    assert hashlib.sha256(vol.tobytes()).hexdigest() == case["volume_sha256"]
    eb = case["bytes_per_channel"] * case["channels"]
    v = gc.volume_desc(case["size"], case["B"], case["c"], eb, case["channels"], case["bb"])
    bricks = orc.brick_level(vol, tuple(case["size"]), v, tuple(case["nb_big"]))
    assert bricks.size == case["bytes"]
    assert hashlib.sha256(bricks.tobytes()).hexdigest() == case["sha256"]
    if "bricks_zlib_b64" in case:
        ref = np.frombuffer(zlib.decompress(base64.b64decode(case["bricks_zlib_b64"])), dtype=np.uint8)
        assert np.array_equal(ref, bricks)


def general_bricks(vol, size, B, c, bb, nb_big, eb):
    """Independent numpy statement: voxel (lx,ly,lz) of small brick b is level
    voxel b*(B-2c) - c + l, zero outside the level; bricks starting outside the
    level are all zero."""
    X, Y, Z = size
    raw = vol.reshape(Z, Y, X, eb)
    Beff = B - 2 * c
    nbs = [nb_big[a] * bb[a] for a in range(3)]
    pad = np.zeros((nbs[2] * Beff + 2 * c + B, nbs[1] * Beff + 2 * c + B, nbs[0] * Beff + 2 * c + B, eb), raw.dtype)
    pad[c:c + Z, c:c + Y, c:c + X] = raw
    out = np.zeros((nb_big[2], nb_big[1], nb_big[0], bb[2] * B, bb[1] * B, bb[0] * B, eb), raw.dtype)
    for sz in range(nbs[2]):
        for sy in range(nbs[1]):
            for sx in range(nbs[0]):
                blk = pad[sz * Beff:sz * Beff + B, sy * Beff:sy * Beff + B, sx * Beff:sx * Beff + B]
                if sx * Beff >= X or sy * Beff >= Y or sz * Beff >= Z:
                    blk = np.zeros_like(blk)  # never visited by the reference's loops
                gz, gy, gx = sz // bb[2], sy // bb[1], sx // bb[0]
                iz, iy, ix = sz % bb[2], sy % bb[1], sx % bb[0]
                out[gz, gy, gx, iz * B:(iz + 1) * B, iy * B:(iy + 1) * B, ix * B:(ix + 1) * B] = blk
    return out.reshape(-1).view(np.uint8)


@pytest.mark.parametrize("name", ["u8_small", "u16_b32", "u8x2_c2_bb2", "u8_bb213"])
def test_bricker_general_formula_matches_reference(orc, name):
    """The closed form the GPU bricker implements equals the reference's loops."""
    case = next(c for c in load("bricker.json")["cases"] if c["name"] == name)
    vol = volume_of(orc, case)
    eb = case["bytes_per_channel"] * case["channels"]
    got = general_bricks(vol.reshape(-1).view(np.uint8).reshape(-1, eb), case["size"], case["B"], case["c"],
                         case["bb"], case["nb_big"], eb)
    assert hashlib.sha256(got.tobytes()).hexdigest() == case["sha256"]


@pytest.mark.parametrize("dims,eb,nc,dtype", [((64, 48, 32), 1, 1, np.uint8), ((40, 32, 16), 2, 1, np.uint16),
                                              ((32, 16, 8), 2, 2, np.uint8)])
def test_oracle_mip_threads_equal_one_thread(orc, dims, eb, nc, dtype):
    """The all-cores mip restatement (the CPU baseline's second figure) gives
    the single-thread result byte for byte."""
    rng = np.random.default_rng(3)
    n = dims[0] * dims[1] * dims[2] * eb // np.dtype(dtype).itemsize
    src = rng.integers(0, np.iinfo(dtype).max, size=n, dtype=dtype)
    assert np.array_equal(orc.mip_level(src, dims, eb, nc), orc.mip_level(src, dims, eb, nc, threads=0))


def test_brick_origins_never_alias():
    """The install finds a brick's page-directory entry from its float origin
    x / (V * (1 / (B - 2c))) + FLT_EPSILON (CacheManagerKernels.cu:75-86):
    for every brick count up to 4000 per axis and the brick sizes / coverings
    in use, distinct bricks land on distinct entries, so an install list
    (distinct requests) never names one entry twice.  The install's
    lowest-index-wins owner word (the serial order of reference_new_bricks)
    therefore only guards against lists that name an entry twice by hand."""
    import numpy as np

    f32 = np.float32
    eps = f32(1.1920928955078125e-7)
    for B, c in ((8, 1), (16, 0), (16, 1), (16, 2), (32, 1), (32, 2), (64, 1)):
        one_over = f32(1.0) / f32(B - 2 * c)
        for nb in range(1, 4001):
            x = np.arange(nb, dtype=np.float32)
            origin = (x / (f32(nb * (B - 2 * c)) * one_over)).astype(np.float32) + eps
            entry = (origin * f32(nb)).astype(np.float32).astype(np.int64)
            assert np.array_equal(entry, np.arange(nb)), (B, c, nb)
