"""The reference's on-disk brick store: bricks.xml byte for byte against the
files the reference's own MetaData::write_bricks_xml produced (golden), brick
files round-tripped through LZ4, and files written by the reference's
process_bricking (compiled from its sources into oracle/_ref) read back by
this library.  Host code only: no kernel is launched."""
import os
import subprocess

import numpy as np
import pytest

import scenario

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "bricks_xml")
REFDRIVER = os.path.join(ROOT, "oracle", "_ref", "refdriver")

# (golden file, brick size, covering, encoded bytes, channels, size, big brick, empty keys)
XML_CASES = [("c1_u8.xml", 16, 1, 1, 1, (256, 256, 256), (1, 1, 1), ()),
             ("c5_u8x2.xml", 16, 2, 2, 2, (96, 80, 64), (2, 2, 2), (281474976776192, 65537))]


def need_lz4(gc):
    if not gc.lz4_available():
        pytest.skip("liblz4 is not installed")


@pytest.mark.parametrize("case", XML_CASES, ids=[c[0] for c in XML_CASES])
def test_bricks_xml_matches_reference(gc, tmp_path, case):
    name, B, c, eb, nc, size, bb, empty = case
    vol = gc.volume_desc(size, B, c, eb, nc, bb)
    layout = gc.compute_layout(vol)
    gc.write_bricks_xml(tmp_path, vol, layout, empty)
    path = tmp_path / f"bricks_{B}_{B}_{B}" / "bricks.xml"
    assert path.read_bytes() == open(os.path.join(GOLDEN, name), "rb").read()
    ini, real, keys = gc.read_bricks_xml(path)
    assert ini == [tuple(layout.initial[l]) for l in range(layout.nb_levels)]
    assert real == [tuple(layout.real[l]) for l in range(layout.nb_levels)]
    assert keys == list(empty)


@pytest.mark.parametrize("size,bpc,nc,B,c,bb", [((64, 48, 40), 1, 1, 16, 1, (1, 1, 1)),
                                                ((48, 40, 36), 1, 2, 16, 2, (2, 2, 2)),
                                                ((40, 40, 40), 2, 1, 8, 1, (2, 1, 1))])
def test_brick_files_round_trip(gc, orc, tmp_path, size, bpc, nc, B, c, bb):
    need_lz4(gc)
    vol = gc.volume_desc(size, B, c, bpc * nc, nc, bb)
    layout = gc.compute_layout(vol)
    o = scenario.orc_volume(orc, size, bpc, 3, 5, channels=nc)
    store, offs = scenario.orc_store(orc, gc, o.reshape(-1).view(np.uint8), vol, layout)
    gc.write_brick_files(tmp_path, vol, layout, store, offs, threads=4)
    back = np.zeros_like(store)
    gc.read_brick_files(tmp_path, vol, layout, back, offs, threads=3)
    assert np.array_equal(back, store)
    # a missing brick file is reported, not read as zeros
    victim = tmp_path / f"bricks_{B}_{B}_{B}" / "L0" / "L0_0_0_0.raw"
    victim.unlink()
    with pytest.raises(gc.GcError, match="missing brick file"):
        gc.read_brick_files(tmp_path, vol, layout, back, offs)


@pytest.mark.skipif(not os.path.exists(REFDRIVER), reason="reference driver not built (needs the reference sources)")
@pytest.mark.parametrize("dims,B,c,bb,eb,nc", [((70, 52, 36), 16, 1, (1, 1, 1), 1, 1),
                                               ((48, 40, 32), 16, 2, (2, 2, 2), 2, 2)])
def test_reads_brick_files_written_by_reference(gc, orc, tmp_path, dims, B, c, bb, eb, nc):
    """The reference's process_bricking writes a level's LZ4 brick files; this
    library reads them into exactly the bytes the reference wrote."""
    need_lz4(gc)
    rng = np.random.default_rng(11)
    vol_bytes = rng.integers(0, 256, size=dims[0] * dims[1] * dims[2] * eb, dtype=np.uint8)
    work = tmp_path / "ref"
    work.mkdir()
    (work / "vol.raw").write_bytes(vol_bytes.tobytes())
    out = tmp_path / "ref_bricks.bin"
    r = subprocess.run([REFDRIVER, "brick", str(work) + "/", "0", *map(str, dims), str(B), str(c), *map(str, bb),
                        str(eb), str(nc), "vol.raw", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nbig = tuple(int(v) for v in r.stdout.split())
    ref = np.fromfile(out, dtype=np.uint8)
    # a one-level layout naming the reference's big-brick grid
    vol = gc.volume_desc(dims, B, c, eb, nc, bb)
    layout = gc.Layout()
    layout.nb_levels = 1
    for a in range(3):
        layout.nb_big_bricks[0][a] = nbig[a]
    back = np.zeros_like(ref)
    gc.read_brick_files(work, vol, layout, back, [0])
    assert np.array_equal(back, ref)
