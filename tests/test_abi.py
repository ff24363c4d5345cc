"""C-ABI surface and host logic (CPU only: no kernel is launched)."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gc_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(gc_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(gc):
    names = declared_functions()
    assert len(names) >= 30
    lib = ctypes.CDLL(gc.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python mirror binds exactly those
    assert set(names) == set(gc._SIGS), set(names) ^ set(gc._SIGS)


def test_version_and_errors(gc):
    assert b"sm_103a" in gc.lib.gc_version()
    bad = gc.VolumeDesc()
    with pytest.raises(gc.GcError, match="volume size"):
        gc.compute_layout(bad)


def test_config_file_roundtrip(gc, tmp_path):
    # the reference's own configuration format (config/config_skull.cfg)
    cfg = tmp_path / "vol.cfg"
    cfg.write_text("""<Fields>
    <Field key="BrickSize" value="16"/>
    <Field key="BigBrickSizeX" value="2"/> <Field key="BigBrickSizeY" value="2"/>
    <Field key="BigBrickSizeZ" value="2"/>
    <!-- <Field key="VoxelCovering" value="9"/> -->
    <Field key="VoxelCovering" value="2"/>
    <Field key="NumberEncodedBytes" value="2" /><Field key="NumberChannels" value="2" />
    <Field key="size_X" value="4096" /><Field key="size_Y" value="4096" /><Field key="size_Z" value="4096" />
    <Field key="downScale_X" value="2" /><Field key="downScale_Y" value="2" /><Field key="downScale_Z" value="2" />
    <Field key="Compositing" value="DVR" />
</Fields>""")
    c = gc.Configuration(cfg)
    assert c.get_field("Compositing") == "DVR"
    assert c.get_field("Missing") is None
    v = c.volume_desc()
    assert tuple(v.size) == (4096, 4096, 4096) and v.brick_size == 16 and v.covering == 2
    assert tuple(v.big_brick_size) == (2, 2, 2) and v.encoded_bytes == 2 and v.channels == 2
    c.add_field("BrickSize", "not-a-number")
    with pytest.raises(gc.GcError):
        c.volume_desc()
    c2 = gc.Configuration()
    c2.add_field("BrickSize", "16")
    with pytest.raises(gc.GcError, match="Missing BigBrickSizeX"):
        c2.volume_desc()
    with pytest.raises(gc.GcError):
        gc.Configuration(tmp_path / "absent.cfg")


def test_pool_dims_matches_reference_formula(gc):
    # Application.cu:79-93 with vram_size = 9500 MiB and the benchmark caps
    def ref(B, eb, vram):
        n = vram // (B ** 3 * eb)
        e = int(np.cbrt(float(n)))
        d = [e, e, e]
        a = 0
        while d[0] * d[1] * d[2] < n:
            d[a] += 1
            a = (a + 1) % 3
        return tuple(d)

    for (B, eb, vram) in [(16, 1, 9500 << 20), (16, 2, 2 << 30), (32, 2, 4 << 30), (16, 2, 8 << 30), (16, 1, 24 << 30)]:
        vol = gc.volume_desc((256, 256, 256), brick_size=B, encoded_bytes=eb, channels=1)
        assert gc.pool_dims(vol, vram) == ref(B, eb, vram)
    vol = gc.volume_desc((2048,) * 3, brick_size=32, encoded_bytes=2)
    assert gc.pool_dims(vol, 4 << 30) == (41, 40, 40)   # 65,600 slots, rounding over the cap
    vol = gc.volume_desc((2048,) * 3, brick_size=16, encoded_bytes=2)
    assert gc.pool_dims(vol, 2 << 30) == (64, 64, 64)


def test_brick_key_layout(gc):
    # get_key (BrickKey.cpp:15-25): uint16 {level, x, y, z} in memory order
    k = gc.brick_key(3, 17, 2, 65535)
    assert np.frombuffer(np.uint64(k).tobytes(), dtype=np.uint16).tolist() == [3, 17, 2, 65535]


def test_view_matrix_is_gl_rotation(gc):
    m = np.array(gc.view_matrix((30.0, -45.0), (0.1, -0.2, 3.0)), dtype=np.float64).reshape(3, 4)
    ax, ay = math.radians(-30.0), math.radians(45.0)
    rx = np.array([[1, 0, 0], [0, math.cos(ax), -math.sin(ax)], [0, math.sin(ax), math.cos(ax)]])
    ry = np.array([[math.cos(ay), 0, math.sin(ay)], [0, 1, 0], [-math.sin(ay), 0, math.cos(ay)]])
    r = rx @ ry
    assert np.allclose(m[:, :3], r, atol=1e-6)
    assert np.allclose(m[:, 3], r @ -np.array([0.1, -0.2, 3.0]), atol=1e-6)
    # eye at (0,0,d) looking down -z: origin = translation column
    m2 = np.array(gc.look_at((0.0, 0.0, 4.0)), dtype=np.float64).reshape(3, 4)
    assert np.allclose(m2[:, 3], [0, 0, 4]) and np.allclose(m2[:, 2], [0, 0, 1])


def tf_reference(points, samples):
    """TransferFunction::getSample (TransferFunction.cpp:127-157), float32."""
    f = np.float32
    out = np.zeros((samples, 4), dtype=np.float32)
    for i in range(samples):
        x = f(i) / f(samples)
        pos = next((j for j, p in enumerate(points) if f(p[0]) > x), len(points))
        prev = (0.0, 0.0, *points[0][2:]) if pos == 0 else points[pos - 1]
        nxt = (1.0, 0.0, *points[-1][2:]) if pos == len(points) else points[pos]
        t = (x - f(prev[0])) / (f(nxt[0]) - f(prev[0]))
        for k, (a, b) in enumerate(((prev[2], nxt[2]), (prev[3], nxt[3]), (prev[4], nxt[4]), (prev[1], nxt[1]))):
            out[i, k] = f(a) + (f(b) - f(a)) * t
    return out


def test_transfer_function_samples(gc):
    pts = [(0.20, 0.10, 0, 0, 1), (0.35, 0.70, 0, 1, 1), (0.45, 1.0, 0, 1, 0), (0.70, 1.0, 1, 1, 0), (1.0, 1.0, 1, 0, 0)]
    got = np.array(gc.TransferFunction.build(pts, 128), dtype=np.float32).reshape(-1, 4)
    assert np.array_equal(got, tf_reference(pts, 128))
    grey = np.array(gc.TransferFunction.greyRamp(128), dtype=np.float32).reshape(-1, 4)
    assert grey[0].tolist() == [0, 0, 0, 0] and abs(grey[127, 3] - 127 / 128) < 1e-6


def test_layout_product_equals_oracle(gc, orc):
    for size, B, c, bb, eb, nc in [((256,) * 3, 16, 1, (1, 1, 1), 1, 1), ((2048,) * 3, 32, 1, (1, 1, 1), 2, 1),
                                   ((97, 64, 33), 16, 2, (2, 1, 3), 2, 1), ((4096, 4096, 2048), 16, 1, (1, 1, 1), 1, 1)]:
        v = gc.volume_desc(size, B, c, eb, nc, bb)
        a, b = gc.compute_layout(v), orc.layout(v)
        assert bytes(a) == bytes(b)


# ctypes mirrors of the C structs (product binding, and the oracle's copies)
STRUCTS = {"gc_volume_desc": "VolumeDesc", "gc_layout": "Layout", "gc_blob": "Blob", "gc_generator": "Generator",
           "gc_cache_desc": "CacheDesc", "gc_cache_info": "CacheInfo", "gc_cache_stats": "CacheStats",
           "gc_view": "View", "gc_batch_desc": "BatchDesc", "gc_batch_stats": "BatchStats",
           "gc_batch_result": "BatchResult", "gc_tf_point": "TfPoint"}


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes structure has the size and field offsets the C compiler
    gives the header's struct (a mismatch would pass garbage through the ABI)."""
    import ctypes
    import shutil
    import subprocess

    import gcgb300 as gc

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gc_gb300.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, _ in getattr(gc, pyname)._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(ROOT, "include")
    subprocess.run(["gcc", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    c_layout = {(a, b): int(c) for a, b, c in (l.split() for l in out if l)}
    for cname, pyname in STRUCTS.items():
        cls = getattr(gc, pyname)
        assert ctypes.sizeof(cls) == c_layout[(cname, "sizeof")], cname
        for field, _ in cls._fields_:
            assert getattr(cls, field).offset == c_layout[(cname, field)], (cname, field)
    from oracle import oracle as orc

    for cname, pyname in (("gc_view", "View"), ("gc_cache_desc", "CacheDesc"), ("gc_volume_desc", "VolumeDesc"),
                          ("gc_layout", "Layout")):
        assert ctypes.sizeof(getattr(orc, pyname)) == c_layout[(cname, "sizeof")], ("oracle", cname)


def test_no_alloc_miss_list_rejects_misaligned_pointers(gc):
    """gc_miss_list_noalloc reads the request words and writes the list 16
    bytes at a time: pointers without that alignment are rejected before any
    device work (the addresses below are never dereferenced)."""
    vol = gc.volume_desc((64, 64, 64), 16, 1, 1, 1)
    layout = gc.compute_layout(vol)
    n = sum(layout.nb_bricks[l][0] for l in range(layout.nb_levels)) * layout.nb_bricks[0][1] * layout.nb_bricks[0][2]
    for req, lst, tot in ((0x10004, 0x20000, 0x30000), (0x10000, 0x20008, 0x30000), (0x10000, 0x20000, 0x30002)):
        with pytest.raises(gc.GcError, match="aligned") as e:
            gc.miss_list_noalloc(req, n, 1, layout, 50, lst, tot)
        assert e.value.code == 1  # GC_ERR_INVALID
