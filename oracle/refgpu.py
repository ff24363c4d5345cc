"""ctypes binding of the reference's own GPU code run headless
(oracle/_ref/librefgpu.so, built by oracle/build.py from a staged copy of the
reference's sources together with oracle/ref_gpu_driver.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/ and the reference-baseline legs of
bench.py, never by the product.  It pins the CUDA-only parts of the path --
mip pyramid, empty bricks, the GPU cache's state machine and the ray caster --
against the reference's implementation on the same inputs.

The reference keeps its configuration in a process-wide singleton and this
driver one open cache per process: use one RefGpu at a time.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

DUMP_MRPD, DUMP_LRU, DUMP_USAGE, DUMP_REQUESTS, DUMP_POOL = 0, 1, 2, 3, 4
LRU_DTYPE = np.dtype([("cx", "<u4"), ("cy", "<u4"), ("cz", "<u4"), ("level", "<u4"),
                      ("vx", "<f4"), ("vy", "<f4"), ("vz", "<f4")])

_lib = None


def available():
    """True when a staged copy of the reference exists (the harness can be built)."""
    return _build.reference_gpu_staged()


def load():
    """Build (if needed) and load librefgpu.so; raises when the build fails."""
    global _lib
    if _lib is None:
        path = _build.build_reference_gpu()
        if path is None:
            raise RuntimeError("no staged copy of the reference under oracle/_ref/src")
        lib = C.CDLL(path)
        lib.refgpu_last_error.restype = C.c_char_p
        u32p = C.POINTER(C.c_uint32)
        lib.refgpu_config_load.argtypes = [C.c_char_p]
        lib.refgpu_preprocess.argtypes = [C.c_float]
        lib.refgpu_mipmap.argtypes = []
        lib.refgpu_preprocess_timed.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.refgpu_open.argtypes = [C.c_char_p, u32p, C.c_int]
        lib.refgpu_render.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_float,
                                      C.POINTER(C.c_float), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.refgpu_update.argtypes = [C.POINTER(C.c_int), C.c_uint32]
        lib.refgpu_timestamp.argtypes = [u32p]
        lib.refgpu_info.argtypes = [u32p, u32p, u32p, u32p, u32p]
        lib.refgpu_dump.argtypes = [C.c_int, C.c_void_p, C.c_size_t]
        lib.refgpu_asked.argtypes = [u32p, C.c_uint32, u32p, u32p]
        lib.refgpu_completude.argtypes = [C.POINTER(C.c_float)]
        lib.refgpu_lod_tables.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), u32p]
        _lib = lib
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference: " + _lib.refgpu_last_error().decode())


def write_config(path, fields):
    """A configuration file in the reference's format (config/config_skull.cfg)."""
    with open(path, "w") as f:
        f.write("<Fields>\n")
        for k, v in fields.items():
            f.write(f'    <Field key="{k}" value="{v}"/>\n')
        f.write("</Fields>\n")


class RefGpu:
    """One volume preprocessed by the reference and, after open(), its
    CacheManager.  workdir receives <workdir>/vol/vol.raw (the level-0
    voxels), the reference's mipmap/ files, brick files and bricks.xml."""

    def __init__(self, workdir, size, brick_size, covering, encoded_bytes, big_brick=(1, 1, 1), channels=1):
        self.lib = load()
        self.workdir = os.path.join(os.path.abspath(workdir), "")
        self.voldir = os.path.join(self.workdir, "vol", "")
        self.size = tuple(size)
        self.B, self.c, self.eb = brick_size, covering, encoded_bytes
        self.cfg = os.path.join(self.workdir, "volume.cfg")
        os.makedirs(self.voldir, exist_ok=True)
        write_config(self.cfg, {
            "BrickSize": brick_size, "BigBrickSizeX": big_brick[0], "BigBrickSizeY": big_brick[1],
            "BigBrickSizeZ": big_brick[2], "VoxelCovering": covering, "NumberEncodedBytes": encoded_bytes,
            "NumberChannels": channels, "size_X": size[0], "size_Y": size[1], "size_Z": size[2],
            "downScale_X": 2, "downScale_Y": 2, "downScale_Z": 2,
            "WorkingDirectory": self.workdir, "VolumeFile": "vol.raw"})
        self.opened = False

    def preprocess(self, level0_bytes, empty_threshold=0.0):
        """Application::pre_process on these voxels: mip files, brick files,
        empty bricks with the threshold, bricks.xml."""
        with open(os.path.join(self.voldir, "vol.raw"), "wb") as f:
            f.write(np.ascontiguousarray(level0_bytes).tobytes())
        _check(self.lib.refgpu_config_load(self.cfg.encode()))
        _check(self.lib.refgpu_preprocess(C.c_float(empty_threshold)))

    def write_volume(self, level0_bytes):
        """The level-0 voxels as the reference's volume file."""
        with open(os.path.join(self.voldir, "vol.raw"), "wb") as f:
            f.write(np.ascontiguousarray(level0_bytes).tobytes())

    def mipmap(self):
        """Mipmapper::process alone on the volume file (the mip files)."""
        _check(self.lib.refgpu_config_load(self.cfg.encode()))
        _check(self.lib.refgpu_mipmap())

    def preprocess_timed(self):
        """Mipmapper::process then process_bricking of every level (LZ4 brick
        files, one thread per level) on the volume file; (mip s, bricking s)."""
        _check(self.lib.refgpu_config_load(self.cfg.encode()))
        m, b = C.c_double(0.0), C.c_double(0.0)
        _check(self.lib.refgpu_preprocess_timed(C.byref(m), C.byref(b)))
        return m.value, b.value

    def mip_level(self, level, dims):
        dt = np.uint8 if self.eb == 1 else np.uint16
        a = np.fromfile(os.path.join(self.voldir, "mipmap", f"L{level}.raw"), dtype=dt)
        assert a.size == dims[0] * dims[1] * dims[2], (level, a.size, dims)
        return a

    @property
    def bricks_xml(self):
        return os.path.join(self.voldir, f"bricks_{self.B}_{self.B}_{self.B}", "bricks.xml")

    def open(self, cache_size, gpu=0):
        _check(self.lib.refgpu_config_load(self.cfg.encode()))
        _check(self.lib.refgpu_open(self.cfg.encode(), (C.c_uint32 * 3)(*cache_size), gpu))
        self.opened = True
        md, cs, b, eb, nl = (C.c_uint32 * 3)(), (C.c_uint32 * 3)(), C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(self.lib.refgpu_info(md, cs, b, eb, nl))
        self.mrpd_dims = tuple(md)
        self.cache_size = tuple(cs)
        self.nlevels = nl.value
        self.nslots = cs[0] * cs[1] * cs[2]

    def close(self):
        if self.opened:
            _check(self.lib.refgpu_close())
            self.opened = False

    def render(self, inv_view, w, h, tstep, tf128, mode, rgba_ptr, tbuf_ptr, state_ptr):
        tf = np.ascontiguousarray(tf128, dtype=np.float32).reshape(-1)
        assert tf.size == 128 * 4, "the reference's transfer function has 128 RGBA samples"
        _check(self.lib.refgpu_render((C.c_float * 12)(*inv_view), w, h, C.c_float(tstep),
                                      tf.ctypes.data_as(C.POINTER(C.c_float)), mode, rgba_ptr, tbuf_ptr, state_ptr))

    def update(self, wait_ms=60000):
        conv = C.c_int()
        _check(self.lib.refgpu_update(C.byref(conv), wait_ms))
        return bool(conv.value)

    def timestamp(self):
        ts = C.c_uint32()
        _check(self.lib.refgpu_timestamp(C.byref(ts)))
        return ts.value

    def dump(self, what):
        if what == DUMP_MRPD:
            out = np.empty(self.mrpd_dims[0] * self.mrpd_dims[1] * self.mrpd_dims[2] * 4, np.uint32)
        elif what == DUMP_LRU:
            out = np.empty(self.nslots, LRU_DTYPE)
        elif what == DUMP_USAGE:
            out = np.empty(self.nslots, np.uint32)
        elif what == DUMP_REQUESTS:
            out = np.empty(self.mrpd_dims[0] * self.mrpd_dims[1] * self.mrpd_dims[2], np.uint32)
        elif what == DUMP_POOL:
            out = np.empty(self.nslots * self.B ** 3, np.uint8 if self.eb == 1 else np.uint16)
        else:
            raise ValueError(what)
        _check(self.lib.refgpu_dump(what, out.ctypes.data, out.nbytes))
        return out

    def asked(self, max_entries=4096):
        out = np.zeros(max_entries * 4, np.uint32)
        n, ne = C.c_uint32(), C.c_uint32()
        _check(self.lib.refgpu_asked(out.ctypes.data_as(C.POINTER(C.c_uint32)), max_entries, C.byref(n),
                                     C.byref(ne)))
        return out[:4 * min(n.value, max_entries)].reshape(-1, 4), ne.value

    def completude(self):
        f = C.c_float()
        _check(self.lib.refgpu_completude(C.byref(f)))
        return f.value

    def lod_tables(self):
        inv = np.zeros(64 * 3, np.float32)
        st = np.zeros(64, np.float32)
        n = C.c_uint32()
        _check(self.lib.refgpu_lod_tables(inv.ctypes.data_as(C.POINTER(C.c_float)),
                                          st.ctypes.data_as(C.POINTER(C.c_float)), C.byref(n)))
        return inv[:3 * n.value].reshape(-1, 3), st[:n.value]
