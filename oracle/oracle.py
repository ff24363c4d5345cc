"""ctypes binding of the CPU oracle (libgcoracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  The structures mirror include/gc_gb300.h; they
are declared here again so that the oracle does not depend on the product's
Python module.  Structures of the product module convert with `conv()`.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

MAX_LEVELS = 16
U3 = C.c_uint32 * 3
L3 = (C.c_uint32 * 3) * MAX_LEVELS


class VolumeDesc(C.Structure):
    _fields_ = [("size", U3), ("brick_size", C.c_uint32), ("big_brick_size", U3), ("covering", C.c_uint32),
                ("encoded_bytes", C.c_uint32), ("channels", C.c_uint32), ("downscale", U3)]


class Layout(C.Structure):
    _fields_ = [("nb_levels", C.c_uint32), ("initial", L3), ("real", L3), ("nb_bricks", L3),
                ("nb_big_bricks", L3), ("mip", L3)]


class Blob(C.Structure):
    _fields_ = [("cx", C.c_int32), ("cy", C.c_int32), ("cz", C.c_int32), ("k", C.c_uint64 * 3),
                ("r", C.c_int32 * 3), ("amplitude", C.c_int32)]


class Generator(C.Structure):
    _fields_ = [("size", U3), ("bytes_per_channel", C.c_uint32), ("channels", C.c_uint32),
                ("channel", C.c_uint32), ("field", C.c_uint32), ("seed", C.c_uint32),
                ("noise_amplitude", C.c_int32), ("nblobs", C.c_uint32), ("blobs", C.POINTER(Blob))]


class CacheDesc(C.Structure):
    _fields_ = [("volume", VolumeDesc), ("layout", Layout), ("cache_size", U3), ("max_requests", C.c_uint32),
                ("flags", C.c_uint32), ("gpu", C.c_int32), ("pt_block", C.c_uint32), ("pt_slots", C.c_uint32)]


class View(C.Structure):
    _fields_ = [("inv_view", C.c_float * 12), ("width", C.c_uint32), ("height", C.c_uint32),
                ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3), ("tstep", C.c_float),
                ("focal", C.c_float), ("early_alpha", C.c_float), ("mode", C.c_uint32), ("sampler", C.c_uint32),
                ("tf_width", C.c_uint32), ("tf", C.c_void_p), ("rgba", C.c_void_p), ("tbuf", C.c_void_p),
                ("state", C.c_void_p), ("status", C.c_void_p), ("volume", C.c_uint32), ("tf_height", C.c_uint32),
                ("fallback", C.c_uint32)]


LRU_DTYPE = np.dtype([("cx", "<u4"), ("cy", "<u4"), ("cz", "<u4"), ("level", "<u4"), ("vx", "<f4"),
                      ("vy", "<f4"), ("vz", "<f4")])

vp = C.c_void_p
P = C.POINTER
_SIGS = {
    "orc_blobs": ([C.c_uint32, C.c_uint32, P(C.c_uint32), C.c_float, C.c_float, C.c_int32, C.c_int32, P(Blob)],
                  C.c_int),
    "orc_generate": ([P(Generator), vp], None),
    "orc_layout": ([P(VolumeDesc), P(Layout)], C.c_int),
    "orc_mip_level": ([vp, vp, P(C.c_uint32), C.c_uint32, C.c_uint32], None),
    "orc_mip_level_mt": ([vp, vp, P(C.c_uint32), C.c_uint32, C.c_uint32, C.c_int], None),
    "orc_brick_level": ([vp, P(C.c_uint32), P(VolumeDesc), P(C.c_uint32), vp], None),
    "orc_empty": ([vp, C.c_uint64, C.c_uint64, C.c_uint32, C.c_float, vp], None),
    "orc_cache_create": ([P(CacheDesc)], vp),
    "orc_cache_destroy": ([vp], None),
    "orc_cache_set_source": ([vp, vp, P(C.c_uint64), P(C.c_uint64), C.c_size_t], None),
    "orc_cache_update": ([vp], C.c_int),
    "orc_lru_update": ([vp], None),
    "orc_request_list": ([vp, vp, C.c_uint32], C.c_uint32),
    "orc_completude": ([vp], C.c_float),
    "orc_timestamp": ([vp], C.c_uint32),
    "orc_set_timestamp": ([vp, C.c_uint32], None),
    "orc_mrpd": ([vp], vp), "orc_requests": ([vp], vp), "orc_usage": ([vp], vp),
    "orc_lru_records": ([vp], vp), "orc_pool": ([vp], vp),
    "orc_cache_dims": ([vp, P(C.c_uint32), P(C.c_uint32), P(C.c_uint64)], None),
    "orc_pt_dims": ([vp, P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)], None),
    "orc_pt_top": ([vp], vp), "orc_pt_table": ([vp], vp), "orc_pt_order": ([vp], vp),
    "orc_pt_usage": ([vp], vp), "orc_pt_keys": ([vp], vp),
    "orc_render": ([vp, P(View), vp, vp, vp, vp, C.c_int], None),
    "orc_render_f64": ([vp, P(View), vp, vp, vp, vp, vp, vp, C.c_int], None),
    "orc_pow": ([C.c_float, C.c_float], C.c_float),
    "orc_sample_normalized": ([vp, C.c_uint32, C.c_float, C.c_float, C.c_float, P(C.c_float)], C.c_int),
}


def _load():
    path = _build.build_oracle()
    lib = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


lib = _load()


def conv(cls, obj):
    """Re-type a structure of the product module (same C layout)."""
    return cls.from_buffer_copy(bytes(obj))


def ptr(a):
    return vp(a.ctypes.data)


def blobs(seed, n, size, smin, smax, amin, amax):
    arr = (Blob * max(1, n))()
    lib.orc_blobs(seed, n, U3(*size), smin, smax, amin, amax, arr)
    return arr


def generate(size, bpc, seed, blob_arr, nblobs, noise_amplitude, channels=1, channel=0, field=0, out=None):
    dt = np.uint8 if bpc == 1 else np.uint16
    if out is None:
        out = np.zeros((size[2], size[1], size[0], channels), dtype=dt)
    g = Generator(U3(*size), bpc, channels, channel, field, seed, noise_amplitude, nblobs, C.cast(blob_arr, P(Blob)))
    lib.orc_generate(C.byref(g), ptr(out))
    return out


def layout(vol):
    L = Layout()
    lib.orc_layout(C.byref(conv(VolumeDesc, vol)), C.byref(L))
    return L


def mip_level(src, dims, eb, nc, threads=1):
    """threads: host threads over the z pairs (<= 0: all)."""
    dt = src.dtype
    out = np.zeros(((dims[2] // 2) * (dims[1] // 2) * (dims[0] // 2) * eb) // dt.itemsize, dtype=dt)
    if threads == 1:
        lib.orc_mip_level(ptr(np.ascontiguousarray(src)), ptr(out), U3(*dims), eb, nc)
    else:
        lib.orc_mip_level_mt(ptr(np.ascontiguousarray(src)), ptr(out), U3(*dims), eb, nc, threads)
    return out


def brick_level(level, dims, vol, nb_big, out=None):
    """out: optional uint8 array (e.g. a slice of a whole store) receiving the bricks."""
    v = conv(VolumeDesc, vol)
    B = v.brick_size
    big = B ** 3 * v.big_brick_size[0] * v.big_brick_size[1] * v.big_brick_size[2] * v.encoded_bytes
    n = nb_big[0] * nb_big[1] * nb_big[2] * big
    if out is None:
        out = np.zeros(n, dtype=np.uint8)
    assert out.dtype == np.uint8 and out.size == n and out.flags.c_contiguous
    lib.orc_brick_level(ptr(np.ascontiguousarray(level)), U3(*dims), C.byref(v), U3(*nb_big), ptr(out))
    return out


def empty_flags(bricks, nbig, values_per_big, cb, threshold):
    flags = np.zeros(nbig, dtype=np.uint8)
    lib.orc_empty(ptr(bricks), nbig, values_per_big, cb, threshold, ptr(flags))
    return flags


class Cache:
    """Oracle cache state machine (the loader completes before the next frame)."""

    def __init__(self, desc):
        self.desc = conv(CacheDesc, desc)
        self.h = lib.orc_cache_create(C.byref(self.desc))
        md, ns, pb = U3(), C.c_uint32(), C.c_uint64()
        lib.orc_cache_dims(self.h, md, C.byref(ns), C.byref(pb))
        self.mrpd_dims = tuple(md)
        self.nslots = ns.value
        self.pool_bytes = pb.value
        self.nentries = md[0] * md[1] * md[2]
        td, ts_, tb = U3(), C.c_uint32(), C.c_uint32()
        lib.orc_pt_dims(self.h, td, C.byref(ts_), C.byref(tb))
        self.pt_dims, self.pt_slots, self.pt_block = tuple(td), ts_.value, tb.value
        self.pt_words = td[0] * td[1] * td[2]
        self._keep = []

    def set_source(self, bricks, level_offsets, empty_keys=()):
        offs = (C.c_uint64 * MAX_LEVELS)(*[int(o) for o in level_offsets])
        keys = (C.c_uint64 * max(1, len(empty_keys)))(*[int(k) for k in empty_keys])
        self._keep.append((bricks, offs, keys))
        lib.orc_cache_set_source(self.h, ptr(bricks), offs, keys, len(empty_keys))

    def update(self):
        return bool(lib.orc_cache_update(self.h))

    def lru_update(self):
        lib.orc_lru_update(self.h)

    def request_list(self, maxreq):
        out = np.zeros((maxreq, 4), dtype=np.uint32)
        n = lib.orc_request_list(self.h, ptr(out), maxreq)
        return n, out[: min(n, maxreq)]

    def completude(self):
        return lib.orc_completude(self.h)

    @property
    def timestamp(self):
        return lib.orc_timestamp(self.h)

    @timestamp.setter
    def timestamp(self, ts):
        lib.orc_set_timestamp(self.h, ts)

    def _arr(self, fn, dtype, count):
        p = fn(self.h)
        return np.ctypeslib.as_array(C.cast(p, P(np.ctypeslib.as_ctypes_type(dtype))), shape=(count,))

    def mrpd(self):
        return self._arr(lib.orc_mrpd, np.uint32, self.nentries * 4).reshape(-1, 4)

    def requests(self):
        return self._arr(lib.orc_requests, np.uint32, self.nentries)

    def usage(self):
        return self._arr(lib.orc_usage, np.uint32, self.nslots)

    def lru(self):
        raw = self._arr(lib.orc_lru_records, np.uint8, self.nslots * 28)
        return raw.view(LRU_DTYPE)

    def pool(self):
        return self._arr(lib.orc_pool, np.uint8, self.pool_bytes)

    # two-level directory state (the layouts of the GC_DUMP_PT_* dumps)
    def pt_top(self):
        return self._arr(lib.orc_pt_top, np.uint32, self.pt_words)

    def pt_table(self):
        return self._arr(lib.orc_pt_table, np.uint32, self.pt_slots * self.pt_block ** 3 * 4).reshape(-1, 4)

    def pt_order(self):
        return self._arr(lib.orc_pt_order, np.uint32, self.pt_slots)

    def pt_usage(self):
        return self._arr(lib.orc_pt_usage, np.uint32, self.pt_slots)

    def pt_keys(self):
        return self._arr(lib.orc_pt_keys, np.uint32, self.pt_slots * 4).reshape(-1, 4)

    def render(self, view, tf, rgba, tbuf, state, threads=0):
        v = conv(View, view)
        lib.orc_render(self.h, C.byref(v), ptr(tf), ptr(rgba), ptr(tbuf), ptr(state), threads)

    def render_f64(self, view, tf, rgba, tbuf, state, usage, req, threads=0):
        v = conv(View, view)
        lib.orc_render_f64(self.h, C.byref(v), ptr(tf), ptr(rgba), ptr(tbuf), ptr(state), ptr(usage), ptr(req),
                           threads)

    def sample_normalized(self, level, x, y, z):
        """(status, value) of one K_CacheManager::get_normalized sample."""
        out = C.c_float(-1.0)
        st = lib.orc_sample_normalized(self.h, level, x, y, z, C.byref(out))
        return st, out.value

    def close(self):
        if self.h:
            lib.orc_cache_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def pow_(x, k):
    return lib.orc_pow(x, k)
