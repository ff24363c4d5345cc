"""Python host mirror of the GB300 out-of-core volume path.

Binds the C ABI of libgcgb300.so (include/gc_gb300.h) with ctypes and wraps it
in classes named after the reference's interface:

  Configuration          GcCore/include/GcCore/libData/Configuration.hpp:18-87
  compute_layout         Mipmapper::fill_metaData + init_meta_data
  Mipmapper              GcCore/include/GcCore/cuda/libPreprocessor/Mipmapper.hpp:35-108
  process_bricking       GcCore/include/GcCore/libPreprocessor/Bricker_v2.hpp:13-41
  CacheManager           GcCore/include/GcCore/cuda/libGPUCache/CacheManager.hpp:38-128
  TransferFunction       Applications/DVR-ray-caster/src/TransferFunction.cpp:16-157

Device memory, streams and events come from PyTorch (plumbing only): every
function takes raw device pointers (int) and a cudaStream_t (int, 0 = legacy
stream).  Errors raise GcError with the library's message.  There is no
fallback: if the shared library is missing, importing this module fails.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgcgb300.so")

MAX_LEVELS = 16
OK = 0
BRICK_SUCCESS, BRICK_UNKNOWN, BRICK_EMPTY = 0, 1, 2
MODE_DVR, MODE_MOP = 0, 1
SAMPLER_REFERENCE, SAMPLER_TRILINEAR = 0, 1
CACHE_SYNC_LOADER = 1
CACHE_STAGED_UPLOAD = 2
DUMP_MRPD, DUMP_LRU, DUMP_USAGE, DUMP_REQUESTS, DUMP_POOL = 0, 1, 2, 3, 4
DUMP_PT_TOP, DUMP_PT_POOL, DUMP_PT_LRU, DUMP_PT_USAGE, DUMP_PT_KEYS = 5, 6, 7, 8, 9
MISS_LIST_FAILED = 0xFFFFFFFF  # gc_miss_list_noalloc: a bounded wait of the scan ran out

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


class CacheInfo(C.Structure):
    _fields_ = [("mrpd_dims", U3), ("nb_slots", C.c_uint32), ("slot_voxels", C.c_uint32),
                ("level_offset", C.c_uint32 * MAX_LEVELS), ("pool_bytes", C.c_uint64), ("pt_block", C.c_uint32),
                ("pt_slots", C.c_uint32), ("pt_dims", U3), ("pt_level_offset", C.c_uint32 * MAX_LEVELS)]


class CacheStats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("requests_raised", C.c_uint64), ("requests_served", C.c_uint64),
                ("bricks_installed", C.c_uint64), ("bricks_empty", C.c_uint64), ("bytes_h2d", C.c_uint64),
                ("load_errors", C.c_uint64), ("last_requests", C.c_uint32), ("last_used", C.c_uint32),
                ("device_error", C.c_uint32), ("load_cycles", C.c_uint64), ("loader_host_ns", C.c_uint64),
                ("upload_ns", C.c_uint64), ("upload_direct", C.c_uint32), ("samples", C.c_uint64),
                ("rays_marched", C.c_uint64)]


class View(C.Structure):
    _fields_ = [("inv_view", C.c_float * 12), ("width", C.c_uint32), ("height", C.c_uint32),
                ("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3), ("tstep", C.c_float),
                ("focal", C.c_float), ("early_alpha", C.c_float), ("mode", C.c_uint32), ("sampler", C.c_uint32),
                ("tf_width", C.c_uint32), ("tf", C.c_void_p), ("rgba", C.c_void_p), ("tbuf", C.c_void_p),
                ("state", C.c_void_p), ("status", C.c_void_p), ("volume", C.c_uint32), ("tf_height", C.c_uint32),
                ("fallback", C.c_uint32)]


class CacheDeviceView(C.Structure):
    _fields_ = [("mrpd", C.c_void_p), ("requests", C.c_void_p), ("usage", C.c_void_p), ("pool", C.c_void_p),
                ("slot_bytes", C.c_uint64), ("mrpd_dims", C.c_uint32 * 3), ("pool_slots", C.c_uint32 * 3),
                ("brick_size", C.c_uint32), ("covering", C.c_uint32), ("voxel_bytes", C.c_uint32),
                ("timestamp", C.c_uint32), ("n_levels", C.c_uint32), ("level_offset", C.c_uint32 * MAX_LEVELS),
                ("level_bricks", (C.c_uint32 * 3) * MAX_LEVELS), ("level_voxels", (C.c_uint32 * 3) * MAX_LEVELS),
                ("level_initial_over_real", (C.c_float * 3) * MAX_LEVELS), ("pt_top", C.c_void_p),
                ("pt_pool", C.c_void_p), ("pt_usage", C.c_void_p), ("pt_shift", C.c_uint32),
                ("pt_dims", C.c_uint32 * 3), ("pt_level_offset", C.c_uint32 * MAX_LEVELS)]


class BatchDesc(C.Structure):
    _fields_ = [("max_views", C.c_uint32), ("max_pixels", C.c_uint64), ("max_passes", C.c_uint32),
                ("max_occupancy", C.c_float), ("max_admit", C.c_uint32), ("park_above", C.c_float),
                ("reorder_window", C.c_uint32), ("overlap_loads", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("ticks", C.c_uint64), ("render_ticks", C.c_uint64), ("view_passes", C.c_uint64),
                ("install_ticks", C.c_uint64), ("graph_replays", C.c_uint64), ("parked", C.c_uint64),
                ("render_ms", C.c_double),
                ("tick_ms", C.c_double),
                ("wait_ms", C.c_double)]


class BatchResult(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("passes", C.c_uint32), ("converged", C.c_uint32), ("latency_ms", C.c_double)]


class TfPoint(C.Structure):
    _fields_ = [("value", C.c_float), ("alpha", C.c_float), ("r", C.c_float), ("g", C.c_float), ("b", C.c_float)]


LOADER_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                        C.c_size_t)

vp = C.c_void_p
P = C.POINTER
# name -> argtypes (restype is int unless listed in _RESTYPES)
_SIGS = {
    "gc_last_error": [], "gc_version": [], "gc_device_count": [P(C.c_int)], "gc_kernel_launches": [],
    "gc_config_create": [P(vp)], "gc_config_destroy": [vp], "gc_config_load": [vp, C.c_char_p],
    "gc_config_set": [vp, C.c_char_p, C.c_char_p], "gc_config_get": [vp, C.c_char_p, C.c_char_p, C.c_size_t],
    "gc_config_volume_desc": [vp, P(VolumeDesc)], "gc_layout_compute": [P(VolumeDesc), P(Layout)],
    "gc_pool_dims": [P(VolumeDesc), C.c_uint64, P(C.c_uint32)],
    "gc_generator_blobs": [C.c_uint32, C.c_uint32, P(C.c_uint32), C.c_float, C.c_float, C.c_int32, C.c_int32,
                           P(Blob)],
    "gc_generate_volume": [P(Generator), vp, vp],
    "gc_mip_level": [vp, vp, P(C.c_uint32), C.c_uint32, C.c_uint32, vp],
    "gc_mip_build": [vp, P(Layout), P(C.c_uint64), C.c_uint32, C.c_uint32, vp],
    "gc_bricks_build": [vp, P(C.c_uint32), P(VolumeDesc), P(C.c_uint32), vp, vp],
    "gc_bricks_empty": [vp, C.c_uint64, P(VolumeDesc), C.c_float, vp, vp],
    "gc_brick_value_bins": [P(VolumeDesc), P(Layout), C.c_uint32, vp, vp, vp],
    "gc_cache_set_volume_brick_bins": [vp, C.c_uint32, P(C.c_uint64), C.c_uint64],
    "gc_brick_key": [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32],
    "gc_cache_create": [P(CacheDesc), P(vp)], "gc_cache_destroy": [vp],
    "gc_cache_set_source_host": [vp, vp, C.c_uint64, P(C.c_uint64), P(C.c_uint64), C.c_size_t],
    "gc_cache_set_source_callback": [vp, LOADER_FN, vp, P(C.c_uint64), C.c_size_t],
    "gc_cache_set_volume_source_host": [vp, C.c_uint32, vp, C.c_uint64, P(C.c_uint64), P(C.c_uint64), C.c_size_t],
    "gc_cache_set_volume_source_device": [vp, C.c_uint32, vp, P(C.c_uint64), P(C.c_uint64), C.c_size_t],
    "gc_cache_set_volume_source_callback": [vp, C.c_uint32, LOADER_FN, vp, P(C.c_uint64), C.c_size_t],
    "gc_cache_create_shared": [P(CacheDesc), P(VolumeDesc), P(Layout), C.c_uint32, P(vp)],
    "gc_render_empty_skip": [C.c_int],
    "gc_cache_set_volume_source_files": [vp, C.c_uint32, C.c_char_p, P(C.c_uint64), C.c_size_t, C.c_uint32],
    "gc_lz4_available": [],
    "gc_brick_files_write": [C.c_char_p, P(VolumeDesc), P(Layout), vp, C.c_uint64, P(C.c_uint64), C.c_uint32],
    "gc_brick_files_read": [C.c_char_p, P(VolumeDesc), P(Layout), vp, C.c_uint64, P(C.c_uint64), C.c_uint32],
    "gc_bricks_xml_write": [C.c_char_p, P(VolumeDesc), P(Layout), P(C.c_uint64), C.c_size_t],
    "gc_bricks_xml_read": [C.c_char_p, P(C.c_uint32), P(C.c_uint32 * 3), P(C.c_uint32 * 3), P(C.c_uint64),
                           C.c_size_t, P(C.c_size_t)],
    "gc_cache_volume_levels": [vp, C.c_uint32, P(C.c_uint32), P(C.c_uint32)],
    "gc_cache_device_view_get": [vp, C.c_uint32, P(CacheDeviceView)],
    "gc_cache_update": [vp, vp, P(C.c_int)], "gc_cache_completude": [vp, vp, P(C.c_float)],
    "gc_cache_timestamp": [vp, P(C.c_uint32)], "gc_cache_info_get": [vp, P(CacheInfo)],
    "gc_cache_stats_get": [vp, P(CacheStats)], "gc_cache_dump": [vp, C.c_int, vp, C.c_size_t],
    "gc_cache_load_buffer": [vp, C.c_int, vp, C.c_size_t],
    "gc_cache_last_misses": [vp, P(C.c_uint32), C.c_uint32, P(C.c_uint32), P(C.c_uint32)],
    "gc_view_matrix": [P(C.c_float), P(C.c_float), P(C.c_float)],
    "gc_look_at": [P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_float)],
    "gc_tf_build": [P(TfPoint), C.c_uint32, C.c_uint32, P(C.c_float)],
    "gc_render": [vp, P(View), vp], "gc_render_batch": [vp, P(View), C.c_uint32, vp],
    "gc_batch_create": [vp, P(BatchDesc), P(vp)], "gc_batch_destroy": [vp],
    "gc_batch_submit": [vp, P(View), C.c_uint64], "gc_batch_stats_get": [vp, P(BatchStats)], "gc_batch_tick": [vp, vp, P(C.c_uint32), P(C.c_uint32)],
    "gc_batch_poll": [vp, P(BatchResult), C.c_uint32, P(C.c_uint32)],
    "gc_miss_list_noalloc": [vp, C.c_uint64, C.c_uint32, P(Layout), C.c_uint32, vp, vp, vp],
    "gc_render_tuning_set": [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32],
    "gc_render_tuning_get": [P(C.c_uint32)],
    "gc_render_precision_set": [C.c_int], "gc_render_precision_get": [P(C.c_int)],
}
_RESTYPES = {"gc_last_error": C.c_char_p, "gc_version": C.c_char_p, "gc_brick_key": C.c_uint64,
             "gc_kernel_launches": C.c_uint64}


class GcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[gc error {code}] {msg}")
        self.code = code


def load(path=LIB_PATH):
    if not os.path.exists(path):
        raise ImportError(f"{path} is not built; run __graft_entry__.build()")
    lib = C.CDLL(path)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    return lib


lib = load()


def check(rc):
    if rc != OK:
        raise GcError(rc, lib.gc_last_error().decode())
    return rc


def u3(v):
    return U3(*[int(x) for x in v])


# ---------------------------------------------------------------------------
class Configuration:
    """Key/value configuration (Configuration::get_field / add_field)."""

    def __init__(self, path=None):
        self._h = vp()
        check(lib.gc_config_create(C.byref(self._h)))
        if path:
            self.load(path)

    def load(self, path):
        check(lib.gc_config_load(self._h, str(path).encode()))

    def add_field(self, key, value):
        check(lib.gc_config_set(self._h, key.encode(), str(value).encode()))

    def get_field(self, key):
        buf = C.create_string_buffer(4096)
        rc = lib.gc_config_get(self._h, key.encode(), buf, len(buf))
        return buf.value.decode() if rc == OK else None

    def volume_desc(self):
        d = VolumeDesc()
        check(lib.gc_config_volume_desc(self._h, C.byref(d)))
        return d

    def __del__(self):
        if getattr(self, "_h", None):
            lib.gc_config_destroy(self._h)
            self._h = None


def volume_desc(size, brick_size=16, covering=1, encoded_bytes=1, channels=1, big_brick=(1, 1, 1)):
    return VolumeDesc(u3(size), brick_size, u3(big_brick), covering, encoded_bytes, channels, u3((2, 2, 2)))


def compute_layout(vol):
    L = Layout()
    check(lib.gc_layout_compute(C.byref(vol), C.byref(L)))
    return L


def pool_dims(vol, pool_bytes):
    out = U3()
    check(lib.gc_pool_dims(C.byref(vol), int(pool_bytes), out))
    return tuple(out)


def render_tuning(scheduler=None, tile_w=None, threads=None, blocks_per_sm=None):
    """Reads, and optionally sets, the ray caster's launch configuration."""
    cur = (C.c_uint32 * 4)()
    check(lib.gc_render_tuning_get(cur))
    new = [cur[0] if scheduler is None else scheduler, cur[1] if tile_w is None else tile_w,
           cur[2] if threads is None else threads, cur[3] if blocks_per_sm is None else blocks_per_sm]
    check(lib.gc_render_tuning_set(*new))
    return tuple(new)


def miss_list_noalloc(requests_ptr, n_entries, timestamp, layout, max_requests, out_list_ptr, out_total_ptr,
                      stream=0):
    """Miss list of a request buffer without any device allocation (for
    callers that cannot allocate: stream capture, hard frame deadlines, hosts
    that own all device memory).  See gc_miss_list_noalloc for the limits."""
    check(lib.gc_miss_list_noalloc(vp(requests_ptr), int(n_entries), int(timestamp), C.byref(layout),
                                   int(max_requests), vp(out_list_ptr), vp(out_total_ptr), vp(stream)))


def kernel_launches():
    return int(lib.gc_kernel_launches())


def brick_key(level, x, y, z):
    return int(lib.gc_brick_key(level, x, y, z))


def generator_blobs(seed, nblobs, size, sigma_min, sigma_max, amp_min, amp_max):
    arr = (Blob * max(1, nblobs))()
    check(lib.gc_generator_blobs(seed, nblobs, u3(size), sigma_min, sigma_max, amp_min, amp_max, arr))
    return arr


def make_generator(size, bytes_per_channel, seed, blobs, noise_amplitude, channels=1, channel=0, field=0):
    g = Generator(u3(size), bytes_per_channel, channels, channel, field, seed, noise_amplitude, len(blobs),
                  C.cast(blobs, P(Blob)))
    g._keep = blobs
    return g


def generate_volume(gen, dst_ptr, stream=0):
    check(lib.gc_generate_volume(C.byref(gen), vp(dst_ptr), vp(stream)))


# ---------------------------------------------------------------------------
class Mipmapper:
    """Device-resident mip pyramid (Mipmapper::process)."""

    @staticmethod
    def down_scale(src_ptr, dst_ptr, dims, encoded_bytes, channels, stream=0):
        check(lib.gc_mip_level(vp(src_ptr), vp(dst_ptr), u3(dims), encoded_bytes, channels, vp(stream)))

    @staticmethod
    def process(pyramid_ptr, layout, level_offsets, encoded_bytes, channels, stream=0):
        offs = (C.c_uint64 * MAX_LEVELS)(*[int(o) for o in level_offsets])
        check(lib.gc_mip_build(vp(pyramid_ptr), C.byref(layout), offs, encoded_bytes, channels, vp(stream)))


def process_bricking(level_ptr, level_dims, vol, nb_big_bricks, out_ptr, stream=0):
    """Bricks one level on the device (process_bricking)."""
    check(lib.gc_bricks_build(vp(level_ptr), u3(level_dims), C.byref(vol), u3(nb_big_bricks), vp(out_ptr),
                              vp(stream)))


def process_empty(bricks_ptr, nb_big, vol, threshold, flags_ptr, stream=0):
    check(lib.gc_bricks_empty(vp(bricks_ptr), int(nb_big), C.byref(vol), float(threshold), vp(flags_ptr),
                              vp(stream)))


def brick_value_bins(vol, layout, level, level_ptr, bins_ptr, stream=0):
    """Value bins of every brick of one level (nb_bricks.x*y*z uint64 words,
    x fastest) from the level's big bricks in device memory."""
    check(lib.gc_brick_value_bins(C.byref(vol), C.byref(layout), level, vp(level_ptr), vp(bins_ptr), vp(stream)))


def pyramid_offsets(layout, encoded_bytes, align=256):
    """Byte offsets of each level in one device buffer (level 0 first)."""
    offs, off = [], 0
    for l in range(layout.nb_levels):
        offs.append(off)
        n = layout.mip[l][0] * layout.mip[l][1] * layout.mip[l][2] * encoded_bytes
        off += (n + align - 1) // align * align
    return offs, off


def brick_store_offsets(layout, vol):
    """Byte offsets of each level's big bricks in a flat brick store."""
    B = vol.brick_size
    big = B ** 3 * vol.big_brick_size[0] * vol.big_brick_size[1] * vol.big_brick_size[2] * vol.encoded_bytes
    offs, off = [], 0
    for l in range(layout.nb_levels):
        offs.append(off)
        nb = layout.nb_big_bricks[l]
        off += nb[0] * nb[1] * nb[2] * big
    return offs, off, big


def pre_process(vol, layout, level0, stream=0, empty_threshold=None, store="host", pin=False, timings=None,
                value_bins=None, host_out=None):
    """Application::pre_process (Applications/DVR-ray-caster/src/Application.cu:148-197)
    run on the device: mip pyramid, bricking of every level and empty flags.

    level0 is a CUDA tensor holding the level-0 voxels (any dtype, contiguous).
    Returns (bricks, level_offsets, empty_keys): the big bricks of every level in
    one uint8 tensor (host memory unless store == "device"; pinned when pin),
    their per-level byte offsets, and the gc_brick_key of every big brick whose
    values are all below empty_threshold (none when it is None, like the
    reference's default threshold 0).  timings (a dict) receives the seconds
    of the device mip build, the device bricking and the store copy.
    value_bins (a list) receives one numpy uint64 array: the value bins of
    every brick of every level, in the order CacheManager.set_brick_bins takes.
    host_out: a host uint8 tensor of the store's size receiving the bricks
    (e.g. a mapping shared by several processes); returned in place of a new
    host tensor.
    """
    import time

    import numpy as np
    import torch

    eb, nc = vol.encoded_bytes, vol.channels
    for l in range(layout.nb_levels):
        if tuple(layout.mip[l]) != tuple(layout.initial[l]):
            raise GcError(1, "mip level sizes differ from the metadata sizes (dimension <= 2)")
    offs, total = pyramid_offsets(layout, eb)
    dev = level0.device
    pyr = torch.empty(total, dtype=torch.uint8, device=dev)
    n0 = level0.numel() * level0.element_size()
    pyr[:n0].copy_(level0.reshape(-1).view(torch.uint8))
    # the store is allocated before the timed stages (a cudaMalloc of tens of
    # GB is not bricking work)
    soffs, stotal, big = brick_store_offsets(layout, vol)
    bricks = torch.empty(stotal, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    Mipmapper.process(pyr.data_ptr(), layout, offs, eb, nc, stream)
    torch.cuda.synchronize(dev)
    t1 = time.perf_counter()
    for l in range(layout.nb_levels):
        process_bricking(pyr.data_ptr() + offs[l], layout.initial[l], vol, layout.nb_big_bricks[l],
                         bricks.data_ptr() + soffs[l], stream)
    torch.cuda.synchronize(dev)
    t_bricks = time.perf_counter()
    empty_keys = []
    if empty_threshold is not None:
        for l in range(layout.nb_levels):
            nb = layout.nb_big_bricks[l]
            n = nb[0] * nb[1] * nb[2]
            flags = torch.empty(n, dtype=torch.uint8, device=dev)
            process_empty(bricks.data_ptr() + soffs[l], n, vol, empty_threshold, flags.data_ptr(), stream)
            torch.cuda.synchronize(dev)
            for i in torch.nonzero(flags).flatten().tolist():
                x, y, z = i % nb[0], (i // nb[0]) % nb[1], i // (nb[0] * nb[1])
                empty_keys.append(brick_key(l, x, y, z))
    if value_bins is not None:
        counts = [layout.nb_bricks[l][0] * layout.nb_bricks[l][1] * layout.nb_bricks[l][2]
                  for l in range(layout.nb_levels)]
        bins = torch.empty(sum(counts), dtype=torch.int64, device=dev)
        at = 0
        for l in range(layout.nb_levels):
            brick_value_bins(vol, layout, l, bricks.data_ptr() + soffs[l], bins.data_ptr() + 8 * at, stream)
            at += counts[l]
        torch.cuda.synchronize(dev)
        value_bins.append(bins.cpu().numpy().view(np.uint64))
    torch.cuda.synchronize(dev)
    t2 = time.perf_counter()
    if timings is not None:
        timings.update(mip_s=t1 - t0, brick_s=t_bricks - t1, flags_bins_s=t2 - t_bricks, level0_bytes=n0,
                       pyramid_bytes=sum(layout.mip[l][0] * layout.mip[l][1] * layout.mip[l][2] * eb
                                         for l in range(layout.nb_levels)), store_bytes=stotal)
    del pyr
    if store == "device":
        return bricks, soffs, empty_keys
    if host_out is not None:
        if host_out.numel() * host_out.element_size() != stotal or host_out.device.type != "cpu":
            raise GcError(1, f"host_out must be a host tensor of {stotal} bytes")
        host = host_out.view(torch.uint8).reshape(-1)
    else:
        host = torch.empty(stotal, dtype=torch.uint8, pin_memory=pin)
    host.copy_(bricks)
    if timings is not None:
        timings["copy_s"] = time.perf_counter() - t2
    del bricks
    return host, soffs, empty_keys


# ---------------------------------------------------------------------------
def view_matrix(rotation_deg, translation):
    out = (C.c_float * 12)()
    check(lib.gc_view_matrix((C.c_float * 2)(*rotation_deg), (C.c_float * 3)(*translation), out))
    return list(out)


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    out = (C.c_float * 12)()
    check(lib.gc_look_at((C.c_float * 3)(*eye), (C.c_float * 3)(*target), (C.c_float * 3)(*up), out))
    return list(out)


class TransferFunction:
    """Piecewise-linear RGBA transfer function (TransferFunction::getSample)."""

    @staticmethod
    def build(points, samples):
        arr = (TfPoint * max(1, len(points)))(*[TfPoint(*p) for p in points])
        out = (C.c_float * (4 * samples))()
        check(lib.gc_tf_build(arr, len(points), samples, out))
        return list(out)

    @staticmethod
    def defaultColorful(samples=128):
        return TransferFunction.build([(0.20, 0.10, 0, 0, 1), (0.35, 0.70, 0, 1, 1), (0.45, 1.0, 0, 1, 0),
                                       (0.70, 1.0, 1, 1, 0), (1.0, 1.0, 1, 0, 0)], samples)

    @staticmethod
    def greyRamp(samples=128):
        return TransferFunction.build([(0.0, 0.0, 0, 0, 0), (1.0, 1.0, 1, 1, 1)], samples)


def make_view(inv_view, width, height, tf_ptr, tf_width, rgba_ptr, tbuf_ptr, state_ptr, tstep=2.0 / 256.0,
              focal=2.0, early_alpha=0.95, mode=MODE_DVR, sampler=SAMPLER_REFERENCE,
              bbox_min=(-1.0, -1.0, -1.0), bbox_max=(1.0, 1.0, 1.0), status_ptr=0, volume=0, tf_height=0,
              fallback=0):
    return View((C.c_float * 12)(*inv_view), width, height, (C.c_float * 3)(*bbox_min), (C.c_float * 3)(*bbox_max),
                tstep, focal, early_alpha, mode, sampler, tf_width, vp(tf_ptr), vp(rgba_ptr), vp(tbuf_ptr),
                vp(state_ptr), vp(status_ptr or None), volume, tf_height, fallback)


RENDER_EXACT, RENDER_FAST = 0, 1


def render_precision(precision=None):
    """Set (RENDER_EXACT / RENDER_FAST) and/or return the ray caster's arithmetic."""
    if precision is not None:
        check(lib.gc_render_precision_set(int(precision)))
    out = C.c_int()
    check(lib.gc_render_precision_get(C.byref(out)))
    return out.value


def render_empty_skip(enable):
    """Empty-space skipping of the ray caster (on by default; same images)."""
    check(lib.gc_render_empty_skip(1 if enable else 0))


def lz4_available():
    """True when liblz4 (the codec of the reference's brick files) can be loaded."""
    return bool(lib.gc_lz4_available())


def _store_ptr(store, nbytes):
    if hasattr(store, "data_ptr"):
        return store.data_ptr(), store.numel() * store.element_size()
    if hasattr(store, "ctypes"):
        return store.ctypes.data, store.nbytes
    return int(store), int(nbytes)


def write_brick_files(volume_dir, vol, layout, store, level_offsets, threads=0, nbytes=None):
    """BricksManager::write_brick for every big brick of the store (LZ4 HC 9)."""
    ptr, size = _store_ptr(store, nbytes)
    offs = (C.c_uint64 * MAX_LEVELS)(*[int(o) for o in level_offsets])
    check(lib.gc_brick_files_write(str(volume_dir).encode(), C.byref(vol), C.byref(layout), vp(ptr), size, offs,
                                   threads))


def read_brick_files(volume_dir, vol, layout, store, level_offsets, threads=0, nbytes=None):
    """BricksManager::load_brick for every big brick, into the store."""
    ptr, size = _store_ptr(store, nbytes)
    offs = (C.c_uint64 * MAX_LEVELS)(*[int(o) for o in level_offsets])
    check(lib.gc_brick_files_read(str(volume_dir).encode(), C.byref(vol), C.byref(layout), vp(ptr), size, offs,
                                  threads))


def write_bricks_xml(volume_dir, vol, layout, empty_keys=()):
    keys = (C.c_uint64 * max(1, len(empty_keys)))(*[int(k) for k in empty_keys])
    check(lib.gc_bricks_xml_write(str(volume_dir).encode(), C.byref(vol), C.byref(layout), keys, len(empty_keys)))


def read_bricks_xml(path, max_empty=1 << 20):
    """(level initial sizes, level real sizes, empty keys) of a bricks.xml."""
    n = C.c_uint32()
    ini = (C.c_uint32 * 3 * MAX_LEVELS)()
    real = (C.c_uint32 * 3 * MAX_LEVELS)()
    keys = (C.c_uint64 * max_empty)()
    ne = C.c_size_t()
    check(lib.gc_bricks_xml_read(str(path).encode(), C.byref(n), ini, real, keys, max_empty, C.byref(ne)))
    return ([tuple(ini[l]) for l in range(n.value)], [tuple(real[l]) for l in range(n.value)],
            list(keys[: min(ne.value, max_empty)]))


# ---------------------------------------------------------------------------
class CacheManager:
    """GPU brick cache + ray caster entry (CacheManager<T> + RayCastDVR)."""

    def __init__(self, vol, layout, cache_size, max_requests=50, sync_loader=True, gpu=0, staged_upload=False,
                 shared=None, pt_block=0, pt_slots=0):
        """shared: [(volume_desc, layout), ...] for one cache over several
        volumes sharing the pool (vol/layout are then the first of them).
        pt_block, pt_slots: a two-level page directory (one word per
        pt_block^3 bricks, a table pool of pt_slots blocks); 0: one level."""
        flags = (CACHE_SYNC_LOADER if sync_loader else 0) | (CACHE_STAGED_UPLOAD if staged_upload else 0)
        self.desc = CacheDesc(vol, layout, u3(cache_size), max_requests, flags, gpu, pt_block, pt_slots)
        self._h = vp()
        if shared:
            vols = (VolumeDesc * len(shared))(*[v for v, _ in shared])
            lays = (Layout * len(shared))(*[l for _, l in shared])
            check(lib.gc_cache_create_shared(C.byref(self.desc), vols, lays, len(shared), C.byref(self._h)))
        else:
            check(lib.gc_cache_create(C.byref(self.desc), C.byref(self._h)))
        info = CacheInfo()
        check(lib.gc_cache_info_get(self._h, C.byref(info)))
        self.info = info
        self._keep = []

    @property
    def handle(self):
        return self._h

    def volume_levels(self, volume):
        base, n = C.c_uint32(), C.c_uint32()
        check(lib.gc_cache_volume_levels(self._h, volume, C.byref(base), C.byref(n)))
        return base.value, n.value

    def set_source_host(self, store, level_offsets, empty_keys=(), nbytes=None, volume=0):
        """`store`: a host torch tensor or numpy array holding the brick store
        (or a raw address, with `nbytes`).  The store must outlive the cache."""
        if hasattr(store, "data_ptr"):
            ptr, size = store.data_ptr(), store.numel() * store.element_size()
        elif hasattr(store, "ctypes"):
            ptr, size = store.ctypes.data, store.nbytes
        else:
            if nbytes is None:
                raise ValueError("nbytes is required with a raw store address")
            ptr, size = int(store), int(nbytes)
        offs = (C.c_uint64 * MAX_LEVELS)(*[int(o) for o in level_offsets])
        keys = (C.c_uint64 * max(1, len(empty_keys)))(*[int(k) for k in empty_keys])
        self._keep.append((offs, keys, store))
        check(lib.gc_cache_set_volume_source_host(self._h, volume, vp(ptr), size, offs, keys, len(empty_keys)))

    def set_source_device(self, pyramid_ptr, level_offsets, empty_keys=(), volume=0, keep=None):
        """A device-resident mip pyramid (level l at byte offset level_offsets[l],
        e.g. from Mipmapper.process) as the brick source: missing bricks are cut
        from it on the device.  `keep`: an object holding the pyramid alive."""
        offs = (C.c_uint64 * MAX_LEVELS)(*[int(o) for o in level_offsets])
        keys = (C.c_uint64 * max(1, len(empty_keys)))(*[int(k) for k in empty_keys])
        self._keep.append((offs, keys, keep))
        check(lib.gc_cache_set_volume_source_device(self._h, volume, vp(pyramid_ptr), offs, keys, len(empty_keys)))

    def drop_sources(self):
        """Releases this object's references to the brick sources given so
        far (host stores, pyramids, key arrays).  The cache keeps the pointers:
        call update() only after giving a source again."""
        self._keep.clear()

    def set_brick_bins(self, bins, volume=0):
        """Value bins of every brick of the volume (pre_process(value_bins=...)):
        missing bricks the transfer function cannot make visible are stepped
        through, not loaded.  None or empty removes them."""
        import numpy as np

        a = np.ascontiguousarray(np.asarray([] if bins is None else bins, dtype=np.uint64))
        self._keep.append(a)
        check(lib.gc_cache_set_volume_brick_bins(self._h, volume, a.ctypes.data_as(P(C.c_uint64)), a.size))

    def set_source_files(self, volume_dir, empty_keys=(), volume=0, threads=0):
        """The reference's brick files under volume_dir, read by the loader."""
        keys = (C.c_uint64 * max(1, len(empty_keys)))(*[int(k) for k in empty_keys])
        self._keep.append(keys)
        check(lib.gc_cache_set_volume_source_files(self._h, volume, str(volume_dir).encode(), keys, len(empty_keys),
                                                   threads))

    def set_source_callback(self, fn, empty_keys=(), volume=0):
        cb = LOADER_FN(fn)
        keys = (C.c_uint64 * max(1, len(empty_keys)))(*[int(k) for k in empty_keys])
        self._keep.append((cb, keys))
        check(lib.gc_cache_set_volume_source_callback(self._h, volume, cb, None, keys, len(empty_keys)))

    def update(self, stream=0):
        conv = C.c_int()
        check(lib.gc_cache_update(self._h, vp(stream), C.byref(conv)))
        return bool(conv.value)

    def completude(self, stream=0):
        f = C.c_float()
        check(lib.gc_cache_completude(self._h, vp(stream), C.byref(f)))
        return f.value

    def timestamp(self):
        t = C.c_uint32()
        check(lib.gc_cache_timestamp(self._h, C.byref(t)))
        return t.value

    def stats(self):
        s = CacheStats()
        check(lib.gc_cache_stats_get(self._h, C.byref(s)))
        return s

    def dump(self, what, buf):
        """Copies one state buffer into a writable host buffer (numpy array):
        DUMP_MRPD / LRU / USAGE / REQUESTS / POOL, and for a two-level page
        directory DUMP_PT_TOP / PT_POOL / PT_LRU / PT_USAGE / PT_KEYS (sizes and
        layouts in include/gc_gb300.h)."""
        check(lib.gc_cache_dump(self._h, what, vp(buf.ctypes.data), buf.nbytes))
        return buf

    def last_misses(self, max_entries=None):
        """(total flagged, list of (x, y, z, level)) of the last request scan."""
        import numpy as np

        m = max_entries or self.desc.max_requests
        out = np.zeros((m, 4), dtype=np.uint32)
        n, tot = C.c_uint32(), C.c_uint32()
        check(lib.gc_cache_last_misses(self._h, out.ctypes.data_as(P(C.c_uint32)), m, C.byref(n), C.byref(tot)))
        return tot.value, out[: n.value]

    def device_view(self, volume=0):
        """The device-side handle (gc_cache_device_view) of one volume, for a
        user kernel sampling with gc_sample_normalized; valid until the next
        update."""
        v = CacheDeviceView()
        check(lib.gc_cache_device_view_get(self._h, volume, C.byref(v)))
        return v

    def load_buffer(self, what, buf):
        check(lib.gc_cache_load_buffer(self._h, what, vp(buf.ctypes.data), buf.nbytes))

    def render(self, view, stream=0):
        check(lib.gc_render(self._h, C.byref(view), vp(stream)))

    def render_batch(self, views, stream=0):
        arr = (View * len(views))(*views)
        check(lib.gc_render_batch(self._h, arr, len(views), vp(stream)))

    def close(self):
        if getattr(self, "_h", None):
            lib.gc_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Batch:
    """Continuous batching of views over one cache (gc_batch_*)."""

    def __init__(self, cache, max_views=64, max_pixels=1 << 24, max_passes=0, max_occupancy=0.0, max_admit=0,
                 park_above=0.0, reorder_window=0, overlap_loads=False):
        self.cache = cache
        self._h = vp()
        d = BatchDesc(max_views, max_pixels, max_passes, max_occupancy, max_admit, park_above, reorder_window,
                      1 if overlap_loads else 0)
        check(lib.gc_batch_create(cache.handle, C.byref(d), C.byref(self._h)))

    def submit(self, view, tag):
        check(lib.gc_batch_submit(self._h, C.byref(view), int(tag)))

    def tick(self, stream=0):
        a, q = C.c_uint32(), C.c_uint32()
        check(lib.gc_batch_tick(self._h, vp(stream), C.byref(a), C.byref(q)))
        return a.value, q.value

    def poll(self, max_results=4096):
        arr = (BatchResult * max_results)()
        n = C.c_uint32()
        check(lib.gc_batch_poll(self._h, arr, max_results, C.byref(n)))
        return [(r.tag, r.passes, bool(r.converged), r.latency_ms) for r in arr[: n.value]]

    def stats(self):
        st = BatchStats()
        check(lib.gc_batch_stats_get(self._h, C.byref(st)))
        return st

    def close(self):
        if getattr(self, "_h", None):
            lib.gc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


AUTOTUNE_CANDIDATES = [(sched, tw, th, bps) for sched in (1, 0) for tw in (8, 4, 16) for th in (128, 64, 256)
                       for bps in (0, 4)]


def autotune_render(cache, views, clear, stream=0, candidates=None, repeats=3, cache_file=None, key=None,
                    per_view=False):
    """Chooses the ray caster's launch configuration (scheduler, ray-tile
    shape, threads per block, blocks per SM) by timing `views` (a list of View
    whose bricks are resident) under each candidate, applies the fastest and
    returns (best, timings).  The views render in one launch (the batched
    form), or with per_view one launch each, timed in sum (the plain per-view
    path).  `clear()` restarts the views' progressive buffers before each timed
    render.  With cache_file and key, a previous choice for the same key is
    reused without timing.  Images do not depend on the choice."""
    import json
    import torch

    if cache_file and key and os.path.exists(cache_file):
        try:
            with open(cache_file) as f:
                known = json.load(f)
            if key in known:
                best = tuple(known[key]["best"])
                render_tuning(*best)
                return best, known[key].get("timings_ms", {})
        except (OSError, ValueError, KeyError):
            pass
    arr = (View * len(views))(*views)
    s = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
    timings = {}
    for cand in candidates or AUTOTUNE_CANDIDATES:
        render_tuning(*cand)
        ms = []
        for r in range(repeats + 1):
            clear()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            if per_view:
                for i in range(len(views)):
                    check(lib.gc_render(cache.handle, C.byref(arr[i]), vp(stream)))
            else:
                check(lib.gc_render_batch(cache.handle, arr, len(views), vp(stream)))
            b.record(s)
            b.synchronize()
            if r:
                ms.append(a.elapsed_time(b))
        timings[str(cand)] = sorted(ms)[len(ms) // 2]
    best = min(timings, key=timings.get)
    best = tuple(int(x) for x in best.strip("()").split(","))
    render_tuning(*best)
    if cache_file and key:
        try:
            known = {}
            if os.path.exists(cache_file):
                with open(cache_file) as f:
                    known = json.load(f)
            known[key] = {"best": list(best), "timings_ms": timings}
            os.makedirs(os.path.dirname(os.path.abspath(cache_file)), exist_ok=True)
            with open(cache_file, "w") as f:
                json.dump(known, f, indent=1)
        except (OSError, ValueError):
            pass
    return best, timings
