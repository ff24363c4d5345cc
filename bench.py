"""Benchmark of the out-of-core volume path on one GB300.

Metric: Mrays/s of converged views (W*H primary rays per view) with p50/p99
view latency, for the plain per-view path (value, e2e) and the batched form.

  python bench.py [--steps K] [--warmup W] [--impl ours|reference] [--config c2]

A step renders one view to convergence, the way the reference's own benchmark
counts time until "Frame done" (ref:bench.sh:39-55): restart the progressive
buffers (the camera moved), then repeat {render, cache update} until the
update reports an empty miss list.  Each iteration pages the missing bricks in
from host memory (miss scan -> loader -> upload on a side stream -> install).
Rays are counted once per converged view.  The first `warmup` views of the
path warm the cache; the `steps` timed views are spread evenly over the rest
of the path (config.timed_views), so a fly-through's close-up end counts as
much as its far start.  Both arms time the same views and print the same
`config`.

Workloads (seeded synthetic volumes with the shapes of the benchmark configs;
no public dataset is used):
  c2  (plain, the bench line's value)  2048^3 u16 (16 GiB), BrickSize 16,
      covering 1, 2 GiB pool, 1024^2 views along a fly-through zooming from 3.0x
      to 0.3x the diagonal, fov 45 deg, TF with 3 Gaussian alpha bumps,
      early termination at alpha 0.99.
  c3  (batched, reported under "batched")  the same volume with BrickSize 32
      and a 4 GiB pool; batches of 64 views on a sphere at 0.5-3.0x the
      diagonal with sizes uniform over {256^2, 512^2, 1024^2, 1920x1080}, all
      views of a batch in one persistent launch sharing the cache's miss list;
      the same views are also rendered one at a time (plain) for the ratio.
  c1  256^3 u8 (small; used for profiling).
  c4  (serving, --config c4)  three volumes (1024^3 u8, 2048^3 u16,
      4096x4096x2048 u8) in one 24 GiB shared pool; Poisson requests at 200/s
      with a random volume, camera, size and one of 4 transfer functions;
      latency from arrival to retirement.
The pool and page directory exceed L2 (129 MB) for c2/c3/c4.  Bricks are paged
in by a gather kernel reading the host store over the host link where the
device can (--upload staged: host copies + cudaMemcpyAsync).  The host brick
stores are page-locked (--pageable-stores: pageable; c4's always pageable).

value  : views rendered into device buffers.
e2e    : the same through the C ABI with the converged RGBA frame read back
         into pinned host memory inside the timed region; brick bytes paged in
         (H2D) and the frame (D2H) are counted per step.
--impl reference runs the CPU port of the same method (the oracle's FP32
ray-march + cache state machine, all host threads) over the same views, with
its brick store built on the host by the oracle: that process loads no GPU
library.
"""
import argparse
import json
import math
import os
import platform
import statistics
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gpu-out-of-core-volume-data_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

VOL2048 = dict(size=(2048, 2048, 2048), bpc=2, nblobs=32, sigma=(40.0, 300.0), amp=(60 * 257, 200 * 257),
               noise=20 * 257, seed=2)
CONFIGS = {
    "c1": dict(size=(256, 256, 256), bpc=1, nblobs=8, sigma=(10.0, 40.0), amp=(60, 200), noise=20, seed=1, B=16,
               c=1, pool_bytes=None, pool_slots=(21, 21, 21), W=512, H=512, frames=36, path="orbit",
               dist=(2.0, 2.0), tf="ramp", early=0.99, fov=45.0),
    "c2": dict(VOL2048, B=16, c=1, pool_bytes=2 << 30, pool_slots=None, W=1024, H=1024, frames=120, path="fly",
               dist=(3.0, 0.3), tf="bumps", early=0.99, fov=45.0),
    "c3": dict(VOL2048, B=32, c=1, pool_bytes=4 << 30, pool_slots=None, batch=64,
               sizes=((256, 256), (512, 512), (1024, 1024), (1920, 1080)), dist=(0.5, 3.0), tf="bumps",
               early=0.99, fov=45.0),
    # large stress: 4096^3 x 2 u8 channels (blob field + independent noise field), covering 2, big
    # bricks 2^3, 8 GiB pool, 2048^2 views on a path through the interior, 2D TF.  Its bricked store
    # (~375 GB with covering 2) fits no host memory here; the volume's mip pyramid (146 GiB) stays on
    # the device and missing bricks are cut from it (run_stress; --config c5 runs the plain loop on a
    # 2048^3 x 2 host store instead)
    "c5": dict(size=(4096, 4096, 4096), bpc=1, channels=2, nblobs=32, sigma=(80.0, 600.0), amp=(60, 200), noise=20,
               seed=5, B=16, c=2, bb=(2, 2, 2), pool_bytes=8 << 30, pool_slots=None, W=2048, H=2048, frames=240,
               path="cross", dist=(0.0, 0.0), tf="2d", early=0.99, fov=45.0, cap=256),
    "c5_host": dict(size=(2048, 2048, 2048), bpc=1, channels=2, nblobs=32, sigma=(40.0, 300.0), amp=(60, 200),
                    noise=20, seed=5, B=16, c=2, bb=(2, 2, 2), pool_bytes=8 << 30, pool_slots=None, W=2048, H=2048,
                    frames=240, path="cross", dist=(0.0, 0.0), tf="2d", early=0.99, fov=45.0, cap=256),
    # serving: three resident volumes sharing one 24 GiB pool, Poisson requests
    "c4": dict(B=16, c=1, pool_bytes=24 << 30, rate=200.0, duration=6.0, batch=64,
               sizes=((256, 256), (512, 512), (1024, 1024), (1920, 1080)), dist=(0.5, 3.0), early=0.99, fov=45.0,
               volumes=(dict(size=(1024, 1024, 1024), bpc=1, nblobs=16, sigma=(20.0, 150.0), amp=(60, 200),
                             noise=20, seed=11),
                        dict(VOL2048, seed=12),
                        dict(size=(4096, 4096, 2048), bpc=1, nblobs=48, sigma=(80.0, 600.0), amp=(60, 200),
                             noise=20, seed=13))),
}
DIAG = 2.0 * math.sqrt(3.0)
PIXEL_BYTES = 44  # RGBA 4 + t 4+4 + colour state 16+16 per pixel and launch
# DRAM bytes (read + write) of the c2 roofline launch (view 42, converged, after
# an L2 flush), from one ncu capture of this command:
#   ncu --set full --clock-control none --nvtx --nvtx-include roofline/ -k regex:render_kernel -c 1
#       python bench.py --roofline-only --steps 3 --tuning 0,16,128,0
# (profiles/render_kernel_c2_1024x1024.md).  None for the other configs.
ROOFLINE_TRAFFIC = {"c2": 106_319_872}
BRICK_BINS = {}  # value bins of every brick, by brick-store address


def workload(name, cfg):
    """(workload text, voxel dtype, data text) of a plain per-view config."""
    n = cfg["size"][0]
    dt = "u8" if cfg["bpc"] == 1 else "u16"
    nc = cfg.get("channels", 1)
    if nc > 1:
        dt = f"{dt}x{nc}"
    vol = f"{n}^3 {dt}"
    if cfg["path"] == "orbit":
        how = f"{cfg['W']}^2 views on a {cfg['frames']}-view orbit at {cfg['dist'][0]}x the diagonal"
    elif cfg["path"] == "cross":
        how = (f"{cfg['W']}^2 views along a {cfg['frames']}-view path through the interior, 2D transfer function, "
               f"covering {cfg['c']}, big bricks {cfg.get('bb')}")
    else:
        how = (f"{cfg['W']}^2 views along a {cfg['frames']}-view fly-through from {cfg['dist'][0]}x to "
               f"{cfg['dist'][1]}x the diagonal")
    core = "in-core" if cfg["pool_slots"] else "out-of-core"
    return (f"{name}: {vol} {core}, plain per-view path, {how}, each rendered to convergence", dt,
            f"synthetic (seeded blobs + value noise, {vol}; no public dataset)")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def pool_slots(cfg):
    """Pool slots of a config: given, or the cube of slots holding pool_bytes
    of bricks grown round-robin per axis (Application.cu:85-93, the same
    formula as gc_pool_dims)."""
    if cfg.get("pool_slots"):
        return tuple(cfg["pool_slots"])
    eb = cfg["bpc"] * cfg.get("channels", 1)
    entries = cfg["pool_bytes"] // (cfg["B"] ** 3 * eb)
    edge = int(round(entries ** (1.0 / 3.0)))
    while edge ** 3 > entries:
        edge -= 1
    while (edge + 1) ** 3 <= entries:
        edge += 1
    d, axis = [edge, edge, edge], 0
    while d[0] * d[1] * d[2] < entries:
        d[axis] += 1
        axis = (axis + 1) % 3
    return tuple(d)


def timed_views(cfg, steps, warmup):
    """The path views a run times: after views 0 .. warmup-1 (the warm-up),
    `steps` views spread evenly over the rest of the path, so that the far
    views at its start and the close-up views at its end both count."""
    n = cfg["frames"]
    return [warmup + (i * (n - warmup)) // steps for i in range(steps)]


def bench_config(name, cfg, args):
    """The `config` object of the bench line: static parameters only, the same
    for the GPU arm and the reference arm."""
    wl = workload(name, cfg)[0]
    pool = pool_slots(cfg)
    eb = cfg["bpc"] * cfg.get("channels", 1)
    l2 = {"c2": "inputs > L2 (2 GiB pool, 103 MB page directory, 28 GiB host brick store)",
          "c5_host": "inputs > L2 (8 GiB pool, 43 GiB host brick store)"}.get(
        name, "in-core volume; L2 not flushed (the c1 case is for profiling)")
    return {"workload": wl, "brick_size": cfg["B"], "covering": cfg["c"], "pool_slots": list(pool),
            "pool_gib": round(pool[0] * pool[1] * pool[2] * cfg["B"] ** 3 * eb / 2 ** 30, 3),
            "view": [cfg["W"], cfg["H"]], "max_requests": args.max_requests, "early_alpha": cfg["early"],
            "warmup_views": list(range(args.warmup)), "timed_views": timed_views(cfg, args.steps, args.warmup),
            "l2": l2}


def tf2d_table(seed=5, width=64, height=64):
    """2D RGBA table (height rows of width entries) for two-channel volumes:
    alpha from seeded bumps over channel 0, modulated along channel 1."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, width)[None, :]
    y = np.linspace(0.0, 1.0, height)[:, None]
    a = np.zeros((height, width))
    for _ in range(3):
        c, w, h = rng.uniform(0.2, 0.9), rng.uniform(0.04, 0.1), rng.uniform(0.2, 0.7)
        a = a + h * np.exp(-0.5 * ((x - c) / w) ** 2) * (0.3 + 0.7 * y)
    rgb = np.stack([np.broadcast_to(np.clip(0.2 + x, 0, 1), a.shape), np.broadcast_to(np.clip(1.0 - y, 0, 1), a.shape),
                    0.5 + 0.5 * np.sin(5 * x + 3 * y)], -1)
    return np.concatenate([rgb, np.clip(a, 0, 1)[..., None]], -1).astype(np.float32)


def tf_table(kind, seed=3):
    x = np.linspace(0.0, 1.0, 256)
    if kind == "ramp":  # alpha 0 up to value 40, ramp to 0.6 at 255
        v = x * 255.0
        a = np.where(v <= 40, 0.0, 0.6 * np.clip((v - 40) / 215.0, 0, 1))
        rgb = np.stack([np.clip(0.2 + 1.2 * x, 0, 1), 0.3 + 1.2 * x * (1 - x), 1.0 - x], 1)
    else:  # three seeded Gaussian alpha bumps
        rng = np.random.default_rng(seed)
        a = np.zeros_like(x)
        for _ in range(3):
            c, w, h = rng.uniform(0.2, 0.9), rng.uniform(0.02, 0.08), rng.uniform(0.2, 0.8)
            a += h * np.exp(-0.5 * ((x - c) / w) ** 2)
        rgb = np.stack([np.clip(0.3 + x, 0, 1), np.clip(1.2 - x, 0, 1), 0.5 + 0.5 * np.sin(6 * x)], 1)
    return np.concatenate([rgb, np.clip(a, 0, 1)[:, None]], 1).astype(np.float32)


def look_at_host(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    """gc_look_at restated on the host (double arithmetic on the float inputs,
    rounded to float like the C ABI), so that the CPU arm needs no GPU library:
    columns (right, up, -forward, eye) of the 3x4 inverse view matrix."""
    f32 = lambda v: float(np.float32(v))  # noqa: E731
    e, t, u = [f32(x) for x in eye], [f32(x) for x in target], [f32(x) for x in up]

    def norm(v):
        n = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
        return [v[0] / n, v[1] / n, v[2] / n]

    def cross(a, b):
        return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]

    fw = norm([t[a] - e[a] for a in range(3)])
    r = norm(cross(fw, u))
    uu = cross(r, fw)
    out = []
    for a in range(3):
        out += [f32(r[a]), f32(uu[a]), f32(-fw[a]), e[a]]
    return out


def path_camera(look_at, cfg, f, rank=0):
    """Camera of view f of the config's path; look_at is gc.look_at or look_at_host."""
    n = cfg["frames"]
    t = (f % n) / max(1, n - 1)
    if cfg["path"] == "cross":  # through the interior, looking ahead along the path
        a, b = (-0.85, -0.25, -0.8), (0.85, 0.3, 0.8)
        eye = tuple(p + (q - p) * t for p, q in zip(a, b))
        ahead = tuple(e + (q - p) * 0.5 for e, p, q in zip(eye, a, b))
        return look_at(eye, ahead)
    if cfg["path"] == "orbit":
        ang = 2 * math.pi * ((f + rank * 7) % n) / n
        d = cfg["dist"][0] * DIAG
        return look_at((d * math.sin(ang) * math.cos(0.3), d * math.sin(0.3), d * math.cos(ang) * math.cos(0.3)))
    d = (cfg["dist"][0] + (cfg["dist"][1] - cfg["dist"][0]) * t) * DIAG
    ang = 0.6 * t + 0.4 * rank
    dirv = (math.sin(ang) * 0.8, 0.35, math.cos(ang))
    nrm = math.sqrt(sum(c * c for c in dirv))
    eye = tuple(d * c / nrm for c in dirv)
    target = tuple(0.15 * math.sin(3 * t + rank) * c for c in (1.0, 0.5, 0.2))
    return look_at(eye, target)


def batch_views(gc, cfg, seed, n):
    """n seeded (matrix, W, H): cameras on a sphere looking at the centre."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        d = rng.uniform(*cfg["dist"]) * DIAG
        up = (0.0, 1.0, 0.0) if abs(v[1]) < 0.95 else (1.0, 0.0, 0.0)
        W, H = cfg["sizes"][int(rng.integers(0, len(cfg["sizes"])))]
        out.append((gc.look_at(tuple(float(c) * d for c in v), (0.0, 0.0, 0.0), up), W, H))
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc, self.path = None, None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-i",
                                          dev, "-lms", "100"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        self.proc.wait(timeout=5)
        rows = [[p.strip() for p in line.split(",")] for line in open(self.path)]
        rows = [r for r in rows if len(r) >= 9]
        os.remove(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [v for v in (num(r[1]) for r in rows) if v is not None]
        mx = [v for v in (num(r[2]) for r in rows) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


PIN_STORES = True  # brick stores in page-locked host memory (--pageable-stores: not)
LAST_PREPROCESS = {}  # stage timings of the last make_store (device mip, bricking, store copy)


SHM_DIR = "/dev/shm"


def host_register(torch, t):
    """Page-locks a host tensor's pages for this process (cudaHostRegister);
    False where that is not possible (no device, or the call fails)."""
    if not torch.cuda.is_available():
        return False
    return int(torch.cuda.cudart().cudaHostRegister(t.data_ptr(), t.numel() * t.element_size(), 0)) == 0


def node_shared_store(torch, key, nbytes, fill):
    """One host brick store for all replicas of a node.  With one process,
    fill(out) gets a host tensor of nbytes (page-locked when PIN_STORES) and
    returns the bins of every brick.  With several (torchrun), the rank with
    LOCAL_RANK 0 runs fill on a tensor mapping a file in /dev/shm, the other
    ranks map the same file after a barrier (the pages exist once on the
    node, each process page-locks its own mapping), and the file's name is
    removed once every rank holds its mapping.  The bins travel beside it.
    Returns (store tensor, bins)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world == 1:
        out = torch.empty(nbytes, dtype=torch.uint8, pin_memory=PIN_STORES)
        return out, fill(out)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    path = os.path.join(SHM_DIR, f"gc_store_{os.environ.get('MASTER_PORT', '0')}_{key}")
    if local == 0:
        mm = np.memmap(path, dtype=np.uint8, mode="w+", shape=(nbytes,))
        out = torch.from_numpy(mm)
        if PIN_STORES:
            host_register(torch, out)
        bins = fill(out)
        mm.flush()
        np.save(path + ".bins.npy", np.asarray(bins, dtype=np.uint64))
    rank_barrier()
    if local != 0:
        mm = np.memmap(path, dtype=np.uint8, mode="r+", shape=(nbytes,))
        out = torch.from_numpy(mm)
        if PIN_STORES:
            host_register(torch, out)
        bins = np.load(path + ".bins.npy")
    rank_barrier()
    if local == 0:
        os.remove(path)
        os.remove(path + ".bins.npy")
    return out, bins


def make_store(gc, torch, cfg):
    """Synthetic volume generated on the device, pre-processed (mip + bricks) on
    the device, brick store moved to host memory (the out-of-core source);
    replicas on one node share one store (node_shared_store)."""
    size, bpc = cfg["size"], cfg["bpc"]
    nc = cfg.get("channels", 1)
    vol = gc.volume_desc(size, cfg["B"], cfg["c"], bpc * nc, nc, cfg.get("bb", (1, 1, 1)))
    layout = gc.compute_layout(vol)
    offs, nbytes, _ = gc.brick_store_offsets(layout, vol)
    t0 = time.time()
    key = f"{size[0]}x{size[1]}x{size[2]}_{bpc}x{nc}_B{cfg['B']}c{cfg['c']}_s{cfg['seed']}"
    store, bins = node_shared_store(torch, key, nbytes, lambda out: build_store(gc, torch, cfg, vol, layout, out))
    BRICK_BINS[store.data_ptr()] = bins
    t2 = time.time()
    log(f"volume {size} B{cfg['B']}: store of {store.numel() / 2**30:.2f} GiB of bricks in {t2 - t0:.2f}s")
    return vol, layout, store, offs, t2 - t0


def build_store(gc, torch, cfg, vol, layout, out):
    """The volume generated and pre-processed on the device, its bricks copied
    into the host tensor `out`; returns the bins of every brick."""
    size, bpc = cfg["size"], cfg["bpc"]
    nc = cfg.get("channels", 1)
    t0 = time.time()
    blobs = gc.generator_blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0],
                               cfg["amp"][1])
    dev = torch.empty(size[0] * size[1] * size[2] * bpc * nc, dtype=torch.uint8, device="cuda")
    gc.generate_volume(gc.make_generator(size, bpc, cfg["seed"], blobs, cfg["noise"], channels=nc, channel=0,
                                         field=0), dev.data_ptr())
    for ch in range(1, nc):  # further channels: an independent noise field
        gc.generate_volume(gc.make_generator(size, bpc, cfg["seed"] + ch, blobs, cfg["noise"] * 4, channels=nc,
                                             channel=ch, field=1), dev.data_ptr())
    torch.cuda.synchronize()
    t1 = time.time()
    tm = {}
    bins = []
    gc.pre_process(vol, layout, dev, timings=tm, value_bins=bins, host_out=out)
    LAST_PREPROCESS.clear()
    LAST_PREPROCESS.update(tm)
    del dev
    torch.cuda.empty_cache()
    log(f"volume {size} B{cfg['B']}: generated {t1 - t0:.2f}s, pre-processed {time.time() - t1:.2f}s")
    return bins[0]


class Session:
    """One cache + the buffers of its views, driven through the C ABI."""

    staged = False  # GC_CACHE_STAGED_UPLOAD for every session (--upload staged)
    brick_bins = False  # give the cache the value bins of every brick (--brick-bins)

    def __init__(self, gc, torch, cfg, vol, layout, store, offs, max_requests, sync=True, pt=(0, 0)):
        self.gc, self.torch, self.cfg = gc, torch, cfg
        self.pool = cfg["pool_slots"] or gc.pool_dims(vol, cfg["pool_bytes"])
        self.cm = gc.CacheManager(vol, layout, self.pool, max_requests=max_requests, sync_loader=sync,
                                  staged_upload=Session.staged, pt_block=pt[0], pt_slots=pt[1])
        self.cm.set_source_host(store, offs)
        if Session.brick_bins:
            self.cm.set_brick_bins(BRICK_BINS[store.data_ptr()])
        self.vol = vol
        tf = tf2d_table() if cfg["tf"] == "2d" else tf_table(cfg["tf"])
        self.tfh, self.tfw = (tf.shape[0], tf.shape[1]) if tf.ndim == 3 else (0, tf.shape[0])
        self.tf = torch.from_numpy(tf.reshape(-1)).cuda()
        self.stream = torch.cuda.Stream()
        self.sp = self.stream.cuda_stream
        self.focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
        self.bufs = {}

    def buffers(self, i, W, H):
        key = (i, W, H)
        if key not in self.bufs:
            t = self.torch
            self.bufs[key] = (t.zeros(W * H, dtype=t.int32, device="cuda"),
                              t.zeros(W * H, dtype=t.float32, device="cuda"),
                              t.zeros(W * H * 4, dtype=t.float32, device="cuda"),
                              t.empty(W * H, dtype=t.int32, pin_memory=True))
        return self.bufs[key]

    def views(self, specs):
        out, bufs = [], []
        for i, (m, W, H) in enumerate(specs):
            b = self.buffers(i, W, H)
            bufs.append(b)
            out.append(self.gc.make_view(m, W, H, self.tf.data_ptr(), self.tfw, b[0].data_ptr(), b[1].data_ptr(),
                                         b[2].data_ptr(), tstep=2.0 / 256.0, focal=self.focal,
                                         early_alpha=self.cfg["early"], tf_height=self.tfh))
        return out, bufs

    def converge(self, specs, e2e=False, cap=64, render_events=None):
        """Render the views to convergence; returns (iterations, converged)."""
        torch = self.torch
        views, bufs = self.views(specs)
        it, conv = 0, False
        with torch.cuda.stream(self.stream):
            for b in bufs:  # camera moved: restart progressive rendering (VolumeRayCaster.cu:320-329)
                b[1].zero_()
                b[2].zero_()
            while not conv and it < cap:
                if render_events is not None:
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(self.stream)
                if len(views) == 1:
                    self.cm.render(views[0], self.sp)
                else:
                    self.cm.render_batch(views, self.sp)
                if render_events is not None:
                    e1.record(self.stream)
                    render_events.append((e0, e1))
                conv = self.cm.update(self.sp)
                it += 1
            if e2e:
                for b in bufs:
                    b[3].copy_(b[0], non_blocking=True)
        return it, conv

    def close(self):
        self.cm.close()


def autotune(gc, torch, S, specs, args, per_view=False):
    """Autotunes the ray caster's launch configuration on converged views
    (per_view: one launch per view, as the plain path renders)."""
    S.converge(specs, cap=S.cfg.get("cap", 64))
    views, bufs = S.views(specs)

    def clear():
        for b in bufs:
            b[1].zero_()
            b[2].zero_()

    with torch.cuda.stream(S.stream):
        best, timings = gc.autotune_render(S.cm, views, clear, stream=S.sp, repeats=3, per_view=per_view)
    log(f"autotune: best {best} of {len(timings)} ({min(timings.values()):.3f} ms vs default "
        f"{timings.get(str((1, 8, 128, 0)), float('nan')):.3f} ms)")
    return best, timings


def rank_barrier():
    """Barrier across the replicas (torchrun ranks); a no-op for one process."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of `values` over the replicas (the slowest rank's
    time); the values themselves for one process."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def timed(torch, stream, fn, steps):
    """Per-step latencies (CUDA events on the launch stream) and wall time,
    bracketed by a barrier across replicas and a device synchronize."""
    lat, info = [], []
    rank_barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        info.append(fn(i))
        b.record(stream)
        lat.append((a, b))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    rank_barrier()
    return wall, [x.elapsed_time(y) for x, y in lat], info


def pct(v, q):
    return round(float(np.percentile(v, q)), 4)


def run_ours(args):
    import torch

    import gcgb300 as gc

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    cfg = CONFIGS[args.config]
    gc.render_precision(gc.RENDER_FAST if args.precision == "fast" else gc.RENDER_EXACT)
    vol, layout, store, offs, prep_s = make_store(gc, torch, cfg)
    W, H = cfg["W"], cfg["H"]
    spec = lambda f: [(path_camera(gc.look_at, cfg, f, rank), W, H)]  # noqa: E731
    views = timed_views(cfg, args.steps, args.warmup)
    assert tuple(pool_slots(cfg)) == tuple(gc.pool_dims(vol, cfg["pool_bytes"]) if cfg["pool_bytes"] else cfg["pool_slots"])
    # the reference arm computes the same cameras without the GPU library
    assert all(path_camera(gc.look_at, cfg, f, rank) == path_camera(look_at_host, cfg, f, rank)
               for f in list(range(args.warmup)) + views)

    def plain_pass(e2e):
        """Fresh cache; warm-up views, then the timed views (same views for value and e2e)."""
        S = Session(gc, torch, cfg, vol, layout, store, offs, args.max_requests)
        for f in range(args.warmup):
            S.converge(spec(f), cap=cfg.get("cap", 64))
        s0, l0 = S.cm.stats(), gc.kernel_launches()
        ev = None if e2e else []
        render_events[:] = [] if ev is None else [ev]
        torch.cuda.nvtx.range_push("timed_e2e" if e2e else "timed")
        wall, lat, info = timed(torch, S.stream, lambda i: S.converge(spec(views[i]), e2e=e2e,
                                                                      cap=cfg.get("cap", 64), render_events=ev),
                                args.steps)
        torch.cuda.nvtx.range_pop()
        launches = gc.kernel_launches() - l0
        s1 = S.cm.stats()
        return S, wall, lat, info, launches, s0, s1

    # ray-caster launches of the last timed value pass, bracketed by CUDA
    # events on the launch stream: the live split of a step's time (the launch
    # list under ncu serialises launches and slows the upload's host reads)
    render_events = []

    # clock samples from here to the end of the timed passes (the sampler's
    # start-up overlaps the autotuning, not a timed pass)
    clocks = ClockSampler()
    clocks.start()
    # launch configuration: autotuned once, on three views spread along the
    # path (near, middle, far), in a cache of its own
    T = Session(gc, torch, cfg, vol, layout, store, offs, args.max_requests)
    n = cfg.get("frames", 120)
    tuned = [autotune(gc, torch, T, [spec(f)[0] for f in (n // 6, n // 2, 5 * n // 6)], args, per_view=True)]
    T.close()
    S_e, wall_e, lat_e, _, _, s0_e, s1_e = plain_pass(True)
    S_e.close()
    S, wall, lat, info, launches, s0, s1 = plain_pass(False)
    torch.cuda.synchronize()
    render_ms_total = sum(a.elapsed_time(b) for a, b in render_events[0])
    render_launches = len(render_events[0])
    with_bins = None
    if not args.brick_bins:
        # the same views with the value bins of every brick given to the cache:
        # invisible missing bricks are stepped through, not loaded (images
        # within the reference's own resume rounding; not its request sequence)
        Session.brick_bins = True
        S_b, wall_b, _, info_b, _, s0_b, s1_b = plain_pass(False)
        Session.brick_bins = False
        S_b.close()
        with_bins = (wall_b, info_b, cache_delta(s0_b, s1_b))
    clk = clocks.stop()
    wall, wall_e = max_over_ranks([wall, wall_e], device="cuda")  # replicas: the slowest rank's time
    rays = W * H * args.steps * world
    if with_bins:
        wall_b, info_b, cd_b = with_bins
        wall_b, = max_over_ranks([wall_b], device="cuda")
        with_bins = {"value": round(rays / wall_b / 1e6, 3), "unit": "Mrays/s",
                     "ms_per_step": round(1e3 * wall_b / args.steps, 4),
                     "iterations_per_view": round(statistics.mean(i for i, _ in info_b), 2),
                     "brick_h2d_bytes_per_step": int(cd_b["brick_h2d_bytes"] / args.steps), "cache": cd_b}
    iters = [i for i, _ in info]
    conv = sum(1 for _, c in info if c)

    # Roofline of the dominant kernel: a fixed view of the path (the last timed
    # view of the default run), converged, re-rendered from scratch (full work
    # per launch) after an L2 flush, 5 launches timed with CUDA events.
    last = spec(cfg.get("roofline_frame", 42))
    S.converge(last, cap=cfg.get("cap", 64))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > L2 (126 MB)
    samples0, marched0 = S.cm.stats().samples, S.cm.stats().rays_marched
    ev = []
    torch.cuda.nvtx.range_push("roofline")
    for _ in range(5):
        views, bufs = S.views(last)
        with torch.cuda.stream(S.stream):
            bufs[0][1].zero_()
            bufs[0][2].zero_()
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(S.stream)
            S.cm.render(views[0], S.sp)
            e1.record(S.stream)
            ev.append((e0, e1))
            S.cm.update(S.sp)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    touched = S.cm.stats().last_used
    samples = (S.cm.stats().samples - samples0) / len(ev)
    rays_hit = (S.cm.stats().rays_marched - marched0) / len(ev)
    render_ms = statistics.median([a.elapsed_time(b) for a, b in ev])
    # the same launch with empty-space skipping off (identical image), for the record
    gc.render_empty_skip(False)
    ev_off = []
    for _ in range(3):
        views, bufs = S.views(last)
        with torch.cuda.stream(S.stream):
            bufs[0][1].zero_()
            bufs[0][2].zero_()
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(S.stream)
            S.cm.render(views[0], S.sp)
            e1.record(S.stream)
            ev_off.append((e0, e1))
            S.cm.update(S.sp)
    torch.cuda.synchronize()
    gc.render_empty_skip(True)
    render_ms_noskip = statistics.median([a.elapsed_time(b) for a, b in ev_off])
    # the roofline view's image from each ray-caster build (from scratch, same
    # cache state) for the parity check against the oracle
    images = {}
    for name, prec in (("exact", gc.RENDER_EXACT), ("fast", gc.RENDER_FAST)):
        gc.render_precision(prec)
        views, bufs = S.views(last)
        with torch.cuda.stream(S.stream):
            bufs[0][1].zero_()
            bufs[0][2].zero_()
            S.cm.render(views[0], S.sp)
        torch.cuda.synchronize()
        images[name] = bufs[0][0].cpu().numpy().view(np.uint32).copy()
    gc.render_precision(gc.RENDER_FAST if args.precision == "fast" else gc.RENDER_EXACT)
    algo = touched * cfg["B"] ** 3 * vol.encoded_bytes + W * H * PIXEL_BYTES
    peak, peak_kind = measured_peak()
    achieved = algo / (render_ms / 1e3) / 1e9

    wl, dt, data_txt = workload(args.config, cfg)
    pool_bytes = S.cm.info.pool_bytes
    out = {
        "metric": "Mrays/s", "value": round(rays / wall / 1e6, 3), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * wall / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dt, "data": data_txt,
        "config": bench_config(args.config, cfg, args),
        "setup": {"pool_gib": round(pool_bytes / 2**30, 3), "brick_bins": bool(args.brick_bins), "loader": "sync",
                  "ray_caster_build": args.precision,
                  "upload": "gather kernel reading the host store" if S.cm.stats().upload_direct
                  else "staged host copies + cudaMemcpyAsync",
                  "stores": "pinned" if PIN_STORES else "pageable", "preprocess_s": round(prep_s, 2)},
        "preprocess": {"mip_build_s": round(LAST_PREPROCESS.get("mip_s", 0.0), 4),
                       "mip_build_gbs": round((2 * LAST_PREPROCESS.get("pyramid_bytes", 0) - LAST_PREPROCESS.get(
                           "level0_bytes", 0)) / max(LAST_PREPROCESS.get("mip_s", 1e-9), 1e-9) / 1e9, 1),
                       "bricking_s": round(LAST_PREPROCESS.get("brick_s", 0.0), 4),
                       "bricking_gbs": round((LAST_PREPROCESS.get("pyramid_bytes", 0) + LAST_PREPROCESS.get(
                           "store_bytes", 0)) / max(LAST_PREPROCESS.get("brick_s", 1e-9), 1e-9) / 1e9, 1),
                       "bricking_frac": round((LAST_PREPROCESS.get("pyramid_bytes", 0) + LAST_PREPROCESS.get(
                           "store_bytes", 0)) / max(LAST_PREPROCESS.get("brick_s", 1e-9), 1e-9) / 1e9
                           / measured_peak()[0], 3),
                       "value_bins_s": round(LAST_PREPROCESS.get("flags_bins_s", 0.0), 4),
                       "store_copy_s": round(LAST_PREPROCESS.get("copy_s", 0.0), 4),
                       "note": "device mip pyramid (every level read once, every coarser level written: "
                               "2 x pyramid - level 0 bytes, over the mip time); device bricking (every level "
                               "read once + the brick store written, over the bricking time; fraction of the "
                               "measured HBM peak); value bins of every brick; copy of the brick store to host "
                               "memory"},
        "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
        "iterations_per_view": {"mean": round(statistics.mean(iters), 2), "max": max(iters)},
        "converged_views": f"{conv}/{args.steps}",
        "e2e": {"value": round(rays / wall_e / 1e6, 3), "unit": "Mrays/s",
                "h2d_bytes_per_step": int((s1_e.bytes_h2d - s0_e.bytes_h2d) / args.steps) + 700,
                "d2h_bytes_per_step": W * H * 4, "latency_ms": {"p50": pct(lat_e, 50), "p99": pct(lat_e, 99)}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": ROOFLINE_TRAFFIC.get(args.config),
                     "kernel": "render_pixels_kernel" if gc.render_tuning()[0] == 1 else "render_kernel",
                     "peak_kind": peak_kind, "algorithmic_bytes_per_launch": int(algo),
                     "launch_ms": round(render_ms, 4), "launch_ms_without_empty_skip": round(render_ms_noskip, 4),
                     "touched_bricks": int(touched), "samples_per_launch": int(samples),
                     "rays_hit_box_per_launch": int(rays_hit),
                     "gather_bytes_per_launch": int(samples * (8 * vol.encoded_bytes + 16)),
                     "gather_gbs": round(samples * (8 * vol.encoded_bytes + 16) / (render_ms / 1e3) / 1e9, 1),
                     "note": f"view {cfg.get('roofline_frame', 42)} of the {args.config} path, converged, "
                             f"re-rendered after an L2 flush; compulsory bytes = touched bricks x B^3 x "
                             f"{vol.encoded_bytes} B + {PIXEL_BYTES} B/pixel"},
        "render_tuning": {"scheduler_tile_threads_bps": list(tuned[0][0]) if tuned else None,
                          "candidates_timed": len(tuned[0][1]) if tuned else 0},
        "gpu_launches": int(launches),
        "cache": cache_delta(s0, s1),
        "step_split": {"render_ms_per_step": round(render_ms_total / args.steps, 3),
                       "other_ms_per_step": round(1e3 * wall / args.steps - render_ms_total / args.steps, 3),
                       "render_launches_per_step": round(render_launches / args.steps, 2),
                       "note": "ray-caster launches timed with CUDA events on the launch stream; other = the "
                               "cache updates (LRU, miss scan, host resolve, brick upload, install)"},
        "clocks": clk,
    }
    if with_bins:
        out["with_brick_bins"] = with_bins
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(gc, S, cfg, last, args, images)
        out["parity_max_abs"] = out["cpu_baseline"]["parity"]["max_abs_rgba"]
    if rank == 0:
        try:
            out["page_table"] = page_table_leg(gc, torch, cfg, vol, layout, store, offs, args, last, render_ms,
                                               images["fast" if args.precision == "fast" else "exact"], S)
        except Exception as e:  # a reported leg: its failure does not void the line
            out["page_table"] = {"unavailable": f"{type(e).__name__}: {e}"[:300]}
    S.close()
    del store, S
    release_memory(torch)
    if rank == 0 and not args.no_reference_gpu:
        try:
            out["reference_gpu_build"] = reference_gpu_baseline(gc, torch, args)
        except Exception as e:  # a reported baseline: its failure does not void the line
            out["reference_gpu_build"] = {"unavailable": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0 and not args.no_batched:
        try:
            out["batched"] = run_batched(gc, torch, args)
        except Exception as e:  # a reported leg: its failure does not void the line
            out["batched"] = {"unavailable": f"{type(e).__name__}: {e}"[:300]}
        release_memory(torch)
    if rank == 0 and not args.no_serving:
        try:
            out["serving"] = run_serving_sweep(gc, torch, args)
        except Exception as e:
            out["serving"] = {"unavailable": f"{type(e).__name__}: {e}"[:300]}
        release_memory(torch)
    if rank == 0 and not args.no_stress:
        try:
            out["stress"] = run_stress(gc, torch, args)
        except Exception as e:  # a reported stress leg: its failure does not void the line
            out["stress"] = {"unavailable": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


PT_BLOCK, PT_SLOTS = 8, 4096


def page_table_leg(gc, torch, cfg, vol, layout, store, offs, args, spec, render_ms_one, image_one, S1):
    """The roofline view through a two-level page directory (PT_BLOCK^3 bricks
    per directory word, a table pool of PT_SLOTS blocks): rendered to
    convergence from a cold cache over the same store, then re-rendered from
    scratch after an L2 flush 5 times (CUDA events); the image must equal the
    one-level cache's."""
    S = Session(gc, torch, cfg, vol, layout, store, offs, args.max_requests, pt=(PT_BLOCK, PT_SLOTS))
    try:
        it, conv = S.converge(spec, cap=256)  # from a cold cache
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        ev = []
        for _ in range(5):
            views, bufs = S.views(spec)
            with torch.cuda.stream(S.stream):
                bufs[0][1].zero_()
                bufs[0][2].zero_()
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(S.stream)
                S.cm.render(views[0], S.sp)
                e1.record(S.stream)
                ev.append((e0, e1))
        torch.cuda.synchronize()
        img = bufs[0][0].cpu().numpy().view(np.uint32)
        info, info1 = S.cm.info, S1.cm.info
        flat = info1.mrpd_dims[0] * info1.mrpd_dims[1] * info1.mrpd_dims[2] * 16
        two = info.pt_dims[0] * info.pt_dims[1] * info.pt_dims[2] * 4 + PT_SLOTS * PT_BLOCK ** 3 * 16
        ms = statistics.median([a.elapsed_time(b) for a, b in ev])
        return {"pt_block": PT_BLOCK, "pt_slots": PT_SLOTS, "iterations_to_converge": it, "converged": bool(conv),
                "launch_ms": round(ms, 4), "launch_ms_one_level": round(render_ms_one, 4),
                "launch_ratio": round(ms / render_ms_one, 3),
                "image_equal_to_one_level": bool(np.array_equal(img, image_one)),
                "directory_bytes": {"one_level": int(flat), "two_level": int(two)},
                "note": "the roofline view through the two-level page directory (directory word per "
                        f"{PT_BLOCK}^3 bricks, table pool of {PT_SLOTS} blocks), converged from a cold cache, "
                        "re-rendered after an L2 flush; launch_ms_one_level is the roofline launch above"}
    finally:
        S.close()


def release_memory(torch):
    """Returns cached device blocks and cached page-locked host blocks (the
    brick stores of a finished leg) to the system before the next leg."""
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    host_empty = getattr(torch._C, "_host_emptyCache", None)
    if host_empty is not None:
        host_empty()


def cache_delta(s0, s1):
    """Loader and upload figures between two gc_cache_stats snapshots."""
    up_ms = (s1.upload_ns - s0.upload_ns) / 1e6
    nbytes = s1.bytes_h2d - s0.bytes_h2d
    return {"bricks_installed": int(s1.bricks_installed - s0.bricks_installed), "brick_h2d_bytes": int(nbytes),
            "load_cycles": int(s1.load_cycles - s0.load_cycles),
            "loader_host_ms": round((s1.loader_host_ns - s0.loader_host_ns) / 1e6, 2),
            "upload_ms": round(up_ms, 2), "upload_gbs": round(nbytes / (up_ms / 1e3) / 1e9, 1) if up_ms > 0 else None,
            "upload_route": "gather" if s1.upload_direct else "staged",
            "samples": int(s1.samples - s0.samples),
            "device_error": int(s1.device_error)}


def batched_pass(gc, torch, cfg, data, views, warm, args):
    """The batched form over `views`: continuous batching with the
    asynchronous loader on a fresh cache.  Returns (result dict, wall s)."""
    vol, layout, store, offs = data
    rays = sum(W * H for _, W, H in views)
    S = Session(gc, torch, cfg, vol, layout, store, offs, args.max_requests, sync=False)
    B = gc.Batch(S.cm, max_views=cfg["batch"], max_pixels=args.batch_pixels, max_passes=args.batch_cap,
                 max_occupancy=args.occupancy, max_admit=args.admit, park_above=args.park,
                 reorder_window=args.reorder, overlap_loads=args.overlap)

    def run_all(vs, base):
        for i, (m, W, H) in enumerate(vs):
            b = S.buffers(base + i, W, H)
            B.submit(gc.make_view(m, W, H, S.tf.data_ptr(), 256, b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr(),
                                  tstep=2.0 / 256.0, focal=S.focal, early_alpha=cfg["early"]), base + i)
        out, ticks = [], 0
        while len(out) < len(vs):
            B.tick(S.sp)
            out += B.poll()
            ticks += 1
        return out, ticks

    run_all(warm, 10000)
    for i, (_, W, H) in enumerate(views):  # every view's buffers exist before the clock starts
        S.buffers(i, W, H)
    torch.cuda.synchronize()
    s0 = S.cm.stats()
    b0 = B.stats()
    torch.cuda.nvtx.range_push("batched")
    t0 = time.perf_counter()
    out, ticks = run_all(views, 0)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    s1 = S.cm.stats()
    b1 = B.stats()
    lat = [r[3] for r in out]
    res = {"value": round(rays / wall / 1e6, 3), "wall_s": round(wall, 4), "ticks": ticks,
           "view_latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
           "passes_per_view": round(statistics.mean(r[1] for r in out), 2),
           "converged_views": f"{sum(1 for r in out if r[2])}/{len(views)}",
           "ticks_detail": {"render_ticks": b1.render_ticks - b0.render_ticks,
                            "install_ticks": b1.install_ticks - b0.install_ticks,
                            "graph_replays": b1.graph_replays - b0.graph_replays,
                            "view_passes": b1.view_passes - b0.view_passes,
                            "render_ms": round(b1.render_ms - b0.render_ms, 2),
                            "tick_host_ms": round(b1.tick_ms - b0.tick_ms, 2),
                            "loader_wait_ms": round(b1.wait_ms - b0.wait_ms, 2)},
           "cache": cache_delta(s0, s1)}
    B.close()
    S.close()
    return res, wall


def plain_views_pass(gc, torch, cfg, data, views, warm, args):
    """The plain per-view loop (synchronous loader, one view per launch, each
    to convergence) over the same views on a fresh cache."""
    vol, layout, store, offs = data
    rays = sum(W * H for _, W, H in views)
    S = Session(gc, torch, cfg, vol, layout, store, offs, args.max_requests)
    for v in warm:
        S.converge([v], cap=args.batch_cap)
    s0 = S.cm.stats()
    wall, lat, info = timed(torch, S.stream, lambda i: S.converge([views[i]], cap=args.batch_cap), len(views))
    s1 = S.cm.stats()
    res = {"value": round(rays / wall / 1e6, 3), "wall_s": round(wall, 4),
           "view_latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
           "converged_views": f"{sum(1 for _, c in info if c)}/{len(views)}",
           "iterations_per_view": round(statistics.mean(i for i, _ in info), 2),
           "cache": cache_delta(s0, s1)}
    S.close()
    return res, wall


def c3_views(gc, cfg, nb):
    views = [v for b in range(nb) for v in batch_views(gc, cfg, 100 + b, cfg["batch"])]
    return views, batch_views(gc, cfg, 99, 8)


def run_c3(args):
    """`--config c3` alone: the batched form over the c3 views (and, unless
    --no-plain, the plain loop over the same views), one JSON line."""
    import torch

    import gcgb300 as gc

    cfg = CONFIGS["c3"]
    vol, layout, store, offs, prep_s = make_store(gc, torch, cfg)
    data = (vol, layout, store, offs)
    views, warm = c3_views(gc, cfg, args.batches)
    rays = sum(W * H for _, W, H in views)
    tune_b, tune_p = c3_tunings(gc, torch, cfg, data, warm, args)
    best = tune_b
    gc.render_tuning(*tune_b)
    batched, wall = batched_pass(gc, torch, cfg, data, views, warm, args)
    out = {"metric": "Mrays/s", "value": batched["value"], "unit": "Mrays/s", "n_gpus": 1, "steps": len(views),
           "warmup": len(warm), "ms_per_step": round(1e3 * wall / len(views), 4), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u16",
           "data": "synthetic (seeded blobs + value noise, 2048^3 u16; no public dataset)",
           "config": {"workload": f"c3: {len(views)} views, batched (continuous batching), each to convergence",
                      "rays": int(rays), "reorder": args.reorder, "occupancy": args.occupancy,
                      "admit": args.admit, "park_above": args.park, "overlap_loads": bool(args.overlap), "brick_bins": bool(args.brick_bins),
                      "render_tuning": list(best),
                      "preprocess_s": round(prep_s, 2)},
           "batched": batched}
    if not args.no_plain:
        gc.render_tuning(*tune_p)
        plain, _ = plain_views_pass(gc, torch, cfg, data, views, warm, args)
        out["plain_same_views"] = plain
        out["ratio"] = round(batched["value"] / plain["value"], 3)
    if not args.brick_bins:  # both arms again with brick value bins given to the caches
        Session.brick_bins = True
        gc.render_tuning(*tune_b)
        bb_, _ = batched_pass(gc, torch, cfg, data, views, warm, args)
        bins = {"batched": bb_}
        if not args.no_plain:
            gc.render_tuning(*tune_p)
            bins["plain_same_views"], _ = plain_views_pass(gc, torch, cfg, data, views, warm, args)
            bins["ratio"] = round(bb_["value"] / bins["plain_same_views"]["value"], 3)
        Session.brick_bins = False
        out["with_brick_bins"] = bins
    print(json.dumps(out), flush=True)


STRESS_VIEWS = 3  # views of the c5 path the default run renders


def run_stress(gc, torch, args, nviews=STRESS_VIEWS):
    """c5 at its configured size.  The 4096^3 x 2-channel volume (128 GiB) is
    generated on the device and its mip pyramid built there (146 GiB, kept
    resident); an 8 GiB cache takes its bricks from that pyramid: each missing
    big brick is cut from its level on the device with the bricker's rule
    (gc_cache_set_volume_source_device) -- no brick store exists.  Views of
    the path through the interior, 2048^2, 2D transfer function, each to
    convergence (at most `cap` iterations)."""
    cfg = CONFIGS["c5"]
    size, nc = cfg["size"], cfg["channels"]
    eb = cfg["bpc"] * nc
    vol = gc.volume_desc(size, cfg["B"], cfg["c"], eb, nc, cfg["bb"])
    layout = gc.compute_layout(vol)
    poffs, total = gc.pyramid_offsets(layout, eb)
    torch.cuda.empty_cache()
    pyr = torch.empty(total, dtype=torch.uint8, device="cuda")
    blobs = gc.generator_blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0],
                               cfg["amp"][1])
    t0 = time.perf_counter()
    gc.generate_volume(gc.make_generator(size, cfg["bpc"], cfg["seed"], blobs, cfg["noise"], channels=nc, channel=0,
                                         field=0), pyr.data_ptr())
    for ch in range(1, nc):
        gc.generate_volume(gc.make_generator(size, cfg["bpc"], cfg["seed"] + ch, blobs, cfg["noise"] * 4,
                                             channels=nc, channel=ch, field=1), pyr.data_ptr())
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    gc.Mipmapper.process(pyr.data_ptr(), layout, poffs, eb, nc)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    level0 = size[0] * size[1] * size[2] * eb
    pyramid_bytes = sum(layout.mip[l][0] * layout.mip[l][1] * layout.mip[l][2] * eb for l in range(layout.nb_levels))
    pool = pool_slots(cfg)
    cm = gc.CacheManager(vol, layout, pool, max_requests=args.max_requests, sync_loader=True)
    cm.set_source_device(pyr.data_ptr(), poffs, keep=pyr)
    tf = tf2d_table()
    tfh, tfw = tf.shape[0], tf.shape[1]
    tf_dev = torch.from_numpy(tf.reshape(-1).copy()).cuda()
    W, H = cfg["W"], cfg["H"]
    bufs = [torch.zeros(W * H * k, dtype=dt, device="cuda") for dt, k in ((torch.int32, 1), (torch.float32, 1),
                                                                        (torch.float32, 4))]
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
    frames = [timed_views(cfg, nviews, 1)[i] for i in range(nviews)]
    stream = torch.cuda.Stream()
    lat, iters, conv = [], [], 0
    s0 = cm.stats()
    torch.cuda.synchronize()
    a = time.perf_counter()
    for f in frames:
        v = gc.make_view(path_camera(gc.look_at, cfg, f), W, H, tf_dev.data_ptr(), tfw, *[b.data_ptr() for b in bufs],
                         tstep=2.0 / 256.0, focal=focal, early_alpha=cfg["early"], tf_height=tfh)
        b0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for b in bufs[1:]:
                b.zero_()
            it, ok = 0, False
            while not ok and it < cfg["cap"]:
                cm.render(v, stream.cuda_stream)
                ok = cm.update(stream.cuda_stream)
                it += 1
        stream.synchronize()
        lat.append(1e3 * (time.perf_counter() - b0))
        iters.append(it)
        conv += int(ok)
    wall = time.perf_counter() - a
    s1 = cm.stats()
    cm.close()
    del pyr
    torch.cuda.empty_cache()
    return {"workload": f"c5: 4096^3 x 2 u8 channels (128 GiB), B16, covering 2, big bricks 2^3, {list(pool)} pool "
                        f"slots (8 GiB), {W}x{H} views {frames} of the {cfg['frames']}-view path through the interior, "
                        f"2D transfer function, each to convergence (<= {cfg['cap']} iterations); bricks cut on "
                        f"demand from the device-resident mip pyramid",
            "value": round(W * H * len(frames) / wall / 1e6, 3), "unit": "Mrays/s",
            "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
            "iterations_per_view": iters, "converged_views": f"{conv}/{len(frames)}",
            "bricks_installed": int(s1.bricks_installed - s0.bricks_installed),
            "brick_bytes_cut": int((s1.bricks_installed - s0.bricks_installed) * cfg["B"] ** 3 * eb),
            "host_upload_bytes": int(s1.bytes_h2d - s0.bytes_h2d),
            "generate_s": round(t1 - t0, 2),
            "mip_build": {"s": round(t2 - t1, 4), "pyramid_gib": round(pyramid_bytes / 2**30, 1),
                          "gbs": round((2 * pyramid_bytes - level0) / (t2 - t1) / 1e9, 1),
                          "note": "every level read once and every coarser level written, over the build time"}}


def run_preprocess_only(args):
    """`--preprocess-only`: the device pre-processing of the c2 volume type
    (u16, B16, covering 1) at --size^3 with the brick store kept on the device
    (twice; the second timed): mip pyramid, bricking of every level, value
    bins.  For profiler captures of the mip and bricking kernels (1024^3: about
    8 GB on the device).  Prints one JSON line with the stage timings."""
    import torch

    import gcgb300 as gc

    cfg = CONFIGS["c2"]
    n = args.size
    size = (n, n, n)
    vol = gc.volume_desc(size, cfg["B"], cfg["c"], cfg["bpc"], 1, (1, 1, 1))
    layout = gc.compute_layout(vol)
    blobs = gc.generator_blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0] * n / 2048,
                               cfg["sigma"][1] * n / 2048, cfg["amp"][0], cfg["amp"][1])
    d = torch.empty(n ** 3 * cfg["bpc"], dtype=torch.uint8, device="cuda")
    gc.generate_volume(gc.make_generator(size, cfg["bpc"], cfg["seed"], blobs, cfg["noise"]), d.data_ptr())
    tm = {}
    for _ in range(2):
        bricks, _, _ = gc.pre_process(vol, layout, d, timings=tm, store="device", value_bins=[])
        del bricks
    torch.cuda.synchronize()
    peak = measured_peak()[0]
    mip_gbs = (2 * tm["pyramid_bytes"] - tm["level0_bytes"]) / tm["mip_s"] / 1e9
    brick_gbs = (tm["pyramid_bytes"] + tm["store_bytes"]) / tm["brick_s"] / 1e9
    print(json.dumps({"preprocess_only": {"volume": f"{n}^3 u16, B16, covering 1", "mip_s": round(tm["mip_s"], 5),
                                          "mip_gbs": round(mip_gbs, 1), "mip_frac": round(mip_gbs / peak, 3),
                                          "bricking_s": round(tm["brick_s"], 5), "bricking_gbs": round(brick_gbs, 1),
                                          "bricking_frac": round(brick_gbs / peak, 3),
                                          "value_bins_s": round(tm["flags_bins_s"], 5)}}), flush=True)


def run_roofline_only(args):
    """`--roofline-only`: the c2 roofline launch alone, for ncu captures.  The
    volume's mip pyramid is built on the device and serves as the brick source
    (nothing is read from host memory under the profiler); views roofline-2
    .. roofline are rendered to convergence, the pyramid is released (the
    pool then holds every brick the view needs; no update follows), and the
    roofline view is re-rendered from scratch after an L2 flush `--steps`
    times inside the NVTX range "roofline" (about 3 GB held on the device).
    Prints one JSON line with the launch times (CUDA events)."""
    import torch

    import gcgb300 as gc

    gc.render_precision(gc.RENDER_FAST if args.precision == "fast" else gc.RENDER_EXACT)
    cfg = CONFIGS["c2"]
    size, eb = cfg["size"], cfg["bpc"]
    vol = gc.volume_desc(size, cfg["B"], cfg["c"], eb, 1, (1, 1, 1))
    layout = gc.compute_layout(vol)
    poffs, total = gc.pyramid_offsets(layout, eb)
    pyr = torch.empty(total, dtype=torch.uint8, device="cuda")
    blobs = gc.generator_blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0],
                               cfg["amp"][1])
    gc.generate_volume(gc.make_generator(size, eb, cfg["seed"], blobs, cfg["noise"]), pyr.data_ptr())
    gc.Mipmapper.process(pyr.data_ptr(), layout, poffs, eb, 1)
    torch.cuda.synchronize()
    if args.tuning:
        gc.render_tuning(*[int(x) for x in args.tuning.split(",")])
    cm = gc.CacheManager(vol, layout, pool_slots(cfg), max_requests=args.max_requests, sync_loader=True,
                         pt_block=args.pt_block, pt_slots=args.pt_slots if args.pt_block else 0)
    cm.set_source_device(pyr.data_ptr(), poffs, keep=pyr)
    tf = torch.from_numpy(tf_table(cfg["tf"]).reshape(-1).copy()).cuda()
    W, H = cfg["W"], cfg["H"]
    bufs = [torch.zeros(W * H * k, dtype=dt, device="cuda") for dt, k in ((torch.int32, 1), (torch.float32, 1),
                                                                        (torch.float32, 4))]
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
    stream = torch.cuda.Stream()
    frame = cfg.get("roofline_frame", 42)
    iters = []
    for f in (frame - 2, frame - 1, frame):
        v = gc.make_view(path_camera(gc.look_at, cfg, f), W, H, tf.data_ptr(), 256, *[b.data_ptr() for b in bufs],
                         tstep=2.0 / 256.0, focal=focal, early_alpha=cfg["early"])
        with torch.cuda.stream(stream):
            bufs[1].zero_()
            bufs[2].zero_()
            it, ok = 0, False
            while not ok and it < 128:
                cm.render(v, stream.cuda_stream)
                ok = cm.update(stream.cuda_stream)
                it += 1
        stream.synchronize()
        iters.append(it)
    cm.drop_sources()
    del pyr
    torch.cuda.empty_cache()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times = []
    s0 = cm.stats().samples
    torch.cuda.nvtx.range_push("roofline")
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            bufs[1].zero_()
            bufs[2].zero_()
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            cm.render(v, stream.cuda_stream)
            e1.record(stream)
        stream.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.nvtx.range_pop()
    st = cm.stats()
    print(json.dumps({"roofline_only": {"view": frame, "iterations_to_converge": iters,
                                        "launch_ms": [round(t, 4) for t in times],
                                        "samples_per_launch": (st.samples - s0) / max(1, args.steps),
                                        "tuning": list(gc.render_tuning()),
                                        "pt_block": args.pt_block,
                                        "device_gb_reserved": round(torch.cuda.memory_reserved() / 1e9, 2)}}),
          flush=True)
    cm.close()


def run_c5(args):
    """`--config c5`: the stress leg alone, printed as its own line."""
    import torch

    import gcgb300 as gc

    gc.render_precision(gc.RENDER_FAST if args.precision == "fast" else gc.RENDER_EXACT)
    r = run_stress(gc, torch, args, nviews=args.steps)
    print(json.dumps({"metric": "Mrays/s", "value": r.get("value"), "unit": "Mrays/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": 0, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "u8x2", "data": "synthetic (seeded blob field + noise field)",
                      "config": {"workload": r.get("workload")}, "stress": r}), flush=True)


def run_c4(args):
    """`--config c4`: the serving form.  Three volumes are generated and
    pre-processed on the device and kept as host brick stores; one cache holds
    all three in a shared 24 GiB pool.  Requests arrive as a Poisson stream
    (seeded) over `duration` seconds, each with a random volume, camera,
    resolution and one of 4 transfer functions; each is submitted to the
    continuous batch at its arrival time and retired when converged.  Latency =
    arrival -> retirement; Mrays/s = rays of all requests / time to the last
    retirement.  The three stores (85 GiB) stay in pageable host memory: page-
    locking them would hold half of the host's memory."""
    import torch

    import gcgb300 as gc

    global PIN_STORES
    PIN_STORES = False
    cfg = CONFIGS["c4"]
    vols, stores, prep = c4_stores(gc, torch, cfg)
    out = c4_serve(gc, torch, cfg, vols, stores, args)
    out["config"]["preprocess_s"] = round(prep, 2)
    print(json.dumps(out), flush=True)


def c4_stores(gc, torch, cfg):
    """The three c4 volumes generated and pre-processed on the device; host stores."""
    vols, stores = [], []
    prep = 0.0
    for vc in cfg["volumes"]:
        vcfg = dict(vc, B=cfg["B"], c=cfg["c"])
        vol, layout, store, offs, prep_s = make_store(gc, torch, vcfg)
        vols.append((vol, layout))
        stores.append((store, offs))
        prep += prep_s
    return vols, stores, prep


def c4_serve(gc, torch, cfg, vols, stores, args):
    """One serving run over a fresh shared cache; returns the JSON object."""
    widest = max(vols, key=lambda v: v[0].encoded_bytes)[0]
    pool = gc.pool_dims(widest, cfg["pool_bytes"])
    cm = gc.CacheManager(vols[0][0], vols[0][1], pool, max_requests=args.max_requests, sync_loader=False,
                         shared=vols, staged_upload=args.upload == "staged")
    for k, (store, offs) in enumerate(stores):
        cm.set_source_host(store, offs, volume=k)
        if Session.brick_bins:
            cm.set_brick_bins(BRICK_BINS[store.data_ptr()], volume=k)
    tfs = [torch.from_numpy(tf_table(kind, seed).reshape(-1)).cuda()
           for kind, seed in (("ramp", 0), ("bumps", 3), ("bumps", 4), ("bumps", 5))]
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
    rng = np.random.default_rng(2026)
    reqs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / args.rate)
        if t > args.duration:
            break
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        d = rng.uniform(*cfg["dist"]) * DIAG
        up = (0.0, 1.0, 0.0) if abs(v[1]) < 0.95 else (1.0, 0.0, 0.0)
        W, H = cfg["sizes"][int(rng.integers(0, len(cfg["sizes"])))]
        reqs.append((t, int(rng.integers(0, len(vols))), gc.look_at(tuple(float(c) * d for c in v), (0.0, 0.0, 0.0),
                                                                    up), W, H, int(rng.integers(0, len(tfs)))))
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    B = gc.Batch(cm, max_views=cfg["batch"], max_pixels=args.batch_pixels, max_passes=args.batch_cap,
                 max_occupancy=args.occupancy, max_admit=args.admit, reorder_window=args.reorder,
                 park_above=args.park, overlap_loads=args.overlap)
    bufs, lat, passes, conv, rays_done = {}, [], [], 0, 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nxt = 0
    torch.cuda.nvtx.range_push("serving")
    while len(lat) < len(reqs):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt][0] <= now:  # arrivals so far
            _, vol_i, m, W, H, tf_i = reqs[nxt]
            with torch.cuda.stream(stream):
                b = (torch.empty(W * H, dtype=torch.int32, device="cuda"),
                     torch.empty(W * H, dtype=torch.float32, device="cuda"),
                     torch.empty(W * H * 4, dtype=torch.float32, device="cuda"))
            bufs[nxt] = b
            B.submit(gc.make_view(m, W, H, tfs[tf_i].data_ptr(), 256, b[0].data_ptr(), b[1].data_ptr(),
                                  b[2].data_ptr(), tstep=2.0 / 256.0, focal=focal, early_alpha=cfg["early"],
                                  volume=vol_i), nxt)
            nxt += 1
        active, queued = B.tick(sp)
        for tag, npass, ok, _ in B.poll():
            _, _, _, W, H, _ = reqs[tag]
            lat.append(1e3 * (time.perf_counter() - t0 - reqs[tag][0]))  # arrival -> retirement
            passes.append(npass)
            conv += int(ok)
            rays_done += W * H
            del bufs[tag]
        if active == 0 and queued == 0 and nxt < len(reqs):
            time.sleep(max(0.0, min(0.002, reqs[nxt][0] - (time.perf_counter() - t0))))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    st, bs = cm.stats(), B.stats()
    rays = sum(W * H for _, _, _, W, H, _ in reqs)
    out = {"metric": "Mrays/s", "value": round(rays / wall / 1e6, 3), "unit": "Mrays/s", "n_gpus": 1,
           "steps": len(reqs), "warmup": 0, "ms_per_step": round(1e3 * wall / len(reqs), 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8+u16",
           "data": "synthetic (seeded blobs + value noise; 1024^3 u8, 2048^3 u16, 4096x4096x2048 u8)",
           "config": {"workload": f"c4: serving, {len(reqs)} Poisson requests at {args.rate}/s over "
                                  f"{args.duration} s, 3 volumes in one shared pool {list(pool)} "
                                  f"({cm.info.pool_bytes / 2**30:.1f} GiB), sizes {list(cfg['sizes'])}, 4 TFs",
                      "offered_mrays_per_s": round(rays / args.duration / 1e6, 2), "reorder": args.reorder,
                      "occupancy": args.occupancy, "admit": args.admit, "park_above": args.park,
                      "overlap_loads": bool(args.overlap), "brick_bins": bool(args.brick_bins),
                      "upload": "staged" if args.upload == "staged" else "gather",
                      "stores": "pinned" if PIN_STORES else "pageable",
                      "max_passes": args.batch_cap},
           "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
           "passes_per_request": round(statistics.mean(passes), 2), "converged": f"{conv}/{len(reqs)}",
           "ticks": {"render_ticks": bs.render_ticks, "graph_replays": bs.graph_replays, "parked": bs.parked,
                     "render_ms": round(bs.render_ms, 1), "loader_wait_ms": round(bs.wait_ms, 1)},
           "cache": {"bricks_installed": int(st.bricks_installed), "brick_h2d_bytes": int(st.bytes_h2d),
                     "upload_gbs": round(st.bytes_h2d / (st.upload_ns / 1e9) / 1e9, 1) if st.upload_ns else None,
                     "device_error": int(st.device_error)}}
    B.close()
    cm.close()
    return out


SERVING_RATES = (25.0, 50.0, 75.0, 100.0, 200.0)  # requests per second tried by the default run
SERVING_SECONDS = 2.0
SERVING_P99_MS = 1000.0  # a rate is sustained while the p99 latency stays below this
SERVING_KEEP_UP = 0.95  # ... and the server keeps up with at least this share of the offered rays


def run_serving_sweep(gc, torch, args):
    """The serving form (c4) in the default run: the three volumes in one
    shared pool, Poisson arrivals at each rate of SERVING_RATES for
    SERVING_SECONDS, each on a fresh cache; per rate the served Mrays/s
    (rays of all requests over the time to the last retirement), p50/p99
    latency (arrival -> retirement) and upload GB/s, and the highest rate the
    server sustains: it serves at least SERVING_KEEP_UP of the offered rays
    per second with a p99 latency under SERVING_P99_MS (no queue building
    up).  Requests that reach the pass cap without converging (a close view
    whose working set the pool cannot hold) retire with their preview image
    and are counted in `converged`."""
    global PIN_STORES
    pinned = PIN_STORES
    PIN_STORES = False
    cfg = CONFIGS["c4"]
    vols, stores, prep = c4_stores(gc, torch, cfg)
    PIN_STORES = pinned
    rates, sustained = [], None
    for rate in SERVING_RATES:
        a = argparse.Namespace(**vars(args))
        a.rate, a.duration = rate, SERVING_SECONDS
        r = c4_serve(gc, torch, cfg, vols, stores, a)
        offered = r["config"]["offered_mrays_per_s"]
        ok = (r["value"] >= SERVING_KEEP_UP * offered and r["latency_ms"]["p99"] is not None
              and r["latency_ms"]["p99"] <= SERVING_P99_MS)
        rates.append({"rate_per_s": rate, "requests": r["steps"], "offered_mrays_per_s": offered,
                      "served_mrays_per_s": r["value"], "latency_ms": r["latency_ms"], "converged": r["converged"],
                      "passes_per_request": r["passes_per_request"], "upload_gbs": r["cache"]["upload_gbs"],
                      "sustained": ok})
        if ok:
            sustained = rate
    del stores
    return {"workload": f"c4: 1024^3 u8 + 2048^3 u16 + 4096x4096x2048 u8 (seeds 11-13) in one shared 24 GiB pool; "
                        f"Poisson requests over {SERVING_SECONDS} s per rate, random volume, camera (0.5-3.0x the "
                        f"diagonal), size {list(cfg['sizes'])} and one of 4 transfer functions; continuous batching",
            "rates": rates, "sustained_rate_per_s": sustained,
            "sustained_means": f"served >= {SERVING_KEEP_UP:.0%} of the offered Mrays/s, p99 <= {SERVING_P99_MS:.0f} ms",
            "sustained_p99_ms": next((x["latency_ms"]["p99"] for x in rates if x["rate_per_s"] == sustained), None),
            "preprocess_s": round(prep, 1), "stores": "pageable host memory (85 GiB)"}


def c3_tunings(gc, torch, cfg, data, warm, args):
    """Launch tunings of the two c3 arms, each for its own launch shape, on
    the warm-up views in a cache of their own: the batched arm on one launch
    of 8 views, the plain arm on one launch per view (4 views)."""
    vol, layout, store, offs = data
    T = Session(gc, torch, cfg, vol, layout, store, offs, args.max_requests)
    tune_b, _ = autotune(gc, torch, T, warm[:8], args)
    tune_p, _ = autotune(gc, torch, T, warm[:4], args, per_view=True)
    T.close()
    return tune_b, tune_p


def run_batched(gc, torch, args):
    """c3: the same views rendered batched (continuous batching, all views
    that can progress in one persistent launch per tick) and plain (one view
    per launch, to convergence), each on a fresh cache."""
    cfg = CONFIGS["c3"]
    vol, layout, store, offs, prep_s = make_store(gc, torch, cfg)
    data = (vol, layout, store, offs)
    views, warm = c3_views(gc, cfg, args.batches)
    rays = sum(W * H for _, W, H in views)
    tune_b, tune_p = c3_tunings(gc, torch, cfg, data, warm, args)
    gc.render_tuning(*tune_b)
    batched, _ = batched_pass(gc, torch, cfg, data, views, warm, args)
    gc.render_tuning(*tune_p)
    plain, _ = plain_views_pass(gc, torch, cfg, data, views, warm, args)
    batched["render_tuning"], plain["render_tuning"] = list(tune_b), list(tune_p)
    bins = None
    if not args.brick_bins:  # both arms again with brick value bins given to the caches
        Session.brick_bins = True
        gc.render_tuning(*tune_b)
        bb_, _ = batched_pass(gc, torch, cfg, data, views, warm, args)
        gc.render_tuning(*tune_p)
        bp_, _ = plain_views_pass(gc, torch, cfg, data, views, warm, args)
        Session.brick_bins = False
        bins = {"batched": bb_, "plain_same_views": bp_, "ratio": round(bb_["value"] / bp_["value"], 3)}
    out = {"config": {"workload": f"c3: {len(views)} views ({args.batches} x {cfg['batch']}), sizes "
                                   f"{list(cfg['sizes'])}, cameras at 0.5-3.0x diagonal; BrickSize 32, 4 GiB pool; "
                                   f"all submitted at t0, continuous batching with a {args.batch_pixels} pixel "
                                   f"budget, admission while demand (used + missing) <= {args.occupancy} of the "
                                   f"pool, <= {args.admit} admissions per tick, "
                                   f"asynchronous loader" + (", overlapped loads" if args.overlap else ""),
                       "preprocess_s": round(prep_s, 2), "rays": int(rays)},
            "unit": "Mrays/s", "batched": batched, "plain_same_views": plain,
            "ratio": round(batched["value"] / plain["value"], 3)}
    if bins:
        out["with_brick_bins"] = bins
    return out


def reference_gpu_baseline(gc, torch, args, views=12):
    """The reference's own CUDA build (oracle/_ref/librefgpu.so: its
    Mipmapper, CacheManager<uchar1> and RayCastDVR compiled for sm_103a) timed
    on this GPU beside our plain path on the same c1 views, each rendered to
    convergence.  Both run the reference's fixed parameters -- 128-entry
    transfer function, early termination at alpha 0.95, focal length 2, 50
    brick requests per cycle -- so both caches go through the same frame
    sequence (their states are equal frame by frame, tests/test_gpu_reference.py)
    and the times compare the two implementations of the same work."""
    from oracle import refgpu

    if not refgpu.available():
        return {"unavailable": "no staged copy of the reference sources (oracle/_ref/src)"}
    cfg = dict(CONFIGS["c1"])
    size, W, H = cfg["size"], cfg["W"], cfg["H"]
    vol = gc.volume_desc(size, cfg["B"], cfg["c"], 1, 1)
    layout = gc.compute_layout(vol)
    blobs = gc.generator_blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0],
                               cfg["amp"][1])
    dev = torch.empty(size[0] * size[1] * size[2], dtype=torch.uint8, device="cuda")
    gc.generate_volume(gc.make_generator(size, 1, cfg["seed"], blobs, cfg["noise"]), dev.data_ptr())
    torch.cuda.synchronize()
    tmp = tempfile.mkdtemp(prefix="refgpu_")
    ref = refgpu.RefGpu(tmp, size, cfg["B"], cfg["c"], 1)
    t0 = time.perf_counter()
    ref.preprocess(dev.cpu().numpy())
    ref_pre = time.perf_counter() - t0
    store, offs, _ = gc.pre_process(vol, layout, dev)
    pool = pool_slots(cfg)
    ref.open(pool)
    tf = tf_table(cfg["tf"])
    tf128 = np.ascontiguousarray(tf[np.round(np.linspace(0, tf.shape[0] - 1, 128)).astype(int)])
    tf_dev = torch.from_numpy(tf128.reshape(-1).copy()).cuda()
    bufs = [torch.zeros((W * H + W + 16) * k, dtype=dt, device="cuda")
            for dt, k in ((torch.int32, 1), (torch.float32, 1), (torch.float32, 4))]
    cams = [path_camera(gc.look_at, cfg, f) for f in range(views)]

    def run_ref():
        frames = 0
        for m in cams:
            for b in bufs[1:]:
                b.zero_()
            for _ in range(2000):
                ref.render(m, W, H, 2.0 / 256.0, tf128, 0, *[b.data_ptr() for b in bufs])
                frames += 1
                if ref.update():
                    break
        return frames

    def run_ours(max_requests):
        cm = gc.CacheManager(vol, layout, pool, max_requests=max_requests, sync_loader=True)
        cm.set_source_host(store, offs)
        frames = 0
        torch.cuda.synchronize()
        a = time.perf_counter()
        for m in cams:
            for b in bufs[1:]:
                b.zero_()
            v = gc.make_view(m, W, H, tf_dev.data_ptr(), 128, *[b.data_ptr() for b in bufs])  # early 0.95, focal 2
            for _ in range(2000):
                cm.render(v)
                frames += 1
                if cm.update():
                    break
        torch.cuda.synchronize()
        el = time.perf_counter() - a
        cm.close()
        return frames, el

    a = time.perf_counter()
    ref_frames = run_ref()
    ref_s = time.perf_counter() - a
    ref.close()
    # mip-pyramid build: the reference's Mipmapper (file in, 512 MB chunks through
    # the device, files out) vs the device pyramid build, on a 512^3 x 2-channel
    # u8 volume (the c5 voxel type)
    msize = (512, 512, 512)
    mvol = gc.volume_desc(msize, 16, 2, 2, 2, (2, 2, 2))
    mlayout = gc.compute_layout(mvol)
    mblobs = gc.generator_blobs(5, 8, msize, 10.0, 75.0, 60, 200)
    mpoffs, mtotal = gc.pyramid_offsets(mlayout, 2)
    mpyr = torch.empty(mtotal, dtype=torch.uint8, device="cuda")
    gc.generate_volume(gc.make_generator(msize, 1, 5, mblobs, 20, channels=2, channel=0, field=0), mpyr.data_ptr())
    gc.generate_volume(gc.make_generator(msize, 1, 6, mblobs, 80, channels=2, channel=1, field=1), mpyr.data_ptr())
    torch.cuda.synchronize()
    raw = mpyr[: msize[0] * msize[1] * msize[2] * 2].cpu().numpy()
    mdir = tempfile.mkdtemp(prefix="refmip_")
    mref = refgpu.RefGpu(mdir, msize, 16, 2, 2, big_brick=(2, 2, 2), channels=2)
    mref.write_volume(raw)
    ref_mip_s, ref_brick_s = mref.preprocess_timed()
    gc.Mipmapper.process(mpyr.data_ptr(), mlayout, mpoffs, 2, 2)  # warm
    torch.cuda.synchronize()
    a = time.perf_counter()
    gc.Mipmapper.process(mpyr.data_ptr(), mlayout, mpoffs, 2, 2)
    torch.cuda.synchronize()
    our_mip_s = time.perf_counter() - a
    # bricking of every level into a device store (the reference: LZ4 files)
    msoffs, mstotal, _ = gc.brick_store_offsets(mlayout, mvol)
    mstore = torch.empty(mstotal, dtype=torch.uint8, device="cuda")
    our_brick_s = []
    for _ in range(2):
        torch.cuda.synchronize()
        a = time.perf_counter()
        for l in range(mlayout.nb_levels):
            gc.process_bricking(mpyr.data_ptr() + mpoffs[l], mlayout.initial[l], mvol, mlayout.nb_big_bricks[l],
                                mstore.data_ptr() + msoffs[l])
        torch.cuda.synchronize()
        our_brick_s.append(time.perf_counter() - a)
    our_brick_s = our_brick_s[-1]
    del mstore
    mdims = [tuple(mlayout.mip[l]) for l in range(mlayout.nb_levels)]
    mbytes = sum(d[0] * d[1] * d[2] * 2 for d in mdims)
    same = all(np.array_equal(mref.mip_level(l, d).view(np.uint8),
                              mpyr[mpoffs[l]: mpoffs[l] + d[0] * d[1] * d[2] * 2].cpu().numpy())
               for l, d in enumerate(mdims) if l > 0)
    shutil.rmtree(mdir, ignore_errors=True)
    mip = {"volume": "512^3 x 2 u8 channels", "pyramid_bytes": int(mbytes), "levels_identical": bool(same),
           "reference_s": round(ref_mip_s, 4), "ours_s": round(our_mip_s, 5),
           "reference_gbs": round((2 * mbytes - raw.nbytes) / ref_mip_s / 1e9, 2),
           "ours_gbs": round((2 * mbytes - raw.nbytes) / our_mip_s / 1e9, 1),
           "what": "the reference's Mipmapper::process (reads the level file, 512 MB chunks through the device, "
                   "writes the level files) vs gc_mip_build on the device-resident volume; bytes = every level read "
                   "once + every coarser level written",
           "bricking": {"reference_s": round(ref_brick_s, 4), "ours_s": round(our_brick_s, 5),
                        "store_bytes": int(mstotal),
                        "reference_gbs": round((mbytes + mstotal) / ref_brick_s / 1e9, 3),
                        "ours_gbs": round((mbytes + mstotal) / our_brick_s / 1e9, 1),
                        "what": "the reference's process_bricking of every level (one host thread per level, "
                                "LZ4-HC brick files, covering 2, big bricks 2^3) vs gc_bricks_build of every level "
                                "into a device store; bytes = every level read + the store written"}}
    del mpyr
    ours_frames, ours_s = run_ours(50)
    ours8k_frames, ours8k_s = run_ours(args.max_requests)
    rays = W * H * views
    return {"workload": f"c1 volume and orbit (first {views} views, {W}x{H}), each view to convergence, with the "
                        f"reference's fixed parameters: 128-entry transfer function, early termination 0.95, focal "
                        f"length 2, 50 requests per cycle; fresh caches of {list(pool)} slots",
            "reference_gpu": {"value": round(rays / ref_s / 1e6, 3), "unit": "Mrays/s", "frames": ref_frames,
                              "ms_per_frame": round(1e3 * ref_s / ref_frames, 3),
                              "preprocess_s": round(ref_pre, 2),
                              "what": "the reference's CacheManager<uchar1> + RayCastDVR built for sm_103a, its "
                                      "request handler loading its own LZ4 brick files"},
            "ours_same_requests": {"value": round(rays / ours_s / 1e6, 3), "unit": "Mrays/s", "frames": ours_frames,
                                   "ms_per_frame": round(1e3 * ours_s / ours_frames, 3)},
            "ours_max_requests": {"value": round(rays / ours8k_s / 1e6, 3), "unit": "Mrays/s",
                                  "frames": ours8k_frames, "max_requests": args.max_requests},
            "ratio_same_requests": round(ref_s / ours_s, 2), "mip_build": mip}


def vol_bytes_per_voxel(cfg):
    return cfg["bpc"] * cfg.get("channels", 1)


ARM_PARTS = {"0xd4f": "Neoverse-V2", "0xd40": "Neoverse-V1", "0xd0c": "Neoverse-N1", "0xd49": "Neoverse-N2"}


def host_cpu():
    """The host CPU's model name (x86: /proc/cpuinfo "model name"; Arm: the
    implementer's part number) for the CPU baselines."""
    try:
        with open("/proc/cpuinfo") as f:
            lines = f.read().splitlines()
        for line in lines:
            if line.lower().startswith("model name") and ":" in line:
                return line.split(":", 1)[1].strip()
        for line in lines:
            if line.startswith("CPU part") and ":" in line:
                part = line.split(":", 1)[1].strip().lower()
                return f"{platform.machine()} {ARM_PARTS.get(part, 'part ' + part)}"
    except Exception:  # a reported detail: never fails the line
        pass
    return platform.machine()


def cpu_baseline(gc, S, cfg, spec, args, images):
    """The oracle's FP32 ray-march (all host threads) on a bounded sample of
    converged c2 views, reading a snapshot of the GPU's cache state; its image
    is compared with the GPU's images of the same view (images: build name ->
    RGBA8 array)."""
    from oracle import oracle as orc

    (m, W, H), = spec
    oc = orc.Cache(S.cm.desc)
    S.cm.dump(gc.DUMP_MRPD, oc.mrpd())
    S.cm.dump(gc.DUMP_POOL, oc.pool())
    tf_np = S.tf.cpu().numpy()
    rgba = np.zeros(W * H, np.uint32)
    tb = np.zeros(W * H, np.float32)
    st = np.zeros(W * H * 4, np.float32)
    v = gc.make_view(m, W, H, 0, S.tfw, 0, 0, 0, tstep=2.0 / 256.0, focal=S.focal, early_alpha=cfg["early"],
                     tf_height=S.tfh)
    frames = 0
    t0 = time.perf_counter()
    while True:
        tb[:] = 0
        st[:] = 0
        oc.render(v, tf_np, rgba, tb, st)
        frames += 1
        el = time.perf_counter() - t0
        if el > args.cpu_seconds:
            break
    oc.close()
    # parity: the GPU's renders of this view (from scratch, same cache state)
    # against the oracle's render of it
    parity = {"vs": "the FP32 oracle's render of the same view from the GPU's cache state (units of 1/255)",
              "pixels": int(W * H)}
    for name, img in images.items():
        dif = np.abs(img.view(np.uint8).astype(np.int32) - rgba.view(np.uint8).astype(np.int32)).reshape(-1, 4).max(1)
        parity[name] = {"max_abs_rgba": int(dif.max()), "pixels_differing": int(np.count_nonzero(dif)),
                        "pixels_beyond_1": int(np.count_nonzero(dif > 1))}
    parity["max_abs_rgba"] = parity["exact"]["max_abs_rgba"]
    # the CPU restatement of the mip reduction (down_sampling_inner) on a bounded
    # 512 x 512 x 64 sample of the same voxel type, single thread
    nc = cfg.get("channels", 1)
    sample = np.random.default_rng(1).integers(0, 255, size=512 * 512 * 64 * vol_bytes_per_voxel(cfg),
                                               dtype=np.uint8)
    t1 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t1 < 2.0:
        orc.mip_level(sample, (512, 512, 64), vol_bytes_per_voxel(cfg), nc)
        reps += 1
    mip_cpu = reps * sample.nbytes * 1.125 / (time.perf_counter() - t1) / 1e9
    # the same over all host cores (z pairs split between threads)
    t1 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t1 < 2.0:
        orc.mip_level(sample, (512, 512, 64), vol_bytes_per_voxel(cfg), nc, threads=0)
        reps += 1
    mip_cpu_all = reps * sample.nbytes * 1.125 / (time.perf_counter() - t1) / 1e9
    # the CPU restatement of process_bricking (checked against the reference's
    # own bricker), one thread, on a bounded 256 x 256 x 128 level of the voxel type
    bdims = (256, 256, 128)
    bvol = gc.volume_desc(bdims, cfg["B"], cfg["c"], vol_bytes_per_voxel(cfg), nc, cfg.get("bb", (1, 1, 1)))
    blay = gc.compute_layout(bvol)
    level = np.random.default_rng(2).integers(0, 255, size=bdims[0] * bdims[1] * bdims[2] * vol_bytes_per_voxel(cfg),
                                              dtype=np.uint8)
    t1 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t1 < 2.0:
        orc.brick_level(level, bdims, bvol, tuple(blay.nb_big_bricks[0]))
        reps += 1
    brick_cpu = reps * level.nbytes / (time.perf_counter() - t1) / 1e9
    return {"value": round(W * H * frames / el / 1e6, 4), "unit": "Mrays/s", "cores": os.cpu_count(),
            "cpu_model": host_cpu(),
            "mip_cpu_gbs_1thread": round(mip_cpu, 2), "mip_cpu_gbs_all_cores": round(mip_cpu_all, 2),
            "bricking_cpu_gbs_1thread": round(brick_cpu, 3),
            "kind": "port", "sample": f"{frames} renders of one converged {W}x{H} {args.config} view from the GPU's cache "
                                      f"snapshot (oracle FP32 ray-march, {os.cpu_count()} threads)",
            "parity": parity}


def make_store_cpu(cfg):
    """The brick store of a config built on the host cores by the oracle alone
    (generator, mip restatement, bricker restatement checked against the
    reference's own bricker): no GPU library is loaded."""
    from oracle import oracle as orc

    size, bpc, nc = cfg["size"], cfg["bpc"], cfg.get("channels", 1)
    eb = bpc * nc
    u3 = orc.U3
    vol = orc.VolumeDesc(u3(*size), cfg["B"], u3(*cfg.get("bb", (1, 1, 1))), cfg["c"], eb, nc, u3(2, 2, 2))
    layout = orc.layout(vol)
    t0 = time.time()
    blobs = orc.blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0],
                      cfg["amp"][1])
    level = orc.generate(size, bpc, cfg["seed"], blobs, cfg["nblobs"], cfg["noise"], channels=nc)
    for ch in range(1, nc):
        orc.generate(size, bpc, cfg["seed"] + ch, blobs, cfg["nblobs"], cfg["noise"] * 4, channels=nc, channel=ch,
                     field=1, out=level)
    level = level.reshape(-1)
    t1 = time.time()
    big = cfg["B"] ** 3 * int(np.prod(cfg.get("bb", (1, 1, 1)))) * eb
    offs, total = [], 0
    for l in range(layout.nb_levels):
        offs.append(total)
        total += int(np.prod(layout.nb_big_bricks[l])) * big
    store = np.empty(total, np.uint8)
    for l in range(layout.nb_levels):
        if l > 0:
            level = orc.mip_level(level, tuple(layout.initial[l - 1]), eb, nc, threads=0)
        n = int(np.prod(layout.nb_big_bricks[l])) * big
        orc.brick_level(level.view(np.uint8), tuple(layout.initial[l]), vol, tuple(layout.nb_big_bricks[l]),
                        out=store[offs[l]:offs[l] + n])
    log(f"volume {size} B{cfg['B']} on the host: generated {t1 - t0:.1f}s, mip + bricks {time.time() - t1:.1f}s "
        f"({total / 2**30:.2f} GiB)")
    return vol, layout, store, offs


def run_reference(args):
    """The reference arm: the CPU port of the plain path (the oracle's FP32
    ray-march + cache state machine on all host cores), each of the GPU arm's
    timed views rendered to convergence.  Loads only the oracle library."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import oracle as orc

    cfg = CONFIGS[args.config]
    vol, layout, store, offs = make_store_cpu(cfg)
    pool = pool_slots(cfg)
    desc = orc.CacheDesc(vol, layout, orc.U3(*pool), args.max_requests, 1, 0)  # GC_CACHE_SYNC_LOADER
    oc = orc.Cache(desc)
    oc.set_source(store, offs)
    W, H = cfg["W"], cfg["H"]
    tf = tf2d_table() if cfg["tf"] == "2d" else tf_table(cfg["tf"])
    tfh, tfw = (tf.shape[0], tf.shape[1]) if tf.ndim == 3 else (0, tf.shape[0])
    tf = np.ascontiguousarray(tf.reshape(-1))
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
    rgba = np.zeros(W * H, np.uint32)
    tb = np.zeros(W * H, np.float32)
    st = np.zeros(W * H * 4, np.float32)
    F3 = orc.C.c_float * 3

    def view_to_convergence(f):
        m = path_camera(look_at_host, cfg, f)
        v = orc.View((orc.C.c_float * 12)(*m), W, H, F3(-1, -1, -1), F3(1, 1, 1), 2.0 / 256.0, focal, cfg["early"],
                     0, 0, tfw, None, None, None, None, None, 0, tfh, 0)
        tb[:] = 0
        st[:] = 0
        for it in range(cfg.get("cap", 64)):
            oc.render(v, tf, rgba, tb, st)
            if oc.update():
                return it + 1, True
        return cfg.get("cap", 64), False

    views = timed_views(cfg, args.steps, args.warmup)
    for f in range(args.warmup):
        view_to_convergence(f)
    lat, info = [], []
    t0 = time.perf_counter()
    for f in views:
        a = time.perf_counter()
        info.append(view_to_convergence(f))
        lat.append(1e3 * (time.perf_counter() - a))
    el = time.perf_counter() - t0
    value = W * H * len(views) / el / 1e6
    wl, dt, data_txt = workload(args.config, cfg)
    sample = (f"the {len(views)} views the GPU arm times, each to convergence after {args.warmup} warm-up views: "
              f"oracle FP32 ray-march + cache state machine, {os.cpu_count()} threads")
    out = {"impl": "reference", "metric": "Mrays/s", "value": round(value, 4), "unit": "Mrays/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * el / args.steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dt, "data": data_txt,
           "config": bench_config(args.config, cfg, args),
           "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
           "iterations_per_view": {"mean": round(statistics.mean(i for i, _ in info), 2),
                                   "max": max(i for i, _ in info)},
           "converged_views": f"{sum(1 for _, c in info if c)}/{len(views)}",
           "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": os.cpu_count(),
                            "cpu_model": host_cpu(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    oc.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=["c1", "c2", "c3", "c4", "c5", "c5_host"], default="c2",
                    help="c2: the plain out-of-core line (+ the c3 batched object); c1: small in-core plain case; "
                         "c3: the batched form alone; c4: serving (three volumes, shared pool, Poisson requests); "
                         "c5: two-channel 2D-TF stress at 4096^3 from the device-resident pyramid; "
                         "c5_host: the same at 2048^3 from a host brick store (plain loop)")
    ap.add_argument("--rate", type=float, default=200.0, help="c4: request arrivals per second")
    ap.add_argument("--duration", type=float, default=6.0, help="c4: seconds of arrivals")
    ap.add_argument("--max-requests", type=int, default=8192)
    ap.add_argument("--batches", type=int, default=3)
    ap.add_argument("--batch-cap", type=int, default=256)
    ap.add_argument("--batch-pixels", type=int, default=16 << 20)
    ap.add_argument("--occupancy", type=float, default=0.45)
    ap.add_argument("--admit", type=int, default=4)
    ap.add_argument("--upload", choices=["auto", "staged"], default="auto",
                    help="brick upload route: auto = gather kernel reading the host store where the device can, "
                         "staged = host copies into pinned staging + cudaMemcpyAsync")
    ap.add_argument("--reorder", type=int, default=192,
                    help="batched admission: locality window over queued views (0: arrival order)")
    ap.add_argument("--pageable-stores", dest="pin_stores", action="store_false",
                    help="keep the host brick stores in pageable memory (read by the gather kernel where the "
                         "device accesses pageable memory) instead of page-locked memory")
    ap.add_argument("--park", type=float, default=0.0,
                    help="batched/serving: park the newest view while demand exceeds this fraction of the pool")
    ap.add_argument("--brick-bins", action="store_true",
                    help="give each cache the value bins of every brick: missing bricks the transfer function "
                         "cannot make visible are stepped through, not loaded (same images; not the reference's "
                         "request sequence)")
    ap.add_argument("--no-overlap", dest="overlap", action="store_false",
                    help="batched/serving: one brick load at a time (default: loads overlap rendering through "
                         "two miss lists with in-flight marks)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--precision", choices=["exact", "fast"], default="fast",
                    help="ray-caster build: exact (the FP32 oracle's operations, bit for bit) or fast (FMA "
                         "contraction, rsqrtf, hardware log2/exp2; validated against the FP64 oracle and the "
                         "reference's ray caster)")
    ap.add_argument("--no-stress", action="store_true",
                    help="skip the c5 stress leg (4096^3 x 2 channels) of the default run")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the serving (c4) rate sweep of the default run")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the reference's own CUDA build timed beside our plain path (c1 views)")
    ap.add_argument("--no-plain", action="store_true", help="c3: skip the plain loop over the same views")
    ap.add_argument("--pt-block", type=int, default=0,
                    help="--roofline-only: a two-level page directory with this block size (0: one level)")
    ap.add_argument("--pt-slots", type=int, default=PT_SLOTS, help="--roofline-only: table-pool blocks")
    ap.add_argument("--roofline-only", action="store_true",
                    help="only the c2 roofline launch, --steps times, bricks from the device pyramid (for ncu)")
    ap.add_argument("--preprocess-only", action="store_true",
                    help="only the device pre-processing (mip, bricks, bins) of a --size^3 u16 volume (for ncu)")
    ap.add_argument("--size", type=int, default=2048, help="--preprocess-only: volume edge")
    ap.add_argument("--tuning", default=None,
                    help="ray-caster launch tuning 'scheduler,tile_w,threads,blocks_per_sm' for --roofline-only")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 20
    args.warmup = max(3, args.warmup)
    Session.staged = args.upload == "staged"
    Session.brick_bins = args.brick_bins
    global PIN_STORES
    PIN_STORES = args.pin_stores
    if args.config != "c2":
        args.no_batched = True
        args.no_serving = True
        args.no_stress = True
    if args.impl == "reference" and args.config in ("c3", "c4"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference arm covers the plain configs "
                                                              "(c1, c2); c3 is the batched form"}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    elif args.config == "c3":
        run_c3(args)
    elif args.config == "c4":
        run_c4(args)
    elif args.config == "c5":
        run_c5(args)
    elif args.roofline_only:
        run_roofline_only(args)
    elif args.preprocess_only:
        run_preprocess_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
