"""Benchmark of the out-of-core volume path on one GB300.

Metric: Mrays/s (primary rays W*H per view per frame) with p50/p99 frame
latency, plain per-view path; the batched form is reported beside it.

  python bench.py [--config c2] [--steps K] [--warmup W] [--impl ours|reference]

Workloads (seeded synthetic volumes with the shapes of the benchmark configs;
no public dataset is used):
  c1  256^3 u8, BrickSize 16, covering 1, 512^2 views orbiting at 2x the
      diagonal, fov 45 deg, TF ramp (alpha 0 at 40 -> 0.6 at 255), early alpha 0.99
  c2  2048^3 u16 (16 GiB), BrickSize 16, covering 1, 2 GiB pool, 1024^2 views
      on a fly-through zooming from 3.0x to 0.3x the diagonal, TF with 3
      Gaussian alpha bumps
A step is one frame: render (camera parameters go host -> device with the
call), cache update (LRU update, miss scan or brick install; missed bricks go
up from pinned host memory on a side stream), and for e2e the RGBA frame read
back into pinned host memory.  Inputs larger than L2 (the pool and the page
directory) are touched every frame.

--impl reference runs the CPU port of the same method (the oracle's FP32
ray-march + cache state machine, all host threads) on a bounded sample.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gpu-out-of-core-volume-data_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

CONFIGS = {
    "c1": dict(size=(256, 256, 256), bpc=1, nblobs=8, sigma=(10.0, 40.0), amp=(60, 200), noise=20, seed=1, B=16,
               c=1, pool_bytes=None, pool_slots=(21, 21, 21), W=512, H=512, frames=36, path="orbit",
               dist=(2.0, 2.0), tf="ramp", early=0.99, fov=45.0),
    "c2": dict(size=(2048, 2048, 2048), bpc=2, nblobs=32, sigma=(40.0, 300.0), amp=(60 * 257, 200 * 257),
               noise=20 * 257, seed=2, B=16, c=1, pool_bytes=2 << 30, pool_slots=None, W=1024, H=1024, frames=120,
               path="fly", dist=(3.0, 0.3), tf="bumps", early=0.99, fov=45.0),
}
DIAG = 2.0 * math.sqrt(3.0)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def tf_table(kind, seed=3):
    x = np.linspace(0.0, 1.0, 256)
    if kind == "ramp":
        v = x * 255.0
        a = np.where(v <= 40, 0.0, 0.6 * np.clip((v - 40) / 215.0, 0, 1))
        rgb = np.stack([np.clip(0.2 + 1.2 * x, 0, 1), 0.3 + 1.2 * x * (1 - x), 1.0 - x], 1)
    else:
        rng = np.random.default_rng(seed)
        a = np.zeros_like(x)
        for _ in range(3):
            c, w, h = rng.uniform(0.2, 0.9), rng.uniform(0.02, 0.08), rng.uniform(0.2, 0.8)
            a += h * np.exp(-0.5 * ((x - c) / w) ** 2)
        rgb = np.stack([np.clip(0.3 + x, 0, 1), np.clip(1.2 - x, 0, 1), 0.5 + 0.5 * np.sin(6 * x)], 1)
    return np.concatenate([rgb, np.clip(a, 0, 1)[:, None]], 1).astype(np.float32)


def camera(gc, cfg, f, rank=0):
    n = cfg["frames"]
    t = (f % n) / max(1, n - 1)
    if cfg["path"] == "orbit":
        ang = 2 * math.pi * ((f + rank * 7) % n) / n
        d = cfg["dist"][0] * DIAG
        eye = (d * math.sin(ang) * math.cos(0.3), d * math.sin(0.3), d * math.cos(ang) * math.cos(0.3))
        return gc.look_at(eye)
    d = (cfg["dist"][0] + (cfg["dist"][1] - cfg["dist"][0]) * t) * DIAG
    ang = 0.6 * t + 0.4 * rank
    dirv = (math.sin(ang) * 0.8, 0.35, math.cos(ang))
    nrm = math.sqrt(sum(c * c for c in dirv))
    eye = tuple(d * c / nrm for c in dirv)
    target = tuple(0.15 * math.sin(3 * t + rank) * c for c in (1.0, 0.5, 0.2))
    return gc.look_at(eye, target)


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        self.proc.wait(timeout=5)
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.remove(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def build_scene(gc, torch, cfg, max_requests, sync):
    size, bpc = cfg["size"], cfg["bpc"]
    vol = gc.volume_desc(size, cfg["B"], cfg["c"], bpc, 1)
    layout = gc.compute_layout(vol)
    t0 = time.time()
    blobs = gc.generator_blobs(cfg["seed"], cfg["nblobs"], size, cfg["sigma"][0], cfg["sigma"][1], cfg["amp"][0],
                               cfg["amp"][1])
    dev = torch.empty(size[0] * size[1] * size[2] * bpc, dtype=torch.uint8, device="cuda")
    gc.generate_volume(gc.make_generator(size, bpc, cfg["seed"], blobs, cfg["noise"]), dev.data_ptr())
    torch.cuda.synchronize()
    t1 = time.time()
    store, offs, _ = gc.pre_process(vol, layout, dev)
    del dev
    torch.cuda.empty_cache()
    t2 = time.time()
    log(f"volume {size} generated in {t1 - t0:.2f}s, pre-processed ({store.numel() / 2**30:.2f} GiB bricks) "
        f"in {t2 - t1:.2f}s")
    pool = cfg["pool_slots"] or gc.pool_dims(vol, cfg["pool_bytes"])
    cm = gc.CacheManager(vol, layout, pool, max_requests=max_requests, sync_loader=sync)
    cm.set_source_host(store.data_ptr(), offs)
    return vol, layout, store, offs, cm, pool, (t2 - t0)


def run_ours(args, cfg):
    import torch

    import gcgb300 as gc

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    vol, layout, store, offs, cm, pool, prep_s = build_scene(gc, torch, cfg, args.max_requests, sync=False)
    W, H = cfg["W"], cfg["H"]
    tf = torch.from_numpy(tf_table(cfg["tf"]).reshape(-1)).cuda()
    rgba = torch.zeros(W * H, dtype=torch.int32, device="cuda")
    tbuf = torch.zeros(W * H, dtype=torch.float32, device="cuda")
    state = torch.zeros(W * H * 4, dtype=torch.float32, device="cuda")
    host_rgba = torch.empty(W * H, dtype=torch.int32, pin_memory=True)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)

    def view(f):
        return gc.make_view(camera(gc, cfg, f, rank), W, H, tf.data_ptr(), 256, rgba.data_ptr(), tbuf.data_ptr(),
                            state.data_ptr(), tstep=2.0 / 256.0, focal=focal, early_alpha=cfg["early"])

    def frame(f, e2e, ev):
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            tbuf.zero_()   # camera moved: restart progressive rendering (VolumeRayCaster.cu:320-329)
            state.zero_()
            ev[1].record(stream)
            cm.render(view(f), sp)
            ev[2].record(stream)
            cm.update(sp)
            if e2e:
                host_rgba.copy_(rgba, non_blocking=True)
            ev[3].record(stream)

    def loop(k, start, e2e):
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(k)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(k):
            frame(start + i, e2e, evs[i])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        lat = [evs[i][0].elapsed_time(evs[i][3]) for i in range(k)]
        rend = [evs[i][1].elapsed_time(evs[i][2]) for i in range(k)]
        return wall, lat, rend

    for f in range(args.warmup):
        frame(f, True, [torch.cuda.Event(enable_timing=True) for _ in range(4)])
    torch.cuda.synchronize()
    s0 = cm.stats()
    launches0 = gc.kernel_launches()
    clocks = ClockSampler()
    clocks.start()
    wall_dev, lat_dev, rend_dev = loop(args.steps, args.warmup, e2e=False)
    launches_dev = gc.kernel_launches() - launches0
    s1 = cm.stats()
    wall_e2e, lat_e2e, rend_e2e = loop(args.steps, args.warmup + args.steps, e2e=True)
    s2 = cm.stats()
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([wall_dev, wall_e2e], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        wall_dev, wall_e2e = t.tolist()
    rays = W * H * args.steps * world
    value = rays / wall_dev / 1e6
    e2e = rays / wall_e2e / 1e6

    # roofline of the dominant kernel (dvr_march): compulsory bytes per launch =
    # touched bricks * B^3 * bytes + W*H * (4 RGBA + 20 state read + 20 state write)
    frame(args.warmup + 2 * args.steps, False, [torch.cuda.Event(enable_timing=True) for _ in range(4)])
    torch.cuda.synchronize()
    touched = cm.stats().last_used
    algo_bytes = touched * cfg["B"] ** 3 * vol.encoded_bytes + W * H * 44
    avg_render_s = statistics.mean(rend_dev) / 1e3
    peak, peak_kind = measured_peak()
    achieved = algo_bytes / avg_render_s / 1e9
    gather = None

    out = {
        "metric": "Mrays/s", "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * wall_dev / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u16" if cfg["bpc"] == 2 else "u8",
        "data": "synthetic (seeded blobs + value noise, benchmark-config shapes)",
        "config": {"workload": f"{args.config}: plain per-view out-of-core frame loop", "volume": list(cfg["size"]),
                   "bytes_per_voxel": cfg["bpc"], "brick_size": cfg["B"], "covering": cfg["c"],
                   "pool_slots": list(pool), "view": [W, H], "frames_in_path": cfg["frames"],
                   "max_requests": args.max_requests, "loader": "async", "l2": "pool and page directory > L2",
                   "preprocess_s": round(prep_s, 2)},
        "latency_ms": {"p50": round(statistics.median(lat_dev), 4),
                       "p99": round(float(np.percentile(lat_dev, 99)), 4)},
        "e2e": {"value": round(e2e, 3), "unit": "Mrays/s",
                "h2d_bytes_per_step": int((s2.bytes_h2d - s1.bytes_h2d) / args.steps) + 700,
                "d2h_bytes_per_step": W * H * 4,
                "latency_ms": {"p50": round(statistics.median(lat_e2e), 4),
                               "p99": round(float(np.percentile(lat_e2e, 99)), 4)}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": None,
                     "kernel": "render_kernel (dvr_march)", "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": int(algo_bytes), "avg_launch_ms": round(avg_render_s * 1e3, 4),
                     "touched_bricks": int(touched)},
        "gpu_launches": int(launches_dev),
        "cache": {"bricks_installed": int(s1.bricks_installed - s0.bricks_installed),
                  "requests_raised": int(s1.requests_raised - s0.requests_raised),
                  "brick_h2d_bytes": int(s1.bytes_h2d - s0.bytes_h2d), "device_error": int(s2.device_error)},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(gc, cm, cfg, vol, layout, store, offs, tf, args)
    if rank == 0:
        print(json.dumps(out), flush=True)
    cm.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(gc, cm, cfg, vol, layout, store, offs, tf, args):
    """The oracle's FP32 ray-march (all host threads) on a bounded sample of the
    same frames, reading a snapshot of the GPU's cache state."""
    from oracle import oracle as orc

    W, H = cfg["W"], cfg["H"]
    oc = orc.Cache(cm.desc)
    cm.dump(gc.DUMP_MRPD, oc.mrpd())
    cm.dump(gc.DUMP_POOL, oc.pool())
    tf_np = tf.cpu().numpy()
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
    rgba = np.zeros(W * H, np.uint32)
    tb = np.zeros(W * H, np.float32)
    st = np.zeros(W * H * 4, np.float32)
    frames = 0
    t0 = time.perf_counter()
    while True:
        v = gc.make_view(camera(gc, cfg, frames), W, H, 0, 256, 0, 0, 0, focal=focal, early_alpha=cfg["early"])
        tb[:] = 0
        st[:] = 0
        oc.render(v, tf_np, rgba, tb, st)
        frames += 1
        el = time.perf_counter() - t0
        if el > args.cpu_seconds or frames >= cfg["frames"]:
            break
    oc.close()
    return {"value": round(W * H * frames / el / 1e6, 4), "unit": "Mrays/s", "cores": os.cpu_count(),
            "kind": "port", "sample": f"{frames} frames of {W}x{H} on the GPU's converged-so-far cache state "
                                      f"(FP32 ray-march of the oracle, {os.cpu_count()} threads)"}


def run_reference(args, cfg):
    """CPU port of the whole frame loop (render + cache update) on the host."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch

    import gcgb300 as gc
    from oracle import oracle as orc

    # inputs: the same brick store (built on the device; bytes identical to the
    # oracle's own mip + bricker, see tests/test_gpu_preprocess.py)
    vol, layout, store, offs, cm, pool, prep_s = build_scene(gc, torch, cfg, args.max_requests, sync=True)
    oc = orc.Cache(cm.desc)
    cm.close()
    st_np = store.numpy()
    oc.set_source(st_np, offs)
    W, H = cfg["W"], cfg["H"]
    tf = tf_table(cfg["tf"])
    focal = 1.0 / math.tan(math.radians(cfg["fov"]) / 2)
    rgba = np.zeros(W * H, np.uint32)
    tb = np.zeros(W * H, np.float32)
    st = np.zeros(W * H * 4, np.float32)

    def frame(f):
        v = gc.make_view(camera(gc, cfg, f), W, H, 0, 256, 0, 0, 0, focal=focal, early_alpha=cfg["early"])
        tb[:] = 0
        st[:] = 0
        oc.render(v, tf, rgba, tb, st)
        oc.update()

    for f in range(args.warmup):
        frame(f)
    lat = []
    t0 = time.perf_counter()
    for i in range(args.steps):
        a = time.perf_counter()
        frame(args.warmup + i)
        lat.append(1e3 * (time.perf_counter() - a))
    el = time.perf_counter() - t0
    value = W * H * args.steps / el / 1e6
    out = {"impl": "reference", "metric": "Mrays/s", "value": round(value, 4), "unit": "Mrays/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * el / args.steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "u16" if cfg["bpc"] == 2 else "u8", "data": "synthetic",
           "config": {"workload": f"{args.config}: plain per-view out-of-core frame loop on host cores",
                      "volume": list(cfg["size"]), "view": [W, H], "max_requests": args.max_requests},
           "latency_ms": {"p50": round(statistics.median(lat), 3), "p99": round(float(np.percentile(lat, 99)), 3)},
           "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
                            "sample": f"{args.steps} frames of {W}x{H}: oracle FP32 ray-march + cache update, "
                                      f"{os.cpu_count()} threads"},
           "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    oc.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=None)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="c2")
    ap.add_argument("--max-requests", type=int, default=8192)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    cfg = CONFIGS[args.config]
    if args.steps is None:
        args.steps = cfg["frames"] if args.impl == "ours" else 3
    if args.warmup is None:
        args.warmup = 3
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
