"""Shared scenario builders for the parity tests (seeded synthetic volumes,
brick stores, cameras).  Both the CUDA path and the oracle are fed the same
inputs; nothing here decides pass or fail."""
import math

import numpy as np


def volume_params(size, bpc):
    m = min(size)
    smin, smax = max(1.0, 0.04 * m), max(1.5, 0.16 * m)
    if bpc == 1:
        return smin, smax, 60, 200, 20
    return smin, smax, 60 * 257, 200 * 257, 20 * 257


def gpu_volume(gc, torch, size, bpc, seed, nblobs, channels=1):
    smin, smax, amin, amax, noise = volume_params(size, bpc)
    blobs = gc.generator_blobs(seed, nblobs, size, smin, smax, amin, amax)
    n = size[0] * size[1] * size[2] * bpc * channels
    t = torch.empty(n, dtype=torch.uint8, device="cuda")
    gc.generate_volume(gc.make_generator(size, bpc, seed, blobs, noise, channels=channels, channel=0, field=0),
                       t.data_ptr())
    for ch in range(1, channels):
        gc.generate_volume(gc.make_generator(size, bpc, seed + ch, blobs, noise * 4,
                                             channels=channels, channel=ch, field=1), t.data_ptr())
    torch.cuda.synchronize()
    return t


def orc_volume(orc, size, bpc, seed, nblobs, channels=1):
    smin, smax, amin, amax, noise = volume_params(size, bpc)
    b = orc.blobs(seed, nblobs, size, smin, smax, amin, amax)
    vol = orc.generate(size, bpc, seed, b, nblobs, noise, channels=channels, channel=0, field=0)
    for ch in range(1, channels):
        orc.generate(size, bpc, seed + ch, b, nblobs, noise * 4, channels=channels, channel=ch, field=1, out=vol)
    return vol


def orc_store(orc, gc, vol_bytes, desc, layout):
    """Brick store built by the oracle: mip levels then bricks of every level."""
    eb, nc = desc.encoded_bytes, desc.channels
    cb = eb // nc
    dt = {1: np.uint8, 2: np.uint16, 4: np.float32}[cb]
    level = np.ascontiguousarray(vol_bytes).view(dt)
    parts, offs, off = [], [], 0
    for l in range(layout.nb_levels):
        dims = tuple(layout.initial[l])
        if l > 0:
            level = orc.mip_level(level, tuple(layout.initial[l - 1]), eb, nc)
        b = orc.brick_level(level.view(np.uint8), dims, desc, tuple(layout.nb_big_bricks[l]))
        offs.append(off)
        off += b.size
        parts.append(b)
    return np.concatenate(parts), offs


def orbit_camera(gc, frame, nframes, distance, elevation_deg=20.0):
    a = 2 * math.pi * frame / nframes
    e = math.radians(elevation_deg)
    eye = (distance * math.cos(e) * math.sin(a), distance * math.sin(e), distance * math.cos(e) * math.cos(a))
    return gc.look_at(eye)


def ramp_tf(width=256, lo=40, hi=255, amax=0.6):
    """256-entry piecewise-linear RGBA: alpha 0 up to value lo, ramp to amax at hi."""
    tf = np.zeros((width, 4), dtype=np.float32)
    for i in range(width):
        v = i * 255.0 / (width - 1)
        a = 0.0 if v <= lo else amax * min(1.0, (v - lo) / (hi - lo))
        t = i / (width - 1)
        tf[i] = (min(1.0, 0.2 + 1.2 * t), 0.3 + 0.6 * t * (1 - t) * 2, 1.0 - t, a)
    return tf


def bumps_tf(seed, width=256, nbumps=3):
    """RGBA with `nbumps` seeded Gaussian alpha bumps."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, width)
    a = np.zeros(width)
    for _ in range(nbumps):
        c, w, h = rng.uniform(0.2, 0.9), rng.uniform(0.02, 0.08), rng.uniform(0.2, 0.8)
        a += h * np.exp(-0.5 * ((x - c) / w) ** 2)
    tf = np.stack([np.clip(0.3 + x, 0, 1), np.clip(1.2 - x, 0, 1), 0.5 + 0.5 * np.sin(6 * x), np.clip(a, 0, 1)], 1)
    return tf.astype(np.float32)


def tf2d(seed, width=64, height=48):
    """2D RGBA table for two-channel volumes (row-major, height rows of width
    entries): alpha from seeded bumps over channel 0, modulated along channel 1."""
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
