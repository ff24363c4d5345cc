"""Generates the golden fixtures of tests/golden/ from the reference's own code.

Run where the reference checkout exists (it is not needed afterwards):
    python tests/golden/make_golden.py
It builds oracle/_ref/refdriver from the reference's CPU sources
(oracle/build.py) and records:
  layout.json   init_meta_data / level sizes of every benchmark geometry and of
                a few ragged shapes (refdriver layout)
  bricker.json  process_bricking output of seeded synthetic volumes: the
                generator parameters, the big-brick counts and the SHA-256 of
                the decompressed big bricks in (z, y, x) order (refdriver brick);
                the smallest case also stores the bricks themselves (zlib, base64)
  bricks_xml/   MetaData::write_bricks_xml output for two geometries
Synthetic volumes come from the oracle's generator, which the tests re-run.
"""
import base64
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle import oracle as orc  # noqa: E402

LAYOUTS = [
    # size, B, c, big brick, encoded bytes, channels
    ((256, 256, 256), 16, 1, (1, 1, 1), 1, 1),
    ((2048, 2048, 2048), 16, 1, (1, 1, 1), 2, 1),
    ((2048, 2048, 2048), 32, 1, (1, 1, 1), 2, 1),
    ((1024, 1024, 1024), 16, 1, (1, 1, 1), 1, 1),
    ((4096, 4096, 2048), 16, 1, (1, 1, 1), 1, 1),
    ((4096, 4096, 4096), 16, 2, (2, 2, 2), 2, 2),
    ((300, 200, 100), 16, 1, (1, 1, 1), 1, 1),
    ((97, 64, 33), 16, 2, (2, 1, 3), 2, 1),
    ((64, 64, 64), 8, 1, (2, 2, 2), 4, 1),
]

# (name, size, bytes/channel, channels, seed, nblobs, sigma, amp, noise, B, c, big brick)
BRICKS = [
    ("u8_small", (40, 36, 28), 1, 1, 3, 4, (4.0, 10.0), (60, 200), 20, 16, 1, (1, 1, 1)),
    ("u8_64", (64, 64, 64), 1, 1, 1, 8, (10.0, 40.0), (60, 200), 20, 16, 1, (1, 1, 1)),
    ("u16_64", (64, 64, 64), 2, 1, 7, 6, (6.0, 20.0), (60 * 257, 200 * 257), 20 * 257, 16, 1, (1, 1, 1)),
    ("u16_b32", (70, 50, 40), 2, 1, 9, 5, (5.0, 15.0), (60 * 257, 200 * 257), 20 * 257, 32, 1, (1, 1, 1)),
    ("u8x2_c2_bb2", (48, 40, 36), 1, 2, 11, 5, (5.0, 12.0), (60, 200), 20, 16, 2, (2, 2, 2)),
    ("u8_bb213", (50, 30, 45), 1, 1, 13, 5, (5.0, 12.0), (60, 200), 20, 8, 1, (2, 1, 3)),
]


def make_volume(size, bpc, nch, seed, nblobs, sigma, amp, noise):
    b = orc.blobs(seed, nblobs, size, sigma[0], sigma[1], amp[0], amp[1])
    vol = orc.generate(size, bpc, seed, b, nblobs, noise, channels=nch, channel=0, field=0)
    for ch in range(1, nch):
        orc.generate(size, bpc, seed + ch, b, 0, noise * 4, channels=nch, channel=ch, field=1, out=vol)
    return vol


def main():
    obuild.build_oracle()
    drv = obuild.build_reference(force=True)
    if drv is None:
        raise SystemExit("reference checkout or liblz4 not available")
    out = {"layouts": []}
    for size, B, c, bb, eb, nc in LAYOUTS:
        r = subprocess.run([drv, "layout", *map(str, size), str(B), str(c), *map(str, bb), str(eb), str(nc)],
                           capture_output=True, text=True, check=True, cwd=tempfile.gettempdir())
        rows = [list(map(int, line.split())) for line in r.stdout.strip().splitlines()]
        out["layouts"].append({"size": size, "B": B, "c": c, "bb": bb, "eb": eb, "nc": nc,
                               "levels": [{"initial": row[1:4], "real": row[4:7], "nb_bricks": row[7:10],
                                           "nb_big_bricks": row[10:13]} for row in rows]})
    with open(os.path.join(HERE, "layout.json"), "w") as f:
        json.dump(out, f, indent=1)

    cases = []
    for name, size, bpc, nch, seed, nblobs, sigma, amp, noise, B, c, bb in BRICKS:
        vol = make_volume(size, bpc, nch, seed, nblobs, sigma, amp, noise)
        eb = bpc * nch
        work = tempfile.mkdtemp(prefix="gcgold_")
        try:
            vol.tofile(os.path.join(work, "vol.raw"))
            res = os.path.join(work, "bricks.bin")
            r = subprocess.run([drv, "brick", work, "0", *map(str, size), str(B), str(c), *map(str, bb), str(eb),
                                str(nch), "unused", res], capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit(f"refdriver failed for {name}: {r.stderr}")
            nbig = list(map(int, r.stdout.split()))
            data = np.fromfile(res, dtype=np.uint8)
        finally:
            shutil.rmtree(work)
        case = {"name": name, "size": size, "bytes_per_channel": bpc, "channels": nch, "seed": seed,
                "nblobs": nblobs, "sigma": sigma, "amp": amp, "noise": noise, "B": B, "c": c, "bb": bb,
                "nb_big": nbig, "bytes": int(data.size), "sha256": hashlib.sha256(data.tobytes()).hexdigest(),
                "volume_sha256": hashlib.sha256(vol.tobytes()).hexdigest()}
        if name == "u8_small":
            case["bricks_zlib_b64"] = base64.b64encode(zlib.compress(data.tobytes(), 9)).decode()
        cases.append(case)
        print(name, nbig, case["sha256"][:16])
    with open(os.path.join(HERE, "bricker.json"), "w") as f:
        json.dump({"cases": cases}, f, indent=1)

    xml_dir = os.path.join(HERE, "bricks_xml")
    os.makedirs(xml_dir, exist_ok=True)
    for tag, args in (("c1_u8", ["16", "1", "1", "1", "256", "256", "256", "1", "1", "1"]),
                      ("c5_u8x2", ["16", "2", "2", "2", "96", "80", "64", "2", "2", "2", "281474976776192", "65537"])):
        work = tempfile.mkdtemp(prefix="gcxml_")
        try:
            subprocess.run([drv, "xml", work + "/", *args], check=True, capture_output=True)
            shutil.copy(os.path.join(work, "bricks_" + "_".join([args[0]] * 3), "bricks.xml"),
                        os.path.join(xml_dir, tag + ".xml"))
        finally:
            shutil.rmtree(work)


if __name__ == "__main__":
    main()
