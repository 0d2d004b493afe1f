"""Generate the golden image fixtures (tests/golden/data/images.npz and the
"images" entry of tests/golden/images.json) from the REFERENCE itself.

The buffers come from oracle/_ref/ffr_ref (the reference's buffer path,
seeded streams) and the pixels from oracle/_ref/ffr_img_ref: the reference's
own src/ffr_img.cpp -- render_image (:199-309) over ImageRenderer
(src/renderers/image_renderer.hpp:111-191) -- compiled by
oracle/build_ref.sh with project-written Boost shims and an unencoded image
writer in place of libpng.  Both binaries exist only where the reference
tree was present at build time; the fixtures are committed so nothing else
needs them.

Usage: python tests/golden/make_golden_images.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "ffr_ref")
IMG = os.path.join(ROOT, "oracle", "_ref", "ffr_img_ref")
FLAMES = os.path.join(HERE, "flames")

# (flame, seed, streams, samples, traj_len, settle) of each buffer
BUFFERS = {
    "c2small": ("c2small", 31, 64, 2_000_000, 5000, 20),
    "color": ("color", 32, 64, 1_000_000, 4000, 20),
    "julia3": ("julia3", 33, 64, 1_500_000, 3000, 20),
}
# (name, buffer, ffr-img options)
CASES = [
    ("c2small_gray8", "c2small", ["-g"]),
    ("c2small_gray8_g22", "c2small", ["-g", "-y", "2.2"]),
    ("c2small_gray16_g045", "c2small", ["-g", "-b", "16", "-y", "0.45"]),
    ("c2small_mono", "c2small", ["-m"]),
    ("julia3_gray16", "julia3", ["-g", "-b", "16"]),
    ("color_rgb8", "color", ["-c"]),
    ("color_rgb16_g15", "color", ["-c", "-b", "16", "-y", "1.5"]),
    ("color_gray8", "color", ["-g", "-y", "2.0"]),
]


def read_image(path: str) -> np.ndarray:
    raw = open(path, "rb").read()
    assert raw[:8] == b"FFRIMG1\n", raw[:8]
    w, h, ch, b = np.frombuffer(raw[8:24], dtype="<u4")
    dt = np.dtype("<u1" if b == 1 else "<u2")
    px = np.frombuffer(raw[24:], dtype=dt).reshape(h, w, ch)
    return px if ch == 3 else px[:, :, 0]


def main() -> int:
    for b in (REF, IMG):
        if not os.path.exists(b):
            print(f"{b} is absent: run oracle/build_ref.sh where the reference exists",
                  file=sys.stderr)
            return 1
    out, meta = {}, {"buffers": {}, "images": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for key, (flame, seed, streams, n, L, settle) in BUFFERS.items():
            fpath = os.path.join(FLAMES, flame + ".json")
            bpath = os.path.join(tmp, key + ".buf")
            subprocess.run([REF, "render", fpath, str(seed), str(streams), str(n), str(L),
                            str(settle), str(10**9), bpath], check=True,
                           stdout=subprocess.DEVNULL)
            out["buf_" + key] = np.fromfile(bpath, dtype=np.uint64)
            meta["buffers"][key] = {"flame": flame, "seed": seed, "streams": streams,
                                    "samples": n, "traj_len": L, "settle": settle}
        for name, key, opts in CASES:
            flame = BUFFERS[key][0]
            ipath = os.path.join(tmp, name + ".img")
            r = subprocess.run([IMG, "-f", os.path.join(FLAMES, flame + ".json"),
                                "-i", os.path.join(tmp, key + ".buf"), "-o", ipath, *opts],
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"ffr_img_ref {name}: {r.stderr}")
            out["img_" + name] = read_image(ipath)
            bounds = [l for l in r.stderr.splitlines() if "bounds:" in l]
            meta["images"][name] = {"buffer": key, "options": opts, "stderr_bounds": bounds}
    np.savez_compressed(os.path.join(HERE, "data", "images.npz"), **out)
    with open(os.path.join(HERE, "images.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(f"wrote {len(CASES)} images from {len(BUFFERS)} buffers")
    return 0


if __name__ == "__main__":
    sys.exit(main())
