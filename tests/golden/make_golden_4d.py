"""Generate the four-dimensional golden fixtures (tests/golden/flames/d4_*.json,
tests/golden/data/d4.npz, tests/golden/d4.json) from the REFERENCE itself.

The reference's BufferRenderer, Flame, XForm, Point and variation templates
are generic over the dimension count; its ffr-buf CLI instantiates 1..3
only (src/ffr_buf.cpp:134-141).  oracle/_ref/ffr_ref (oracle/build_ref.sh)
also instantiates 4, so these vectors come from the reference's own code at
dims = 4: renders (counts and statistics), single-step outputs and a
trajectory trace per flame.

Flames:
  d4_simplex   the 4-D analogue of the Sierpinski triangle: five maps
               x -> (x + v_k) / 2 toward the vertices of a 4-simplex;
               linear only (bit-exact in FP64)
  d4_mixed     linear + noise (randDirection<4>: two gaussian pairs),
               julia on axes (1, 3), sinusoidal, spherical, swirl on axes
               (0, 2), a post-affine and a final xform
Usage: python tests/golden/make_golden_4d.py
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
FLAMES = os.path.join(HERE, "flames")


def simplex() -> dict:
    verts = [(1, 1, 1, -1 / 5 ** 0.5), (1, -1, -1, -1 / 5 ** 0.5), (-1, 1, -1, -1 / 5 ** 0.5),
             (-1, -1, 1, -1 / 5 ** 0.5), (0, 0, 0, 4 / 5 ** 0.5)]
    xfs = [{"weight": 0.2, "variations": [{"name": "linear", "weight": 1.0}],
            "pre_affine": {"A": [[0.5 if i == j else 0.0 for j in range(4)] for i in range(4)],
                           "b": [0.5 * c for c in v]}} for v in verts]
    return {"dimensions": 4, "size": [24, 24, 24, 24], "bounds": [[-1.1, 1.1]] * 3 + [[-0.5, 1.8]],
            "xforms": xfs}


def mixed() -> dict:
    eye = lambda s: [[s if i == j else 0.0 for j in range(4)] for i in range(4)]  # noqa: E731
    return {
        "dimensions": 4, "size": [16, 14, 12, 10], "bounds": [[-2, 2]] * 4,
        "xforms": [
            {"weight": 1.0, "variations": [{"name": "linear", "weight": 0.6},
                                           {"name": "noise", "weight": 0.3}],
             "pre_affine": {"A": [[0.5, 0.1, 0, 0], [0, 0.5, 0.1, 0], [0, 0, 0.5, 0.1],
                                  [0.1, 0, 0, 0.5]], "b": [0.3, -0.2, 0.1, 0.0]}},
            {"weight": 0.7, "variations": [{"name": "julia", "weight": 0.5, "axis_x": 1,
                                            "axis_y": 3},
                                           {"name": "sinusoidal", "weight": 0.5}],
             "pre_affine": {"A": eye(0.6), "b": [-0.4, 0.2, 0.0, 0.3]}},
            {"weight": 0.5, "variations": [{"name": "spherical", "weight": 0.8},
                                           {"name": "swirl", "weight": 0.2, "axis_x": 0,
                                            "axis_y": 2}],
             "post_affine": {"A": eye(0.9), "b": [0.1, 0.1, -0.1, 0.0]}}],
        "final_xform": {"variations": [{"name": "linear", "weight": 0.9},
                                       {"name": "blur", "weight": 0.1}],
                        "pre_affine": {"A": eye(1.0), "b": [0.05, 0.0, 0.0, -0.05]}},
    }


# (flame, seed, streams, samples, traj_len, settle)
RENDERS = [("d4_simplex", 41, 64, 400_000, 2000, 20),
           ("d4_simplex", 42, 8, 30_000, 1000, 53),
           ("d4_mixed", 43, 64, 200_000, 1000, 20)]


def ref(*args):
    r = subprocess.run([REF, *map(str, args)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ffr_ref {' '.join(map(str, args))}: {r.stderr}")
    return r.stdout


def main() -> int:
    if not os.path.exists(REF):
        print(f"{REF} is absent: run oracle/build_ref.sh where the reference exists",
              file=sys.stderr)
        return 1
    flames = {"d4_simplex": simplex(), "d4_mixed": mixed()}
    out, meta = {}, {"renders": [], "flames": {}}
    g = np.random.Generator(np.random.PCG64(44))
    with tempfile.TemporaryDirectory() as tmp:
        for name, fl in flames.items():
            path = os.path.join(FLAMES, name + ".json")
            with open(path, "w") as f:
                json.dump(fl, f, indent=1)
            nxf = len(fl["xforms"])
            pts = g.uniform(-1.5, 1.5, size=(257, 4))
            inp = os.path.join(tmp, "in.bin")
            pts.astype(np.float64).tofile(inp)
            steps = {}
            for xi in list(range(nxf)) + ([-1] if "final_xform" in fl else []):
                o = os.path.join(tmp, f"step{xi}.bin")
                ref("step", path, xi, 777, inp, o)
                steps[str(xi)] = np.fromfile(o, dtype=np.float64).reshape(-1, 4)
            tr = ref("trace", path, 999, 20, 64).split("\n")
            ids, tp = [], []
            for line in tr:
                if not line.strip():
                    continue
                p = line.split()
                ids.append(int(p[0]))
                tp.append([np.frombuffer(int(h, 16).to_bytes(8, "little"), dtype=np.float64)[0]
                           for h in p[1:]])
            out[f"{name}_step_in"] = pts
            for k, v in steps.items():
                out[f"{name}_step_{k.replace('-', 'm')}"] = v
            out[f"{name}_trace_ids"] = np.array(ids, dtype=np.int64)
            out[f"{name}_trace_pts"] = np.array(tp, dtype=np.float64)
            meta["flames"][name] = {"xforms": nxf, "final": "final_xform" in fl}
        for k, (name, seed, streams, n, L, settle) in enumerate(RENDERS):
            path = os.path.join(FLAMES, name + ".json")
            b = os.path.join(tmp, f"r{k}.buf")
            st = json.loads(ref("render", path, seed, streams, n, L, settle, 10**9, b))
            out[f"render{k}"] = np.fromfile(b, dtype=np.uint64)
            meta["renders"].append({"key": f"render{k}", "flame": name, "seed": seed,
                                    "streams": streams, "samples": n, "traj_len": L,
                                    "settle": settle, "stats": st})
    np.savez_compressed(os.path.join(HERE, "data", "d4.npz"), **out)
    with open(os.path.join(HERE, "d4.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(f"wrote {len(RENDERS)} renders and {len(flames)} flames")
    return 0


if __name__ == "__main__":
    sys.exit(main())
