"""Flames for the per-flame kernel tests (FFR_KERNEL_JIT).

Every variation of the reference (the per-variation fixtures under
golden/flames/var, with their parameters) placed in multi-type flames:
xforms of two variations each, so every slot of the generated kernels
holds several types, with and without pre/post affines (3-D), a final
xform, and a colour variant.  The weights are 0.5 per variation; bad
values are allowed (the tests compare kernels, not attractors).
"""
import glob
import json
import os

import numpy as np

from conftest import GOLDEN

VAR_DIR = os.path.join(GOLDEN, "flames", "var")


def fixture_variation(path):
    """The tested variation of one per-variation fixture (its first one)."""
    with open(path) as f:
        v = dict(json.load(f)["xforms"][0]["variations"][0])
    v["weight"] = 0.5
    return v


def variations(dims):
    return [fixture_variation(p)
            for p in sorted(glob.glob(os.path.join(VAR_DIR, f"v{dims}_*.json")))]


def grouped(dims, per_flame, seed=0, final=False, color=False):
    """Flames of dims dimensions covering every fixture variation of that
    dimension count, per_flame variations (two per xform) each."""
    vs = variations(dims)
    g = np.random.Generator(np.random.PCG64(seed + 10 * dims))
    size = {1: [256], 2: [96, 64], 3: [24, 24, 24]}[dims]
    out = []
    for f0 in range(0, len(vs), per_flame):
        chunk = vs[f0:f0 + per_flame]
        xfs = []
        for k in range(0, len(chunk), 2):
            x = {"weight": float(1.0 + (k % 3)), "variations": chunk[k:k + 2]}
            # 3-D: every third xform without a pre-affine, every second with
            # a post-affine (has_pre / has_post both ways)
            if dims < 3 or k % 3:
                a = g.uniform(-0.6, 0.6, size=(dims, dims + 1))
                x["pre_affine"] = {"A": a[:, :dims].tolist(), "b": a[:, dims].tolist()}
            if dims == 3 and k % 2 == 0:
                a = np.eye(3) + g.normal(0.0, 0.1, size=(3, 3))
                x["post_affine"] = {"A": a.tolist(), "b": [0.0, 0.1, -0.1]}
            if color:
                x["color"] = [float(g.uniform()) for _ in range(3)]
            xfs.append(x)
        f = {"dimensions": dims, "size": size, "bounds": [[-2.0, 2.0]] * dims,
             "xforms": xfs}
        if final:
            f["final_xform"] = {"variations": [dict(chunk[0]), dict(chunk[-1])]}
        if color:
            f["color_dimensions"] = 3
            f["color_speed"] = 0.3
        out.append(json.dumps(f))
    return out


def cases():
    """name -> flame text: all 98 2-D types in four flames (one with a
    final xform), the 20 N-D types in 1-D, the 46 3-D types in two flames,
    and a colour flame."""
    c = {}
    for i, t in enumerate(grouped(2, 26, final=True)):
        c[f"d2_group{i}"] = t
    for i, t in enumerate(grouped(1, 20)):
        c[f"d1_group{i}"] = t
    for i, t in enumerate(grouped(3, 24)):
        c[f"d3_group{i}"] = t
    c["d2_color"] = grouped(2, 12, seed=5, color=True)[1]
    return c
