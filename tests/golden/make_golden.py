"""Generate the golden fixtures in tests/golden/ from the REFERENCE itself.

Runs oracle/_ref/ffr_ref -- the reference's own hot-path code compiled from
its sources by oracle/build_ref.sh (only possible where the reference tree
exists; the fixtures are committed so nothing else needs it).  Writes:

  flames/<name>.json   test flames (seeded generators + hand-written edge cases)
  data/<name>.npz      per flame: normalised-flame dump, renders (counts,
                       colour sums, statistics), traces, single-step outputs
  data/kat.npz         Isaac<u64,4> words per key
  manifest.json        parameters of every case and the reference's stats

Usage: python tests/golden/make_golden.py
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
sys.path.insert(0, os.path.join(ROOT, "flame-fractal-renderer_gb300"))
import flames as gen  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ffr_ref")
FLAMES = os.path.join(HERE, "flames")
DATA = os.path.join(HERE, "data")

KAT_KEYS = [0, 1, 2, 0xFFFFFFFFFFFFFFFF, 0x0123456789ABCDEF, 12345678901234567,
            0x8000000000000000]


def ref(*args, capture=True):
    r = subprocess.run([REF, *map(str, args)], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ffr_ref {' '.join(map(str, args))}: {r.stderr}")
    return r.stdout


def hexd(s: str) -> float:
    return float(np.frombuffer(int(s, 16).to_bytes(8, "little"), dtype=np.float64)[0])


def edge_flames() -> dict:
    f = {}
    f["line1d"] = {
        "dimensions": 1, "size": [128], "bounds": [[-2, 2]],
        "xforms": [
            {"weight": 2, "variations": [{"name": "linear", "weight": 0.5},
                                         {"name": "sinusoidal", "weight": 0.4}],
             "pre_affine": {"A": [[0.9]], "b": [0.3]}},
            {"weight": 1.5, "variations": [{"name": "spherical", "weight": 0.7}],
             "pre_affine": {"A": [[1.2]], "b": [-0.5]}},
            {"weight": 1, "variations": [{"name": "linear", "weight": -0.6}]},
        ]}
    f["color"] = {
        "dimensions": 2, "size": [80, 60], "bounds": [[-1.5, 1.5], [-1.2, 1.2]],
        "color_dimensions": 3, "color_speed": 0.4,
        "xforms": [
            {"weight": 1.0, "color": [1, 0, 0],
             "variations": [{"name": "linear", "weight": 1.0}],
             "pre_affine": {"A": [[0.5, 0], [0, 0.5]], "b": [0.0, 0.5]}},
            {"weight": 1.0, "color": [0, 1, 0], "color_speed": 0.9,
             "variations": [{"name": "linear", "weight": 0.8},
                            {"name": "spherical", "weight": 0.1}],
             "pre_affine": {"A": [[0.5, 0.1], [0, 0.5]], "b": [-0.5, -0.5]}},
            {"weight": 1.0,
             "variations": [{"name": "horseshoe", "weight": 0.3},
                            {"name": "linear", "weight": 0.5}],
             "pre_affine": {"A": [[0.5, 0], [-0.1, 0.5]], "b": [0.5, -0.5]}},
        ],
        "final_xform": {"color": [0.2, 0.2, 1.0], "color_speed": 0.25,
                        "variations": [{"name": "linear", "weight": 0.9},
                                       {"name": "spherical", "weight": 0.05}],
                        "post_affine": {"A": [[1, 0.1], [0, 1]], "b": [0.05, 0]}},
    }
    f["ties"] = {
        "dimensions": 2, "size": [64, 48], "bounds": [[-2, 2], [-1.5, 1.5]],
        "xforms": [
            {"weight": 1, "variations": [{"name": "linear", "weight": 0.6}],
             "pre_affine": {"A": [[0.6, 0.2], [-0.2, 0.6]], "b": [0.4, 0.1]}},
            {"weight": 0, "variations": [{"name": "linear", "weight": 1}]},
            {"weight": 2, "variations": [{"name": "linear", "weight": 0.5},
                                         {"name": "julia", "weight": 0.0}],
             "pre_affine": {"b": [-0.4, 0.2]}},
            {"weight": 1, "variations": [{"name": "spherical", "weight": 0.3},
                                         {"name": "linear", "weight": 0.4}]},
            {"weight": 1, "variations": [{"name": "horseshoe", "weight": 0.4}],
             "post_affine": {"A": [[0.8, 0], [0, 0.8]]}},
            {"weight": 2, "variations": [{"name": "linear", "weight": -0.5}]},
        ]}
    f["badval"] = {
        "dimensions": 2, "size": [32, 32], "bounds": [[-1, 1], [-1, 1]],
        "xforms": [
            {"weight": 0.7, "variations": [{"name": "linear", "weight": 1}],
             "pre_affine": {"A": [[2, 0.1], [0, 2]], "b": [0.1, 0]}},
            {"weight": 0.3, "variations": [{"name": "linear", "weight": 1}],
             "pre_affine": {"A": [[0.5, 0], [0.1, 0.5]], "b": [0, 0.1]}},
        ]}
    f["julia3"] = {
        "dimensions": 2, "size": [100, 100], "bounds": [[-1.6, 1.6], [-1.6, 1.6]],
        "xforms": [
            {"weight": 1, "variations": [{"name": "julia", "weight": 1.0}],
             "pre_affine": {"A": [[0.8, 0], [0, 0.8]], "b": [0.1, 0.2]}},
            {"weight": 1, "variations": [{"name": "julia", "weight": 0.7},
                                         {"name": "polar", "weight": 0.2}],
             "pre_affine": {"A": [[0.6, -0.3], [0.3, 0.6]], "b": [-0.3, 0.0]}},
        ],
        "final_xform": {"variations": [{"name": "swirl", "weight": 0.8}]}}
    return f


FLAME_SET = {
    "sierpinski": gen.sierpinski_2d(size=(64, 64)),
    "tetra": gen.tetrahedron_3d(size=(32, 32, 32)),
    "alg2d": gen.random_2d(3, k=5, size=(96, 54),
                           variations=["linear", "spherical", "horseshoe"]),
    "c2small": gen.random_2d(7, k=6, size=(192, 108)),
    "rand3d": gen.random_3d(5, k=4, size=(24, 24, 24)),
}

# (flame, seed, streams, samples, traj_len, settle, bad_limit, mode)
RENDERS = [
    ("sierpinski", 1, 64, 100000, 1000, 20, 256, "mirror"),
    ("sierpinski", 2, 4, 30000, 1000, 53, 256, "seeded"),
    ("tetra", 3, 32, 50000, 500, 20, 256, "mirror"),
    ("alg2d", 5, 16, 50000, 2000, 20, 256, "mirror"),
    ("alg2d", 6, 3, 20000, 777, 53, 256, "seeded"),
    ("c2small", 7, 16, 50000, 2000, 20, 256, "mirror"),
    ("rand3d", 9, 16, 40000, 2000, 20, 256, "mirror"),
    ("line1d", 11, 8, 20000, 1000, 53, 256, "seeded"),
    ("line1d", 12, 8, 20000, 999, 20, 256, "mirror"),
    ("color", 13, 8, 20000, 1000, 20, 256, "mirror"),
    ("ties", 15, 8, 20000, 1000, 20, 256, "mirror"),
    ("badval", 17, 8, 20000, 1000, 20, 1000000000, "mirror"),
    ("julia3", 19, 8, 20000, 1000, 20, 256, "mirror"),
    ("heavy", 23, 64, 200000, 500, 20, 256, "mirror"),
]

# parameters for every variation that takes any (keys as the reference reads them)
VAR_PARAMS = {
    "bent": lambda d: {"scales_neg": [2.0, 0.5, 1.5][:d], "scales_pos": [1.0, 1.0, 0.8][:d]},
    "rectangles": lambda d: {"params": [0.3, 0.5, 0.0][:d]},
    "fisheye": lambda d: {"addval": 1.0},
    "bubble": lambda d: {"addval": 4.0},
    "separation": lambda d: {"params": [0.2, 0.3, 0.1][:d], "inside": [0.1, -0.2, 0.05][:d]},
    "splits": lambda d: {"params": [0.1, 0.2, 0.15][:d]},
    "modulus": lambda d: {"params": [0.6, 0.4, 0.5][:d]},
    "celln": lambda d: {"sizes": [0.5, 0.7, 0.3][:d]},
    "spherical_p": lambda d: {"norm": 1.5},
    "unit_sphere_p": lambda d: {"norm": 3.0},
    "disc2": lambda d: {"rotation": 0.7, "twist": 0.4},
    "waves": lambda d: {"xfreq": 2.0, "xscale": 0.3, "yfreq": 3.0, "yscale": 0.2},
    "fan": lambda d: {"x": 0.4, "y": 0.3},
    "rings": lambda d: {"value": 0.6},
    "blob": lambda d: {"low": 0.3, "high": 1.1, "waves": 5},
    "pdj": lambda d: {"a": 1.1, "b": -1.3, "c": 0.9, "d": 1.7},
    "perspective": lambda d: {"distance": 2.5, "angle": 0.6},
    "julian": lambda d: {"power": 3, "dist": 1.2},
    "juliascope": lambda d: {"power": -2.5, "dist": 0.8},
    "radial_blur": lambda d: {"angle": 0.4, "flam3_weight": 0.5},
    "pie": lambda d: {"slices": 6, "rotation": 0.3, "thickness": 0.5},
    "ngon": lambda d: {"sides": 5, "power": 2.0, "corners": 0.3, "circle": 1.0},
    "curl": lambda d: {"c1": 0.4, "c2": 0.2},
    "arch": lambda d: {"flam3_weight": 0.7},
    "rays": lambda d: {"flam3_weight": 0.7},
    "blade": lambda d: {"flam3_weight": 0.7},
    "secant": lambda d: {"flam3_weight": 0.7},
    "twintrian": lambda d: {"flam3_weight": 0.7},
    "scry": lambda d: {"flam3_weight": 0.7},
    "auger": lambda d: {"freq": 2.0, "flam3_weight": 0.6, "scale": 1.0, "sym": 0.4},
    "flux": lambda d: {"spread": 0.3, "flam3_weight": 0.4},
    "mobius": lambda d: {"a": [0.6, 0.2], "b": [0.1, -0.3], "c": [0.3, 0.1], "d": [1.0, 0.2]},
    "split": lambda d: {"xsize": 0.4, "ysize": 0.6},
    "stripes": lambda d: {"space": 0.3, "warp": 0.5},
    "wedge": lambda d: {"swirl": 0.3, "count": 3, "angle": 0.5, "hole": 0.1},
    "wedge_julia": lambda d: {"angle": 0.4, "count": 2, "power": 3, "dist": 1.0},
    "wedge_sph": lambda d: {"angle": 0.4, "count": 2, "swirl": 0.2, "hole": 0.05},
    "whorl": lambda d: {"inside": 0.3, "outside": 0.5, "flam3_weight": 0.8},
    "supershape": lambda d: {"n1": 2.0, "m": 5, "n2": 1.5, "n3": 1.5, "rnd": 0.2, "holes": 0.1},
    "flower": lambda d: {"petals": 4, "holes": 0.2},
    "conic": lambda d: {"eccen": 0.7, "holes": 0.1},
    "parabola": lambda d: {"height": 0.8, "width": 1.2},
    "bipolar": lambda d: {"shift": 0.3},
    "boarders": lambda d: {"prob": 0.6},
    "cell": lambda d: {"size": 0.4},
    "cpow": lambda d: {"r": 1.2, "i": 0.3, "power": 2.5},
    "curve": lambda d: {"xamp": 0.3, "yamp": 0.4, "xlen": 0.6, "ylen": 0.8},
    "escher": lambda d: {"beta": 0.7},
    "lazysusan": lambda d: {"x": 0.2, "y": -0.1, "spin": 0.5, "twist": 0.3, "space": 0.4,
                            "flam3_weight": 0.6},
    "loonie": lambda d: {"flam3_weight": 0.9},
    "oscope": lambda d: {"frequency": 2.0, "amplitude": 0.5, "damping": 0.3, "separation": 0.2},
    "popcorn": lambda d: {"x": 0.2, "y": 0.15, "c": 0.8},
}

ND_VARS = ["linear", "sinusoidal", "spherical", "bent", "rectangles", "fisheye",
           "bubble", "noise", "blur", "gaussian_blur", "square_noise", "separation",
           "splits", "pre_blur", "modulus", "celln", "spherical_p", "unit_sphere",
           "unit_sphere_p", "unit_cube"]
TWO_D_VARS = [
    "swirl", "horseshoe", "polar", "polar2", "handkerchief", "heart", "disc",
    "disc2", "waves", "fan", "rings", "spiral", "hyperbolic", "diamond", "ex",
    "julia", "exponential", "power", "cosine", "blob", "pdj", "cylinder",
    "perspective", "julian", "juliascope", "radial_blur", "pie", "ngon",
    "curl", "arch", "tangent", "rays", "blade", "secant", "twintrian",
    "cross", "exp", "log", "sin", "cos", "tan", "sec", "csc", "cot", "sinh",
    "cosh", "tanh", "sech", "csch", "coth", "auger", "flux", "mobius", "scry",
    "split", "stripes", "wedge", "wedge_julia", "wedge_sph", "whorl",
    "supershape", "flower", "conic", "parabola", "bipolar", "boarders",
    "butterfly", "cell", "cpow", "curve", "edisc", "elliptic", "escher",
    "foci", "lazysusan", "loonie", "oscope", "popcorn"]


def var_obj(name, dims, weight, axes=None):
    v = {"name": name, "weight": weight}
    v.update(VAR_PARAMS.get(name, lambda d: {})(dims))
    if axes is not None:
        v["axis_x"], v["axis_y"] = axes
    return v


def variation_flame(name, dims, axes=None):
    """Two xforms: the variation under test (weight 0.7) plus linear, then a
    plain contraction, so trajectories stay bounded."""
    A = {1: [[0.6]], 2: [[0.6, 0.2], [-0.1, 0.7]],
         3: [[0.6, 0.2, 0.0], [-0.1, 0.7, 0.1], [0.05, 0.0, 0.65]]}[dims]
    b = [0.1, -0.05, 0.03][:dims]
    I5 = [[0.5 if i == k else 0.0 for k in range(dims)] for i in range(dims)]
    return {
        "dimensions": dims, "size": [32] * dims if dims < 3 else [16] * 3,
        "bounds": [[-2.0, 2.0]] * dims,
        "xforms": [
            {"weight": 1.0, "pre_affine": {"A": A, "b": b},
             "variations": [var_obj(name, dims, 0.7, axes),
                            {"name": "linear", "weight": 0.3}]},
            {"weight": 0.5, "pre_affine": {"A": I5, "b": [-0.3, 0.2, 0.1][:dims]},
             "variations": [{"name": "linear", "weight": 1.0}]},
        ]}


def variation_set():
    out = {}
    for n in ND_VARS:
        for d in (1, 2, 3):
            out[f"v{d}_{n}"] = variation_flame(n, d)
    for n in TWO_D_VARS:
        out[f"v2_{n}"] = variation_flame(n, 2)
    for k, n in enumerate(TWO_D_VARS):
        if k % 3 == 0:
            out[f"v3_{n}"] = variation_flame(n, 3, axes=(2, 0) if k % 2 else (1, 2))
    return out


INVALID = {
    "no_xforms": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[]}',
    "all_zero": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":0,"variations":[]}]}',
    "neg_weight": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":-1,"variations":[]}]}',
    "bad_bounds": '{"dimensions":2,"size":[4,4],"bounds":[[1,0],[0,1]],"xforms":[{"weight":1,"variations":[]}]}',
    "big_bounds": '{"dimensions":2,"size":[4,4],"bounds":[[-2e10,1],[0,1]],"xforms":[{"weight":1,"variations":[]}]}',
    "size_zero": '{"dimensions":2,"size":[0,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[]}]}',
    "size_big": '{"dimensions":2,"size":[65536,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[]}]}',
    "size_len": '{"dimensions":2,"size":[4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[]}]}',
    "unknown_var": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[{"name":"nope","weight":1}]}]}',
    "swirl_1d": '{"dimensions":1,"size":[4],"bounds":[[0,1]],"xforms":[{"weight":1,"variations":[{"name":"swirl","weight":1}]}]}',
    "axes_missing_3d": '{"dimensions":3,"size":[4,4,4],"bounds":[[0,1],[0,1],[0,1]],"xforms":[{"weight":1,"variations":[{"name":"swirl","weight":1}]}]}',
    "axes_same_3d": '{"dimensions":3,"size":[4,4,4],"bounds":[[0,1],[0,1],[0,1]],"xforms":[{"weight":1,"variations":[{"name":"swirl","weight":1,"axis_x":1,"axis_y":1}]}]}',
    "color_range": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"color_dimensions":1,"xforms":[{"weight":1,"color":[2],"variations":[]}]}',
    "color_len": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"color_dimensions":2,"xforms":[{"weight":1,"color":[0.5],"variations":[]}]}',
    "color_dims_float": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"color_dimensions":1.0,"xforms":[{"weight":1,"variations":[]}]}',
    "too_many_colors": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"color_dimensions":128,"xforms":[{"weight":1,"variations":[]}]}',
    "affine_shape": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[],"pre_affine":{"A":[[1,0]]}}]}',
    "weight_string": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":"1","variations":[]}]}',
    "syntax": '{"dimensions":2,"size":[4,4],,}',
    "trailing": '{"dimensions":2,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[]}]} x',
    "unterminated_comment": '{"dimensions":2 /* ,"size":[4,4]}',
    "dims_float": '{"dimensions":2.0,"size":[4,4],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[]}]}',
}

VALID_EDGE = {
    "comments": '// line comment\n{"dimensions":2, /* block */ "size":[4.9,4],"bounds":[[0,1],[0,1]],\n"xforms":[{"weight":1,"variations":[{"name":"linear","weight":1}]}]} // tail\n',
    "int_floats": '{"dimensions":2,"size":[8,8],"bounds":[[-1,1],[-1e0,1.0]],"xforms":[{"weight":3,"variations":[{"name":"linear","weight":1}],"pre_affine":{"A":[[1,0],[0,1]],"b":[0,0]}}]}',
    "dup_key": '{"dimensions":2,"size":[4,4],"size":[8,8],"bounds":[[0,1],[0,1]],"xforms":[{"weight":1,"variations":[]}]}',
}


def main():
    if not os.path.exists(REF):
        subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")])
    os.makedirs(FLAMES, exist_ok=True)
    os.makedirs(DATA, exist_ok=True)
    allf = dict(FLAME_SET)
    allf.update(edge_flames())
    # a density piled up at one fixed point (the kernels' hot-cell table);
    # last, so the seeded inputs of the flames above stay as they were
    allf["heavy"] = gen.heavy_point_2d(size=(64, 64))
    manifest = {"kat": {}, "flames": {}, "renders": [], "invalid": {}, "valid_edge": {}}
    # KATs
    kat = {}
    for k in KAT_KEYS:
        words = [int(w, 16) for w in ref("kat", k, 100).split()]
        kat[f"k{k:016x}"] = np.array(words, dtype=np.uint64)
    np.savez_compressed(os.path.join(DATA, "kat.npz"), **kat)
    manifest["kat"] = {"keys": [f"{k:016x}" for k in KAT_KEYS], "words": 100}
    rng = np.random.Generator(np.random.PCG64(2024))
    for name, fl in allf.items():
        path = os.path.join(FLAMES, name + ".json")
        with open(path, "w") as f:
            json.dump(fl, f, indent=1)
        dump = json.loads(ref("flame", path))
        arrays = {}
        dims = dump["dims"]
        nx = len(dump["xforms"])
        # single steps on seeded points, every xform and the final one
        pts = rng.uniform(-1.5, 1.5, size=(256, dims))
        arrays["step_in"] = pts
        with tempfile.TemporaryDirectory() as td:
            pin = os.path.join(td, "in.bin")
            pout = os.path.join(td, "out.bin")
            pts.astype(np.float64).tofile(pin)
            xis = list(range(nx)) + ([-1] if dump["has_final"] else [])
            for xi in xis:
                ref("step", path, xi, 777, pin, pout)
                arrays[f"step_out_{xi}"] = np.fromfile(pout, dtype=np.float64).reshape(-1, dims)
        # one trajectory trace
        lines = ref("trace", path, 12345, 20, 300).strip().split("\n")
        arrays["trace_ids"] = np.array([int(l.split()[0]) for l in lines], dtype=np.int32)
        arrays["trace_pts"] = np.array([[hexd("0x" + h) for h in l.split()[1:]] for l in lines])
        manifest["flames"][name] = {
            "dims": dims, "xform_ids": dump["xform_ids"],
            "color_dims": dump["color_dims"],
            "order": [x["id"] for x in dump["xforms"]],
            "weights": [x["weight"] for x in dump["xforms"]],
            "xfcw": dump["xfcw"], "mult_d": dump["mult_d"],
            "mult_i": dump["mult_i"], "cells": dump["cells"],
            "has_final": dump["has_final"],
            "var_weights": [x["var_weights"] for x in dump["xforms"]],
            "pre": [x["pre"] for x in dump["xforms"]],
            "post": [x["post"] for x in dump["xforms"]],
            "has_pre": [x["has_pre"] for x in dump["xforms"]],
            "has_post": [x["has_post"] for x in dump["xforms"]],
            "steps": xis,
        }
        np.savez_compressed(os.path.join(DATA, name + ".npz"), **arrays)
    for i, (name, seed, streams, n, L, settle, bvl, mode) in enumerate(RENDERS):
        path = os.path.join(FLAMES, name + ".json")
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "o.buf")
            args = ["render", path, seed, streams, n, L, settle, bvl, out]
            if mode == "seeded":
                args.append("seeded")
            st = json.loads(ref(*args))
            raw = np.fromfile(out, dtype=np.uint64)
        cd = manifest["flames"][name]["color_dims"]
        cells = manifest["flames"][name]["cells"]
        raw = raw.reshape(cells, 1 + cd)
        key = f"render{i}"
        np.savez_compressed(os.path.join(DATA, key + ".npz"), counts=raw[:, 0],
                            colors=raw[:, 1:].copy().view(np.float64))
        manifest["renders"].append({
            "key": key, "flame": name, "seed": seed, "streams": streams,
            "samples": n, "traj_len": L, "settle": settle, "bad_limit": bvl,
            "mode": mode, "stats": st})
    for name, text in INVALID.items():
        with tempfile.TemporaryDirectory() as td:
            p = os.path.join(td, "f.json")
            with open(p, "w") as f:
                f.write(text)
            r = subprocess.run([REF, "flame", p], stdout=subprocess.PIPE,
                               stderr=subprocess.PIPE, text=True)
        manifest["invalid"][name] = {"text": text, "rejected": r.returncode != 0,
                                     "message": r.stderr.strip()}
    for name, text in VALID_EDGE.items():
        with tempfile.TemporaryDirectory() as td:
            p = os.path.join(td, "f.json")
            with open(p, "w") as f:
                f.write(text)
            r = subprocess.run([REF, "flame", p], stdout=subprocess.PIPE,
                               stderr=subprocess.PIPE, text=True)
        manifest["valid_edge"][name] = {"text": text, "ok": r.returncode == 0,
                                        "dump": json.loads(r.stdout) if r.returncode == 0 else None}
    # every variation: flame, single steps, a trace and a small render
    manifest["vflames"] = {}
    vdir = os.path.join(FLAMES, "var")
    ddir = os.path.join(DATA, "var")
    os.makedirs(vdir, exist_ok=True)
    os.makedirs(ddir, exist_ok=True)
    vrng = np.random.Generator(np.random.PCG64(4242))
    for name, fl in variation_set().items():
        path = os.path.join(vdir, name + ".json")
        with open(path, "w") as f:
            json.dump(fl, f)
        dims = fl["dimensions"]
        arrays = {}
        pts = vrng.uniform(-1.5, 1.5, size=(128, dims))
        arrays["step_in"] = pts
        with tempfile.TemporaryDirectory() as td:
            pin = os.path.join(td, "in.bin")
            pout = os.path.join(td, "out.bin")
            pts.astype(np.float64).tofile(pin)
            ref("step", path, 0, 777, pin, pout)
            arrays["step_out"] = np.fromfile(pout, dtype=np.float64).reshape(-1, dims)
            lines = ref("trace", path, 999, 20, 100).strip().split("\n")
            arrays["trace_ids"] = np.array([int(l.split()[0]) for l in lines], dtype=np.int32)
            arrays["trace_pts"] = np.array([[hexd("0x" + h) for h in l.split()[1:]]
                                            for l in lines])
            out = os.path.join(td, "o.buf")
            st = json.loads(ref("render", path, 21, 8, 20000, 1000, 20, 10**9, out))
            arrays["counts"] = np.fromfile(out, dtype=np.uint64)
        np.savez_compressed(os.path.join(ddir, name + ".npz"), **arrays)
        manifest["vflames"][name] = {"dims": dims, "stats": st,
                                     "render": [21, 8, 20000, 1000, 20, 10**9]}
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("golden fixtures written", file=sys.stderr)


if __name__ == "__main__":
    main()
