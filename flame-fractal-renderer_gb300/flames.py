"""Seeded generators of flame JSON documents (the benchmark workloads).

Each function returns a dict in the reference's flame JSON format
(FLAME_JSON.md of the reference project).  Randomness comes from numpy's
PCG64 generator seeded explicitly, so the same seed gives the same flame on
every machine.

  sierpinski_2d      3 xforms, weight 1/3, A = 0.5 I, b = 0.5 v_i with
                     v = (0,1), (-1,-1), (1,-1); linear; bounds [-1,1]^2
  tetrahedron_3d     4 xforms, weight 0.25, A = 0.5 I, b = 0.5 v_i with v_i
                     the vertices (1,1,1), (1,-1,-1), (-1,1,-1), (-1,-1,1)
  random_2d          k xforms, weights Dirichlet(1); pre-affine entries
                     U[-1,1]; post-affine identity + N(0, 0.1); 2 variations
                     per xform drawn without replacement from TIER_A with
                     weights Dirichlet(1); bounds [-2,2] x [-1.125,1.125]
  random_3d          the 3-D analogue (2-D variations act on a random plane,
                     given by axis_x / axis_y)
  random_2d(..., variations=OTHER_2D)
                     the same with twelve parameterless variations outside
                     the benchmark seven (the per-flame kernel workload)
  batch_jobs         the 256-flame batch: random_2d flames with 2..8 xforms,
                     square buffers of side log-uniform in [256, 2048],
                     sample counts log-uniform in [1e7, 1e9]
  serving_requests   a Poisson request stream: 80% random 2-D flames
                     (buffers 512..1920 x 512..1080, 1e7..1e9 samples), 15%
                     random 3-D flames (4..6 xforms, cubes of side 128..384),
                     5% continuations adding 1e8 samples to a resident buffer
"""
from __future__ import annotations

import numpy as np

TIER_A = ["linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "julia"]
TWO_D = {"swirl", "horseshoe", "polar", "julia"}
# twelve 2-D variations outside the benchmark seven that take no parameters
# (the per-flame kernel workload: random_2d(seed, variations=OTHER_2D))
OTHER_2D = ["handkerchief", "heart", "disc", "spiral", "hyperbolic", "diamond", "ex",
            "exponential", "cosine", "power", "cylinder", "tangent"]


def _f(x) -> float:
    return float(x)


def sierpinski_2d(size=(1024, 1024)) -> dict:
    verts = [(0.0, 1.0), (-1.0, -1.0), (1.0, -1.0)]
    xfs = []
    for v in verts:
        xfs.append({
            "weight": 1.0 / 3.0,
            "variations": [{"name": "linear", "weight": 1.0}],
            "pre_affine": {"A": [[0.5, 0.0], [0.0, 0.5]], "b": [0.5 * v[0], 0.5 * v[1]]},
        })
    return {"dimensions": 2, "size": list(size), "bounds": [[-1.0, 1.0], [-1.0, 1.0]],
            "xforms": xfs}


def heavy_point_2d(size=(640, 360)) -> dict:
    """Three contractions by 1/2 with weights 0.9 / 0.05 / 0.05: the measure
    piles up at the heavy map's fixed point, so a few cells hold most samples
    (a flame for the hot-cell table).  Linear maps only: FP64 renders are
    bit-exact against the oracle."""
    def xf(w, bx, by):
        return {"weight": w, "variations": [{"name": "linear", "weight": 1.0}],
                "pre_affine": {"A": [[0.5, 0.0], [0.0, 0.5]], "b": [bx, by]}}
    return {"dimensions": 2, "size": list(size), "bounds": [[-1.0, 1.0], [-1.0, 1.0]],
            "xforms": [xf(0.9, 0.13, 0.21), xf(0.05, -0.5, 0.4), xf(0.05, 0.45, -0.5)]}


def tetrahedron_3d(size=(512, 512, 512)) -> dict:
    verts = [(1, 1, 1), (1, -1, -1), (-1, 1, -1), (-1, -1, 1)]
    xfs = []
    for v in verts:
        xfs.append({
            "weight": 0.25,
            "variations": [{"name": "linear", "weight": 1.0}],
            "pre_affine": {"A": [[0.5, 0, 0], [0, 0.5, 0], [0, 0, 0.5]],
                           "b": [0.5 * v[0], 0.5 * v[1], 0.5 * v[2]]},
        })
    return {"dimensions": 3, "size": list(size),
            "bounds": [[-1.0, 1.0], [-1.0, 1.0], [-1.0, 1.0]], "xforms": xfs}


def random_2d(seed: int, k: int = 6, size=(1920, 1080), variations=TIER_A,
              nvars: int = 2, bounds=((-2.0, 2.0), (-1.125, 1.125))) -> dict:
    g = np.random.Generator(np.random.PCG64(seed))
    w = g.dirichlet(np.ones(k))
    xfs = []
    for i in range(k):
        pre = g.uniform(-1.0, 1.0, size=(2, 3))
        post = np.eye(2) + g.normal(0.0, 0.1, size=(2, 2))
        postb = g.normal(0.0, 0.1, size=2)
        names = list(g.choice(len(variations), size=nvars, replace=False))
        vw = g.dirichlet(np.ones(nvars))
        xfs.append({
            "weight": _f(w[i]),
            "variations": [{"name": variations[n], "weight": _f(vw[j])}
                           for j, n in enumerate(names)],
            "pre_affine": {"A": [[_f(pre[0, 0]), _f(pre[0, 1])], [_f(pre[1, 0]), _f(pre[1, 1])]],
                           "b": [_f(pre[0, 2]), _f(pre[1, 2])]},
            "post_affine": {"A": [[_f(post[0, 0]), _f(post[0, 1])],
                                  [_f(post[1, 0]), _f(post[1, 1])]],
                            "b": [_f(postb[0]), _f(postb[1])]},
        })
    return {"dimensions": 2, "size": list(size),
            "bounds": [list(bounds[0]), list(bounds[1])], "xforms": xfs}


def random_3d(seed: int, k: int = 4, size=(256, 256, 256), variations=TIER_A,
              nvars: int = 2) -> dict:
    g = np.random.Generator(np.random.PCG64(seed))
    w = g.dirichlet(np.ones(k))
    xfs = []
    for i in range(k):
        pre = g.uniform(-1.0, 1.0, size=(3, 4))
        post = np.eye(3) + g.normal(0.0, 0.1, size=(3, 3))
        postb = g.normal(0.0, 0.1, size=3)
        names = list(g.choice(len(variations), size=nvars, replace=False))
        vw = g.dirichlet(np.ones(nvars))
        vs = []
        for j, n in enumerate(names):
            v = {"name": variations[n], "weight": _f(vw[j])}
            if variations[n] in TWO_D:
                ax = g.choice(3, size=2, replace=False)
                v["axis_x"], v["axis_y"] = int(ax[0]), int(ax[1])
            vs.append(v)
        xfs.append({
            "weight": _f(w[i]),
            "variations": vs,
            "pre_affine": {"A": [[_f(pre[r, c]) for c in range(3)] for r in range(3)],
                           "b": [_f(pre[r, 3]) for r in range(3)]},
            "post_affine": {"A": [[_f(post[r, c]) for c in range(3)] for r in range(3)],
                            "b": [_f(postb[r]) for r in range(3)]},
        })
    return {"dimensions": 3, "size": list(size),
            "bounds": [[-2.0, 2.0], [-2.0, 2.0], [-2.0, 2.0]], "xforms": xfs}


def _log_uniform(g, lo: float, hi: float) -> float:
    return float(np.exp(g.uniform(np.log(lo), np.log(hi))))


def batch_jobs(seed: int = 11, n: int = 256, side=(256, 2048), samples=(1e7, 1e9)):
    """[(flame, samples)] of the batched-launch workload."""
    g = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        k = int(g.integers(2, 9))
        s = int(round(_log_uniform(g, *side)))
        m = int(round(_log_uniform(g, *samples)))
        out.append((random_2d(seed * 100_003 + i, k=k, size=(s, s)), m))
    return out


def serving_requests(seed: int = 23, rate: float = 200.0, duration: float = 60.0,
                     samples=(1e7, 1e9), cont_samples: int = 10**8):
    """[(arrival_s, kind, flame or None, samples)], kind in {"2d", "3d",
    "cont"}; arrivals are a Poisson process of `rate` per second."""
    g = np.random.Generator(np.random.PCG64(seed))
    out = []
    t = 0.0
    i = 0
    while True:
        t += float(g.exponential(1.0 / rate))
        if t >= duration:
            break
        u = float(g.uniform())
        if u < 0.80:
            w = int(round(_log_uniform(g, 512, 1920)))
            h = int(round(_log_uniform(g, 512, 1080)))
            k = int(g.integers(2, 9))
            out.append((t, "2d", random_2d(seed * 1_000_003 + i, k=k, size=(w, h)),
                        int(round(_log_uniform(g, *samples)))))
        elif u < 0.95:
            c = int(round(_log_uniform(g, 128, 384)))
            k = int(g.integers(4, 7))
            out.append((t, "3d", random_3d(seed * 1_000_003 + i, k=k, size=(c, c, c)),
                        int(round(_log_uniform(g, *samples)))))
        else:
            out.append((t, "cont", None, cont_samples))
        i += 1
    return out
