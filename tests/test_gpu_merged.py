"""The FP32 merged form (ProgHeader::merged) and its kernel instantiations.

Every kernel computes the same operations for a merged program -- the plain
render kernel in its variation-set instantiations (1: a branch per type the
flame uses; 2: all seven types without branches, thresholds in registers),
the xform-sorted kernel through the general instantiation, the batch kernel
-- so FP32 buffers, statistics and xform choices are identical across them.
These cases aim at the edges of that claim:

  * a julia of weight 0 still draws its word (the reference calls it and
    multiplies by 0): xform choices stay the oracle's;
  * points beyond the merged form's range (sum t_i^2 >= 1e36) fall back to
    per-slot evaluation in both instantiations alike;
  * flames using 2, 4 and 7 of the seven types (set 1 and set 2), with and
    without a final xform, in one batch and alone;
  * a 3-D flame whose 2-D types act on per-variation planes.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TYPES = ["linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "julia"]


def flame(types_per_xform, final=None, scale=1.0, size=(160, 90)):
    g = np.random.Generator(np.random.PCG64(len(types_per_xform) * 7 + len(str(final))))
    xfs = []
    for k, names in enumerate(types_per_xform):
        pre = g.uniform(-1.0, 1.0, size=(2, 3))
        xfs.append({
            "weight": float(1.0 + k),
            "variations": [{"name": n, "weight": float(w)} for n, w in names],
            "pre_affine": {"A": [[float(pre[0, 0]) * scale, float(pre[0, 1])],
                                 [float(pre[1, 0]), float(pre[1, 1]) * scale]],
                           "b": [float(pre[0, 2]), float(pre[1, 2])]},
        })
    f = {"dimensions": 2, "size": list(size), "bounds": [[-2.0, 2.0], [-1.2, 1.2]],
         "xforms": xfs}
    if final:
        f["final_xform"] = {"variations": [{"name": n, "weight": float(w)} for n, w in final]}
    return json.dumps(f)


CASES = {
    "two_types": flame([[("linear", 0.7), ("sinusoidal", 0.3)], [("spherical", 1.0)]]),
    "four_types_julia": flame([[("julia", 0.6), ("linear", 0.4)], [("swirl", 0.5),
                                                                   ("spherical", 0.5)],
                               [("julia", 0.3), ("sinusoidal", 0.7)]]),
    "all_seven_final": flame([[("linear", 0.5), ("julia", 0.5)], [("sinusoidal", 0.4),
                                                                 ("spherical", 0.6)],
                              [("swirl", 0.3), ("horseshoe", 0.7)], [("polar", 0.5),
                                                                     ("julia", 0.5)],
                              [("horseshoe", 0.2), ("linear", 0.8)]],
                             final=[("linear", 0.9), ("julia", 0.1)]),
    # julia at weight 0 still draws; and a type twice in one xform
    "julia_weight_zero": flame([[("julia", 0.0), ("linear", 1.0)], [("swirl", 0.6),
                                                                   ("polar", 0.2),
                                                                   ("polar", 0.2)],
                                [("sinusoidal", 0.5), ("horseshoe", 0.5)],
                                [("spherical", 1.0), ("julia", 0.0)],
                                [("linear", 1.0)]]),
    # pre-affines scaled by 1e19: sum t_i^2 passes 1e36, the per-slot path
    "huge_points": flame([[("linear", 0.5), ("swirl", 0.5)], [("julia", 0.5),
                                                             ("spherical", 0.5)],
                          [("polar", 0.5), ("horseshoe", 0.5)],
                          [("sinusoidal", 1.0)], [("linear", 1.0)]], scale=1e19),
}


def render(ffr, text, kernel, n=3_000_000, seed=5):
    with ffr.BufferRenderer(text, precision=ffr.FP32, settle=20, streams=4096,
                            traj_len=n // 4096 + 1, kernel=kernel) as r:
        s = r.render(n, seed, bad_limit=10**12)
        return s, r.counts()


def random_3d_text():
    import importlib.util
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location(
        "ffr_flames_t", os.path.join(here, "..", "flame-fractal-renderer_gb300", "flames.py"))
    fl = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fl)
    # 2-D types on random planes of a 3-D flame (the serving stream's 3-D jobs)
    return json.dumps(fl.random_3d(5, k=5, size=(64, 64, 64)))


CASES["random_3d_planes"] = random_3d_text()
# more xforms than the registers hold thresholds for (shared-memory choice)
CASES["ten_xforms"] = flame([[(TYPES[(k + j) % 7], 0.5) for j in (0, 3)] for k in range(10)])


@pytest.mark.parametrize("name", sorted(CASES))
def test_merged_plain_equals_sorted(ffr, name):
    """The merged instantiations (plain kernel) against the general one
    (xform-sorted kernel): identical FP32 buffers and statistics."""
    text = CASES[name]
    sp, cp = render(ffr, text, ffr.KERNEL_PLAIN)
    ss, cs = render(ffr, text, ffr.KERNEL_SORTED)
    assert sp.kernel == ffr.KERNEL_PLAIN and ss.kernel == ffr.KERNEL_SORTED
    np.testing.assert_array_equal(cp, cs)
    assert sp.samples_plotted == ss.samples_plotted
    assert sp.bad_values == ss.bad_values
    np.testing.assert_array_equal(sp.xf_dist, ss.xf_dist)


@pytest.mark.parametrize("name", ["julia_weight_zero", "four_types_julia", "all_seven_final"])
def test_merged_choices_match_oracle(ffr, fo, name):
    """Julia draws its word whatever its weight: per-xform counts (the
    choices, hence every draw) equal the FP64 oracle's for the same
    streams."""
    text = CASES[name]
    S, N, L = 512, 1_000_000, 977
    of = fo.OracleFlame(fo.load_flame(text))
    ref = fo.render(of, 9, S, N, L, 20, 10**12, threads=16)
    with ffr.BufferRenderer(text, precision=ffr.FP32, settle=20, streams=S, traj_len=L,
                            kernel=ffr.KERNEL_PLAIN) as r:
        s = r.render(N, 9, bad_limit=10**12)
    assert ref.bad == 0 and s.bad_values == 0
    assert s.xf_dist.tolist() == ref.xf_dist.tolist()


def test_merged_batch_equals_solo(ffr):
    """Sets 1 and 2 and a general-kernel flame in one batch (three kernel
    groups): every buffer equals its solo plain render."""
    texts = [CASES["two_types"], CASES["all_seven_final"], CASES["julia_weight_zero"],
             json.dumps({"dimensions": 2, "size": [64, 64], "bounds": [[-2, 2], [-2, 2]],
                         "xforms": [{"weight": 1, "variations": [{"name": "handkerchief",
                                                                  "weight": 1}]},
                                    {"weight": 1, "variations": [{"name": "julia",
                                                                  "weight": 1}]}]})]
    n = [1_000_000, 2_000_000, 1_500_000, 800_000]
    seeds = [3, 4, 5, 6]
    rs = [ffr.BufferRenderer(t, precision=ffr.FP32, settle=20, traj_len=4096,
                             kernel=ffr.KERNEL_PLAIN) for t in texts]
    try:
        with ffr.Batch(rs) as b:
            b.render(n, seeds, bad_limit=10**12)
        got = [r.counts() for r in rs]
    finally:
        for r in rs:
            r.close()
    for t, k, sd, g in zip(texts, n, seeds, got):
        with ffr.BufferRenderer(t, precision=ffr.FP32, settle=20, traj_len=4096,
                                streams=-(-k // 4096), kernel=ffr.KERNEL_PLAIN) as r:
            r.render(k, sd, bad_limit=10**12)
            np.testing.assert_array_equal(g, r.counts())


def test_merged_colour_flame_plain_equals_sorted(ffr):
    """A colour flame in the merged form: counts identical, colour sums equal
    to rounding (their atomic additions come in another order)."""
    f = json.loads(CASES["all_seven_final"])
    f["color_dimensions"] = 3
    f["color_speed"] = 0.4
    for k, x in enumerate(f["xforms"]):
        x["color"] = [((k * 37) % 11) / 10.0, ((k * 53) % 7) / 6.0, 0.25]
    text = json.dumps(f)
    out = []
    for kernel in (ffr.KERNEL_PLAIN, ffr.KERNEL_SORTED):
        with ffr.BufferRenderer(text, precision=ffr.FP32, settle=20, streams=4096,
                                traj_len=500, kernel=kernel) as r:
            r.render(2_000_000, 8, bad_limit=10**12)
            out.append(r.buffer_array())
    np.testing.assert_array_equal(out[0][:, 0], out[1][:, 0])
    np.testing.assert_allclose(out[0][:, 1:].copy().view(np.float64),
                               out[1][:, 1:].copy().view(np.float64), rtol=1e-9, atol=1e-6)
