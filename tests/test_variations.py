"""All 98 variations of src/variations/variations.hpp, one small flame each
(N-D ones in 1-D, 2-D and 3-D; 2-D ones in 2-D and on a 3-D axis plane),
against vectors the reference itself produced (tests/golden/make_golden.py).

CPU (oracle): single step, trajectory trace and render reproduce the
reference exactly on the machine the fixtures were made on (same glibc),
within 1e-12 elsewhere.
GPU (C ABI): xform choices and RNG consumption exact (a wrong draw count
shifts every later choice), single steps within 1e-12 of the reference
(bit-exact where only + - * / sqrt floor rint fmod copysign are involved),
renders bit-exact for those, by statistics otherwise.
"""
import json
import os
import platform

import numpy as np
import pytest

from conftest import GOLDEN, golden_manifest

MAN = golden_manifest()
VF = MAN["vflames"]
EXACT_LIBM = platform.machine() == "x86_64"

# variations whose arithmetic uses only + - * / sqrt floor rint fmod copysign
ALGEBRAIC = {"linear", "spherical", "bent", "rectangles", "fisheye", "bubble",
             "square_noise", "separation", "splits", "modulus", "celln",
             "unit_sphere", "unit_cube", "horseshoe", "hyperbolic", "rings",
             "curl", "cross", "mobius", "scry", "stripes", "boarders",
             "butterfly", "cell", "loonie"}
STEP_REL = 1e-12


def var_of(name):
    return name.split("_", 1)[1]


def npz(name):
    return np.load(os.path.join(GOLDEN, "data", "var", name + ".npz"))


def text(name):
    with open(os.path.join(GOLDEN, "flames", "var", name + ".json")) as f:
        return f.read()


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1.0)


def close(a, b, rel):
    both_nan = np.isnan(a) & np.isnan(b)
    same_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    ok = both_nan | same_inf | (rel_err(np.nan_to_num(a), np.nan_to_num(b)) <= rel)
    return bool(np.all(ok))


@pytest.mark.parametrize("name", sorted(VF))
def test_oracle_variation_matches_reference(fo, name):
    d = npz(name)
    of = fo.OracleFlame(fo.load_flame(text(name)))
    got = fo.step(of, 0, 777, d["step_in"])
    ids, pts = fo.trace(of, 999, 20, len(d["trace_ids"]))
    np.testing.assert_array_equal(ids, d["trace_ids"])
    seed, streams, n, L, settle, bvl = VF[name]["render"]
    r = fo.render(of, seed, streams, n, L, settle, bvl)
    st = VF[name]["stats"]
    assert r.s_iter == st["s_iter"] and r.xf_dist.tolist() == st["xf_dist"]
    assert r.bad == st["bad"]
    if EXACT_LIBM:
        np.testing.assert_array_equal(got, d["step_out"])
        np.testing.assert_array_equal(pts, d["trace_pts"])
        np.testing.assert_array_equal(r.counts, d["counts"])
        assert r.s_plot == st["s_plot"]
    else:
        assert close(got, d["step_out"], STEP_REL)


def test_every_variation_is_covered():
    import flame_oracle as fo
    covered = {var_of(n) for n in VF}
    assert covered == set(fo.ALL_NAMES)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(VF))
def test_gpu_variation_fp64(ffr, name):
    d = npz(name)
    v = var_of(name)
    st = VF[name]["stats"]
    seed, streams, n, L, settle, bvl = VF[name]["render"]
    with ffr.BufferRenderer(text(name), precision=ffr.FP64, settle=settle,
                            streams=streams, traj_len=L) as r:
        got = r.step(0, 777, d["step_in"])
        ids, pts = r.trace(999, 20, len(d["trace_ids"]))
        s = r.render(n, seed, bvl)
        counts = r.counts()
    np.testing.assert_array_equal(ids, d["trace_ids"])
    if v in ALGEBRAIC:
        np.testing.assert_array_equal(got, d["step_out"])
        np.testing.assert_array_equal(pts, d["trace_pts"])
        np.testing.assert_array_equal(counts, d["counts"])
        assert s.samples_plotted == st["s_plot"]
    else:
        assert close(got, d["step_out"], STEP_REL), float(np.nanmax(rel_err(got, d["step_out"])))
    assert s.samples_iterated == st["s_iter"]
    if st["bad"] == 0 and s.bad_values == 0:
        assert s.xf_dist.tolist() == st["xf_dist"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(VF))
def test_gpu_variation_fp32_choices(ffr, name):
    """FP32: same xform choices (hence same RNG consumption) per stream."""
    d = npz(name)
    with ffr.BufferRenderer(text(name), precision=ffr.FP32) as r:
        ids, pts = r.trace(999, 20, len(d["trace_ids"]))
        got = r.step(0, 777, d["step_in"])
    np.testing.assert_array_equal(ids, d["trace_ids"])
    # single-precision step: loose agreement where the reference is finite
    # and well-conditioned
    ref = d["step_out"]
    fin = np.isfinite(ref) & (np.abs(ref) < 1e3)
    err = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)
    assert np.median(err) < 1e-3
