"""Four-dimensional flames.

The reference's BufferRenderer, Flame, XForm, Point and variation templates
take any dimension count; its ffr-buf CLI compiles 1..3
(src/ffr_buf.cpp:134-141).  The golden vectors (tests/golden/make_golden_4d.py)
come from the reference's own templates instantiated at dims = 4: a 4-simplex
IFS (linear only) and a mixed flame with noise (randDirection<4>, gaussian
pairs), julia and swirl on axis planes, sinusoidal, spherical, a post-affine
and a final xform drawing blur's words.

CPU: the oracle reproduces them (exactly on the machine that made them,
within 1e-12 elsewhere).  GPU, through the C ABI: single steps within 1e-12
(exact for the linear flame), trace choices exact, the linear flame's renders
bit-exact with the reference's statistics, the mixed flame's histogram within
3x the oracle noise floor in FP64 and FP32; batches and the serving loop
refuse 4-D flames (ffr_render renders them).
"""
import json
import os
import platform

import numpy as np
import pytest

from conftest import GOLDEN, golden_flame_text

with open(os.path.join(GOLDEN, "d4.json")) as _f:
    META = json.load(_f)
EXACT_LIBM = platform.machine() == "x86_64"
STEP_REL = 1e-12


def data():
    return np.load(os.path.join(GOLDEN, "data", "d4.npz"))


def close(a, b, rel):
    return bool(np.all(np.abs(a - b) <= rel * np.maximum(np.abs(b), 1.0)))


def step_keys(name):
    m = META["flames"][name]
    return list(range(m["xforms"])) + ([-1] if m["final"] else [])


@pytest.mark.parametrize("name", sorted(META["flames"]))
def test_oracle_d4_steps_and_trace(fo, name):
    d = data()
    of = fo.OracleFlame(fo.load_flame(golden_flame_text(name)))
    for xi in step_keys(name):
        got = fo.step(of, xi, 777, d[f"{name}_step_in"])
        want = d[f"{name}_step_{str(xi).replace('-', 'm')}"]
        if EXACT_LIBM or name == "d4_simplex":
            np.testing.assert_array_equal(got, want)
        else:
            assert close(got, want, STEP_REL)
    ids, pts = fo.trace(of, 999, 20, len(d[f"{name}_trace_ids"]))
    np.testing.assert_array_equal(ids, d[f"{name}_trace_ids"])
    if EXACT_LIBM or name == "d4_simplex":
        np.testing.assert_array_equal(pts, d[f"{name}_trace_pts"])


@pytest.mark.parametrize("case", META["renders"], ids=lambda c: c["key"])
def test_oracle_d4_renders(fo, case):
    of = fo.OracleFlame(fo.load_flame(golden_flame_text(case["flame"])))
    r = fo.render(of, case["seed"], case["streams"], case["samples"], case["traj_len"],
                  case["settle"], 10**9)
    st = case["stats"]
    assert r.s_iter == st["s_iter"] and r.xf_dist.tolist() == st["xf_dist"]
    if EXACT_LIBM or case["flame"] == "d4_simplex":
        np.testing.assert_array_equal(r.counts, data()[case["key"]])
        assert r.s_plot == st["s_plot"]


def test_d4_flames_pass_validation_and_5d_is_refused(ffr):
    st, msg = ffr.create_status(golden_flame_text("d4_mixed"))
    # validation passes; without a GPU the create fails at device setup
    assert st in (ffr.FFR_OK, ffr.FFR_ERR_CUDA, ffr.FFR_ERR_OOM), (st, msg)
    f5 = {"dimensions": 5, "size": [2] * 5, "bounds": [[-1, 1]] * 5,
          "xforms": [{"weight": 1, "variations": [{"name": "linear", "weight": 1}]}]}
    st, msg = ffr.create_status(json.dumps(f5))
    assert st == ffr.FFR_ERR_PARSE and "5D not supported" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(META["flames"]))
def test_gpu_d4_steps_and_trace(ffr, name):
    d = data()
    with ffr.BufferRenderer(golden_flame_text(name), precision=ffr.FP64) as r:
        for xi in step_keys(name):
            got = r.step(xi, 777, d[f"{name}_step_in"])
            want = d[f"{name}_step_{str(xi).replace('-', 'm')}"]
            if name == "d4_simplex":
                np.testing.assert_array_equal(got, want)
            else:
                assert close(got, want, STEP_REL), xi
        ids, pts = r.trace(999, 20, len(d[f"{name}_trace_ids"]))
    np.testing.assert_array_equal(ids, d[f"{name}_trace_ids"])
    if name == "d4_simplex":
        np.testing.assert_array_equal(pts, d[f"{name}_trace_pts"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("case", [c for c in META["renders"] if c["flame"] == "d4_simplex"],
                         ids=lambda c: c["key"])
def test_gpu_d4_simplex_render_matches_reference(ffr, case, precision):
    st = case["stats"]
    with ffr.BufferRenderer(golden_flame_text(case["flame"]), precision=precision,
                            settle=case["settle"], streams=case["streams"],
                            traj_len=case["traj_len"]) as r:
        s = r.render(case["samples"], case["seed"], 10**9)
        counts = r.counts()
    assert s.samples_iterated == st["s_iter"]
    assert s.xf_dist.tolist() == st["xf_dist"]
    assert s.ctas >= 1 and s.threads_per_cta > 0 and s.streams_per_thread >= 1
    if precision == 0:
        np.testing.assert_array_equal(counts, data()[case["key"]])
        assert s.samples_plotted == st["s_plot"]
        for i, (lo, hi) in enumerate(st["ext"]):
            want_lo = np.frombuffer(int(lo, 16).to_bytes(8, "little"), dtype=np.float64)[0]
            want_hi = np.frombuffer(int(hi, 16).to_bytes(8, "little"), dtype=np.float64)[0]
            assert s.ext_lo[i] == want_lo and s.ext_hi[i] == want_hi


def tv(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return 0.5 * np.abs(a / a.sum() - b / b.sum()).sum()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_gpu_d4_mixed_histogram_within_noise_floor(ffr, fo, precision):
    """Chaotic through libm: mean TV to three oracle runs within 3x their
    mean pairwise TV, at 10^7 samples from 4096 streams."""
    text = golden_flame_text("d4_mixed")
    of = fo.OracleFlame(fo.load_flame(text))
    n, S = 10_000_000, 4096
    runs = [fo.render(of, seed, S, n, n // S, 20, 10**9, threads=os.cpu_count() or 8)
            for seed in (101, 202, 404)]
    with ffr.BufferRenderer(text, precision=precision, settle=20, streams=S,
                            traj_len=n // S) as r:
        s = r.render(n, 303, bad_limit=10**9)
        got = r.counts()
    assert s.samples_iterated == n
    floor = np.mean([tv(runs[i].counts, runs[j].counts) for i in range(3)
                     for j in range(i + 1, 3)])
    d = np.mean([tv(got, x.counts) for x in runs])
    assert d <= 3.0 * floor, (d, floor)


@pytest.mark.gpu
def test_gpu_d4_batch_and_server_refuse(ffr):
    text = golden_flame_text("d4_simplex")
    with ffr.BufferRenderer(text, precision=1) as r:
        with pytest.raises(ffr.FfrError) as e:
            ffr.Batch([r])
        assert e.value.status == ffr.FFR_ERR_ARG and "1- to 3-dimensional" in e.value.message
    srv = ffr.Server(precision=ffr.FP32, settle=20)
    try:
        with pytest.raises(ffr.FfrError) as e:
            srv.submit(text, 1000, 1)
        assert e.value.status == ffr.FFR_ERR_ARG and "1- to 3-dimensional" in e.value.message
    finally:
        srv.close()
