"""FP32 and transcendental-flame parity by histogram total variation.

Trajectories are chaotic: an ulp of difference in sin/cos/atan2 (glibc
against CUDA in FP64, or any FP32 rounding) grows until the two runs visit
the attractor independently.  The bar is therefore statistical: the
normalised histogram of a GPU run must lie within 3x the noise floor of the
reference arithmetic, the floor being the TV distance between two oracle
(FP64, reference order of operations) runs with different seeds at the same
sample count.  TV(h, g) = 1/2 sum |h/sum h - g/sum g|.
"""
import json

import numpy as np
import pytest

from conftest import golden_flame_text

pytestmark = pytest.mark.gpu

TV_FACTOR = 3.0


def tv(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return 0.5 * np.abs(a / a.sum() - b / b.sum()).sum()


def oracle_pair(fo, text, n, settle=20):
    of = fo.OracleFlame(fo.load_flame(text))
    a = fo.render(of, 101, 4096, n, max(1, n // 4096), settle, 10**9, threads=16)
    b = fo.render(of, 202, 4096, n, max(1, n // 4096), settle, 10**9, threads=16)
    return a, b


CASES = [
    ("c2small", None),
    ("rand3d", None),
    ("julia3", None),
    ("line1d", None),
    ("bench_flame_small", "gen"),
]


def flame_text(flames, name, kind):
    if kind == "gen":
        return json.dumps(flames.random_2d(7, size=(240, 135)))
    return golden_flame_text(name)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("name,kind", CASES)
def test_histogram_tv_within_noise_floor(ffr, fo, flames, name, kind, precision):
    text = flame_text(flames, name, kind)
    n = 20_000_000
    a, b = oracle_pair(fo, text, n)
    floor = tv(a.counts, b.counts)
    with ffr.BufferRenderer(text, precision=precision, settle=20) as r:
        s = r.render(n, 303, bad_limit=10**9)
        got = r.counts()
    d = tv(got, a.counts)
    assert d <= TV_FACTOR * floor, (name, d, floor)
    # binned fraction agrees with the reference arithmetic too
    assert abs(s.samples_plotted / n - a.s_plot / n) < 0.01


@pytest.mark.parametrize("name,kind", CASES)
def test_fp32_xform_distribution_exact(ffr, fo, flames, name, kind):
    """Xform choices are exact per stream in FP32 (integer selection on the
    reference's 53-bit draw), so the per-xform counts equal the oracle's."""
    text = flame_text(flames, name, kind)
    of = fo.OracleFlame(fo.load_flame(text))
    S, N, L = 512, 1_000_000, 977
    ref = fo.render(of, 9, S, N, L, 20, 10**9, threads=16)
    with ffr.BufferRenderer(text, precision=1, settle=20, streams=S, traj_len=L) as r:
        s = r.render(N, 9, bad_limit=10**9)
    if ref.bad == 0 and s.bad_values == 0:
        assert s.xf_dist.tolist() == ref.xf_dist.tolist()
    assert s.samples_iterated == ref.s_iter
