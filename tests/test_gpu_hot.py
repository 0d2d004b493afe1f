"""Hot-cell table (FFR_KERNEL_HOT, and the autotuner's choice of it): the
plain kernel counting a flame's hottest cells in per-CTA shared memory must
give the same buffer as the plain kernel, which in turn matches the oracle.

Tolerances: counts, samples plotted and xform distribution exact; colour
sums within 1e-9 relative (their atomic adds run in a different order).
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLAIN, HOT = 1, 3


def heavy_point_flame(size=(640, 360)):
    import flames
    return flames.heavy_point_2d(size)


def render_pair(ffr, text, precision, samples, seed, S, L, preload=None):
    out = {}
    for k in (PLAIN, HOT):
        with ffr.BufferRenderer(text, precision=precision, settle=20, streams=S,
                                traj_len=L, kernel=k) as r:
            if preload is not None:
                r.add_buffer(preload)
            s = r.render(samples, seed)
            out[k] = (s, r.buffer_array())
    return out


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_hot_equals_plain_on_benchmark_flame(ffr, flames, prec):
    text = json.dumps(flames.random_2d(7))
    p = ffr.FP32 if prec == "fp32" else ffr.FP64
    out = render_pair(ffr, text, p, 40_000_000, 5, 20_000, 2_000)
    (sp, bp), (sh, bh) = out[PLAIN], out[HOT]
    assert sp.hot_cells == 0 and sh.hot_cells > 0
    assert sh.kernel == PLAIN
    np.testing.assert_array_equal(bh, bp)
    assert sh.samples_plotted == sp.samples_plotted
    assert sh.xf_dist.tolist() == sp.xf_dist.tolist()


def test_hot_matches_oracle_fp64(ffr, fo):
    text = json.dumps(heavy_point_flame())
    of = fo.OracleFlame(fo.load_flame(text))
    seed, S, N, L = 11, 4096, 4_000_000, 977
    ref = fo.render(of, seed, S, N, L, 20, threads=8)
    c = ref.counts.astype(np.float64)
    assert np.sort(c)[::-1][:8].sum() > 0.2 * c.sum()     # the flame is hot
    with ffr.BufferRenderer(text, precision=ffr.FP64, settle=20, streams=S, traj_len=L,
                            kernel=HOT) as r:
        s = r.render(N, seed)
        got = r.counts()
    assert s.hot_cells > 0
    np.testing.assert_array_equal(got, ref.counts)
    assert s.samples_plotted == ref.s_plot
    assert s.xf_dist.tolist() == ref.xf_dist.tolist()


def test_hot_cells_carry_into_high_words(ffr, fo):
    """Shared counts flushed into cells near 2^32: the carry is exact."""
    text = json.dumps(heavy_point_flame(size=(64, 64)))
    of = fo.OracleFlame(fo.load_flame(text))
    base = np.full(64 * 64, (1 << 32) - 5000, dtype=np.uint64)
    seed, S, N, L = 3, 2048, 3_000_000, 1000
    ref = fo.render(of, seed, S, N, L, 20)
    with ffr.BufferRenderer(text, precision=ffr.FP64, settle=20, streams=S, traj_len=L,
                            kernel=HOT) as r:
        r.add_buffer(base.tobytes())
        s = r.render(N, seed)
        got = r.counts()
    assert s.hot_cells > 0
    np.testing.assert_array_equal(got, base + ref.counts)
    assert int(got.max()) > (1 << 32)


def test_hot_colour_flame(ffr, flames):
    """Colours still go to the buffer: counts exact, colour sums close."""
    fl = heavy_point_flame()
    for x, col in zip(fl["xforms"], ([1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0])):
        x["color"] = col
    fl["color_dimensions"] = 3
    fl["color_speed"] = 0.5
    text = json.dumps(fl)
    out = render_pair(ffr, text, ffr.FP64, 4_000_000, 8, 4096, 977)
    (sp, bp), (sh, bh) = out[PLAIN], out[HOT]
    assert sh.hot_cells > 0
    np.testing.assert_array_equal(bh[:, 0], bp[:, 0])
    cp = bp[:, 1:].copy().view(np.float64)
    ch = bh[:, 1:].copy().view(np.float64)
    np.testing.assert_allclose(ch, cp, rtol=1e-9, atol=1e-9)


def test_hot_without_hot_cells_is_plain(ffr, flames):
    """A flame without hot cells (uniform Sierpinski) gets no table."""
    text = json.dumps(flames.sierpinski_2d(size=(512, 512)))
    out = render_pair(ffr, text, ffr.FP32, 20_000_000, 2, 8192, 1000)
    (sp, bp), (sh, bh) = out[PLAIN], out[HOT]
    assert sh.hot_cells == 0
    np.testing.assert_array_equal(bh, bp)


def test_autotuner_decision_gives_plain_buffer(ffr, flames):
    """Whatever the autotuner picks (table or not) the buffer is the plain
    kernel's for the same streams and trajectory length."""
    text = json.dumps(flames.random_2d(7))
    with ffr.BufferRenderer(text, precision=ffr.FP32, settle=20, streams=30_000,
                            traj_len=2_000) as r:
        s = r.render(60_000_000, 6)
        auto = r.buffer_array()
    with ffr.BufferRenderer(text, precision=ffr.FP32, settle=20, streams=30_000,
                            traj_len=2_000, kernel=PLAIN) as r:
        r.render(60_000_000, 6)
        plain = r.buffer_array()
    np.testing.assert_array_equal(auto, plain)
    assert s.kernel in (1, 2)
