"""Batched render (ffr_batch_*): many flames of different sizes, dims and
sample counts in one persistent launch per (dims, colour) group, replayed
from a captured CUDA graph.  Each job runs exactly the streams a solo
ffr_render would, so every buffer must equal the solo render's: counts
exactly (FP64 and FP32: per-stream arithmetic is deterministic and integer
adds commute), colour sums within 1e-12 relative (their addition order is
not fixed)."""
import json

import numpy as np
import pytest

from conftest import golden_flame_text

pytestmark = pytest.mark.gpu


def jobs(flames):
    return [
        (json.dumps(flames.sierpinski_2d(size=(300, 200))), 3_000_000, 11),
        (golden_flame_text("alg2d"), 1_000_000, 12),
        (golden_flame_text("color"), 700_000, 13),
        (json.dumps(flames.tetrahedron_3d(size=(64, 64, 64))), 2_000_000, 14),
        (golden_flame_text("julia3"), 500_000, 15),
        (json.dumps(flames.random_2d(7, size=(320, 180))), 4_000_000, 16),
        (golden_flame_text("line1d"), 300_000, 17),
        (golden_flame_text("c2small"), 1, 18),          # a one-sample job
    ]


def solo(ffr, text, n, seed, precision, bad_limit=256):
    """ffr_render of the same job: one trajectory of 4096 samples per stream,
    the decomposition the batch uses when the context leaves streams open."""
    streams = max(1, -(-n // 4096))
    with ffr.BufferRenderer(text, precision=precision, settle=20, traj_len=4096,
                            streams=streams) as r:
        s = r.render(n, seed, bad_limit)
        return r.buffer_array(), s


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_batch_equals_solo(ffr, flames, precision):
    js = jobs(flames)
    rs = [ffr.BufferRenderer(t, precision=precision, settle=20, traj_len=4096) for t, _, _ in js]
    with ffr.Batch(rs) as b:
        status, sts = b.render([n for _, n, _ in js], [s for _, _, s in js])
    assert status == ffr.FFR_OK
    for (t, n, seed), r, st in zip(js, rs, sts):
        got = r.buffer_array()
        want, ws = solo(ffr, t, n, seed, precision)
        np.testing.assert_array_equal(got[:, 0], want[:, 0])
        if got.shape[1] > 1:
            np.testing.assert_allclose(got[:, 1:].copy().view(np.float64),
                                       want[:, 1:].copy().view(np.float64),
                                       rtol=1e-12, atol=1e-9)
        assert st.samples_iterated == ws.samples_iterated == n
        assert st.samples_plotted == ws.samples_plotted
        assert st.xf_dist.tolist() == ws.xf_dist.tolist()
    # the random flame has hot cells: its job counted them in shared memory
    assert sts[5].hot_cells > 0 and sts[5].agg == 0
    for r in rs:
        r.close()


def test_batch_replay_accumulates(ffr, flames):
    """Second launch of the captured graph adds to the buffers: the result is
    the sum of the two solo renders."""
    js = jobs(flames)[:4]
    rs = [ffr.BufferRenderer(t, settle=20, traj_len=4096) for t, _, _ in js]
    with ffr.Batch(rs) as b:
        b.render([n for _, n, _ in js], [s for _, _, s in js])
        b.render([n // 2 for _, n, _ in js], [s + 100 for _, _, s in js])
    for (t, n, seed), r in zip(js, rs):
        first, _ = solo(ffr, t, n, seed, 0)
        second, _ = solo(ffr, t, n // 2, seed + 100, 0)
        np.testing.assert_array_equal(r.counts(), first[:, 0] + second[:, 0])
        r.close()


def test_batch_rejects_mixed_precision(ffr, flames):
    a = ffr.BufferRenderer(json.dumps(flames.sierpinski_2d((16, 16))), precision=0)
    b = ffr.BufferRenderer(json.dumps(flames.sierpinski_2d((16, 16))), precision=1)
    with pytest.raises(ffr.FfrError) as e:
        ffr.Batch([a, b])
    assert e.value.status == ffr.FFR_ERR_ARG
    a.close()
    b.close()


def test_batch_many_flames(ffr, flames):
    """64 random flames of log-uniform sizes and sample counts."""
    g = np.random.Generator(np.random.PCG64(11))
    rs, ns, seeds, texts = [], [], [], []
    for i in range(64):
        side = int(np.exp(g.uniform(np.log(64), np.log(512))))
        n = int(np.exp(g.uniform(np.log(1e4), np.log(1e6))))
        t = json.dumps(flames.random_2d(1000 + i, k=int(g.integers(2, 9)), size=(side, side)))
        texts.append(t)
        rs.append(ffr.BufferRenderer(t, precision=1, settle=20, traj_len=4096))
        ns.append(n)
        seeds.append(500 + i)
    with ffr.Batch(rs) as b:
        status, sts = b.render(ns, seeds, bad_limit=10**9)
    for i in (0, 17, 63):
        want, ws = solo(ffr, texts[i], ns[i], seeds[i], 1, bad_limit=10**9)
        np.testing.assert_array_equal(rs[i].counts(), want[:, 0])
    assert all(st.samples_iterated == n for st, n in zip(sts, ns))
    for r in rs:
        r.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_autotuned_render_with_odd_cell_count(ffr, flames, precision):
    """Renders of 2^25 samples or more are autotuned on a scratch copy of the
    buffer.  With an odd cell count the scratch's statistics block must still
    start 8-byte aligned (its u64 atomics need it), and the autotuned render
    equals a render with the kernel fixed."""
    text = json.dumps(flames.random_2d(11, k=4, size=(723, 723)))
    n = 1 << 25
    S = n // 4096
    with ffr.BufferRenderer(text, precision=precision, settle=20, traj_len=4096,
                            streams=S) as a:
        sa = a.render(n, 5, bad_limit=10**9)
        got = a.counts()
    with ffr.BufferRenderer(text, precision=precision, settle=20, traj_len=4096,
                            streams=S, kernel=ffr.KERNEL_PLAIN) as b:
        sb = b.render(n, 5, bad_limit=10**9)
        want = b.counts()
    np.testing.assert_array_equal(got, want)
    assert sa.samples_plotted == sb.samples_plotted
