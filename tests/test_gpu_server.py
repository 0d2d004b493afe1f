"""Serving loop (ffr_server_*): continuous batching of render jobs with
device-resident buffers and admission by a device-memory budget.

A job of N samples runs ceil(N / traj_len) streams of one trajectory each,
the decomposition ffr_render uses for a context with those streams and that
trajectory length.  Every job must therefore equal that solo render, alone
and in any mix: counts exactly (per-stream arithmetic is deterministic and
integer adds commute), colour sums within 1e-12 relative (their order of
addition is not fixed), statistics exactly."""
import json
import threading
import time

import numpy as np
import pytest

from conftest import golden_flame_text

pytestmark = pytest.mark.gpu

L = 4096
SETTLE = 20


def solo(ffr, text, n, seed, precision, bad_limit=256, traj_len=L):
    streams = max(1, -(-n // traj_len))
    with ffr.BufferRenderer(text, precision=precision, settle=SETTLE, traj_len=traj_len,
                            streams=streams) as r:
        s = r.render(n, seed, bad_limit) if n else None
        return r.buffer_array(), s, (r.cells, r.color_dims, r.dims)


def mix(flames):
    return [
        (json.dumps(flames.sierpinski_2d(size=(300, 200))), 3_000_000, 11),
        (golden_flame_text("alg2d"), 1_000_000, 12),
        (golden_flame_text("color"), 700_000, 13),
        (json.dumps(flames.tetrahedron_3d(size=(64, 64, 64))), 2_000_000, 14),
        (golden_flame_text("julia3"), 500_000, 15),
        (json.dumps(flames.random_2d(7, size=(320, 180))), 4_000_000, 16),
        (golden_flame_text("line1d"), 300_000, 17),
        (golden_flame_text("c2small"), 1, 18),
        (json.dumps(flames.random_3d(5, size=(48, 40, 32))), 1_500_000, 19),
    ]


def check_equal(got, want, st, ws):
    np.testing.assert_array_equal(got[:, 0], want[:, 0])
    if got.shape[1] > 1:
        np.testing.assert_allclose(got[:, 1:].copy().view(np.float64),
                                   want[:, 1:].copy().view(np.float64), rtol=1e-12, atol=1e-9)
    assert st.samples_iterated == ws.samples_iterated
    assert st.samples_plotted == ws.samples_plotted
    assert st.xf_dist.tolist() == ws.xf_dist.tolist()
    np.testing.assert_array_equal(st.ext_lo, ws.ext_lo)
    np.testing.assert_array_equal(st.ext_hi, ws.ext_hi)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_mixed_jobs_equal_solo_renders(ffr, flames, precision):
    """Jobs submitted from another thread while earlier ones run (staggered
    arrivals) each give the solo render's buffer and statistics."""
    js = mix(flames)
    ids = [None] * len(js)
    with ffr.Server(precision=precision, settle=SETTLE, traj_len=L) as srv:
        def client():
            for k, (t, n, seed) in enumerate(js):
                ids[k] = srv.submit(t, n, seed)
                time.sleep(0.002)
        th = threading.Thread(target=client)
        th.start()
        th.join()
        for k, (t, n, seed) in enumerate(js):
            info = srv.wait(ids[k], timeout_ms=120_000)
            assert info.state == ffr.JOB_DONE and info.status == ffr.FFR_OK, info
            want, ws, (cells, r, d) = solo(ffr, t, n, seed, precision)
            got = srv.read(ids[k], cells, r)
            check_equal(got, want, srv.stats(ids[k], d), ws)
            srv.release(ids[k])


def test_same_alone_and_in_mix(ffr, flames):
    """The same job rendered alone on an idle server and inside a mix of 24
    concurrent jobs gives identical counts."""
    text = json.dumps(flames.random_2d(7, size=(480, 270)))
    n, seed = 6_000_000, 77
    with ffr.Server(precision=1, settle=SETTLE) as srv:
        a = srv.submit(text, n, seed)
        srv.wait(a, 120_000)
        alone = srv.read(a, 480 * 270)
    g = np.random.Generator(np.random.PCG64(3))
    with ffr.Server(precision=1, settle=SETTLE, round_chunks=64) as srv:
        others = []
        for i in range(12):
            t = json.dumps(flames.random_2d(100 + i, size=(256, 256)))
            others.append(srv.submit(t, int(g.integers(10**5, 3 * 10**6)), 1000 + i))
        b = srv.submit(text, n, seed)
        for i in range(12):
            t = json.dumps(flames.random_2d(200 + i, size=(200, 120)))
            others.append(srv.submit(t, int(g.integers(10**5, 3 * 10**6)), 2000 + i))
        for j in others + [b]:
            assert srv.wait(j, 120_000).state == ffr.JOB_DONE
        inmix = srv.read(b, 480 * 270)
    np.testing.assert_array_equal(alone, inmix)


def test_continuation_adds_to_resident_buffer(ffr, flames):
    """-i accumulation on the device: a continuation (queued while its parent
    still runs, and one after it finished) adds to the same buffer."""
    text = json.dumps(flames.random_2d(9, size=(256, 144)))
    with ffr.Server(precision=1, settle=SETTLE) as srv:
        a = srv.submit(text, 2_000_000, 1)
        b = srv.continue_(a, 1_000_000, 2)
        srv.wait(b, 120_000)
        srv.wait(a, 120_000)
        c = srv.continue_(a, 500_000, 3)
        assert srv.wait(c, 120_000).state == ffr.JOB_DONE
        got = srv.read(c, 256 * 144)
        np.testing.assert_array_equal(got, srv.read(a, 256 * 144))
        want = sum(solo(ffr, text, n, s, 1)[0] for n, s in ((2_000_000, 1), (1_000_000, 2),
                                                            (500_000, 3)))
        np.testing.assert_array_equal(got, want)
        assert srv.poll(b).parent == a
        for j in (a, b, c):
            srv.release(j)


def test_hot_cell_table_after_first_round(ffr, flames):
    """A job of many rounds on a flame with hot cells counts them in shared
    memory once its buffer's first round is in (the table comes from the
    buffer's own counts); a continuation uses the table from its first
    round.  Both equal their solo renders."""
    text = json.dumps(flames.random_2d(7, size=(640, 360)))
    cells = 640 * 360
    with ffr.Server(precision=1, settle=SETTLE, round_chunks=16) as srv:
        a = srv.submit(text, 40_000_000, 5)
        assert srv.wait(a, 120_000).state == ffr.JOB_DONE
        got_a = srv.read(a, cells)
        st_a = srv.stats(a, 2)
        b = srv.continue_(a, 20_000_000, 6)
        assert srv.wait(b, 120_000).state == ffr.JOB_DONE
        got_b = srv.read(b, cells)
        st_b = srv.stats(b, 2)
    want_a, ws_a, _ = solo(ffr, text, 40_000_000, 5, 1)
    want_b, ws_b, _ = solo(ffr, text, 20_000_000, 6, 1)
    assert st_a.hot_cells > 0 and st_b.hot_cells > 0
    np.testing.assert_array_equal(got_a, want_a)
    np.testing.assert_array_equal(got_b, want_a + want_b)
    check_equal(got_a, want_a, st_a, ws_a)
    assert st_b.samples_plotted == ws_b.samples_plotted


def test_init_buffer_is_added(ffr, flames):
    """submit(init=...) adds a buffer file first (the reference's -i)."""
    text = golden_flame_text("color")
    first, _, (cells, r, _) = solo(ffr, text, 300_000, 5, 0)
    with ffr.Server(precision=0, settle=SETTLE) as srv:
        j = srv.submit(text, 400_000, 6, init=first.tobytes())
        assert srv.wait(j, 120_000).state == ffr.JOB_DONE
        got = srv.read(j, cells, r)
    second, _, _ = solo(ffr, text, 400_000, 6, 0)
    np.testing.assert_array_equal(got[:, 0], first[:, 0] + second[:, 0])
    np.testing.assert_allclose(got[:, 1:].copy().view(np.float64),
                               first[:, 1:].view(np.float64) + second[:, 1:].view(np.float64),
                               rtol=1e-12, atol=1e-9)
    with ffr.Server(precision=0, settle=SETTLE) as srv:
        with pytest.raises(ffr.FfrError) as e:
            srv.submit(text, 10, 1, init=first.tobytes()[:-8])
        assert e.value.status == ffr.FFR_ERR_IO


def test_admission_respects_memory_budget(ffr, flames):
    """With a budget that holds two 1024x1024 buffers (besides the 64 MiB
    read staging), the third job waits in the queue until a finished job's
    buffer is released; the device bytes held never pass the budget and every
    result is still exact."""
    side = 1024
    per = side * side * 4 + 200_000
    budget = (64 << 20) + int(2.5 * per)
    texts = [json.dumps(flames.random_2d(40 + i, size=(side, side))) for i in range(4)]
    with ffr.Server(precision=1, settle=SETTLE, hbm_budget=budget) as srv:
        ids = [srv.submit(t, 1_500_000, 60 + i) for i, t in enumerate(texts)]
        for i in (0, 1):
            assert srv.wait(ids[i], 120_000).state == ffr.JOB_DONE
        time.sleep(0.05)
        # buffers of finished jobs stay resident until released
        assert srv.poll(ids[2]).state == ffr.JOB_QUEUED
        assert srv.poll(ids[3]).state == ffr.JOB_QUEUED
        for i, j in enumerate(ids):
            assert srv.wait(j, 120_000).state == ffr.JOB_DONE
            got = srv.read(j, side * side)
            want, _, _ = solo(ffr, texts[i], 1_500_000, 60 + i, 1)
            np.testing.assert_array_equal(got, want)
            srv.release(j)
        ld = srv.load()
        assert ld["bytes_peak"] <= budget, ld
        assert ld["running"] == 0 and ld["queued"] == 0


def test_too_large_for_budget_is_rejected(ffr, flames):
    """A buffer larger than the whole budget (64 MiB staging + 1 MiB here) is
    refused at submission instead of waiting forever."""
    with ffr.Server(precision=1, settle=SETTLE, hbm_budget=(64 << 20) + (1 << 20)) as srv:
        with pytest.raises(ffr.FfrError) as e:
            srv.submit(json.dumps(flames.random_2d(1, size=(1024, 1024))), 10, 1)
        assert e.value.status == ffr.FFR_ERR_OOM


def test_cancel_queued_and_running(ffr, flames):
    text = json.dumps(flames.random_2d(7, size=(320, 180)))
    with ffr.Server(precision=1, settle=SETTLE, max_active=1) as srv:
        big = srv.submit(text, 10**12, 1)
        queued = srv.submit(text, 10**6, 2)
        time.sleep(0.05)
        assert srv.poll(queued).state == ffr.JOB_QUEUED
        srv.cancel(queued)
        assert srv.poll(queued).state == ffr.JOB_CANCELLED
        srv.cancel(big)
        info = srv.wait(big, 30_000)
        assert info.state == ffr.JOB_CANCELLED
        small = srv.submit(text, 10**6, 3)
        assert srv.wait(small, 60_000).state == ffr.JOB_DONE
        want, _, _ = solo(ffr, text, 10**6, 3, 1)
        np.testing.assert_array_equal(srv.read(small, 320 * 180), want)


def test_round_timeout_cancels_instead_of_hanging(ffr, flames):
    """A round that outlives timeout_ms is asked to stop through the mapped
    cancel flags (the kernels poll them every 4096 samples); its jobs end
    CANCELLED with FFR_ERR_TIMEOUT and the server keeps serving."""
    text = json.dumps(flames.random_2d(7, size=(320, 180)))
    with ffr.Server(precision=1, settle=SETTLE, traj_len=10**7, timeout_ms=20) as srv:
        j = srv.submit(text, 10**10, 1)
        info = srv.wait(j, 60_000)
        assert info.state == ffr.JOB_CANCELLED and info.status == ffr.FFR_ERR_TIMEOUT
    with ffr.Server(precision=1, settle=SETTLE, timeout_ms=5000) as srv:
        k = srv.submit(text, 10**6, 2)
        assert srv.wait(k, 60_000).state == ffr.JOB_DONE


def test_bad_value_limit(ffr):
    text = golden_flame_text("badval")
    with ffr.Server(precision=0, settle=SETTLE) as srv:
        j = srv.submit(text, 200_000, 4, bad_limit=5)
        info = srv.wait(j, 60_000)
        assert info.state == ffr.JOB_DONE and info.status == ffr.FFR_BAD_VALUES
        st = srv.stats(j, 2)
        assert st.bad_values > 5 and len(st.bad_xf) > 0


def test_errors_and_release_rules(ffr, flames):
    with ffr.Server(precision=1, settle=SETTLE) as srv:
        with pytest.raises(ffr.FfrError) as e:
            srv.submit('{"dimensions": 2, "xforms": [}', 10, 1)
        assert e.value.status == ffr.FFR_ERR_PARSE
        text = json.dumps(flames.random_2d(7, size=(64, 64)))
        big = srv.submit(text, 10**11, 1)
        with pytest.raises(ffr.FfrError) as e:
            srv.release(big)
        assert e.value.status == ffr.FFR_ERR_STATE
        srv.cancel(big)
        srv.wait(big, 30_000)
        srv.release(big)
        with pytest.raises(ffr.FfrError) as e:
            srv.poll(big)
        assert e.value.status == ffr.FFR_ERR_ARG
        z = srv.submit(text, 0, 1)
        info = srv.wait(z, 10_000)
        assert info.state == ffr.JOB_DONE
        assert int(srv.read(z, 64 * 64).sum()) == 0


def test_budget_below_staging_is_refused(ffr):
    with pytest.raises(ffr.FfrError) as e:
        ffr.Server(precision=1, hbm_budget=1 << 20)
    assert e.value.status == ffr.FFR_ERR_CUDA


def test_concurrent_and_multi_slice_reads(ffr, flames):
    """Reads from several threads at once (the server has four read slots)
    and reads larger than one 16 MiB staging slice return the exact buffers."""
    import concurrent.futures as cf
    big = json.dumps(flames.random_3d(5, size=(200, 200, 200)))      # 64 MB file: 4 slices
    col = golden_flame_text("color")                                  # colour channels
    small = [json.dumps(flames.random_2d(300 + i, size=(256, 144))) for i in range(6)]
    jobs = [(big, 3_000_000, 1, 200 ** 3, 0), (col, 400_000, 2, 80 * 60, 3)]
    jobs += [(t, 500_000, 10 + i, 256 * 144, 0) for i, t in enumerate(small)]
    with ffr.Server(precision=1, settle=SETTLE) as srv:
        ids = [srv.submit(t, n, seed) for t, n, seed, _, _ in jobs]
        for j in ids:
            assert srv.wait(j, 120_000).state == ffr.JOB_DONE
        with cf.ThreadPoolExecutor(8) as ex:
            got = list(ex.map(lambda a: srv.read(a[0], a[1][3], a[1][4]), zip(ids, jobs)))
    for (t, n, seed, cells, r), g in zip(jobs, got):
        want, _, _ = solo(ffr, t, n, seed, 1)
        np.testing.assert_array_equal(g[:, 0], want[:, 0])
        if r:
            np.testing.assert_allclose(g[:, 1:].copy().view(np.float64),
                                       want[:, 1:].copy().view(np.float64), rtol=1e-12, atol=1e-9)
