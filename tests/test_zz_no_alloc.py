"""ffr_render_noalloc: the render entry point for callers that cannot let a
library call cudaMalloc -- their device memory comes from another allocator
(here torch's caching allocator stands in for it) and they pass in a count
buffer they already own.

Checked through the C ABI against the ordinary entry point (ffr_create +
ffr_render + ffr_read_buffer) on two calls in a row into the same caller
buffer: the second call must start from cleared statistics and add to the
counts the first one left.  The flames are FP64 and built from + - * /
only, so the tolerance our parity tests use for them is exact equality
(colour sums: 1e-12 relative, their addition order differs).

This file is collected last on purpose; it passes alone in a fresh process
and after every other test.
"""
import ctypes
import json

import numpy as np
import pytest

from conftest import golden_flame_text

pytestmark = pytest.mark.gpu


def _noalloc(ffr, text, counts_ptr, colors_ptr, cells, samples, seed, opts):
    lib = ffr.load_library()
    st = ffr.Stats()
    raw = text.encode()
    rc = lib.ffr_render_noalloc(raw, len(raw), ctypes.byref(opts), counts_ptr, colors_ptr,
                                cells, samples, seed, 256, ctypes.byref(st))
    assert rc == ffr.FFR_OK, lib.ffr_last_error(None).decode()
    return st


def _opts(ffr, settle, streams, traj_len):
    o = ffr.Opts()
    ffr.load_library().ffr_default_opts(ctypes.byref(o))
    o.precision, o.settle, o.streams, o.traj_len = ffr.FP64, settle, streams, traj_len
    return o


def test_noalloc_matches_ffr_render_two_calls(ffr, flames):
    torch = pytest.importorskip("torch")
    text = json.dumps(flames.sierpinski_2d(size=(256, 256)))
    settle, streams, traj_len, n = 20, 2048, 700, 3_000_000
    cells = 256 * 256
    buf = torch.zeros(cells, dtype=torch.int32, device="cuda:0")     # caller-owned
    torch.cuda.synchronize()
    o = _opts(ffr, settle, streams, traj_len)
    plotted = 0
    with ffr.BufferRenderer(text, precision=ffr.FP64, settle=settle, streams=streams,
                            traj_len=traj_len) as r:
        for seed in (11, 12):
            st = _noalloc(ffr, text, ctypes.c_void_p(buf.data_ptr()), None, cells, n, seed, o)
            ref = r.render(n, seed)              # accumulates like the caller's buffer
            got = buf.cpu().numpy().view(np.uint32).astype(np.uint64)
            np.testing.assert_array_equal(got, r.counts())
            assert st.samples_iterated == ref.samples_iterated == n
            assert st.samples_plotted == ref.samples_plotted
            assert [st.xf_dist[i] for i in range(3)] == ref.xf_dist.tolist()
            assert [st.ext_lo[i] for i in range(2)] == ref.ext_lo.tolist()
            assert [st.ext_hi[i] for i in range(2)] == ref.ext_hi.tolist()
            assert st.kernel == 1                # FFR_KERNEL_PLAIN
            # the caller's buffer holds every sample both calls binned
            plotted += st.samples_plotted
            assert int(got.sum()) == plotted


def test_noalloc_allocates_no_device_memory(ffr, flames):
    """The defining property: after a first call (which looks up the scratch
    array and loads the kernel), further calls leave the device's free memory
    exactly where it was."""
    torch = pytest.importorskip("torch")
    text = json.dumps(flames.sierpinski_2d(size=(128, 128)))
    buf = torch.zeros(128 * 128, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    o = _opts(ffr, 20, 1024, 500)
    ptr = ctypes.c_void_p(buf.data_ptr())
    _noalloc(ffr, text, ptr, None, 128 * 128, 500_000, 1, o)
    free0, _ = torch.cuda.mem_get_info(0)
    for seed in (2, 3, 4):
        _noalloc(ffr, text, ptr, None, 128 * 128, 500_000, seed, o)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0


def _expanding(dims, size):
    """Every xform triples the point: trajectories leave 1e20 within 45
    steps, so a render records many bad values."""
    eye = [[3.0 if i == j else 0.0 for j in range(dims)] for i in range(dims)]
    return json.dumps({"dimensions": dims, "size": [size] * dims,
                       "bounds": [[-1.0, 1.0]] * dims,
                       "xforms": [{"weight": 1.0, "variations": [{"name": "linear", "weight": 1.0}],
                                   "pre_affine": {"A": eye, "b": [0.1] * dims}}]})


def test_noalloc_bad_value_records_only_the_flames_dims(ffr):
    """Bad-value records of a 2-D call after a 3-D one: the scratch array keeps
    the 3-D call's coordinates, the 2-D call reports only its own two."""
    torch = pytest.importorskip("torch")
    lib = ffr.load_library()
    o = _opts(ffr, 20, 256, 400)
    for dims, size in ((3, 16), (2, 64)):
        text = _expanding(dims, size)
        cells = size ** dims
        buf = torch.zeros(cells, dtype=torch.int32, device="cuda:0")
        torch.cuda.synchronize()
        st = ffr.Stats()
        raw = text.encode()
        rc = lib.ffr_render_noalloc(raw, len(raw), ctypes.byref(o),
                                    ctypes.c_void_p(buf.data_ptr()), None, cells, 100_000, 7,
                                    10**9, ctypes.byref(st))
        assert rc == ffr.FFR_OK, lib.ffr_last_error(None).decode()
        n = st.bad_recorded
        assert n > 100 and st.bad_values >= n
        pts = np.array([[st.bad_pts[k][i] for i in range(3)] for k in range(n)])
        big = ~(np.abs(pts[:, :dims]) <= 1e20)       # beyond the threshold, or NaN
        assert big.any(axis=1).all()
        if dims == 2:
            assert (pts[:, 2] == 0.0).all()


def test_noalloc_rejects_options_it_cannot_honour(ffr, flames):
    torch = pytest.importorskip("torch")
    lib = ffr.load_library()
    raw = json.dumps(flames.sierpinski_2d(size=(8, 8))).encode()
    owned = torch.zeros(64, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    ptr = ctypes.c_void_p(owned.data_ptr())
    for field, value in (("kernel", 2), ("kernel", 3), ("timeout_ms", 100)):
        o = _opts(ffr, 20, 0, 0)
        setattr(o, field, value)
        rc = lib.ffr_render_noalloc(raw, len(raw), ctypes.byref(o), ptr, None, 64, 1000, 1,
                                    256, None)
        assert rc == ffr.FFR_ERR_ARG, field
    # host memory is not the device's: refused before any launch
    host = np.zeros(64, dtype=np.uint32)
    rc = lib.ffr_render_noalloc(raw, len(raw), ctypes.byref(_opts(ffr, 20, 0, 0)),
                                host.ctypes.data_as(ctypes.c_void_p), None, 64, 1000, 1, 256,
                                None)
    assert rc == ffr.FFR_ERR_ARG and b"device memory" in lib.ffr_last_error(None)
    assert (host == 0).all()


def test_noalloc_colour_flame(ffr):
    torch = pytest.importorskip("torch")
    text = golden_flame_text("color")
    settle, streams, traj_len, n = 20, 512, 400, 400_000
    with ffr.BufferRenderer(text, precision=ffr.FP64, settle=settle, streams=streams,
                            traj_len=traj_len) as r:
        cells, r3 = r.cells, r.color_dims
        r.render(n, 5)
        want = r.buffer_array()
    counts = torch.zeros(cells, dtype=torch.int32, device="cuda:0")
    colors = torch.zeros(cells * r3, dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    _noalloc(ffr, text, ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(colors.data_ptr()),
             cells, n, 5, _opts(ffr, settle, streams, traj_len))
    np.testing.assert_array_equal(counts.cpu().numpy().view(np.uint32), want[:, 0])
    np.testing.assert_allclose(colors.cpu().numpy().reshape(cells, r3),
                               want[:, 1:].copy().view(np.float64), rtol=1e-12, atol=1e-9)


def test_noalloc_rejects_oversized_program_and_bad_sizes(ffr, flames):
    torch = pytest.importorskip("torch")
    lib = ffr.load_library()
    big = flames.random_2d(1, k=40, size=(32, 32))       # 21 KB program: fine for ffr_create
    raw = json.dumps(big).encode()
    o = _opts(ffr, 20, 0, 0)
    owned = torch.zeros(32 * 32, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    fake = ctypes.c_void_p(owned.data_ptr())     # every call below is rejected on the host
    rc = lib.ffr_render_noalloc(raw, len(raw), ctypes.byref(o), fake, None, 32 * 32, 1000, 1,
                                256, None)
    assert rc == ffr.FFR_ERR_ARG
    assert b"16384" in lib.ffr_last_error(None)
    small = json.dumps(flames.sierpinski_2d(size=(8, 8))).encode()
    rc = lib.ffr_render_noalloc(small, len(small), ctypes.byref(o), fake, None, 65, 1000, 1,
                                256, None)
    assert rc == ffr.FFR_ERR_ARG and b"cells" in lib.ffr_last_error(None)
    rc = lib.ffr_render_noalloc(small, len(small), ctypes.byref(o), fake, None, 64, 1 << 32, 1,
                                256, None)
    assert rc == ffr.FFR_ERR_ARG
