"""ffr-img side: the device pixel mapping (ffr_render_image), the host PNG
writer (ffr_encode_png) and the ffr-img command line, checked against the
CPU restatement of the reference's render_image (oracle/image_oracle.py).

The pixel mapping runs log and pow in double on the GPU; the oracle uses
numpy's.  They can differ by an ulp, which moves a pixel by one level only
when the scaled value sits on an integer boundary, so the bar is: no pixel
differs by more than 1 and at most 1e-4 of the pixels differ at all."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import golden_flame_text

import image_oracle as io


def test_png_round_trip_gray_and_rgb(ffr):
    g = np.random.Generator(np.random.PCG64(5))
    cases = [
        g.integers(0, 256, size=(7, 13), dtype=np.uint8),
        g.integers(0, 65536, size=(9, 4), dtype=np.uint16),
        g.integers(0, 256, size=(5, 6, 3), dtype=np.uint8),
        g.integers(0, 65536, size=(3, 2, 3), dtype=np.uint16),
        # (254 + 1) * 257 = 65535 raw bytes: exactly one full stored block
        g.integers(0, 256, size=(257, 254), dtype=np.uint8),
        # several stored blocks
        g.integers(0, 65536, size=(300, 200, 3), dtype=np.uint16),
    ]
    for px in cases:
        data = ffr.encode_png(px)
        np.testing.assert_array_equal(io.decode_png(data), px)


def test_png_rejects_bad_geometry(ffr):
    import ctypes
    lib = ffr.load_library()
    n = ctypes.c_size_t()
    px = np.zeros(4, dtype=np.uint8)
    assert lib.ffr_encode_png(px.ctypes.data, 2, 2, 2, 8, None, 0, ctypes.byref(n)) \
        == ffr.FFR_ERR_ARG
    assert lib.ffr_encode_png(px.ctypes.data, 2, 2, 1, 12, None, 0, ctypes.byref(n)) \
        == ffr.FFR_ERR_ARG
    assert lib.ffr_encode_png(px.ctypes.data, 2, 2, 1, 8, None, 0, ctypes.byref(n)) \
        == ffr.FFR_ERR_IO and n.value > 0


@pytest.mark.parametrize("args,msg", [
    (["-y", "0"], "gamma too small"),
    (["-b", "12"], "bits per channel must be 8 or 16"),
])
def test_cli_argument_errors(ffr, tmp_path, args, msg):
    f = tmp_path / "f.json"
    f.write_text(golden_flame_text("alg2d"))
    r = subprocess.run([ffr.IMG_CLI_PATH, "-f", str(f), "-o", str(tmp_path / "o.png"), "-g",
                        "-i", "x"] + args, capture_output=True, text=True)
    assert r.returncode == 1 and msg in r.stderr


def _close(got, want):
    d = np.abs(got.astype(np.int64) - want.astype(np.int64))
    assert d.max() <= 1, d.max()
    assert np.count_nonzero(d) <= max(1, int(1e-4 * d.size)), np.count_nonzero(d)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,bits,gamma", [(0, 8, 1.0), (1, 8, 1.0), (1, 16, 2.2),
                                              (1, 8, 0.45), (2, 8, 1.0), (2, 16, 2.0)])
def test_render_image_matches_oracle(ffr, flames, mode, bits, gamma):
    text = golden_flame_text("color") if mode == 2 else json.dumps(
        flames.random_2d(7, size=(320, 180)))
    with ffr.BufferRenderer(text, precision=1, settle=20) as r:
        r.render(3_000_000, 11, bad_limit=10**9)
        buf = r.buffer_array()
        px, info = r.render_image(mode, gamma, bits)
        w, h = r.size
    colors = buf[:, 1:].copy().view(np.float64) if buf.shape[1] > 1 else None
    want, b = io.image(buf[:, 0], colors, w, h, mode, gamma, bits)
    assert (info.hist_min, info.hist_max) == (b["hist_min"], b["hist_max"])
    assert info.scale_max == pytest.approx(b["scale_max"], rel=1e-15)
    assert px.shape == want.shape and px.dtype == want.dtype
    _close(px, want)


@pytest.mark.gpu
def test_render_image_errors(ffr, flames):
    with ffr.BufferRenderer(json.dumps(flames.random_2d(7, size=(64, 36))), settle=20) as r:
        with pytest.raises(ffr.FfrError) as e:
            r.render_image(1)
        assert e.value.status == ffr.FFR_ERR_STATE and "empty" in e.value.message
        r.render(10_000, 1)
        with pytest.raises(ffr.FfrError) as e:
            r.render_image(2)
        assert "3 color dimensions" in e.value.message
    with ffr.BufferRenderer(json.dumps(flames.tetrahedron_3d((8, 8, 8))), settle=20) as r:
        with pytest.raises(ffr.FfrError) as e:
            r.render_image(1)
        assert "only 2D" in e.value.message


@pytest.mark.gpu
def test_ffr_buf_to_ffr_img_pipeline(ffr, tmp_path):
    """ffr-buf writes a buffer file, ffr-img turns it (twice, like two -i
    inputs) into a PNG whose pixels are the oracle's mapping of the summed
    buffer."""
    f = tmp_path / "flame.json"
    f.write_text(golden_flame_text("color"))
    b = tmp_path / "out.buf"
    subprocess.run([ffr.CLI_PATH, "-f", str(f), "-o", str(b), "-s", "2000000", "--seed", "3",
                    "--settle", "20"], check=True, capture_output=True)
    png = tmp_path / "out.png"
    r = subprocess.run([ffr.IMG_CLI_PATH, "-f", str(f), "-i", str(b), "-i", str(b), "-o",
                        str(png), "-c", "-b", "16", "-y", "1.5"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "histogram bounds:" in r.stderr and "scaler bounds:" in r.stderr
    raw = np.fromfile(b, dtype=np.uint64).reshape(-1, 4)
    counts = raw[:, 0] * 2
    colors = raw[:, 1:].copy().view(np.float64) * 2
    fl = json.loads(golden_flame_text("color"))
    want, _ = io.image(counts, colors, fl["size"][0], fl["size"][1], io.RGB, 1.5, 16)
    _close(io.decode_png(png.read_bytes()), want)
