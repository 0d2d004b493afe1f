"""ffr-img side: the device pixel mapping (ffr_render_image), the host PNG
writer (ffr_encode_png) and the ffr-img command line, checked against the
reference's own ffr-img pixels (tests/golden/data/images.npz, made by
tests/golden/make_golden_images.py from src/ffr_img.cpp compiled into the
oracle) and against the CPU restatement of its render_image
(oracle/image_oracle.py), which is itself checked against those pixels.

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


GOLDEN_IMAGES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
with open(os.path.join(GOLDEN_IMAGES, "images.json")) as _f:
    IMAGES = json.load(_f)


def golden_image_case(name):
    """(flame text, buffer as u64 [cells, 1 + colour dims], mode, gamma,
    bits, reference pixels) of one golden image case."""
    d = np.load(os.path.join(GOLDEN_IMAGES, "data", "images.npz"))
    m = IMAGES["images"][name]
    flame = IMAGES["buffers"][m["buffer"]]["flame"]
    text = golden_flame_text(flame)
    r = json.loads(text).get("color_dimensions", 0)
    buf = d["buf_" + m["buffer"]].reshape(-1, 1 + r)
    opts = m["options"]
    mode = io.RGB if "-c" in opts else (io.MONO if "-m" in opts else io.GRAY)
    gamma = float(opts[opts.index("-y") + 1]) if "-y" in opts else 1.0
    bits = int(opts[opts.index("-b") + 1]) if "-b" in opts else 8
    return text, buf, mode, gamma, bits, d["img_" + name]


@pytest.mark.parametrize("name", sorted(IMAGES["images"]))
def test_image_oracle_matches_reference_pixels(name):
    """The numpy restatement against the reference's own ffr-img output."""
    text, buf, mode, gamma, bits, want = golden_image_case(name)
    w, h = json.loads(text)["size"]
    colors = buf[:, 1:].copy().view(np.float64) if buf.shape[1] > 1 else None
    got, _ = io.image(buf[:, 0], colors, w, h, mode, gamma, bits)
    assert got.shape == want.shape and got.dtype == want.dtype
    _close(got, want)


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
@pytest.mark.parametrize("name", sorted(IMAGES["images"]))
def test_render_image_matches_reference_pixels(ffr, name):
    """The device pixel mapping of a buffer the reference rendered, against
    the pixels the reference's own ffr-img made of it."""
    text, buf, mode, gamma, bits, want = golden_image_case(name)
    with ffr.BufferRenderer(text, precision=0, settle=20) as r:
        r.load_buffer(buf)
        px, info = r.render_image(mode, gamma, bits)
    assert (info.hist_min, info.hist_max) == (int(buf[:, 0].min()), int(buf[:, 0].max()))
    assert px.shape == want.shape and px.dtype == want.dtype
    _close(px, want)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c2small_gray16_g045", "color_rgb8", "c2small_mono"])
def test_ffr_img_cli_matches_reference_pixels(ffr, tmp_path, name):
    """ffr-img on the same buffer file: the PNG decodes to the reference's
    pixels, and the bounds lines match the reference's stderr."""
    text, buf, mode, gamma, bits, want = golden_image_case(name)
    m = IMAGES["images"][name]
    f = tmp_path / "flame.json"
    f.write_text(text)
    b = tmp_path / "in.buf"
    buf.tofile(b)
    png = tmp_path / "out.png"
    r = subprocess.run([ffr.IMG_CLI_PATH, "-f", str(f), "-i", str(b), "-o", str(png),
                        *m["options"]], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for line in m["stderr_bounds"]:
        assert line in r.stderr
    _close(io.decode_png(png.read_bytes()), want)


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
