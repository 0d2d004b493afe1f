"""CPU restatement of the reference's ffr-img pixel mapping -- TEST
INFRASTRUCTURE ONLY (the oracle for ffr_render_image / ffr-img; never on a
product path).

Restates, in numpy double precision:
  render_image                src/ffr_img.cpp:199-309
      histogram bounds         :212-218   (min/max of the u64 counts)
      log scaler bounds        :220-230   (max of log(1 + count); "histogram
                                           is (probably) empty" below eps)
      gamma                    :233       gp = 1 / gamma
      grayscale scaler         :236-242   pow(log(1 + count) / max, gp)
      monochrome               :244-266   count != 0 ? 1.0 : 0.0, 8-bit gray
      colour                   :282-296   ll * (colour_c / count), c = 0..2
  ImageRenderer::renderGrayImage / renderColorImageRGB
                               src/renderers/image_renderer.hpp:139-191
      (pix_t)(value * pix_scale), rows in buffer order
  pix_scale<u8|u16, double> = 2^bits * (1 - 2^-52)
                               src/types/constants.hpp:77-91 with
                               scale_adjust_down_v<double>

The reference converts NaN (an empty cell's 0/0 colour) and values at or
above 2^bits to an integer pixel, which is undefined behaviour in C++; here
(as in the GPU kernel) NaN maps to 0 and values saturate at 2^bits - 1.

Parity: pinned.  The reference's own src/ffr_img.cpp (with ImageRenderer)
is compiled into oracle/_ref/ffr_img_ref by oracle/build_ref.sh, with
project-written Boost.GIL / program_options shims and an unencoded image
writer in place of libpng; tests/golden/make_golden_images.py ran it on
buffers from the reference's buffer path, and tests/test_image.py checks this
restatement against those pixels (identical on every case when generated).
"""
from __future__ import annotations

import numpy as np

MONO, GRAY, RGB = 0, 1, 2


def pix_scale(bits: int) -> float:
    return (256.0 if bits == 8 else 65536.0) * (1.0 - 2.0 ** -52)


def _to_pix(x: np.ndarray, bits: int) -> np.ndarray:
    top = 255.0 if bits == 8 else 65535.0
    x = np.where(np.isnan(x), 0.0, x)
    x = np.clip(x, 0.0, top)
    return np.floor(x).astype(np.uint8 if bits == 8 else np.uint16)


def image(counts: np.ndarray, colors: np.ndarray | None, width: int, height: int,
          mode: int, gamma: float = 1.0, bits: int = 8):
    """(pixels [height, width(, 3)], bounds dict) for a 2-D buffer given as
    u64 counts [cells] and f64 colours [cells, color_dims] (or None)."""
    if gamma < 1e-20:
        raise ValueError("gamma too small")
    if bits not in (8, 16):
        raise ValueError("bits per channel must be 8 or 16")
    counts = np.asarray(counts, dtype=np.uint64)
    h = counts.astype(np.float64)
    hmin, hmax = int(counts.min()), int(counts.max())
    smin, smax = float(np.log(1.0 + float(hmin))), float(np.log(1.0 + float(hmax)))
    bounds = {"hist_min": hmin, "hist_max": hmax, "scale_min": smin, "scale_max": smax}
    if smax < 1e-20:
        raise ValueError("histogram is (probably) empty")
    gp = 1.0 / gamma
    if mode == MONO:
        px = _to_pix(np.where(counts != 0, 1.0, 0.0) * pix_scale(8), 8)
        return px.reshape(height, width), bounds
    with np.errstate(divide="ignore", invalid="ignore"):
        ll = np.power(np.log(1.0 + h) / smax, gp)
        if mode == GRAY:
            return _to_pix(ll * pix_scale(bits), bits).reshape(height, width), bounds
        if colors is None or colors.shape[1] != 3:
            raise ValueError("buffer must use 3 color dimensions")
        rgb = np.stack([(ll * (colors[:, c] / h)) * pix_scale(bits) for c in range(3)], axis=1)
    return _to_pix(rgb, bits).reshape(height, width, 3), bounds


def decode_png(data: bytes) -> np.ndarray:
    """Pixels of a non-interlaced 8/16-bit gray or RGB PNG (test helper)."""
    import struct
    import zlib
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos = 8
    idat = b""
    w = h = bits = ctype = None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF, typ
        if typ == b"IHDR":
            w, h, bits, ctype = struct.unpack(">IIBB", body[:10])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    ch = 3 if ctype == 2 else 1
    raw = zlib.decompress(idat)
    bpp = ch * bits // 8
    rows = np.frombuffer(raw, dtype=np.uint8).reshape(h, 1 + w * bpp)
    assert (rows[:, 0] == 0).all()
    pix = rows[:, 1:]
    if bits == 16:
        pix = pix.reshape(h, w * ch, 2).astype(np.uint16)
        pix = (pix[:, :, 0] << 8) | pix[:, :, 1]
    return pix.reshape(h, w, ch) if ch == 3 else pix.reshape(h, w)
