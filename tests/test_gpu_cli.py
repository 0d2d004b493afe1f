"""The drop-in command line: ffr-buf renders through the C ABI and writes
the reference's buffer file.  For an algebraic flame in FP64 (products, sums
and square roots only, rounded as in the reference) the file is byte-for-byte
the oracle's render of the same streams; -i adds earlier files; the stderr
report carries the reference's lines."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import golden_flame_text

pytestmark = pytest.mark.gpu


def run(ffr, *args):
    return subprocess.run([ffr.CLI_PATH, *map(str, args)], capture_output=True, timeout=600)


@pytest.mark.parametrize("kernel", ["auto", "jit", "jit-sorted"])
@pytest.mark.parametrize("name", ["alg2d", "color"])
def test_ffr_buf_file_equals_oracle(ffr, fo, tmp_path, name, kernel):
    text = golden_flame_text(name)
    f = tmp_path / "flame.json"
    f.write_text(text)
    out = tmp_path / "out.buf"
    S, N, L, seed = 512, 1_000_000, 977, 5
    r = run(ffr, "-f", f, "-o", out, "-s", N, "-b", L, "--streams", S, "--seed", seed,
            "--settle", 53, "--kernel", kernel)
    assert r.returncode == 0, r.stderr.decode()
    err = r.stderr.decode()
    of = fo.OracleFlame(fo.load_flame(text))
    ref = fo.render(of, seed, S, N, L, 53, 256)
    got = out.read_bytes()
    want = ref.file_bytes()
    if json.loads(text).get("color_dimensions", 0):
        # colour sums are added in a different order: counts exact, colours 1e-12
        g = np.frombuffer(got, dtype=np.uint64).reshape(len(ref.counts), -1)
        w = np.frombuffer(want, dtype=np.uint64).reshape(len(ref.counts), -1)
        np.testing.assert_array_equal(g[:, 0], w[:, 0])
        np.testing.assert_allclose(g[:, 1:].copy().view(np.float64),
                                   w[:, 1:].copy().view(np.float64), rtol=1e-12, atol=1e-12)
    else:
        assert got == want
    assert f"samples iterated: {ref.s_iter}" in err
    assert f"samples plotted: {ref.s_plot}" in err
    assert "render done:" in err and "xform selection:" in err


def test_ffr_buf_input_accumulates(ffr, fo, tmp_path):
    text = golden_flame_text("alg2d")
    f = tmp_path / "flame.json"
    f.write_text(text)
    a, b = tmp_path / "a.buf", tmp_path / "b.buf"
    assert run(ffr, "-f", f, "-o", a, "-s", 300_000, "-b", 1000, "--streams", 300, "--seed", 1,
               "--settle", 53).returncode == 0
    r = run(ffr, "-f", f, "-i", a, "-i", a, "-o", b, "-s", 200_000, "-b", 1000, "--streams", 200,
            "--seed", 2, "--settle", 53)
    assert r.returncode == 0, r.stderr.decode()
    of = fo.OracleFlame(fo.load_flame(text))
    first = fo.render(of, 1, 300, 300_000, 1000, 53, 256).counts
    second = fo.render(of, 2, 200, 200_000, 1000, 53, 256).counts
    got = np.frombuffer(b.read_bytes(), dtype=np.uint64)
    np.testing.assert_array_equal(got, 2 * first + second)
    # a short input file is the reference's "error reading file"
    short = tmp_path / "short.buf"
    short.write_bytes(a.read_bytes()[:-8])
    r = run(ffr, "-f", f, "-i", short, "-o", b, "-s", 10)
    assert r.returncode == 1 and b"error reading file" in r.stderr


def test_trajectories_option(ffr, fo, tmp_path):
    """--trajectories T: T streams of one trajectory of ceil(N/T) samples (the
    "N samples from T trajectories" of the Sierpinski configuration)."""
    text = golden_flame_text("alg2d")
    f = tmp_path / "flame.json"
    f.write_text(text)
    out = tmp_path / "out.buf"
    N, T = 500_000, 5_000
    r = run(ffr, "-f", f, "-o", out, "-s", N, "--trajectories", T, "--seed", 9, "--settle", 20)
    assert r.returncode == 0, r.stderr.decode()
    of = fo.OracleFlame(fo.load_flame(text))
    ref = fo.render(of, 9, T, N, N // T, 20, 256)
    assert out.read_bytes() == ref.file_bytes()
    r = run(ffr, "-f", f, "-o", out, "-s", N, "--trajectories", T, "-b", 10)
    assert r.returncode == 1 and b"excludes" in r.stderr
