"""The per-flame kernels (FFR_KERNEL_JIT) on the GPU, through the C ABI.

A per-flame kernel computes what the general kernels compute -- the plain
one with each variation slot's type dispatch narrowed at compile time, the
xform-sorted one with each xform's types fixed -- so for equal streams and
trajectory lengths its buffers and statistics are the general plain
kernel's, bit for bit, in FP64 and FP32: every variation type (the grouped
flames of jit_cases.py), 1 to 4 dimensions, xforms with and without
affines, a final xform.  Colour sums are equal to rounding (CTAs add them
in another order when the two kernels fit different CTA counts per SM).
The oracle-pinned golden renders run through it in test_gpu_parity.py.
"""
import concurrent.futures as cf
import json
import os

import numpy as np
import pytest

import jit_cases
from conftest import golden_flame_text

pytestmark = pytest.mark.gpu

CASES = jit_cases.cases()
CASES["d4_mixed"] = golden_flame_text("d4_mixed")


@pytest.fixture(scope="module")
def prepared(ffr):
    """Compile every case's kernels (plain and xform-sorted) up front, in
    parallel."""
    jobs = [(n, p) for n in sorted(CASES) for p in (ffr.FP64, ffr.FP32)]
    with cf.ThreadPoolExecutor(max(2, min(len(jobs), os.cpu_count() or 2))) as ex:
        res = list(ex.map(lambda j: ffr.jit_prepare(CASES[j[0]], j[1]), jobs))
    assert all(r[0] == ffr.FFR_OK for r in res), [r for r in res if r[0]][:1]
    return True


def render(ffr, text, precision, kernel, n=2_000_000, seed=11, streams=2048, traj=None):
    traj = traj or -(-n // streams)
    with ffr.BufferRenderer(text, precision=precision, settle=20, streams=streams,
                            traj_len=traj, kernel=kernel) as r:
        s = r.render(n, seed, bad_limit=10**12)
        return s, r.buffer_array()


def same_stats(a, b):
    assert a.samples_iterated == b.samples_iterated
    assert a.samples_plotted == b.samples_plotted
    assert a.bad_values == b.bad_values
    assert a.dropped == b.dropped
    np.testing.assert_array_equal(a.xf_dist, b.xf_dist)
    np.testing.assert_array_equal(a.ext_lo, b.ext_lo)
    np.testing.assert_array_equal(a.ext_hi, b.ext_hi)


@pytest.mark.parametrize("kernel", [4, 5], ids=["jit", "jit_sorted"])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_jit_equals_general_kernel(ffr, prepared, name, precision, kernel):
    text = CASES[name]
    if kernel == ffr.KERNEL_JIT_SORTED and json.loads(text)["dimensions"] > 3:
        with pytest.raises(ffr.FfrError) as e:
            render(ffr, text, precision, kernel)
        assert e.value.status == ffr.FFR_ERR_ARG
        return
    sp, bp = render(ffr, text, precision, ffr.KERNEL_PLAIN)
    sj, bj = render(ffr, text, precision, kernel)
    assert sp.kernel == ffr.KERNEL_PLAIN and sj.kernel == kernel
    np.testing.assert_array_equal(bj[:, 0], bp[:, 0])
    same_stats(sj, sp)
    assert sj.samples_iterated == 2_000_000
    if bp.shape[1] > 1:
        np.testing.assert_allclose(bj[:, 1:].copy().view(np.float64),
                                   bp[:, 1:].copy().view(np.float64), rtol=1e-9, atol=1e-6)


def test_jit_merged_fp32_program_runs_merged_kernel(ffr, flames):
    """An FP32 flame of the benchmark types has no per-flame kernel: a JIT
    request runs the precompiled merged instantiation (stats.kernel PLAIN),
    with the plain kernel's buffer."""
    text = json.dumps(flames.random_2d(31, size=(320, 180)))
    sj, bj = render(ffr, text, ffr.FP32, ffr.KERNEL_JIT)
    sp, bp = render(ffr, text, ffr.FP32, ffr.KERNEL_PLAIN)
    assert sj.kernel == ffr.KERNEL_PLAIN
    np.testing.assert_array_equal(bj, bp)


def test_auto_times_a_prepared_kernel(ffr, flames):
    """After ffr_jit_prepare the autotuner times the per-flame kernel too;
    whichever it keeps, the buffer is the general kernel's."""
    fl = flames.random_2d(32, size=(640, 360), variations=["handkerchief", "disc", "heart",
                                                             "spiral", "ex", "julia"])
    text = json.dumps(fl)
    assert ffr.jit_prepare(text, ffr.FP32)[0] == ffr.FFR_OK
    n = 1 << 25
    sa, ba = render(ffr, text, ffr.FP32, ffr.KERNEL_AUTO, n=n, streams=16384)
    sp, bp = render(ffr, text, ffr.FP32, ffr.KERNEL_PLAIN, n=n, streams=16384)
    assert sa.kernel in (ffr.KERNEL_PLAIN, ffr.KERNEL_SORTED, ffr.KERNEL_JIT,
                         ffr.KERNEL_JIT_SORTED)
    assert sa.aux_launches > 0      # the autotuner's probes
    np.testing.assert_array_equal(ba[:, 0], bp[:, 0])


def test_jit_default_plan_matches_plain(ffr, flames):
    """The default plan (no streams given) and a render that keeps the
    context's count bound and stats across calls: JIT and plain agree."""
    fl = flames.random_2d(33, size=(400, 300), variations=["cosine", "disc", "tangent",
                                                             "power", "swirl", "linear"])
    text = json.dumps(fl)
    out = []
    for kernel in (ffr.KERNEL_PLAIN, ffr.KERNEL_JIT):
        with ffr.BufferRenderer(text, precision=ffr.FP32, settle=20, kernel=kernel) as r:
            s1 = r.render(3_000_000, 5, bad_limit=10**12)
            s2 = r.render(3_000_000, 6, bad_limit=10**12)
            out.append((s1.streams, s1.traj_len, s2.samples_plotted, r.counts()))
    assert out[0][:2] == out[1][:2]
    assert out[0][2] == out[1][2]
    np.testing.assert_array_equal(out[0][3], out[1][3])


@pytest.mark.parametrize("auto_seconds", ["0", "-1"], ids=["compiles", "never"])
def test_autotuner_compiles_for_long_renders(ffr, flames, tmp_path, monkeypatch, auto_seconds):
    """A render the autotuner expects to run longer than FFR_JIT_AUTO_SECONDS
    (0 here: every tuned render) gets its per-flame kernels compiled and
    timed (both land in the FFR_JIT_CACHE directory); negative: never.
    Whichever kernel wins, the buffer is the general kernel's."""
    monkeypatch.setenv("FFR_JIT_CACHE", str(tmp_path))
    monkeypatch.setenv("FFR_JIT_AUTO_SECONDS", auto_seconds)
    # a structure no other test compiles (FP64, 5 xforms of other variations)
    fl = flames.random_2d(34 if auto_seconds == "0" else 35, k=5, size=(480, 270),
                          variations=["ex", "diamond", "cylinder", "heart", "power", "cosine"])
    text = json.dumps(fl)
    n = 1 << 25
    sa, ba = render(ffr, text, ffr.FP64, ffr.KERNEL_AUTO, n=n, streams=16384)
    keys = list(tmp_path.glob("ffr_*.key"))
    if auto_seconds == "0":
        assert len(keys) == 2
        assert sa.kernel in (ffr.KERNEL_PLAIN, ffr.KERNEL_SORTED, ffr.KERNEL_JIT,
                             ffr.KERNEL_JIT_SORTED)
    else:
        assert keys == []
        assert sa.kernel in (ffr.KERNEL_PLAIN, ffr.KERNEL_SORTED)
    sp, bp = render(ffr, text, ffr.FP64, ffr.KERNEL_PLAIN, n=n, streams=16384)
    np.testing.assert_array_equal(ba[:, 0], bp[:, 0])
