"""The identities behind the FP64 kernels' integer-pipe rewrites, checked on
IEEE doubles (numpy on the host) over special values: signed zeros,
subnormals, infinities, NaN, the bad-value threshold.  The FP64 kernels
compute the right-hand sides from bit patterns instead of the reference's
arithmetic on the left, so these equalities are what keeps their buffers
bit-identical to the reference's (the GPU golden tests check the buffers).

  0 + y                                   = y, except -0 -> +0
  Affine::apply_to of the 2-D identity    = x_i with -0 -> +0, or NaN when
    (0 + ((0 + 1 x_i) + 0 x_j))             x_i is NaN or x_j is not finite
  a < b, a == b (non-NaN)                 = the same on ord_key(a), ord_key(b)
  lo <= x <= hi (x may be NaN)            = ord_key(lo) <= ord_key(x) <= ord_key(hi)
  !(|x| <= 1e20)                          = (bits(x) & ~sign) > bits(1e20)
"""
import itertools
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

VALUES = np.array([0.0, -0.0, 1.5, -2.25, 1e-310, -1e-310, 5e-324, -5e-324, 1e20, -1e20,
                   1e20 * (1 + 2 ** -52), -1e20 * (1 + 2 ** -52), 3e300, -3e300, np.inf,
                   -np.inf, np.nan, -np.nan, 0.5, -0.5], dtype=np.float64)


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.uint64)


def same(a, b):
    """Bit-identical, or both NaN (NaN payloads are not part of the claim)."""
    a, b = np.float64(a), np.float64(b)
    if np.isnan(a) or np.isnan(b):
        return bool(np.isnan(a) and np.isnan(b))
    return int(bits(a)) == int(bits(b))


def zero_plus(y):
    return np.float64(0.0) if int(bits(y)) == 0x8000000000000000 else np.float64(y)


def test_zero_plus():
    with np.errstate(all="ignore"):
        for y in VALUES:
            assert same(np.float64(0.0) + y, zero_plus(y)), y


def test_identity_affine_two_dims():
    one, zero = np.float64(1.0), np.float64(0.0)
    with np.errstate(all="ignore"):
        for x0, x1 in itertools.product(VALUES, VALUES):
            # Affine::apply_to with A = I, b = 0: ret[i] = b[i] + (0 + A[i][0] x0 + A[i][1] x1)
            ref0 = zero + ((zero + one * x0) + zero * x1)
            ref1 = zero + ((zero + zero * x0) + one * x1)
            rule0 = np.nan if np.isnan(x0) or not np.isfinite(x1) else zero_plus(x0)
            rule1 = np.nan if np.isnan(x1) or not np.isfinite(x0) else zero_plus(x1)
            assert same(ref0, rule0), (x0, x1)
            assert same(ref1, rule1), (x0, x1)


def test_identity_affine_one_dim():
    one, zero = np.float64(1.0), np.float64(0.0)
    with np.errstate(all="ignore"):
        for x in VALUES:
            assert same(zero + (zero + one * x), zero_plus(x)), x


def test_bad_value_bit_test():
    thr = int(bits(np.float64(1e20)))
    for x in VALUES:
        ref = not (abs(x) <= 1e20)
        assert ref == ((int(bits(x)) & 0x7FFFFFFFFFFFFFFF) > thr), x


DRIVER = r"""
#include <cstdio>
#include <cstring>
#include "launch.h"
int main()
{
    double v;
    while (std::scanf("%la", &v) == 1)
        std::printf("%llu\n", ffr::ord_key(v));
    return 0;
}
"""


def test_ord_key_order_and_bounds(tmp_path):
    """launch.h's ord_key (the host/device function the FP64 kernels and the
    bound keys use), compiled with the host compiler."""
    cuda = next((c for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda")
                 if c and os.path.exists(os.path.join(c, "include", "cuda_runtime.h"))), None)
    if cuda is None:
        pytest.skip("CUDA headers not found")
    src = tmp_path / "ord.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "ord"
    subprocess.check_call(["g++", "-std=c++17", "-O1",
                           "-I", os.path.join(ROOT, "flame-fractal-renderer_gb300", "csrc"),
                           "-I", os.path.join(cuda, "include"), str(src), "-o", str(exe)])
    text = "\n".join(float(v).hex() if not np.isnan(v) else ("nan" if not np.signbit(v) else "-nan")
                     for v in VALUES) + "\n"
    out = subprocess.run([str(exe)], input=text, capture_output=True, text=True, check=True)
    keys = [int(k) for k in out.stdout.split()]
    assert len(keys) == len(VALUES)
    key = dict(zip(range(len(VALUES)), keys))
    for i, j in itertools.product(range(len(VALUES)), repeat=2):
        a, b = VALUES[i], VALUES[j]
        if np.isnan(a) or np.isnan(b):
            continue
        assert (a < b) == (key[i] < key[j]), (a, b)
        assert (a == b) == (key[i] == key[j]), (a, b)
    # bounds with finite lo <= hi, any x (NaN: outside)
    finite = [k for k in range(len(VALUES)) if np.isfinite(VALUES[k])]
    for lo, hi in itertools.product(finite, finite):
        if not VALUES[lo] <= VALUES[hi]:
            continue
        for x in range(len(VALUES)):
            ref = bool(VALUES[lo] <= VALUES[x] <= VALUES[hi])
            assert ref == (key[lo] <= key[x] <= key[hi]), (VALUES[lo], VALUES[x], VALUES[hi])
