"""Hot-cell table placement (csrc/hot_cells.cpp, host-only, no GPU): the
candidates a probe collects become a direct-mapped table whose multiplier
sends every kept cell to its own slot.  A small driver compiled against the
library's source reads candidate lists and prints the table."""
import importlib.util
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

PKG = os.path.join(ROOT, "flame-fractal-renderer_gb300")
SLOTS, SLOT_BITS, CELLS_MAX, EMPTY = 256, 8, 64, 0xFFFFFFFF

DRIVER = r"""
#include "launch.h"
#include <cstdio>
#include <vector>
int main()
{
    unsigned long long sum = 0, n = 0;
    while (std::scanf("%llu %llu", &sum, &n) == 2)
    {
        std::vector<unsigned long long> found(n);
        for (auto& f : found)
        {
            unsigned long long count = 0, cell = 0;
            if (std::scanf("%llu %llu", &count, &cell) != 2)
                return 1;
            f = (count << 32) | cell;
        }
        unsigned int mult = 0;
        std::vector<unsigned int> keys;
        if (!ffr::hot_place(found, sum, &mult, keys))
        {
            std::printf("none\n");
            continue;
        }
        std::printf("%u", mult);
        for (unsigned int k : keys)
            std::printf(" %u", k);
        std::printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def placer(tmp_path_factory):
    spec = importlib.util.spec_from_file_location("ffr_build", os.path.join(PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    d = tmp_path_factory.mktemp("hot")
    src = d / "driver.cpp"
    src.write_text(DRIVER)
    exe = d / "driver"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(PKG, "csrc"),
                           "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(b._cuda_home(), "include"), str(src),
                           os.path.join(PKG, "csrc", "hot_cells.cpp"), "-o", str(exe)])

    def run(cases):
        text = "".join(f"{s} {len(c)}\n" + "".join(f"{n} {k}\n" for n, k in c)
                       for s, c in cases)
        out = subprocess.run([str(exe)], input=text, capture_output=True, text=True,
                             check=True).stdout.splitlines()
        res = []
        for line in out:
            if line == "none":
                res.append(None)
            else:
                v = [int(x) for x in line.split()]
                res.append((v[0], v[1:]))
        return res
    return run


def check_table(mult, keys, want_cells):
    assert mult % 2 == 1 and len(keys) == SLOTS
    kept = [k for k in keys if k != EMPTY]
    assert sorted(kept) == sorted(want_cells)
    for slot, k in enumerate(keys):
        if k != EMPTY:
            assert ((k * mult) & 0xFFFFFFFF) >> (32 - SLOT_BITS) == slot


def test_sixty_four_hot_cells_get_distinct_slots(placer):
    g = np.random.Generator(np.random.PCG64(5))
    cells = g.choice(1 << 21, size=64, replace=False).tolist()
    counts = sorted(g.integers(10_000, 1_000_000, size=64).tolist(), reverse=True)
    (res,) = placer([(sum(counts) * 3, list(zip(counts, cells)))])
    check_table(*res, cells)


def test_only_the_hottest_sixty_four_are_kept(placer):
    g = np.random.Generator(np.random.PCG64(6))
    cells = g.choice(1 << 21, size=100, replace=False).tolist()
    counts = list(range(2_000_000, 2_000_000 - 100 * 1000, -1000))   # distinct, descending
    cand = list(zip(counts, cells))
    g.shuffle(cand)                      # the collect kernel returns them in any order
    (res,) = placer([(sum(counts), cand)])
    check_table(*res, cells[:64])


def test_few_very_hot_cells_get_a_table(placer):
    # a density almost entirely in three cells (a point attractor)
    cand = [(900_000, 1234), (50_000, 777_777), (40_000, 5)]
    (res,) = placer([(1_000_000, cand)])
    check_table(*res, [1234, 777_777, 5])


def test_too_little_mass_gives_no_table(placer):
    cand = [(1000, k) for k in range(64)]         # 64 000 of 10^7 samples: 0.64% < 2%
    assert placer([(10_000_000, cand), (1000, [])]) == [None, None]


def test_placement_is_deterministic(placer):
    g = np.random.Generator(np.random.PCG64(7))
    cells = g.choice(1 << 20, size=40, replace=False).tolist()
    cand = [(100_000 - i, c) for i, c in enumerate(cells)]
    a, b = placer([(4_000_000, cand), (4_000_000, cand)])
    assert a == b
