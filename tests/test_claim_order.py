"""Claim order of the persistent batch kernel (interleave_chunks, launch.h;
host-only, no GPU): chunk r of job k sits at key (r + 1/2) / chunks_k, so
every job advances at the same relative pace.  A small driver compiled
against the header prints the order for given chunk counts."""
import importlib.util
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

PKG = os.path.join(ROOT, "flame-fractal-renderer_gb300")

DRIVER = r"""
#include "launch.h"
#include <cstdio>
#include <vector>
int main()
{
    unsigned long long n = 0;
    while (std::scanf("%llu", &n) == 1)
    {
        std::vector<unsigned long long> chunks(n), order;
        for (auto& c : chunks)
            if (std::scanf("%llu", &c) != 1)
                return 1;
        ffr::interleave_chunks(chunks, order);
        std::printf("%zu", order.size());
        for (unsigned long long e : order)
            std::printf(" %llu", e);
        std::printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def order_of(tmp_path_factory):
    spec = importlib.util.spec_from_file_location("ffr_build", os.path.join(PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    d = tmp_path_factory.mktemp("order")
    src = d / "driver.cpp"
    src.write_text(DRIVER)
    exe = d / "driver"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(PKG, "csrc"),
                           "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(b._cuda_home(), "include"), str(src),
                           "-o", str(exe)])

    def run(chunks):
        text = f"{len(chunks)} " + " ".join(str(c) for c in chunks) + "\n"
        out = subprocess.run([str(exe)], input=text, capture_output=True, text=True,
                             check=True).stdout.split()
        n = int(out[0])
        return [(int(e) >> 32, int(e) & 0xFFFFFFFF) for e in out[1:1 + n]]
    return run


@pytest.mark.parametrize("chunks", [[1], [5, 0, 3], [7, 7, 7], [1, 1000, 13, 0, 250],
                                    list(range(1, 40))])
def test_every_chunk_once_in_job_order(order_of, chunks):
    order = order_of(chunks)
    assert sorted(order) == sorted((k, r) for k, c in enumerate(chunks) for r in range(c))
    last = {}
    for k, r in order:
        assert r == last.get(k, -1) + 1        # a job's chunks in ascending order
        last[k] = r


def test_jobs_advance_at_the_same_relative_pace(order_of):
    g = np.random.Generator(np.random.PCG64(3))
    chunks = g.integers(1, 500, size=64).tolist()
    order = order_of(chunks)
    keys = [(r + 0.5) / chunks[k] for k, r in order]
    assert all(a <= b for a, b in zip(keys, keys[1:]))
    # halfway through the order every job is about halfway through its chunks
    half = order[:len(order) // 2]
    done = np.bincount([k for k, _ in half], minlength=len(chunks))
    assert np.all(np.abs(done / np.array(chunks) - 0.5) <= 1.0 / np.array(chunks) + 1e-9)


def test_no_chunks_no_order(order_of):
    assert order_of([0, 0]) == []
