"""Windows of the batch claim order (interleave_chunks with buffer sizes,
launch.h; host-only, no GPU), compiled with the host compiler: every (job,
chunk) pair exactly once, chunks of a job in order, and windows of
consecutive jobs -- at least kMinWindowJobs jobs and min_chunks chunks, more
while the buffers fit kWindowBytes -- one after another."""
import json
import os
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "flame-fractal-renderer_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "launch.h"
using namespace ffr;
int main()
{
    // jobs: chunk counts and buffer bytes (MB)
    unsigned long long chunks_in[] = {@CHUNKS@};
    unsigned long long mb_in[] = {@MBS@};
    const size_t n = sizeof chunks_in / sizeof chunks_in[0];
    std::vector<unsigned long long> chunks(chunks_in, chunks_in + n), bytes(n);
    for (size_t k = 0; k < n; ++k)
        bytes[k] = mb_in[k] << 20;
    std::vector<unsigned long long> order;
    interleave_chunks(chunks, order, @WITH_BYTES@ ? &bytes : nullptr, @MIN_CHUNKS@);
    std::printf("{\"min_jobs\": %zu, \"window_mb\": %llu, \"order\": [", kMinWindowJobs,
                kWindowBytes >> 20);
    for (size_t i = 0; i < order.size(); ++i)
        std::printf("%s[%llu, %llu]", i ? ", " : "", order[i] >> 32, order[i] & 0xffffffffull);
    std::printf("]}\n");
    return 0;
}
"""


def cuda_include():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "include", "cuda_runtime.h")):
            return os.path.join(c, "include")
    pytest.skip("CUDA headers not found")


def run_order(tmp_path, chunks, mbs, with_bytes, min_chunks=0):
    src = (DRIVER.replace("@CHUNKS@", ", ".join(map(str, chunks)))
           .replace("@MBS@", ", ".join(map(str, mbs)))
           .replace("@WITH_BYTES@", "1" if with_bytes else "0")
           .replace("@MIN_CHUNKS@", str(min_chunks)))
    c = tmp_path / "order.cpp"
    c.write_text(src)
    exe = tmp_path / "order"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", CSRC, "-I", cuda_include(),
                           str(c), "-o", str(exe)])
    return json.loads(subprocess.check_output([str(exe)], text=True))


def check_permutation(order, chunks):
    seen = {}
    for job, r in order:
        assert r == seen.get(job, 0), "chunks of a job in order"
        seen[job] = r + 1
    assert seen == {k: c for k, c in enumerate(chunks) if c}


def test_interleaved_without_sizes(tmp_path):
    chunks = [4, 1, 8, 0, 2]
    out = run_order(tmp_path, chunks, [1] * len(chunks), False)
    order = out["order"]
    check_permutation(order, chunks)
    # relative pace: the key (r + 1/2) / chunks never decreases along the order
    keys = [(r + 0.5) / chunks[j] for j, r in order]
    assert keys == sorted(keys)


def test_windows_of_jobs_by_buffer_size(tmp_path):
    # 40 jobs of 10 MB and 5 chunks each: windows of 16 jobs (160 MB > 64 MB,
    # so the minimum count decides), i.e. jobs 0-15, 16-31, 32-39
    chunks, mbs = [5] * 40, [10] * 40
    out = run_order(tmp_path, chunks, mbs, True)
    order = out["order"]
    check_permutation(order, chunks)
    assert out["min_jobs"] == 16 and out["window_mb"] == 64
    windows = [j // 16 for j, _ in order]
    assert windows == sorted(windows), "one window after another"
    # small buffers: more jobs per window while they fit 64 MB (1 MB each)
    out = run_order(tmp_path, [3] * 100, [1] * 100, True)
    first = [j for j, _ in out["order"][:64 * 3]]
    assert max(first) == 63 and min(first) == 0


def test_windows_hold_min_chunks(tmp_path):
    # 40 jobs of one chunk: with min_chunks 30 a window spans 30 jobs
    out = run_order(tmp_path, [1] * 40, [10] * 40, True, min_chunks=30)
    order = out["order"]
    check_permutation(order, [1] * 40)
    assert [j for j, _ in order[:30]] == list(range(30))
    assert sorted(j for j, _ in order[30:]) == list(range(30, 40))
