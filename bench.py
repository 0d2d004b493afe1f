#!/usr/bin/env python3
"""Benchmark of the chaos-game buffer generator on one GB300 (or N replicas).

Workload: the random 2-D flame of the 1920x1080 configuration -- 6 xforms,
weights Dirichlet(1), pre-affine U[-1,1], post-affine I + N(0, 0.1), two
variations per xform from {linear, sinusoidal, spherical, swirl, horseshoe,
polar, julia}, bounds [-2,2] x [-1.125,1.125], 20 settle iterations, seed 7
(flames.random_2d(7)).  A step renders --samples-per-step post-settle samples
(default 10^9) into the device-resident u32 count buffer; the default
10 steps make the 10^10-sample job.

metric  binned (in-bounds) samples per second, whole job
value   device time of the render kernel (CUDA events on the library's
        stream), count buffer already resident; L2 flushed between steps by
        writing a 256 MiB buffer (the buffer itself, 8.3 MB, fits in L2)
e2e     the same metric through the C ABI with host buffers: every step
        creates the context from the JSON text (parse + program upload),
        renders, reads the buffer back into pinned host memory (allocated
        once, before timing) and destroys the context
roofline  bound "l2_atomic": binned samples per launch (one 4-byte atomic
        add each) over the launch's event time, against the rate of 4-byte
        atomic adds at uniformly random cells of a buffer of the same size
        measured in the same run; roofline_hbm: the same adds as 8 B of
        read-modify-write against the measured HBM copy bandwidth
cpu_baseline  the oracle's C restatement of the reference path (FP64,
        all host threads) on a bounded sample of the same workload, with
        its measured speed against the reference's own render()
        (port_vs_reference, oracle/port_vs_reference.py)
batch256  the 256-flame batch in one persistent graph launch (2 timed
        steps, per-flame TV of 8 flames against FP64)
serving  the Poisson request stream three times, each with p50/p99 latency
        and its own clock record: the configured 200 req/s, the same stream
        at 400 req/s (saturated: its served samples/s is the capacity), and
        0.7x that capacity; latency_ms at the top level is the configured
        stream's, with the sustainable one's beside it
per_flame_kernels  the kernels compiled per flame at run time (NVRTC, plain
        and xform-sorted) against the general plain and xform-sorted
        kernels, same streams, identical buffers: a random 2-D flame of
        twelve other variations in FP32 and FP64, the benchmark flame in the
        FP64 mirror (3 steps each, with compile time)

tv      FP32 against FP64 at a fixed sample count: total-variation distance
        between the FP32 histogram and an FP64 (reference arithmetic) one,
        beside the FP64 seed-to-seed noise floor at the same count

--impl reference times that CPU implementation alone, as the reference arm.
--kernel auto|plain|sorted|hot|jit picks the render kernel (default: the
library's autotuner; hot = the plain kernel with the flame's hottest cells
counted in shared memory; jit = the kernel compiled for the flame at run
time) for the default, sierpinski and tetra3d workloads.

Other configurations (--workload; each prints its own JSON line):
  sierpinski  2-D Sierpinski triangle, 1024x1024, 1e8 samples from 1e6
              trajectories of 100, settle 20, seed 1, FP64 (the plain method)
              and FP32; --verify compares the FP64 buffer with the oracle
  tetra3d     Sierpinski tetrahedron, 512^3 u32 buffer (512 MiB), 1e10
              samples in steps of 1e9, FP32, seed 3
  batch256    256 random 2-D flames (2..8 xforms, square buffers of side
              256..2048, 1e7..1e9 samples each, seed 11) in one persistent
              graph-captured launch per step, FP32
  serving     Poisson request stream (200 req/s for 60 s, seed 23) through
              the serving loop: p50/p99 latency and samples/s
  perflame    the per_flame_kernels record alone (--steps renders per kernel)
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "flame-fractal-renderer_gb300"))

import __graft_entry__ as ge  # noqa: E402

METRIC = "binned samples/s"
# the oracle port against the reference's own BufferRenderer::render() on the
# same flame and host (oracle/port_vs_reference.py, FP64, settle 53, the
# reference's automatic batch size; x86-64, 8 cores): the reference sources,
# and so oracle/_ref, exist only where the reference was checked out
PORT_VS_REFERENCE = {"threads_8": 3.47, "threads_4": 2.54, "threads_1": 1.07,
                     "host": "x86-64, 8 cores", "script": "oracle/port_vs_reference.py"}
WORKLOAD = "random 2-D flame, 6 xforms x 2 variations, 1920x1080, 1e10 samples"
# ffr_stats.kernel -> name
KERNEL_NAMES = {1: "plain", 2: "xform-sorted", 4: "per-flame", 5: "per-flame xform-sorted"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def rank_seed(base: int, rank: int) -> int:
    """Seed of one rank's shard: ranks render disjoint ISAAC streams."""
    return base + 1_000_003 * rank


def rank_totals(kern_ms: float, binned: float, wall: float, dist=None, device="cpu"):
    """(max device ms, total binned samples, max wall s) over the job's ranks:
    the whole-job time is the slowest rank's, the work is every rank's."""
    if dist is None:
        return kern_ms, float(binned), wall
    import torch
    t = torch.tensor([kern_ms, float(binned), wall], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return mx[0].item(), sm[1].item(), mx[2].item()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0}, "fallback"


def profile_traffic():
    """Per-launch DRAM traffic (read + write) of the render kernel from the
    committed ncu summary (profiles/chaos_fp32_random2d.md).  The buffer is
    L2-resident, so the traffic is the one fill of the buffer after the L2
    flush and does not depend on the launch's sample count; None when no
    summary exists."""
    p = os.path.join(ROOT, "profiles", "chaos_fp32_random2d.md")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def cpu_port_rate(flame: dict, settle: int, seconds: float, threads: int):
    """Oracle C restatement, FP64, `threads` host threads, about `seconds`."""
    fo = ge._load("flame_oracle", os.path.join(ROOT, "oracle", "flame_oracle.py"))
    of = fo.OracleFlame(fo.load_flame(json.dumps(flame)))
    n = 200_000 * threads
    while True:
        t0 = time.perf_counter()
        r = fo.render(of, 11, 4096, n, max(1, n // 4096), settle, 256, threads)
        dt = time.perf_counter() - t0
        if dt >= seconds * 0.5 or n >= 10**11:
            return r.s_plot / dt, r.s_iter / dt, n, dt
        n = int(n * max(2.0, seconds / max(dt, 1e-3)))


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    flames = ge._load("ffr_flames", os.path.join(ROOT, "flame-fractal-renderer_gb300", "flames.py"))
    ge._load("flame_oracle", os.path.join(ROOT, "oracle", "flame_oracle.py")).build()
    flame = flames.random_2d(7)
    threads = os.cpu_count() or 1
    fo = ge._load("flame_oracle", os.path.join(ROOT, "oracle", "flame_oracle.py"))
    of = fo.OracleFlame(fo.load_flame(json.dumps(flame)))
    # bounded sample per step: about 1 s of the machine's host cores
    per = 10_000_000
    t0 = time.perf_counter()
    fo.render(of, 1, 4096, per, per // 4096, 20, 256, threads)
    dt = time.perf_counter() - t0
    per = max(threads * 1000, int(per * 1.0 / max(dt, 1e-3)))
    for w in range(args.warmup):
        fo.render(of, 100 + w, 4096, per, max(1, per // 4096), 20, 256, threads)
    binned = iters = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        r = fo.render(of, 1000 + k, 4096, per, max(1, per // 4096), 20, 256, threads)
        binned += r.s_plot
        iters += r.s_iter
    dt = time.perf_counter() - t0
    value = binned / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "samples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "samples_per_step": per, "settle": 20,
                   "seed": 7, "flush": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{args.steps} x {per} samples of the workload, FP64",
                         "port_vs_reference": PORT_VS_REFERENCE},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "iterated_per_s": iters / dt,
    }
    print(json.dumps(line), flush=True)


def tv_distance(a, b) -> float:
    """1/2 sum |a/sum a - b/sum b| over all cells."""
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return 0.5 * float(np.abs(a / a.sum() - b / b.sum()).sum())


def tv_check(ffr, text, n, settle, device, seeds=(101, 202, 303)):
    """TV of an FP32 histogram against an FP64 one at n samples, and the FP64
    seed-to-seed noise floor at the same n."""
    hs = []
    for prec, seed in ((ffr.FP64, seeds[0]), (ffr.FP64, seeds[1]), (ffr.FP32, seeds[2])):
        with ffr.BufferRenderer(text, precision=prec, settle=settle, device=device) as r:
            r.render(n, seed, bad_limit=10**12)
            hs.append(r.counts())
    floor = tv_distance(hs[0], hs[1])
    d = tv_distance(hs[2], hs[0])
    return {"samples": n, "fp32_vs_fp64": d, "fp64_noise_floor": floor,
            "ratio": d / floor if floor > 0 else None, "bar": 3.0}


def _flames():
    return ge._load("ffr_flames", os.path.join(ROOT, "flame-fractal-renderer_gb300", "flames.py"))


def _setup_single(args):
    """Single-GPU workloads: rank 0 only (the other ranks exit)."""
    ws, rank, local = dist_env()
    if rank != 0:
        return None
    import torch
    torch.cuda.set_device(local)
    ge.build()
    return ge.package(), local


def _line(args, workload, value, ms_per_step, dtype, config, **extra):
    peaks, _ = measured_peaks()
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": "synthetic (seeded flame generator)",
            "config": dict({"workload": workload}, **config)}
    line.update(extra)
    print(json.dumps(line), flush=True)


def _timed_steps(r, args, samples, seed0, flush=None):
    """args.warmup untimed renders, then args.steps timed ones; returns
    (kernel ms, binned, iterated, last stats, kernels launched while timed)."""
    import torch
    for w in range(args.warmup):
        r.render(samples, seed0 + 10_000 + w, bad_limit=10**12)
    r.clear()
    ms = 0.0
    binned = iters = launches = 0
    s = None
    for k in range(args.steps):
        if flush is not None:
            flush.zero_()
            torch.cuda.synchronize()
        s = r.render(samples, seed0 + k, bad_limit=10**12)
        ms += s.kernel_ms
        binned += s.samples_plotted - s.dropped
        iters += s.samples_iterated
        # the render kernel plus the library's own extra launches (count-bound
        # reductions between accumulating steps)
        launches += 1 + s.aux_launches
    return ms, binned, iters, s, launches


def run_sierpinski(args):
    """2-D Sierpinski triangle, 1024^2, 1e8 samples from 1e6 trajectories of
    100 samples, settle 20, seed 1: the plain FP64 method and FP32."""
    got = _setup_single(args)
    if got is None:
        return
    ffr, dev = got
    import torch
    text = json.dumps(_flames().sierpinski_2d((1024, 1024)))
    N, T, Lt, settle = 10**8, 10**6, 100, 20
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    res = {}
    launches = 0
    sampler = ClockSampler(dev)
    sampler.start()
    kern = {"auto": ffr.KERNEL_AUTO, "plain": ffr.KERNEL_PLAIN, "sorted": ffr.KERNEL_SORTED,
            "hot": ffr.KERNEL_HOT, "jit": ffr.KERNEL_JIT, "jit-sorted": ffr.KERNEL_JIT_SORTED}
    for name, prec in (("fp64", ffr.FP64), ("fp32", ffr.FP32)):
        with ffr.BufferRenderer(text, precision=prec, settle=settle, streams=T, traj_len=Lt,
                                device=dev, kernel=kern[args.kernel]) as r:
            ms, binned, iters, s, n_launch = _timed_steps(r, args, N, 1, flush)
            launches += n_launch
            res[name] = {"value": binned / (ms * 1e-3), "ms_per_step": ms / args.steps,
                         "kernel": KERNEL_NAMES.get(s.kernel)}
            if name == "fp64" and args.verify:
                r.clear()
                r.render(N, 1, bad_limit=10**12)
                gpu = r.counts()
    clocks = sampler.stop()
    verify = None
    if args.verify:
        fo = ge._load("flame_oracle", os.path.join(ROOT, "oracle", "flame_oracle.py"))
        fo.build()
        of = fo.OracleFlame(fo.load_flame(text))
        ref = fo.render(of, 1, T, N, Lt, settle, 10**12, os.cpu_count() or 1)
        import numpy as np
        verify = {"identical_to_oracle": bool(np.array_equal(gpu, ref.counts)),
                  "binned": int(gpu.sum())}
    atom = ffr.measure_atomic_rate(1024 * 1024, 1 << 31, device=dev)
    v = res["fp64"]["value"]
    _line(args, "2-D Sierpinski triangle, 1024x1024, 1e8 samples from 1e6 trajectories",
          v, res["fp64"]["ms_per_step"], "f64",
          {"samples_per_step": N, "trajectories": T, "traj_len": Lt, "settle": settle,
           "seed": 1, "flush": "256 MiB L2 flush between timed steps"},
          fp32=res["fp32"], gpu_launches=launches,
          l2_atomic={"peak_ops_per_s": atom, "frac_fp64": v / atom,
                     "frac_fp32": res["fp32"]["value"] / atom},
          verify=verify, clocks=clocks)


def run_tetra3d(args):
    """Sierpinski tetrahedron, 512^3 u32 buffer, 1e10 samples in steps of
    1e9, FP32, seed 3."""
    got = _setup_single(args)
    if got is None:
        return
    ffr, dev = got
    text = json.dumps(_flames().tetrahedron_3d((512, 512, 512)))
    B, settle = int(args.samples_per_step), 20
    kern = {"auto": ffr.KERNEL_AUTO, "plain": ffr.KERNEL_PLAIN, "sorted": ffr.KERNEL_SORTED,
            "hot": ffr.KERNEL_HOT, "jit": ffr.KERNEL_JIT, "jit-sorted": ffr.KERNEL_JIT_SORTED}
    with ffr.BufferRenderer(text, precision=ffr.FP32, settle=settle, device=dev,
                            kernel=kern[args.kernel]) as r:
        sampler = ClockSampler(dev)
        sampler.start()
        # the 512 MiB buffer exceeds L2: no flush needed between steps
        ms, binned, iters, s, launches = _timed_steps(r, args, B, 3)
        clocks = sampler.stop()
        assert r.histogram()[0] == binned
        import numpy as np
        occupied = int(np.count_nonzero(r.counts()))
    value = binned / (ms * 1e-3)
    peaks, kind = measured_peaks()
    achieved = 8.0 * binned / (ms * 1e-3) / 1e9
    # the hits land on the attractor's occupied cells only: the matching
    # peak is the atomic rate over a buffer of that many cells (L2-resident),
    # not over the whole 512^3 buffer (HBM-bound)
    atom = ffr.measure_atomic_rate(occupied, 1 << 31, device=dev)
    atom_full = ffr.measure_atomic_rate(512 ** 3, 1 << 31, device=dev)
    tv = None if args.no_tv else tv_check(ffr, text, 10**8, settle, dev)
    _line(args, "Sierpinski tetrahedron, 512^3 u32 buffer, 1e10 samples", value,
          ms / args.steps, "f32",
          {"samples_per_step": B, "settle": settle, "seed": 3, "streams": s.streams,
           "traj_len": s.traj_len, "kernel": KERNEL_NAMES.get(s.kernel),
           "flush": "none: the 512 MiB buffer is larger than L2"},
          gpu_launches=launches,
          roofline={"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                    "peak_source": kind},
          l2_atomic={"peak_ops_per_s": atom, "achieved_ops_per_s": value, "frac": value / atom,
                     "what": f"u32 atomic adds at uniformly random cells of a buffer of "
                             f"{occupied} cells (the occupied cells of the 512^3 buffer)",
                     "whole_buffer_peak_ops_per_s": atom_full},
          tv=tv, clocks=clocks, iterated_per_s=iters / (ms * 1e-3))


def batch256_record(ffr, dev, steps, warmup, with_tv=True, n_tv=8, scale=1.0):
    """The 256-flame batch (flames.batch_jobs(11)) in one persistent,
    graph-captured launch per step: binned samples/s over `steps` timed
    steps (L2 flushed between them), per-flame TV against FP64 for n_tv
    flames, and the clocks seen while timing."""
    import torch
    fl = _flames()
    jobs = fl.batch_jobs(11)
    texts = [json.dumps(f) for f, _ in jobs]
    # scale < 1: the same flames with fewer samples (small profiling cases)
    ns = [max(1, int(n * scale)) for _, n in jobs]
    rs = [ffr.BufferRenderer(t, precision=ffr.FP32, settle=20, traj_len=4096, device=dev)
          for t in texts]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    with ffr.Batch(rs) as b:
        for w in range(warmup):
            b.render([max(1, n // 100) for n in ns], [500 + i for i in range(len(ns))],
                     bad_limit=10**12, stats=False)
        for r in rs:
            r.clear()
        sampler = ClockSampler(dev)
        sampler.start()
        ms, binned, iters, aux = 0.0, 0, 0, 0
        for k in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            _, sts = b.render(ns, [1000 * k + i for i in range(len(ns))], bad_limit=10**12)
            ms += sts[0].kernel_ms
            binned += sum(st.samples_plotted - st.dropped for st in sts)
            iters += sum(st.samples_iterated for st in sts)
            aux += sum(st.aux_launches for st in sts)
        clocks = sampler.stop()
        nhot = sum(1 for st in sts if st.hot_cells)
    for r in rs:
        r.close()
    tvs = []
    if with_tv:
        for i in range(0, len(texts), len(texts) // n_tv):
            t = tv_check(ffr, texts[i], 10**8, 20, dev)
            t["flame"] = i
            tvs.append(t)
    return {"value": binned / (ms * 1e-3), "unit": "samples/s", "ms_per_step": ms / steps,
            "steps": steps, "warmup": warmup, "iterated_per_s": iters / (ms * 1e-3),
            "flames": len(texts), "samples_per_step": sum(ns), "settle": 20, "seed": 11,
            "traj_len": 4096, "kernel": "persistent batch (CUDA graph)",
            "hot_cell_tables": f"{nhot} of {len(texts)} jobs",
            "flush": "256 MiB L2 flush between timed steps",
            "gpu_launches": steps * 2 + aux,
            "tv": {"per_flame": tvs,
                   "max_ratio": max((t["ratio"] for t in tvs if t["ratio"]), default=None)},
            "clocks": clocks}


NO_BAD_LIMIT = 10**15


def per_flame_record(ffr, dev, flames, steps=3):
    """The per-flame kernels (NVRTC: KERNEL_JIT, the plain kernel with each
    variation slot's dispatch narrowed; KERNEL_JIT_SORTED, the xform-sorted
    kernel with each xform's types fixed) against the general plain and
    xform-sorted kernels, on flames the precompiled merged instantiations
    do not cover: a random 2-D flame of twelve parameterless variations
    outside the benchmark seven, in FP32 and in the FP64 mirror, and the
    benchmark flame in the FP64 mirror.  All four kernels run the same
    streams (the general plain kernel's default plan), so their buffers must
    be identical.  No bad-value limit: a render the limit stopped would end
    early at a time that depends on the race to the stop flag."""
    import numpy as np
    import torch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    other = flames.random_2d(7, variations=flames.OTHER_2D)
    out = []
    for name, fl, prec, n in (
            ("random 2-D flame of 12 other variations, 1920x1080, FP32", other, ffr.FP32,
             10**9),
            ("random 2-D flame of 12 other variations, 1920x1080, FP64 mirror", other,
             ffr.FP64, 10**8),
            ("benchmark flame (6-xform random 1920x1080), FP64 mirror",
             flames.random_2d(7), ffr.FP64, 10**8)):
        text = json.dumps(fl)
        t0 = time.perf_counter()
        st, msg = ffr.jit_prepare(text, prec)
        prep_s = time.perf_counter() - t0
        if st != ffr.FFR_OK:
            out.append({"flame": name, "error": msg})
            continue
        rec = {"flame": name, "samples_per_step": n, "compile_s": prep_s}
        plan = None
        first = None
        same = True
        for kname, kern in (("general", ffr.KERNEL_PLAIN), ("general_sorted", ffr.KERNEL_SORTED),
                            ("per_flame", ffr.KERNEL_JIT),
                            ("per_flame_sorted", ffr.KERNEL_JIT_SORTED)):
            kw = {} if plan is None else {"streams": plan[0], "traj_len": plan[1]}
            with ffr.BufferRenderer(text, precision=prec, settle=20, device=dev, kernel=kern,
                                    **kw) as r:
                s = r.render(n, 99, bad_limit=NO_BAD_LIMIT)
                if plan is None:
                    plan = (s.streams, s.traj_len)
                r.clear()
                ms, binned, bad = 0.0, 0, 0
                for k in range(steps):
                    flush.zero_()
                    torch.cuda.synchronize()
                    s = r.render(n, 100 + k, bad_limit=NO_BAD_LIMIT)
                    assert s.ok and s.samples_iterated == n and s.kernel == kern
                    ms += s.kernel_ms
                    binned += s.samples_plotted - s.dropped
                    bad += s.bad_values
                rec[kname] = {"value": binned / (ms * 1e-3), "unit": "binned samples/s",
                              "ms_per_step": ms / steps, "bad_values_per_step": bad / steps}
                counts = r.counts()
                if first is None:
                    first = counts
                else:
                    same = same and bool(np.array_equal(first, counts))
        best_g = min(rec["general"]["ms_per_step"], rec["general_sorted"]["ms_per_step"])
        best_p = min(rec["per_flame"]["ms_per_step"], rec["per_flame_sorted"]["ms_per_step"])
        rec["speedup_best_over_best"] = best_g / best_p
        rec["identical_buffers"] = same
        rec["streams"], rec["traj_len"] = plan
        out.append(rec)
    return out


def run_perflame(args):
    """The per-flame kernel record alone (--steps timed renders per kernel)."""
    got = _setup_single(args)
    if got is None:
        return
    ffr, dev = got
    recs = per_flame_record(ffr, dev, _flames(), steps=max(1, args.steps))
    fp32 = recs[0]["per_flame"]
    _line(args, "per-flame kernels: random 2-D flame of 12 other variations, 1920x1080, "
          "FP32 (and FP64 records)", fp32["value"], fp32["ms_per_step"],
          "f32", {"samples_per_step": recs[0]["samples_per_step"], "settle": 20,
                  "flush": "256 MiB L2 flush between timed steps"},
          gpu_launches=4 * len(recs) * max(1, args.steps), per_flame_kernels=recs)


def run_batch256(args):
    """256 random 2-D flames in one persistent, graph-captured launch per step."""
    got = _setup_single(args)
    if got is None:
        return
    ffr, dev = got
    rec = batch256_record(ffr, dev, args.steps, args.warmup, with_tv=not args.no_tv,
                          scale=args.batch_scale)
    _line(args, "256 random 2-D flames (2-8 xforms, 256^2-2048^2, 1e7-1e9 samples) "
          "in one persistent launch", rec["value"], rec["ms_per_step"], "f32",
          {k: rec[k] for k in ("flames", "samples_per_step", "settle", "seed", "traj_len",
                               "kernel", "hot_cell_tables", "flush")},
          gpu_launches=rec["gpu_launches"], tv=rec["tv"], clocks=rec["clocks"],
          iterated_per_s=rec["iterated_per_s"])


def serving_record(ffr, dev, rate, duration, warmup, max_active, with_tv=True, n_tv=4):
    """A Poisson request stream (flames.serving_requests(23, rate, duration))
    through the serving loop (ffr_server_*), every result read back by four
    client threads: binned samples/s from the first submission to the last
    completion, p50/p99 latency (submission to completion, and with the
    read-back), and TV against FP64 for n_tv served 2-D jobs."""
    import queue
    import random
    import numpy as np
    fl = _flames()
    reqs = fl.serving_requests(23, rate, duration)
    texts = [json.dumps(f) if f is not None else None for _, _, f, _ in reqs]
    geo = []
    for _, kind, f, _ in reqs:
        if f is None:
            geo.append(None)
        else:
            cells = 1
            for x in f["size"]:
                cells *= x
            geo.append((cells, f["dimensions"]))
    srv = ffr.Server(precision=ffr.FP32, settle=20, traj_len=4096, device=dev,
                     max_active=max_active)
    # warm-up: a few small jobs of each kind (module load, pool growth)
    for w in range(max(1, warmup)):
        a = srv.submit(texts[0], 10**6, 9000 + w)
        srv.wait(a, 60_000)
        srv.release(a)
    lock = threading.Lock()
    done = queue.Queue()
    pool = []                    # resident continuation targets
    evicted = set()
    info = {}                    # job -> (kind, cells, dims)
    rnd = random.Random(23)
    t_start = time.perf_counter()
    errors = []

    def submitter():
        for i, (t, kind, f, n) in enumerate(reqs):
            dt = t_start + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            try:
                if kind == "cont":
                    with lock:
                        if not pool:
                            continue
                        parent = rnd.choice(pool)
                        j = srv.continue_(parent, n, 50_000 + i)
                        info[j] = ("cont",) + info[parent][1:]
                else:
                    j = srv.submit(texts[i], n, 50_000 + i)
                    with lock:
                        info[j] = (kind,) + geo[i]
                        pool.append(j)
                        if len(pool) > 64:
                            evicted.add(pool.pop(0))
                done.put(j)
            except Exception as e:          # noqa: BLE001
                errors.append(repr(e))
        for _ in range(4):
            done.put(None)

    results = []

    def completer():
        # one host buffer per client thread, grown as needed and reused (a
        # client that writes results out does not fault in fresh pages per read)
        out = np.empty(0, dtype=np.uint64)
        while True:
            j = done.get()
            if j is None:
                return
            try:
                inf = srv.wait(j, 0)
                kind, cells, dims = info[j]
                st = srv.stats(j, dims)
                t0 = time.perf_counter_ns()
                if out.size < cells:
                    out = np.ones(cells, dtype=np.uint64)
                srv.read_into(j, out.ctypes.data, cells * 8)
                t_read = time.perf_counter_ns() - t0
            except Exception as e:          # noqa: BLE001
                errors.append(repr(e))
                continue
            with lock:
                keep = j in pool
                results.append((kind, inf.submit_ns, inf.done_ns, t_read, st.samples_plotted,
                                st.samples_iterated, inf.status))
            if not keep:
                srv.release(j)
                with lock:
                    evicted.discard(j)

    sampler = ClockSampler(dev)
    sampler.start()
    th = [threading.Thread(target=submitter)] + [threading.Thread(target=completer)
                                                  for _ in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.perf_counter() - t_start
    clocks = sampler.stop()
    load = srv.load()
    srv.close()
    lat = np.array([(d - s) * 1e-6 for _, s, d, _, _, _, _ in results])
    lat_read = np.array([(d - s) * 1e-6 + r * 1e-6 for _, s, d, r, _, _, _ in results])
    binned = sum(r[4] for r in results)
    iters = sum(r[5] for r in results)
    first = min(r[1] for r in results)
    last = max(r[2] for r in results)
    span = (last - first) * 1e-9
    offered = sum(n for *_, n in reqs) / duration
    kinds = {}
    for r in results:
        kinds.setdefault(r[0], []).append((r[2] - r[1]) * 1e-6)
    # TV of served FP32 results against FP64: a served job's buffer equals the
    # solo FP32 render with streams = ceil(N / 4096) (tests/test_gpu_server.py),
    # so four 2-D requests of at most 2e8 samples are re-rendered that way
    tvs = []
    if with_tv:
        picks = [i for i, (_, k, _, n) in enumerate(reqs) if k == "2d" and n <= 2 * 10**8][:n_tv]
        for i in picks:
            n = reqs[i][3]
            hs = []
            for prec, seed in ((ffr.FP32, 50_000 + i), (ffr.FP64, 7_000 + i), (ffr.FP64, 8_000 + i)):
                with ffr.BufferRenderer(texts[i], precision=prec, settle=20, traj_len=4096,
                                        streams=-(-n // 4096), device=dev) as r:
                    r.render(n, seed, bad_limit=10**12)
                    hs.append(r.counts())
            floor = tv_distance(hs[1], hs[2])
            d = tv_distance(hs[0], hs[1])
            tvs.append({"request": i, "samples": n, "fp32_vs_fp64": d, "fp64_noise_floor": floor,
                        "ratio": d / floor if floor > 0 else None})
    return {"value": binned / span, "unit": "samples/s", "span_s": span,
            "iterated_per_s": iters / span, "offered_samples_per_s": offered,
            "requests": len(reqs), "completed": len(results), "rate_per_s": rate,
            "duration_s": duration, "seed": 23, "settle": 20, "traj_len": 4096,
            "max_active": max_active,
            "latency_ms": {"p50": float(np.percentile(lat, 50)),
                           "p99": float(np.percentile(lat, 99)),
                           "p50_with_read": float(np.percentile(lat_read, 50)),
                           "p99_with_read": float(np.percentile(lat_read, 99)),
                           "by_kind_p50": {k: float(np.percentile(v, 50)) for k, v in kinds.items()},
                           "by_kind_p99": {k: float(np.percentile(v, 99)) for k, v in kinds.items()}},
            "wall_s": wall,
            "tv": {"served_jobs": tvs,
                   "max_ratio": max((t["ratio"] for t in tvs if t["ratio"]), default=None)},
            "statuses": sorted({r[6] for r in results}), "errors": errors[:5],
            "server_load": load, "clocks": clocks}


def run_serving(args):
    """Poisson request stream through the serving loop (ffr_server_*)."""
    got = _setup_single(args)
    if got is None:
        return
    ffr, dev = got
    rec = serving_record(ffr, dev, args.rate, args.duration, args.warmup, args.max_active,
                         with_tv=not args.no_tv)
    _line(args, f"Poisson serving stream, {args.rate:g} req/s for {args.duration:g} s "
          "(80% 2-D, 15% 3-D, 5% continuations)", rec["value"], rec["span_s"] * 1e3, "f32",
          {k: rec[k] for k in ("requests", "completed", "rate_per_s", "duration_s", "seed",
                               "settle", "traj_len", "max_active")}
          | {"flush": "n/a (a stream of distinct buffers)"},
          latency_ms=rec["latency_ms"], offered_samples_per_s=rec["offered_samples_per_s"],
          iterated_per_s=rec["iterated_per_s"], wall_s=rec["wall_s"], tv=rec["tv"],
          statuses=rec["statuses"], errors=rec["errors"], server_load=rec["server_load"],
          clocks=rec["clocks"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="random2d",
                    choices=["random2d", "sierpinski", "tetra3d", "batch256", "serving",
                             "perflame"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--samples-per-step", type=float, default=1e9)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-tv", action="store_true")
    ap.add_argument("--verify", action="store_true")
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--max-active", type=int, default=256)
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="batch256: multiply every flame's sample count (profiling cases)")
    ap.add_argument("--no-sub", action="store_true",
                    help="default workload only: skip the batch and serving sub-records")
    ap.add_argument("--serving-seconds", type=float, default=10.0,
                    help="default workload: arrival window of the over-capacity stream "
                         "(the sustainable one runs 1.5x as long)")
    ap.add_argument("--kernel", default="auto",
                    choices=["auto", "plain", "sorted", "hot", "jit", "jit-sorted"],
                    help="render kernel (auto: the library's autotuner decides)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "random2d":
        {"sierpinski": run_sierpinski, "tetra3d": run_tetra3d, "batch256": run_batch256,
         "serving": run_serving, "perflame": run_perflame}[args.workload](args)
        return
    ws, rank, local = dist_env()
    import torch
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist = None
    ge.build()
    ffr = ge.package()
    flames = ge._load("ffr_flames", os.path.join(ROOT, "flame-fractal-renderer_gb300", "flames.py"))
    flame = flames.random_2d(7)
    text = json.dumps(flame)
    prec = ffr.FP32 if args.precision == "fp32" else ffr.FP64
    B = int(args.samples_per_step)
    settle = 20
    seed_base = rank_seed(7, rank)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    kern = {"auto": ffr.KERNEL_AUTO, "plain": ffr.KERNEL_PLAIN, "sorted": ffr.KERNEL_SORTED,
            "hot": ffr.KERNEL_HOT, "jit": ffr.KERNEL_JIT, "jit-sorted": ffr.KERNEL_JIT_SORTED}
    r = ffr.BufferRenderer(text, precision=prec, settle=settle, device=local,
                           kernel=kern[args.kernel])
    for w in range(args.warmup):
        r.render(B, seed_base + 10_000 + w)
    r.clear()
    sampler = ClockSampler(local)
    barrier()
    sampler.start()
    t0 = time.perf_counter()
    kern_ms, binned, iters, launches = 0.0, 0, 0, 0
    streams = traj_len = 0
    kernel_used = None
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s = r.render(B, seed_base + k)
        kern_ms += s.kernel_ms
        binned += s.samples_plotted - s.dropped
        iters += s.samples_iterated
        launches += 1 + s.aux_launches
        streams, traj_len = s.streams, s.traj_len
        kernel_used = KERNEL_NAMES.get(s.kernel) + (
            " + warp-merged bins" if s.agg else "") + (
            f" + {s.hot_cells} hot cells in shared memory" if s.hot_cells else "")
    barrier()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    hsum = r.histogram()[0]
    assert hsum == binned, (hsum, binned)
    # max over ranks of the device time; whole-job binned = sum over ranks
    kern_ms_all, binned_all, wall_all = rank_totals(kern_ms, binned, wall, dist,
                                                    device=f"cuda:{local}")
    value = binned_all / (kern_ms_all * 1e-3)
    r.close()

    # end to end through the C ABI: create (JSON -> program upload), render,
    # read back into pinned host memory, every step
    e2e_steps = max(1, min(args.steps, 5))
    # the pinned result buffer is the caller's, allocated once before timing
    # (file layout: one u64 count per cell, no colours in this flame)
    cells = int(flame["size"][0]) * int(flame["size"][1])
    pinned = torch.empty(cells * 8, dtype=torch.uint8).pin_memory()
    e2e_binned = 0
    h2d = d2h = 0
    barrier()
    te = time.perf_counter()
    for k in range(e2e_steps):
        with ffr.BufferRenderer(text, precision=prec, settle=settle, device=local,
                                kernel=kern[args.kernel]) as er:
            assert er.buffer_bytes == pinned.numel()
            s = er.render(B, seed_base + 500 + k)
            st = er._lib.ffr_read_buffer(er._ctx, pinned.data_ptr(), er.buffer_bytes)
            assert st == 0
            e2e_binned += s.samples_plotted - s.dropped
            h2d = len(text.encode())
            d2h = er.buffer_bytes
    barrier()
    e2e_dt = time.perf_counter() - te
    e2e_value = e2e_binned * ws / e2e_dt

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peaks, peak_kind = measured_peaks()
    # per launch of the render kernel: one 4-byte atomic add per binned
    # sample (8 B of read-modify-write), over the launch's average event time
    per_launch_ops = binned / launches
    avg_s = kern_ms / launches * 1e-3
    achieved_hbm = 8.0 * per_launch_ops / avg_s / 1e9
    atom = ffr.measure_atomic_rate(1920 * 1080, 1 << 31, device=local)
    traffic = profile_traffic()
    # the primary bound: the 8.3 MB buffer is L2-resident, so binning is
    # capped by the rate of L2 atomics, measured in this run
    roofline = {"bound": "l2_atomic", "achieved": per_launch_ops / avg_s / 1e9,
                "peak": atom / 1e9, "unit": "G atomic adds/s",
                "frac": per_launch_ops / avg_s / atom,
                "traffic": traffic, "traffic_unit": "DRAM bytes per launch (ncu)",
                "peak_source": "measured in this run: u32 atomic adds at uniformly random "
                               "cells of a 1920x1080 buffer (ffr_measure_atomic_rate)",
                "kernel": f"render kernel ({kernel_used}), FP32"}
    roofline_hbm = {"bound": "hbm", "achieved": achieved_hbm, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": achieved_hbm / peaks["hbm_gbs"],
                    "traffic": traffic, "peak_source": peak_kind,
                    "what": "8 B per binned sample against the HBM copy bandwidth (of "
                            f"{peak_kind}); secondary: every atomic resolves in L2"}
    l2 = {"peak_ops_per_s": atom, "achieved_ops_per_s": binned / (kern_ms * 1e-3),
          "frac": binned / (kern_ms * 1e-3) / atom,
          "what": "u32 atomic adds at uniformly random cells of a 1920x1080 buffer"}

    fp64 = None
    if not args.no_fp64:
        B64 = max(10**7, B // 10)
        with ffr.BufferRenderer(text, precision=ffr.FP64, settle=settle, device=local,
                                kernel=ffr.KERNEL_PLAIN) as r64:
            r64.render(B64, 99)
            ms64, bin64 = 0.0, 0
            for k in range(3):
                flush.zero_()
                torch.cuda.synchronize()
                s = r64.render(B64, 200 + k)
                ms64 += s.kernel_ms
                bin64 += s.samples_plotted - s.dropped
        fp64 = {"value": bin64 / (ms64 * 1e-3), "samples_per_step": B64,
                "kernel": "plain FP64 mirror",
                "fp32_over_fp64": value / ws / (bin64 / (ms64 * 1e-3))}

    tv = None
    if not args.no_tv:
        tv = tv_check(ffr, text, 2 * 10**8, settle, local)

    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        threads = os.cpu_count() or 1
        rate, irate, n, dt = cpu_port_rate(flame, settle, args.cpu_seconds, threads)
        cpu = {"value": rate, "unit": "samples/s", "cores": threads, "kind": "port",
               "sample": f"{n} samples of the workload (FP64, settle 20), {dt:.1f} s",
               "port_vs_reference": PORT_VS_REFERENCE}

    # the batched and serving paths (the 256-flame batch; the Poisson stream
    # over capacity, then at 0.7x the capacity it measured), single GPU only
    batch = serving = per_flame = None
    if ws == 1 and not args.no_sub:
        per_flame = per_flame_record(ffr, local, flames)
        batch = batch256_record(ffr, local, steps=2, warmup=1, with_tv=not args.no_tv)
        # the configured stream (200 req/s); the same stream at twice the
        # rate, whose served samples/s is the loop's capacity when the loop
        # falls behind it (served below 95% of offered); then 0.7 x capacity
        conf = serving_record(ffr, local, 200.0, args.serving_seconds, 1, args.max_active,
                              with_tv=False)
        sat = serving_record(ffr, local, 400.0, max(4.0, args.serving_seconds / 2), 1,
                             args.max_active, with_tv=False)
        per_req = conf["offered_samples_per_s"] / conf["rate_per_s"]
        saturated = sat["iterated_per_s"] < 0.95 * sat["offered_samples_per_s"]
        capacity = max(conf["iterated_per_s"], sat["iterated_per_s"]) / per_req
        rate = round(0.7 * capacity, 1)
        steady = serving_record(ffr, local, rate, args.serving_seconds * 1.5, 1,
                                args.max_active, with_tv=not args.no_tv)
        serving = {
            "configured": dict(conf, what="the configured stream, 200 req/s"),
            "saturated": dict(sat, what="400 req/s: when the loop falls behind, its served "
                              "samples/s is the capacity and latency measures queue growth"),
            "sustainable": dict(steady, what=f"0.7 x the measured capacity "
                                f"({capacity:.1f} req/s = served samples/s / {per_req:.3g} "
                                f"samples per request)"),
            "capacity_req_per_s": capacity,
            "capacity_is_lower_bound": not saturated,
        }

    line = {
        "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": kern_ms_all / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == ffr.FP32 else "f64",
        "data": "synthetic (seeded flame generator)",
        "config": {"workload": WORKLOAD, "samples_per_step": B, "settle": settle,
                   "seed": 7, "streams": streams, "traj_len": traj_len,
                   "kernel": kernel_used,
                   "flush": "256 MiB L2 flush between timed steps",
                   "parallelism": f"replicas{ws}"},
        "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps},
        "gpu_launches": launches,
        "roofline": roofline,
        "roofline_hbm": roofline_hbm,
        "l2_atomic": l2,
        "fp64": fp64,
        "tv": tv,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "iterated_per_s": iters / (kern_ms * 1e-3),
        "wall_s": wall_all,
        "batch256": batch,
        "serving": serving,
        "per_flame_kernels": per_flame,
    }
    if serving:
        # the configured stream's latency (the loop keeps up with it), and
        # the sustainable stream's
        line["latency_ms"] = {"p50": serving["configured"]["latency_ms"]["p50"],
                              "p99": serving["configured"]["latency_ms"]["p99"],
                              "rate_per_s": serving["configured"]["rate_per_s"],
                              "sustainable": {
                                  "p50": serving["sustainable"]["latency_ms"]["p50"],
                                  "p99": serving["sustainable"]["latency_ms"]["p99"],
                                  "rate_per_s": serving["sustainable"]["rate_per_s"]}}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
