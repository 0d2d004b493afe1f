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
        renders, and reads the buffer back into pinned host memory
roofline  binned samples x 8 B (one 4-byte atomic read-modify-write each)
        against measured HBM bandwidth, plus the measured rate of 4-byte
        atomic adds at random cells of a buffer of the same size (l2_atomic)
cpu_baseline  the oracle's C restatement of the reference path (FP64,
        all host threads) on a bounded sample of the same workload

--impl reference times that CPU implementation alone, as the reference arm.
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
WORKLOAD = "random 2-D flame, 6 xforms x 2 variations, 1920x1080, 1e10 samples"


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


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0}, "fallback"


def profile_traffic():
    """Per-launch DRAM traffic of the render kernel from the committed ncu
    summary (profiles/chaos_fp32_random2d.md), scaled to one launch of the
    bench's sample count; None when no summary exists."""
    p = os.path.join(ROOT, "profiles", "chaos_fp32_random2d.md")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_binned_sample:"):
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
                         "sample": f"{args.steps} x {per} samples of the workload, FP64"},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "iterated_per_s": iters / dt,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--samples-per-step", type=float, default=1e9)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
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
    seed_base = 7 + 1_000_003 * rank

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    r = ffr.BufferRenderer(text, precision=prec, settle=settle, device=local)
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
        launches += 1
        streams, traj_len = s.streams, s.traj_len
        kernel_used = {1: "plain", 2: "xform-sorted"}.get(s.kernel) + (
            " + warp-merged bins" if s.agg else "")
    barrier()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    hsum = r.histogram()[0]
    assert hsum == binned, (hsum, binned)
    # max over ranks of the device time; whole-job binned = sum over ranks
    t = torch.tensor([kern_ms, float(binned), wall], dtype=torch.float64, device=f"cuda:{local}")
    if dist:
        mx = t.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        sm = t.clone()
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        kern_ms_all, binned_all, wall_all = mx[0].item(), sm[1].item(), mx[2].item()
    else:
        kern_ms_all, binned_all, wall_all = kern_ms, float(binned), wall
    value = binned_all / (kern_ms_all * 1e-3)
    r.close()

    # end to end through the C ABI: create (JSON -> program upload), render,
    # read back into pinned host memory, every step
    e2e_steps = max(1, min(args.steps, 5))
    pinned = None
    e2e_binned = 0
    h2d = d2h = 0
    barrier()
    te = time.perf_counter()
    for k in range(e2e_steps):
        with ffr.BufferRenderer(text, precision=prec, settle=settle, device=local) as er:
            if pinned is None:
                pinned = torch.empty(er.buffer_bytes, dtype=torch.uint8).pin_memory()
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
    per_launch_bytes = 8.0 * binned / launches
    avg_s = kern_ms / launches * 1e-3
    achieved = per_launch_bytes / avg_s / 1e9
    dram_per_sample = profile_traffic()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "traffic": (dram_per_sample * binned / launches) if dram_per_sample else None,
                "peak_source": peak_kind,
                "kernel": f"render kernel ({kernel_used}), FP32"}
    atom = ffr.measure_atomic_rate(1920 * 1080, 1 << 31, device=local)
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

    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        threads = os.cpu_count() or 1
        rate, irate, n, dt = cpu_port_rate(flame, settle, args.cpu_seconds, threads)
        cpu = {"value": rate, "unit": "samples/s", "cores": threads, "kind": "port",
               "sample": f"{n} samples of the workload (FP64, settle 20), {dt:.1f} s"}

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
        "l2_atomic": l2,
        "fp64": fp64,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "iterated_per_s": iters / (kern_ms * 1e-3),
        "wall_s": wall_all,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
