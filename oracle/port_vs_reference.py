"""Speed of the oracle's C restatement against the reference's own render().

Both run the 1920x1080 random 2-D benchmark flame (flames.random_2d(7)) in
FP64 on the same host cores, with the reference CLI's defaults: 53 settle
iterations and the automatic batch size clamp((N + 255) >> 8, 4096, 2^20)
(src/ffr_buf.cpp:94-101) as the trajectory length.  The reference side is
oracle/_ref/ffr_ref's `bench` subcommand, which calls
BufferRenderer<2>::render() (src/renderers/buffer_renderer.hpp:269-338)
exactly as ffr-buf does; it exists only where the reference sources were
present at build time (oracle/build_ref.sh).

Usage: python oracle/port_vs_reference.py [samples] [threads ...]
Prints one JSON line per thread count: both rates and port / reference.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [HERE, os.path.join(ROOT, "flame-fractal-renderer_gb300")]


def main() -> int:
    import flame_oracle as fo
    import flames
    ref_bin = os.path.join(HERE, "_ref", "ffr_ref")
    if not os.path.exists(ref_bin):
        print("oracle/_ref/ffr_ref is absent (the reference sources were not found "
              "when oracle/build_ref.sh ran)", file=sys.stderr)
        return 1
    fo.build()
    n_total = int(float(sys.argv[1])) if len(sys.argv) > 1 else 2 * 10**8
    thread_counts = [int(t) for t in sys.argv[2:]] or [os.cpu_count() or 1, 1]
    text = json.dumps(flames.random_2d(7))
    path = os.path.join(HERE, "_ref", "random2d_seed7.json")
    with open(path, "w") as f:
        f.write(text)
    of = fo.OracleFlame(fo.load_flame(text))
    for threads in thread_counts:
        n = max(10**6, n_total * threads // max(thread_counts))
        out = subprocess.run([ref_bin, "bench", path, str(n), str(threads)],
                             capture_output=True, text=True, check=True).stdout
        ref = json.loads(out)
        batch = ref["batch"]
        t0 = time.perf_counter()
        port = fo.render(of, 11, max(threads, -(-n // batch)), n, batch, 53, 256, threads)
        dt = time.perf_counter() - t0
        print(json.dumps({
            "flame": "random_2d(7), 1920x1080", "samples": n, "threads": threads,
            "batch": batch, "settle": 53,
            "reference_samples_per_s": ref["samples_per_s"],
            "port_samples_per_s": n / dt,
            "port_over_reference": (n / dt) / ref["samples_per_s"],
            "plotted": {"reference": ref["s_plot"], "port": int(port.s_plot)},
            "cpu": os.uname().machine}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
