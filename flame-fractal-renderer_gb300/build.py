"""Build libffr_gpu.so and the ffr-buf / ffr-img / ffr-serve executables in-tree.

Outputs go to flame-fractal-renderer_gb300/_build/ (git-ignored).  Every
CUDA translation unit is compiled for sm_103a only; the six chaos-kernel
objects (precision x dims) and the host objects compile in parallel.  The
FP64 kernel objects use --fmad=false so products and sums round separately,
as in the reference's double arithmetic.  Only the ffr_* C symbols are
exported (exports.map).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libffr_gpu.so")
CLI = os.path.join(OUT, "ffr-buf")
IMG_CLI = os.path.join(OUT, "ffr-img")
SERVE_CLI = os.path.join(OUT, "ffr-serve")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libffr_gpu.so")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
          if f.endswith((".h", ".hpp", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "ffr_gpu.h"))
    hs.append(os.path.abspath(__file__))
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(force: bool = False, verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers()
    nv_common = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
                 "-I", CSRC, "-I", INCLUDE]
    cxx_common = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
                  "-Wall", "-Wextra", "-I", CSRC, "-I", INCLUDE,
                  "-I", os.path.join(cuda, "include")]
    jobs = []   # (target, deps, cmd)
    for p in (0, 1):
        for d in (1, 2, 3, 4):
            # four dimensions: plain render (kinds 0, 2, 6) and step/trace (5)
            kinds = range(8 if p == 1 else 6) if d < 4 else ([0, 2, 5, 6] if p == 1 else [0, 2, 5])
            for kind in kinds:
                obj = os.path.join(OUT, f"chaos_p{p}_d{d}_k{kind}.o")
                src = os.path.join(CSRC, "chaos_inst.cu")
                extra = ["--fmad=false"] if p == 0 else []
                jobs.append((obj, [src] + hdrs,
                             [nvcc, *nv_common, *extra, f"-DFFR_P={p}", f"-DFFR_D={d}",
                              f"-DFFR_KIND={kind}", "-c", src, "-o", obj]))
    for name in ("buffer_kernels", "image_kernels", "noalloc"):
        src = os.path.join(CSRC, name + ".cu")
        obj = os.path.join(OUT, name + ".o")
        jobs.append((obj, [src] + hdrs, [nvcc, *nv_common, "-c", src, "-o", obj]))
    for name in ("api", "server", "png", "flame", "json", "variations_host", "hot_cells"):
        src = os.path.join(CSRC, name + ".cpp")
        obj = os.path.join(OUT, name + ".o")
        jobs.append((obj, [src] + hdrs, [*cxx_common, "-c", src, "-o", obj]))
    todo = [j for j in jobs if force or _stale(j[0], j[1])]
    if todo:
        workers = min(len(todo), max(2, os.cpu_count() or 2))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = [ex.submit(_run, j[2]) for j in todo]
            for f in futs:
                f.result()
    objs = [j[0] for j in jobs]
    exports = os.path.join(CSRC, "exports.map")
    if force or _stale(LIB, objs + [exports]):
        tmp = LIB + f".tmp{os.getpid()}"
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs,
              "-Xlinker", f"--version-script={exports}", "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    for exe, src in ((CLI, "ffr_buf_cli.cpp"), (IMG_CLI, "ffr_img_cli.cpp"),
                     (SERVE_CLI, "ffr_serve_cli.cpp")):
        cli_src = os.path.join(CSRC, src)
        if force or _stale(exe, [cli_src, LIB, os.path.join(INCLUDE, "ffr_gpu.h"),
                                 os.path.join(INCLUDE, "ffr_wire.h")]):
            tmp = exe + f".tmp{os.getpid()}"
            _run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", INCLUDE, cli_src,
                  "-o", tmp, "-L", OUT, "-lffr_gpu", "-lpthread", "-Wl,-rpath,$ORIGIN"])
            os.replace(tmp, exe)
    if verbose:
        print(f"built {LIB} and {CLI}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
