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


# headers the per-flame kernels (csrc/jit.cpp, NVRTC) include, embedded in
# the library so that it needs no source tree at run time
JIT_HEADERS = ["std_types.h", "variation_ids.h", "flame_program.h", "isaac64.cuh", "launch.h",
               "variations.cuh", "chaos_kernel.cuh", "chaos_sorted.cuh"]
JIT_INC = os.path.join(OUT, "jit_headers.inc")


def _write_jit_headers() -> None:
    """_build/jit_headers.inc: the kernel headers as raw string literals."""
    names, texts = [], []
    for h in JIT_HEADERS:
        with open(os.path.join(CSRC, h)) as f:
            t = f.read()
        if ")FFRJIT\"" in t:
            raise RuntimeError(f"{h} contains the raw-string delimiter")
        names.append(f'"{h}"')
        # split into pieces below the 64 KB literal limit some compilers keep
        pieces = [t[i:i + 30000] for i in range(0, len(t), 30000)] or [""]
        texts.append("\n".join(f'R"FFRJIT({p})FFRJIT"' for p in pieces))
    out = ["// generated by build.py from csrc/: the headers of the per-flame kernels",
           f"constexpr int kJitHeaderCount = {len(names)};",
           "const char* const kJitHeaderNames[] = {" + ", ".join(names) + "};",
           "const char* const kJitHeaderTexts[] = {"]
    out += [t + "," for t in texts]
    out.append("};")
    text = "\n".join(out) + "\n"
    if not os.path.exists(JIT_INC) or open(JIT_INC).read() != text:
        tmp = JIT_INC + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            f.write(text)
        os.replace(tmp, JIT_INC)


def build(force: bool = False, verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers()
    _write_jit_headers()
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
    for name in ("api", "server", "png", "flame", "json", "variations_host", "hot_cells", "jit"):
        src = os.path.join(CSRC, name + ".cpp")
        obj = os.path.join(OUT, name + ".o")
        jobs.append((obj, [src] + hdrs + [JIT_INC], [*cxx_common, "-I", OUT, "-c", src, "-o", obj]))
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
