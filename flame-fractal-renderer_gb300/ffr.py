"""ctypes binding of libffr_gpu.so (include/ffr_gpu.h).

The Python face of the reference's BufferRenderer<dims> interface
(src/renderers/buffer_renderer.hpp:254-584): construct from a flame JSON,
add_buffer / render / write_buffer / histogram, plus the verification entry
points (isaac_words, step, trace).  All work runs in the CUDA library; if it
cannot be loaded this module raises instead of computing anything itself.
"""
from __future__ import annotations

import ctypes
import json
import os
import threading
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libffr_gpu.so")
CLI_PATH = os.path.join(HERE, "_build", "ffr-buf")

FFR_ABI_VERSION = 4
MAX_DIMS = 4
MAX_XFORM_IDS = 4096
MAX_BAD_RECORDS = 4096

FFR_OK, FFR_BAD_VALUES, FFR_ERR_PARSE, FFR_ERR_ARG, FFR_ERR_IO, FFR_ERR_OOM, \
    FFR_ERR_TIMEOUT, FFR_ERR_CUDA, FFR_ERR_STATE = range(9)
STATUS_NAMES = ["FFR_OK", "FFR_BAD_VALUES", "FFR_ERR_PARSE", "FFR_ERR_ARG",
                "FFR_ERR_IO", "FFR_ERR_OOM", "FFR_ERR_TIMEOUT", "FFR_ERR_CUDA",
                "FFR_ERR_STATE"]
FP64, FP32 = 0, 1
KERNEL_AUTO, KERNEL_PLAIN, KERNEL_SORTED, KERNEL_HOT, KERNEL_JIT, KERNEL_JIT_SORTED = (
    0, 1, 2, 3, 4, 5)

# every symbol include/ffr_gpu.h declares
EXPORTS = [
    "ffr_default_opts", "ffr_create", "ffr_destroy", "ffr_jit_prepare", "ffr_last_error",
    "ffr_info", "ffr_size", "ffr_flame_json", "ffr_add_buffer", "ffr_render",
    "ffr_read_buffer", "ffr_load_buffer", "ffr_histogram", "ffr_clear",
    "ffr_isaac_words", "ffr_step", "ffr_trace", "ffr_plan",
    "ffr_measure_atomic_rate", "ffr_render_noalloc", "ffr_batch_create",
    "ffr_batch_destroy", "ffr_batch_render", "ffr_batch_last_error",
    "ffr_server_default_opts", "ffr_server_create", "ffr_server_destroy",
    "ffr_server_last_error", "ffr_server_submit", "ffr_server_continue",
    "ffr_server_poll", "ffr_server_wait", "ffr_server_job_stats", "ffr_server_read",
    "ffr_server_cancel", "ffr_server_release", "ffr_server_load",
    "ffr_render_image", "ffr_encode_png",
]
IMG_CLI_PATH = os.path.join(HERE, "_build", "ffr-img")
SERVE_CLI_PATH = os.path.join(HERE, "_build", "ffr-serve")
IMAGE_MONO, IMAGE_GRAY, IMAGE_RGB = 0, 1, 2

JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED, JOB_CANCELLED = range(5)


class FfrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES[status] if 0 <= status < 9 else status}: {message}")
        self.status = status
        self.message = message


class Opts(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_uint32), ("device", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("kernel", ctypes.c_int32),
                ("settle", ctypes.c_uint64), ("streams", ctypes.c_uint64),
                ("traj_len", ctypes.c_uint64), ("timeout_ms", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("samples_iterated", ctypes.c_uint64),
                ("samples_plotted", ctypes.c_uint64),
                ("bad_values", ctypes.c_uint64), ("dropped", ctypes.c_uint64),
                ("ext_lo", ctypes.c_double * MAX_DIMS),
                ("ext_hi", ctypes.c_double * MAX_DIMS),
                ("xform_ids", ctypes.c_uint64),
                ("xf_dist", ctypes.c_uint64 * MAX_XFORM_IDS),
                ("bad_recorded", ctypes.c_uint64),
                ("bad_xf", ctypes.c_uint64 * MAX_BAD_RECORDS),
                ("bad_pts", (ctypes.c_double * MAX_DIMS) * MAX_BAD_RECORDS),
                ("streams", ctypes.c_uint64), ("traj_len", ctypes.c_uint64),
                ("settle", ctypes.c_uint64), ("kernel_ms", ctypes.c_double),
                ("kernel", ctypes.c_int32), ("agg", ctypes.c_int32),
                ("hot_cells", ctypes.c_int32), ("aux_launches", ctypes.c_int32),
                ("ctas", ctypes.c_uint64), ("streams_per_thread", ctypes.c_uint64),
                ("ctas_per_sm", ctypes.c_int32), ("threads_per_cta", ctypes.c_int32)]


class ImageInfo(ctypes.Structure):
    _fields_ = [("hist_min", ctypes.c_uint64), ("hist_max", ctypes.c_uint64),
                ("scale_min", ctypes.c_double), ("scale_max", ctypes.c_double),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("channels", ctypes.c_uint32), ("bits", ctypes.c_uint32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_uint32), ("device", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("settle", ctypes.c_uint64), ("traj_len", ctypes.c_uint64),
                ("hbm_budget", ctypes.c_uint64), ("max_active", ctypes.c_uint64),
                ("round_chunks", ctypes.c_uint64), ("timeout_ms", ctypes.c_uint64)]


class JobInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("status", ctypes.c_int32),
                ("samples", ctypes.c_uint64), ("buffer_bytes", ctypes.c_uint64),
                ("parent", ctypes.c_uint64), ("submit_ns", ctypes.c_uint64),
                ("admit_ns", ctypes.c_uint64), ("done_ns", ctypes.c_uint64)]


_lib = None
_lock = threading.Lock()


def load_library(path: str = LIB_PATH):
    """Load libffr_gpu.so; raises OSError if it is missing (no fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise OSError(f"libffr_gpu.so not built at {path}; run "
                          "__graft_entry__.build() first")
        L = ctypes.CDLL(path)
        vp, u64, i32, sz = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_size_t
        L.ffr_default_opts.argtypes = [ctypes.POINTER(Opts)]
        L.ffr_default_opts.restype = None
        L.ffr_create.argtypes = [ctypes.c_char_p, sz, ctypes.POINTER(Opts), ctypes.POINTER(vp)]
        L.ffr_destroy.argtypes = [vp]
        L.ffr_destroy.restype = None
        L.ffr_jit_prepare.argtypes = [ctypes.c_char_p, sz, ctypes.POINTER(Opts)]
        L.ffr_last_error.argtypes = [vp]
        L.ffr_last_error.restype = ctypes.c_char_p
        L.ffr_info.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(u64),
                               ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(sz)]
        L.ffr_size.argtypes = [vp, ctypes.POINTER(u64)]
        L.ffr_flame_json.argtypes = [vp]
        L.ffr_flame_json.restype = ctypes.c_char_p
        L.ffr_add_buffer.argtypes = [vp, vp, sz]
        L.ffr_load_buffer.argtypes = [vp, vp, sz]
        L.ffr_read_buffer.argtypes = [vp, vp, sz]
        L.ffr_render.argtypes = [vp, u64, u64, u64, ctypes.POINTER(Stats)]
        L.ffr_histogram.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64),
                                    ctypes.POINTER(u64)]
        L.ffr_clear.argtypes = [vp]
        L.ffr_isaac_words.argtypes = [ctypes.c_int, u64, u64, vp]
        L.ffr_step.argtypes = [vp, ctypes.c_int, u64, u64, vp, vp]
        L.ffr_trace.argtypes = [vp, u64, u64, u64, vp, vp]
        L.ffr_plan.argtypes = [vp, u64, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.ffr_measure_atomic_rate.argtypes = [ctypes.c_int, u64, u64,
                                              ctypes.POINTER(ctypes.c_double)]
        L.ffr_batch_create.argtypes = [ctypes.POINTER(vp), sz, ctypes.POINTER(vp)]
        L.ffr_batch_destroy.argtypes = [vp]
        L.ffr_batch_destroy.restype = None
        L.ffr_batch_render.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64), u64,
                                       ctypes.POINTER(Stats)]
        L.ffr_batch_last_error.argtypes = [vp]
        L.ffr_batch_last_error.restype = ctypes.c_char_p
        L.ffr_render_noalloc.argtypes = [ctypes.c_char_p, sz, ctypes.POINTER(Opts), vp, vp,
                                         u64, u64, u64, u64, ctypes.POINTER(Stats)]
        P = ctypes.POINTER
        L.ffr_server_default_opts.argtypes = [P(ServerOpts)]
        L.ffr_server_default_opts.restype = None
        L.ffr_server_create.argtypes = [P(ServerOpts), P(vp)]
        L.ffr_server_destroy.argtypes = [vp]
        L.ffr_server_destroy.restype = None
        L.ffr_server_last_error.argtypes = [vp]
        L.ffr_server_last_error.restype = ctypes.c_char_p
        L.ffr_server_submit.argtypes = [vp, ctypes.c_char_p, sz, vp, sz, u64, u64, u64, P(u64)]
        L.ffr_server_continue.argtypes = [vp, u64, u64, u64, u64, P(u64)]
        L.ffr_server_poll.argtypes = [vp, u64, P(JobInfo)]
        L.ffr_server_wait.argtypes = [vp, u64, u64, P(JobInfo)]
        L.ffr_server_job_stats.argtypes = [vp, u64, P(Stats)]
        L.ffr_server_read.argtypes = [vp, u64, vp, sz]
        L.ffr_server_cancel.argtypes = [vp, u64]
        L.ffr_server_release.argtypes = [vp, u64]
        L.ffr_server_load.argtypes = [vp, P(u64), P(u64), P(u64), P(u64)]
        L.ffr_render_image.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_uint32,
                                       vp, sz, P(ImageInfo)]
        L.ffr_encode_png.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_uint32, vp, sz, P(sz)]
        for name in EXPORTS:
            f = getattr(L, name)
            if f.restype is ctypes.c_int:      # default: ffr_status
                f.restype = ctypes.c_int
        _lib = L
        return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(lib, ctx, status: int):
    if status not in (FFR_OK, FFR_BAD_VALUES):
        msg = lib.ffr_last_error(ctx).decode("utf-8", "replace")
        raise FfrError(status, msg)
    return status


@dataclass
class RenderStats:
    status: int
    samples_iterated: int
    samples_plotted: int
    bad_values: int
    dropped: int
    ext_lo: np.ndarray
    ext_hi: np.ndarray
    xf_dist: np.ndarray          # by JSON xform id
    bad_xf: np.ndarray
    bad_pts: np.ndarray
    streams: int
    traj_len: int
    settle: int
    kernel_ms: float
    kernel: int
    agg: int
    hot_cells: int = 0
    aux_launches: int = 0
    ctas: int = 0
    streams_per_thread: int = 0
    ctas_per_sm: int = 0
    threads_per_cta: int = 0

    @property
    def ok(self) -> bool:
        return self.status == FFR_OK


def _render_stats(status: int, st: Stats, n: int) -> RenderStats:
    nrec = st.bad_recorded
    ids = int(st.xform_ids)
    return RenderStats(
        status=status, samples_iterated=st.samples_iterated,
        samples_plotted=st.samples_plotted, bad_values=st.bad_values,
        dropped=st.dropped, ext_lo=np.array(st.ext_lo[:n]), ext_hi=np.array(st.ext_hi[:n]),
        xf_dist=np.array(st.xf_dist[:min(ids, MAX_XFORM_IDS)], dtype=np.uint64),
        bad_xf=np.array(st.bad_xf[:nrec], dtype=np.uint64),
        bad_pts=np.array([[st.bad_pts[k][i] for i in range(n)] for k in range(nrec)]).reshape(nrec, n),
        streams=st.streams, traj_len=st.traj_len, settle=st.settle,
        kernel_ms=st.kernel_ms, kernel=st.kernel, agg=st.agg, hot_cells=st.hot_cells,
        aux_launches=st.aux_launches, ctas=st.ctas, streams_per_thread=st.streams_per_thread,
        ctas_per_sm=st.ctas_per_sm, threads_per_cta=st.threads_per_cta)


def isaac_words(key: int, n: int, device: int = 0) -> np.ndarray:
    """Isaac<u64,4> words after setSeed(key), generated on the GPU."""
    lib = load_library()
    out = np.zeros(n, dtype=np.uint64)
    _check(lib, None, lib.ffr_isaac_words(device, key, n, _ptr(out)))
    return out


def measure_atomic_rate(cells: int, ops: int = 1 << 30, device: int = 0) -> float:
    """Relaxed u32 atomic adds per second at random cells (roofline peak)."""
    lib = load_library()
    out = ctypes.c_double()
    _check(lib, None, lib.ffr_measure_atomic_rate(device, cells, ops, ctypes.byref(out)))
    return out.value


class BufferRenderer:
    """GPU BufferRenderer: one flame, one device-resident count buffer."""

    def __init__(self, flame, precision: int = FP64, settle: int = 53,
                 streams: int = 0, traj_len: int = 0, device: int = 0,
                 timeout_ms: int = 0, kernel: int = KERNEL_AUTO):
        self._lib = load_library()
        text = flame if isinstance(flame, str) else json.dumps(flame)
        raw = text.encode("utf-8")
        o = Opts()
        self._lib.ffr_default_opts(ctypes.byref(o))
        o.device, o.precision, o.settle = device, precision, settle
        o.streams, o.traj_len, o.timeout_ms = streams, traj_len, timeout_ms
        o.kernel = kernel
        ctx = ctypes.c_void_p()
        st = self._lib.ffr_create(raw, len(raw), ctypes.byref(o), ctypes.byref(ctx))
        if st != FFR_OK:
            raise FfrError(st, self._lib.ffr_last_error(None).decode("utf-8", "replace"))
        self._ctx = ctx
        d, c, r, b = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_size_t()
        _check(self._lib, self._ctx, self._lib.ffr_info(self._ctx, ctypes.byref(d),
                                                        ctypes.byref(c), ctypes.byref(r),
                                                        ctypes.byref(b)))
        self.dims, self.cells, self.color_dims, self.buffer_bytes = d.value, c.value, r.value, b.value
        size = (ctypes.c_uint64 * MAX_DIMS)()
        _check(self._lib, self._ctx, self._lib.ffr_size(self._ctx, size))
        self.size = [size[i] for i in range(self.dims)]

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.ffr_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def flame_json(self) -> str:
        return self._lib.ffr_flame_json(self._ctx).decode("utf-8")

    def add_buffer(self, data) -> None:
        buf = np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray)) \
            else np.ascontiguousarray(data).view(np.uint8)
        _check(self._lib, self._ctx, self._lib.ffr_add_buffer(self._ctx, _ptr(buf), buf.nbytes))

    def load_buffer(self, data) -> None:
        buf = np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray)) \
            else np.ascontiguousarray(data).view(np.uint8)
        _check(self._lib, self._ctx, self._lib.ffr_load_buffer(self._ctx, _ptr(buf), buf.nbytes))

    def render(self, samples: int, seed: int, bad_limit: int = 256) -> RenderStats:
        st = Stats()
        status = _check(self._lib, self._ctx,
                        self._lib.ffr_render(self._ctx, samples, seed, bad_limit,
                                             ctypes.byref(st)))
        return _render_stats(status, st, self.dims)

    def plan(self, samples: int):
        s, L = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib, self._ctx, self._lib.ffr_plan(self._ctx, samples, ctypes.byref(s),
                                                        ctypes.byref(L)))
        return s.value, L.value

    def write_buffer(self) -> bytes:
        out = np.zeros(self.buffer_bytes, dtype=np.uint8)
        _check(self._lib, self._ctx, self._lib.ffr_read_buffer(self._ctx, _ptr(out), out.nbytes))
        return out.tobytes()

    def buffer_array(self) -> np.ndarray:
        """The file layout as a uint64 [cells, 1 + color_dims] array."""
        out = np.zeros((self.cells, 1 + self.color_dims), dtype=np.uint64)
        _check(self._lib, self._ctx, self._lib.ffr_read_buffer(self._ctx, _ptr(out), out.nbytes))
        return out

    def counts(self) -> np.ndarray:
        return self.buffer_array()[:, 0].copy()

    def histogram(self):
        s, mn, mx = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib, self._ctx, self._lib.ffr_histogram(self._ctx, ctypes.byref(s),
                                                             ctypes.byref(mn), ctypes.byref(mx)))
        return s.value, mn.value, mx.value

    def clear(self) -> None:
        _check(self._lib, self._ctx, self._lib.ffr_clear(self._ctx))

    def render_image(self, mode: int = IMAGE_GRAY, gamma: float = 1.0, bits: int = 8):
        """ffr-img's pixels of the buffer: (array [height, width(, 3)], info)."""
        pbits = 8 if mode == IMAGE_MONO else bits
        ch = 3 if mode == IMAGE_RGB else 1
        dt = np.uint8 if pbits == 8 else np.uint16
        w, h = self.size[0], self.size[1] if self.dims > 1 else 1
        out = np.zeros((h, w, ch), dtype=dt)
        info = ImageInfo()
        _check(self._lib, self._ctx, self._lib.ffr_render_image(
            self._ctx, mode, gamma, bits, _ptr(out), out.nbytes, ctypes.byref(info)))
        return (out if ch == 3 else out[:, :, 0]), info

    def step(self, xf_index: int, key: int, pts: np.ndarray) -> np.ndarray:
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        out = np.zeros_like(pts)
        _check(self._lib, self._ctx, self._lib.ffr_step(self._ctx, xf_index, key,
                                                        pts.shape[0], _ptr(pts), _ptr(out)))
        return out

    def trace(self, key: int, settle: int, n: int):
        ids = np.zeros(n, dtype=np.int32)
        pts = np.zeros((n, self.dims), dtype=np.float64)
        _check(self._lib, self._ctx, self._lib.ffr_trace(self._ctx, key, settle, n,
                                                         _ptr(ids), _ptr(pts)))
        return ids, pts


def encode_png(pixels: np.ndarray) -> bytes:
    """PNG file bytes of a [h, w] or [h, w, 3] u8/u16 array (ffr_encode_png)."""
    lib = load_library()
    a = np.ascontiguousarray(pixels)
    h, w = a.shape[0], a.shape[1]
    ch = 3 if a.ndim == 3 else 1
    bits = 8 * a.dtype.itemsize
    n = ctypes.c_size_t()
    lib.ffr_encode_png(_ptr(a), w, h, ch, bits, None, 0, ctypes.byref(n))
    out = np.zeros(n.value, dtype=np.uint8)
    st = lib.ffr_encode_png(_ptr(a), w, h, ch, bits, _ptr(out), out.nbytes, ctypes.byref(n))
    if st != FFR_OK:
        raise FfrError(st, "ffr_encode_png failed")
    return out.tobytes()


def create_status(flame_text: str, precision: int = FP64):
    """(status, message) of ffr_create without keeping the context."""
    lib = load_library()
    raw = flame_text.encode("utf-8")
    o = Opts()
    lib.ffr_default_opts(ctypes.byref(o))
    o.precision = precision
    ctx = ctypes.c_void_p()
    st = lib.ffr_create(raw, len(raw), ctypes.byref(o), ctypes.byref(ctx))
    msg = lib.ffr_last_error(None).decode("utf-8", "replace")
    if st == FFR_OK:
        lib.ffr_destroy(ctx)
    return st, msg


def jit_prepare(flame_text: str, precision: int = FP64, kernel: int = KERNEL_AUTO):
    """(status, message) of ffr_jit_prepare: compile the flame's per-flame
    kernels with NVRTC, without a device (kernel KERNEL_JIT or
    KERNEL_JIT_SORTED: that one; otherwise both)."""
    lib = load_library()
    raw = flame_text.encode("utf-8")
    o = Opts()
    lib.ffr_default_opts(ctypes.byref(o))
    o.precision = precision
    o.kernel = kernel
    st = lib.ffr_jit_prepare(raw, len(raw), ctypes.byref(o))
    return st, lib.ffr_last_error(None).decode("utf-8", "replace")


class Batch:
    """Several BufferRenderers rendered in one persistent launch per
    (dims, colour) group (ffr_batch_*); each buffer equals a solo render."""

    def __init__(self, renderers):
        self._lib = load_library()
        self.renderers = list(renderers)
        arr = (ctypes.c_void_p * len(self.renderers))(*[r._ctx.value for r in self.renderers])
        out = ctypes.c_void_p()
        st = self._lib.ffr_batch_create(arr, len(self.renderers), ctypes.byref(out))
        if st != FFR_OK:
            raise FfrError(st, self._lib.ffr_last_error(None).decode("utf-8", "replace"))
        self._b = out

    def render(self, samples, seeds, bad_limit: int = 256, stats: bool = True):
        n = len(self.renderers)
        sa = (ctypes.c_uint64 * n)(*samples)
        se = (ctypes.c_uint64 * n)(*seeds)
        sts = (Stats * n)() if stats else None
        status = self._lib.ffr_batch_render(self._b, sa, se, bad_limit, sts)
        if status not in (FFR_OK, FFR_BAD_VALUES):
            raise FfrError(status, self._lib.ffr_batch_last_error(self._b).decode("utf-8", "replace"))
        if not stats:
            return status, None
        out = []
        for i, r in enumerate(self.renderers):
            st = sts[i]
            d = r.dims
            out.append(RenderStats(
                status=status, samples_iterated=st.samples_iterated,
                samples_plotted=st.samples_plotted, bad_values=st.bad_values,
                dropped=st.dropped, ext_lo=np.array(st.ext_lo[:d]),
                ext_hi=np.array(st.ext_hi[:d]),
                xf_dist=np.array(st.xf_dist[:min(int(st.xform_ids), MAX_XFORM_IDS)], dtype=np.uint64),
                bad_xf=np.array(st.bad_xf[:st.bad_recorded], dtype=np.uint64),
                bad_pts=np.zeros((0, d)), streams=st.streams, traj_len=st.traj_len,
                settle=st.settle, kernel_ms=st.kernel_ms, kernel=st.kernel, agg=st.agg,
                hot_cells=st.hot_cells, aux_launches=st.aux_launches))
        return status, out

    def close(self):
        if getattr(self, "_b", None):
            self._lib.ffr_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


@dataclass
class Job:
    id: int
    state: int
    status: int
    samples: int
    buffer_bytes: int
    parent: int
    submit_ns: int
    admit_ns: int
    done_ns: int

    @property
    def finished(self) -> bool:
        return self.state in (JOB_DONE, JOB_FAILED, JOB_CANCELLED)

    @property
    def latency_s(self) -> float:
        return (self.done_ns - self.submit_ns) * 1e-9


class Server:
    """Serving loop (ffr_server_*): jobs submitted at any time run in
    continuously batched rounds with their buffers resident on the device."""

    def __init__(self, precision: int = FP32, settle: int = 53, traj_len: int = 4096,
                 device: int = 0, hbm_budget: int = 0, max_active: int = 256,
                 round_chunks: int = 0, timeout_ms: int = 0):
        self._lib = load_library()
        o = ServerOpts()
        self._lib.ffr_server_default_opts(ctypes.byref(o))
        o.device, o.precision, o.settle, o.traj_len = device, precision, settle, traj_len
        o.hbm_budget, o.max_active, o.round_chunks = hbm_budget, max_active, round_chunks
        o.timeout_ms = timeout_ms
        out = ctypes.c_void_p()
        st = self._lib.ffr_server_create(ctypes.byref(o), ctypes.byref(out))
        if st != FFR_OK:
            raise FfrError(st, self._lib.ffr_last_error(None).decode("utf-8", "replace"))
        self._s = out
        self.settle, self.traj_len = settle, traj_len

    def _check(self, status: int):
        if status not in (FFR_OK, FFR_BAD_VALUES):
            raise FfrError(status, self._lib.ffr_server_last_error(self._s).decode("utf-8", "replace"))
        return status

    def submit(self, flame, samples: int, seed: int, bad_limit: int = 256, init=None) -> int:
        text = flame if isinstance(flame, str) else json.dumps(flame)
        raw = text.encode("utf-8")
        job = ctypes.c_uint64()
        if init is None:
            ip, n = None, 0
        else:
            buf = np.frombuffer(init, dtype=np.uint8) if isinstance(init, (bytes, bytearray)) \
                else np.ascontiguousarray(init).view(np.uint8)
            ip, n = _ptr(buf), buf.nbytes
        self._check(self._lib.ffr_server_submit(self._s, raw, len(raw), ip, n, samples, seed,
                                                bad_limit, ctypes.byref(job)))
        return job.value

    def continue_(self, parent: int, samples: int, seed: int, bad_limit: int = 256) -> int:
        job = ctypes.c_uint64()
        self._check(self._lib.ffr_server_continue(self._s, parent, samples, seed, bad_limit,
                                                  ctypes.byref(job)))
        return job.value

    @staticmethod
    def _job(job: int, i: JobInfo) -> Job:
        return Job(job, i.state, i.status, i.samples, i.buffer_bytes, i.parent, i.submit_ns,
                   i.admit_ns, i.done_ns)

    def poll(self, job: int) -> Job:
        i = JobInfo()
        self._check(self._lib.ffr_server_poll(self._s, job, ctypes.byref(i)))
        return self._job(job, i)

    def wait(self, job: int, timeout_ms: int = 0) -> Job:
        i = JobInfo()
        self._check(self._lib.ffr_server_wait(self._s, job, timeout_ms, ctypes.byref(i)))
        return self._job(job, i)

    def stats(self, job: int, dims: int) -> RenderStats:
        st = Stats()
        status = self._check(self._lib.ffr_server_job_stats(self._s, job, ctypes.byref(st)))
        return _render_stats(status, st, dims)

    def read(self, job: int, cells: int, color_dims: int = 0) -> np.ndarray:
        """The job's buffer in the file layout, uint64 [cells, 1 + color_dims]."""
        out = np.zeros((cells, 1 + color_dims), dtype=np.uint64)
        self._check(self._lib.ffr_server_read(self._s, job, _ptr(out), out.nbytes))
        return out

    def read_into(self, job: int, ptr: int, nbytes: int) -> None:
        self._check(self._lib.ffr_server_read(self._s, job, ctypes.c_void_p(ptr), nbytes))

    def cancel(self, job: int) -> None:
        self._check(self._lib.ffr_server_cancel(self._s, job))

    def release(self, job: int) -> None:
        self._check(self._lib.ffr_server_release(self._s, job))

    def load(self):
        q, r, u, p = (ctypes.c_uint64() for _ in range(4))
        self._check(self._lib.ffr_server_load(self._s, ctypes.byref(q), ctypes.byref(r),
                                              ctypes.byref(u), ctypes.byref(p)))
        return {"queued": q.value, "running": r.value, "bytes_used": u.value,
                "bytes_peak": p.value}

    def close(self):
        if getattr(self, "_s", None):
            self._lib.ffr_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---------------------------------------------------------------- wire client
# Framing of include/ffr_wire.h (little-endian, packed).
WIRE_VERSION = 1
WIRE_SUBMIT, WIRE_CONTINUE, WIRE_WAIT, WIRE_READ, WIRE_POLL, WIRE_CANCEL, WIRE_RELEASE, \
    WIRE_SHUTDOWN = range(1, 9)
WIRE_WITH_BUFFER = 1
_REQ = "<4sIII7Q"           # 72 bytes
_RSP = "<4sIQII7Q"          # 80 bytes


def pack_request(op: int, job: int = 0, samples: int = 0, seed: int = 0, bad_limit: int = 256,
                 timeout_ms: int = 0, flags: int = 0, json_text: bytes = b"",
                 init: bytes = b"") -> bytes:
    import struct
    return struct.pack(_REQ, b"FFRQ", WIRE_VERSION, op, flags, job, samples, seed, bad_limit,
                       timeout_ms, len(json_text), len(init)) + json_text + init


def unpack_response(head: bytes) -> dict:
    import struct
    (magic, status, job, state, job_status, samples, buffer_bytes, parent, submit_ns, admit_ns,
     done_ns, payload_len) = struct.unpack(_RSP, head)
    if magic != b"FFRR":
        raise FfrError(FFR_ERR_IO, "bad response frame")
    return {"status": status, "job": job, "state": state, "job_status": job_status,
            "samples": samples, "buffer_bytes": buffer_bytes, "parent": parent,
            "submit_ns": submit_ns, "admit_ns": admit_ns, "done_ns": done_ns,
            "payload_len": payload_len}


class RemoteServer:
    """Client of ffr-serve over a socket (or any pair of binary streams)."""

    def __init__(self, host: str = "127.0.0.1", port: int = 0, rfile=None, wfile=None):
        import socket
        if rfile is None:
            self._sock = socket.create_connection((host, port))
            self._r = self._sock.makefile("rb")
            self._w = self._sock.makefile("wb")
        else:
            self._sock, self._r, self._w = None, rfile, wfile

    def _call(self, frame: bytes):
        import struct
        self._w.write(frame)
        self._w.flush()
        head = self._r.read(struct.calcsize(_RSP))
        if len(head) != struct.calcsize(_RSP):
            raise FfrError(FFR_ERR_IO, "connection closed")
        rsp = unpack_response(head)
        payload = self._r.read(rsp["payload_len"]) if rsp["payload_len"] else b""
        if rsp["status"] not in (FFR_OK, FFR_BAD_VALUES):
            raise FfrError(rsp["status"], payload.decode("utf-8", "replace"))
        return rsp, payload

    def submit(self, flame, samples: int, seed: int, bad_limit: int = 256, init: bytes = b""):
        text = flame if isinstance(flame, str) else json.dumps(flame)
        return self._call(pack_request(WIRE_SUBMIT, samples=samples, seed=seed,
                                       bad_limit=bad_limit, json_text=text.encode(),
                                       init=init))[0]["job"]

    def continue_(self, parent: int, samples: int, seed: int, bad_limit: int = 256):
        return self._call(pack_request(WIRE_CONTINUE, job=parent, samples=samples, seed=seed,
                                       bad_limit=bad_limit))[0]["job"]

    def wait(self, job: int, timeout_ms: int = 0, with_buffer: bool = False):
        return self._call(pack_request(WIRE_WAIT, job=job, timeout_ms=timeout_ms,
                                       flags=WIRE_WITH_BUFFER if with_buffer else 0))

    def read(self, job: int) -> bytes:
        return self._call(pack_request(WIRE_READ, job=job))[1]

    def poll(self, job: int) -> dict:
        return self._call(pack_request(WIRE_POLL, job=job))[0]

    def cancel(self, job: int) -> None:
        self._call(pack_request(WIRE_CANCEL, job=job))

    def release(self, job: int) -> None:
        self._call(pack_request(WIRE_RELEASE, job=job))

    def shutdown(self) -> None:
        self._call(pack_request(WIRE_SHUTDOWN))

    def close(self):
        for f in (self._r, self._w):
            try:
                f.close()
            except Exception:
                pass
        if self._sock is not None:
            self._sock.close()
