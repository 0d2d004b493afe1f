"""The per-flame kernels (FFR_KERNEL_JIT) on the CPU: ffr_jit_prepare runs
NVRTC without a device, so the generated source of every variation type,
dimension count, final xform and colour flame is compiled here; the disk
cache and the argument checks too.  (Their buffers are checked against the
general kernel on the GPU, test_gpu_jit.py.)"""
import concurrent.futures as cf
import glob
import json
import os
import re

import jit_cases
from conftest import golden_flame_text

CASES = jit_cases.cases()


def test_cases_cover_every_variation():
    names = set()
    for text in CASES.values():
        for x in json.loads(text)["xforms"]:
            names.update(v["name"] for v in x["variations"])
    assert len(names) == 98


def test_prepare_compiles_every_case(ffr):
    """The plain per-flame kernel of every case in both precisions, and the
    xform-sorted one of a flame per dimension count (NVRTC compiles them in
    parallel)."""
    jobs = [(n, p, ffr.KERNEL_JIT) for n in sorted(CASES) for p in (ffr.FP64, ffr.FP32)]
    jobs += [(n, ffr.FP64, ffr.KERNEL_JIT_SORTED) for n in ("d1_group0", "d2_group0",
                                                            "d3_group0")]
    with cf.ThreadPoolExecutor(max(2, min(len(jobs), os.cpu_count() or 2))) as ex:
        res = list(ex.map(lambda j: ffr.jit_prepare(CASES[j[0]], j[1], j[2]), jobs))
    bad = [(j, r) for j, r in zip(jobs, res) if r[0] != ffr.FFR_OK]
    assert not bad, bad[:2]


def test_prepare_four_dimensions(ffr):
    for p in (ffr.FP64, ffr.FP32):
        st, msg = ffr.jit_prepare(golden_flame_text("d4_mixed"), p)
        assert st == ffr.FFR_OK, msg


def test_disk_cache_and_merged_programs(ffr, flames, tmp_path, monkeypatch):
    """FFR_JIT_CACHE holds a cubin and its key (the options and the source)
    per compiled structure; an FP32 flame of the benchmark types has no
    per-flame kernel (its precompiled merged instantiation runs) and
    prepares without compiling."""
    monkeypatch.setenv("FFR_JIT_CACHE", str(tmp_path))
    text = json.dumps(flames.random_2d(424242, k=5))
    assert ffr.jit_prepare(text, ffr.FP32)[0] == ffr.FFR_OK
    assert glob.glob(str(tmp_path / "*")) == []
    st, msg = ffr.jit_prepare(text, ffr.FP64, ffr.KERNEL_JIT)
    assert st == ffr.FFR_OK, msg
    keys = glob.glob(str(tmp_path / "ffr_*.key"))
    cubins = glob.glob(str(tmp_path / "ffr_*.cubin"))
    assert len(keys) == 1 and len(cubins) == 1
    key = open(keys[0]).read()
    # the options, a hash of the kernel headers the library embeds (a rebuilt
    # library never takes another build's cubin) and the source
    assert "--fmad=false" in key and "struct FlameSpec" in key
    assert re.search(r"^headers [0-9a-f]{16}$", key, re.M)
    assert os.path.getsize(cubins[0]) > 1000
    # same structure, other weights and affines: the same kernel
    other = json.loads(text)
    for x in other["xforms"]:
        x["weight"] *= 1.5
        x["pre_affine"]["b"] = [0.25, -0.25]
    assert ffr.jit_prepare(json.dumps(other), ffr.FP64, ffr.KERNEL_JIT)[0] == ffr.FFR_OK
    assert len(glob.glob(str(tmp_path / "ffr_*.key"))) == 1
    # the xform-sorted kernel of the structure: a second entry
    assert ffr.jit_prepare(text, ffr.FP64, ffr.KERNEL_JIT_SORTED)[0] == ffr.FFR_OK
    keys = sorted(glob.glob(str(tmp_path / "ffr_*.key")))
    assert len(keys) == 2
    assert sum("ffr_flame_sorted(" in open(k).read() for k in keys) == 1


def test_prepare_rejects_bad_input(ffr):
    st, msg = ffr.jit_prepare("{not json", ffr.FP64)
    assert st == ffr.FFR_ERR_PARSE
    st, msg = ffr.jit_prepare(json.dumps({"dimensions": 5, "size": [2] * 5,
                                          "bounds": [[-1, 1]] * 5, "xforms": []}), ffr.FP64)
    assert st == ffr.FFR_ERR_PARSE
    import ctypes
    lib = ffr.load_library()
    o = ffr.Opts()
    lib.ffr_default_opts(ctypes.byref(o))
    o.abi_version = 1
    raw = CASES["d1_group0"].encode()
    assert lib.ffr_jit_prepare(raw, len(raw), ctypes.byref(o)) == ffr.FFR_ERR_ARG
    assert lib.ffr_jit_prepare(None, 0, None) == ffr.FFR_ERR_ARG


def test_generated_source_fixes_slot_and_xform_types(ffr, tmp_path, monkeypatch):
    """The per-flame sources (read back from the FFR_JIT_CACHE key files)
    narrow each variation slot to the types it holds over the xforms (plain
    kernel) and write each xform out with its own types (sorted kernel)."""
    monkeypatch.setenv("FFR_JIT_CACHE", str(tmp_path))
    flame = {"dimensions": 2, "size": [32, 32], "bounds": [[-2, 2], [-2, 2]],
             "xforms": [{"weight": 1.0, "variations": [{"name": "handkerchief", "weight": 0.5},
                                                       {"name": "julia", "weight": 0.5}]},
                        {"weight": 0.5, "variations": [{"name": "spherical", "weight": 0.5},
                                                       {"name": "disc", "weight": 0.5}]}],
             "final_xform": {"variations": [{"name": "linear", "weight": 1.0}]}}
    assert ffr.jit_prepare(json.dumps(flame), ffr.FP32)[0] == ffr.FFR_OK
    keys = [open(k).read() for k in glob.glob(str(tmp_path / "ffr_*.key"))]
    plain = [k for k in keys if "ffr_flame_render(" in k]
    sorted_ = [k for k in keys if "ffr_flame_sorted(" in k]
    assert len(plain) == 1 and len(sorted_) == 1
    # slot 0: handkerchief (id 24) and the benchmark types spherical and
    # linear (kTa bits 4 | 1); slot 1: disc (id 26) and julia (bit 64)
    assert "SlotTypes<D, R, 5u, 24>" in plain[0]
    assert "SlotTypes<D, R, 64u, 26>" in plain[0]
    assert "static constexpr int slots = 2;" in plain[0]
    # xforms sorted by weight: xform 0 = handkerchief julia, xform 1 =
    # spherical disc, then the final (linear); 2-D pre-affines absent
    assert "FixedXform<D, R, 64u, false, false, 0, 24, 35>" in sorted_[0]
    assert "FixedXform<D, R, 4u, false, false, 2, 2, 26>" in sorted_[0]
    assert "FixedXform<D, R, 1u, false, false, 4, 0>" in sorted_[0]


def test_sorted_kernel_only_where_the_sorted_kernel_runs(ffr, tmp_path, monkeypatch):
    """Above 16 xforms the xform-sorted kernel does not run: preparing both
    kernels compiles the plain one only, and asking for the sorted one
    alone compiles nothing (renders then refuse FFR_KERNEL_JIT_SORTED)."""
    monkeypatch.setenv("FFR_JIT_CACHE", str(tmp_path))
    flame = {"dimensions": 2, "size": [16, 16], "bounds": [[-2, 2], [-2, 2]],
             "xforms": [{"weight": 1.0 + k, "variations": [{"name": "heart", "weight": 1.0}]}
                        for k in range(20)]}
    text = json.dumps(flame)
    assert ffr.jit_prepare(text, ffr.FP32, ffr.KERNEL_JIT_SORTED)[0] == ffr.FFR_OK
    assert glob.glob(str(tmp_path / "ffr_*.key")) == []
    assert ffr.jit_prepare(text, ffr.FP32)[0] == ffr.FFR_OK
    keys = [open(k).read() for k in glob.glob(str(tmp_path / "ffr_*.key"))]
    assert len(keys) == 1 and "ffr_flame_render(" in keys[0]
