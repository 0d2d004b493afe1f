"""Host-side checks that need no GPU: the C-ABI library loads and exports
every symbol include/ffr_gpu.h declares, flame validation through the ABI
rejects what the reference rejects, the CLI's argument handling, and the
flame generators."""
import json
import os
import re
import subprocess

import pytest

from conftest import ROOT, golden_manifest

MAN = golden_manifest()


def header_functions():
    text = open(os.path.join(ROOT, "include", "ffr_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ffr_[a-z_]+)\s*\(", text)))


def test_header_lists_exports(ffr):
    assert header_functions() == sorted(ffr.EXPORTS)


def test_library_exports_every_declared_symbol(ffr):
    lib = ffr.load_library()
    for name in header_functions():
        assert hasattr(lib, name), name
    out = subprocess.check_output(["nm", "-D", "--defined-only", ffr.LIB_PATH], text=True)
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert exported == set(header_functions())


# the ctypes mirrors of the header's structs, field by field
STRUCTS = {"ffr_opts": "Opts", "ffr_stats": "Stats", "ffr_image_info": "ImageInfo",
           "ffr_server_opts": "ServerOpts", "ffr_job_info": "JobInfo"}


def test_struct_layouts_match_ctypes(ffr, tmp_path):
    """sizeof and every field offset of the header's structs, compiled by
    the C compiler, against the ctypes classes the binding uses."""
    lines = []
    for cname, pyname in STRUCTS.items():
        cls = getattr(ffr, pyname)
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "ffr_gpu.h"\n'
                   "int main(void) {\n" + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src),
                           "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    import ctypes
    for cname, pyname in STRUCTS.items():
        cls = getattr(ffr, pyname)
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)


@pytest.mark.parametrize("name", sorted(MAN["invalid"]))
def test_invalid_flames_rejected_through_abi(ffr, name):
    case = MAN["invalid"][name]
    st, msg = ffr.create_status(case["text"])
    assert st == ffr.FFR_ERR_PARSE, (st, msg)
    assert msg


@pytest.mark.parametrize("name", sorted(MAN["valid_edge"]))
def test_valid_flames_pass_validation(ffr, name):
    st, msg = ffr.create_status(MAN["valid_edge"][name]["text"])
    # parsing happens before any CUDA call: without a GPU the create fails
    # at device setup, never at validation
    assert st in (ffr.FFR_OK, ffr.FFR_ERR_CUDA, ffr.FFR_ERR_OOM), (st, msg)


def test_unknown_variation_message(ffr):
    st, msg = ffr.create_status(MAN["invalid"]["unknown_var"]["text"])
    assert st == ffr.FFR_ERR_PARSE and "unknown variation: nope" in msg


def test_default_opts(ffr):
    import ctypes
    o = ffr.Opts()
    ffr.load_library().ffr_default_opts(ctypes.byref(o))
    assert o.abi_version == ffr.FFR_ABI_VERSION
    assert o.settle == 53 and o.precision == ffr.FP64 and o.streams == 0


def test_abi_version_matches_header(ffr):
    text = open(os.path.join(ROOT, "include", "ffr_gpu.h")).read()
    m = re.search(r"#define FFR_ABI_VERSION (\d+)", text)
    assert m and int(m.group(1)) == ffr.FFR_ABI_VERSION


def test_kernel_option_range(ffr):
    """ffr_create accepts FFR_KERNEL_AUTO..FFR_KERNEL_HOT and rejects other
    values before any device work (so this runs without a GPU)."""
    import ctypes
    lib = ffr.load_library()
    raw = json.dumps({"dimensions": 1, "size": [8], "bounds": [[-1, 1]],
                      "xforms": [{"weight": 1, "variations": [{"name": "linear",
                                                               "weight": 1}]}]}).encode()
    for kernel, rejected in ((-1, True), (6, True), (ffr.KERNEL_HOT, False),
                             (ffr.KERNEL_JIT, False), (ffr.KERNEL_JIT_SORTED, False)):
        o = ffr.Opts()
        lib.ffr_default_opts(ctypes.byref(o))
        o.kernel = kernel
        ctx = ctypes.c_void_p()
        st = lib.ffr_create(raw, len(raw), ctypes.byref(o), ctypes.byref(ctx))
        msg = lib.ffr_last_error(None).decode()
        if st == ffr.FFR_OK:
            lib.ffr_destroy(ctx)
        assert (st == ffr.FFR_ERR_ARG and "kernel" in msg) == rejected, (kernel, st, msg)


def test_isaac_words_rejects_null(ffr):
    lib = ffr.load_library()
    assert lib.ffr_isaac_words(0, 1, 4, None) == ffr.FFR_ERR_ARG


def test_null_context_is_an_argument_error(ffr):
    lib = ffr.load_library()
    assert lib.ffr_render(None, 10, 1, 256, None) == ffr.FFR_ERR_ARG
    assert lib.ffr_read_buffer(None, None, 0) == ffr.FFR_ERR_ARG
    assert lib.ffr_last_error(None)


def run_cli(ffr, args, stdin=None):
    return subprocess.run([ffr.CLI_PATH, *args], input=stdin, stdout=subprocess.PIPE,
                          stderr=subprocess.PIPE)


def test_cli_usage(ffr):
    r = run_cli(ffr, [])
    assert r.returncode == 1 and b"ffr-buf usage" in r.stderr
    r = run_cli(ffr, ["-h"])
    assert r.returncode == 1 and b"--flame" in r.stderr


def test_cli_missing_required(ffr, tmp_path):
    r = run_cli(ffr, ["-o", str(tmp_path / "o.buf")])
    assert r.returncode == 1 and b"--flame" in r.stderr
    r = run_cli(ffr, ["-f", "x.json"])
    assert r.returncode == 1 and b"--output" in r.stderr


def test_cli_bad_option_value(ffr):
    r = run_cli(ffr, ["-f", "-", "-o", "-", "-s", "abc"])
    assert r.returncode == 1 and b"invalid" in r.stderr
    r = run_cli(ffr, ["-f", "-", "-o", "-", "-s", "10", "--kernel", "fast"])
    assert r.returncode == 1 and b"--kernel must be" in r.stderr


def test_cli_rejects_bad_flame(ffr, tmp_path):
    p = tmp_path / "bad.json"
    p.write_text(MAN["invalid"]["bad_bounds"]["text"])
    r = run_cli(ffr, ["-f", str(p), "-o", str(tmp_path / "o.buf")])
    assert r.returncode == 1
    assert b"ERROR:" in r.stderr and b"low >= high" in r.stderr


@pytest.mark.parametrize("args,msg", [
    (["-s", "1000", "-t", "0"], b"BufferRenderer::render(): threads must be positive"),
    (["-s", "1000", "-t", "65536"], b"BufferRenderer::render(): too many threads"),
    (["-s", "1000", "-b", "255"], b"BufferRenderer::render(): batch size too small"),
    (["-s", "1000", "-b", "1"], b"BufferRenderer::render(): batch size too small"),
])
def test_cli_render_argument_checks(ffr, tmp_path, args, msg):
    """render()'s checks of threads and batch size (buffer_renderer.hpp:277-285),
    made before any device work."""
    r = run_cli(ffr, ["-f", str(tmp_path / "none.json"), "-o", str(tmp_path / "o.buf"), *args])
    assert r.returncode == 1 and msg in r.stderr, r.stderr


def test_cli_render_argument_checks_need_samples(ffr, tmp_path):
    """With no samples render() returns before its checks: -t 0 and -b 1 pass
    and the command fails only at the missing flame file."""
    r = run_cli(ffr, ["-f", str(tmp_path / "none.json"), "-o", str(tmp_path / "o.buf"),
                      "-t", "0", "-b", "1"])
    assert r.returncode == 1 and b"BufferRenderer" not in r.stderr
    assert b"cannot open flame file" in r.stderr


@pytest.mark.parametrize("samples,batch", [(1000, 4096), (10**7, 39063), (10**12, 1 << 20),
                                           (0, 4096)])
def test_cli_automatic_batch_size(ffr, tmp_path, samples, batch):
    """-b 0 is the reference's clamp((N + 255) >> 8, 4096, 2^20)
    (ffr_buf.cpp:94-101), echoed before the flame is read."""
    r = run_cli(ffr, ["-f", str(tmp_path / "none.json"), "-o", str(tmp_path / "o.buf"),
                      "-s", str(samples), "-t", "4"])
    assert f"--batch_size 0 ({batch})\n".encode() in r.stderr, r.stderr
    lines = r.stderr.decode().splitlines()
    assert lines.index("--threads 4") + 1 == lines.index(f"--batch_size 0 ({batch})")


def test_cli_explicit_batch_and_trajectories_echo(ffr, tmp_path):
    base = ["-f", str(tmp_path / "none.json"), "-o", str(tmp_path / "o.buf"), "-s", "100000"]
    r = run_cli(ffr, base + ["-b", "300"])
    assert b"--batch_size 300\n" in r.stderr
    # --trajectories: N samples from T trajectories may mean fewer than 256
    # samples each (the project's extension; no batch check applies)
    r = run_cli(ffr, base + ["--trajectories", "1000"])
    assert b"--batch_size 100\n" in r.stderr and b"too small" not in r.stderr
    r = run_cli(ffr, base + ["--trajectories", "10", "-b", "300"])
    assert r.returncode == 1 and b"excludes" in r.stderr


def test_flame_generators_are_seeded(flames):
    a = json.dumps(flames.random_2d(7))
    b = json.dumps(flames.random_2d(7))
    c = json.dumps(flames.random_2d(8))
    assert a == b and a != c
    f3 = flames.random_3d(5)
    for x in f3["xforms"]:
        for v in x["variations"]:
            if v["name"] in flames.TWO_D:
                assert v["axis_x"] != v["axis_y"]


def test_generated_flames_parse_in_oracle(fo, flames):
    for fl in (flames.sierpinski_2d(), flames.tetrahedron_3d(), flames.random_2d(7),
               flames.random_3d(5), flames.heavy_point_2d()):
        f = fo.load_flame(json.dumps(fl))
        assert abs(sum(x.weight for x in f.xforms) / sum(x.weight for x in f.xforms) - 1) == 0


def test_heavy_point_flame_concentrates(fo, flames):
    """The hot-cell test flame (oracle, CPU): its 64 hottest cells hold most
    of the samples, far above the 1/50 a hot-cell table needs."""
    import numpy as np
    of = fo.OracleFlame(fo.load_flame(json.dumps(flames.heavy_point_2d((64, 64)))))
    r = fo.render(of, 1, 256, 200_000, 500, 20)
    c = np.sort(r.counts)[::-1]
    assert c[:64].sum() > 0.9 * c.sum()
