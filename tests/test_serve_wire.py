"""ffr-serve: the serving loop behind the framing of include/ffr_wire.h.

CPU: the frame layout the Python client writes matches the C header's
declared sizes and the command line's argument checks.  GPU: a client on
TCP submits a mix (2-D, 3-D, an initial buffer, a continuation), waits for
the buffers over the wire and checks each against a solo render; a second
connection waits on a job the first submitted; SHUTDOWN stops the process."""
import json
import os
import re
import struct
import subprocess
import time

import numpy as np
import pytest

from conftest import ROOT, golden_flame_text


def test_frame_sizes_match_header(ffr):
    text = open(os.path.join(ROOT, "include", "ffr_wire.h")).read()
    assert "} ffr_wire_request;         /* 72 bytes */" in text
    assert "} ffr_wire_response;        /* 80 bytes */" in text
    assert struct.calcsize(ffr._REQ) == 72 and struct.calcsize(ffr._RSP) == 80
    f = ffr.pack_request(ffr.WIRE_SUBMIT, samples=5, seed=6, json_text=b"{}", init=b"\x01" * 8)
    assert f[:4] == b"FFRQ" and len(f) == 72 + 2 + 8
    ops = dict(re.findall(r"FFR_WIRE_([A-Z]+) = (\d+)", text))
    assert int(ops["SUBMIT"]) == ffr.WIRE_SUBMIT and int(ops["SHUTDOWN"]) == ffr.WIRE_SHUTDOWN


def test_cli_needs_one_transport(ffr):
    r = subprocess.run([ffr.SERVE_CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 1 and "exactly one of --port and --stdio" in r.stderr
    r = subprocess.run([ffr.SERVE_CLI_PATH, "--port", "70000"], capture_output=True, text=True)
    assert r.returncode == 1 and "port out of range" in r.stderr


def _solo(ffr, text, n, seed, precision=1):
    with ffr.BufferRenderer(text, precision=precision, settle=20, traj_len=4096,
                            streams=max(1, -(-n // 4096))) as r:
        if n:
            r.render(n, seed)
        return r.write_buffer()


@pytest.mark.gpu
def test_serve_over_tcp(ffr, flames):
    p = subprocess.Popen([ffr.SERVE_CLI_PATH, "--port", "0", "--settle", "20"],
                         stderr=subprocess.PIPE, text=True)
    try:
        line = ""
        t0 = time.time()
        while "listening on" not in line and time.time() - t0 < 120:
            line = p.stderr.readline()
        port = int(line.strip().rsplit(":", 1)[1])
        c = ffr.RemoteServer("127.0.0.1", port)
        t2 = json.dumps(flames.random_2d(7, size=(320, 180)))
        t3 = json.dumps(flames.random_3d(5, size=(40, 40, 40)))
        tc = golden_flame_text("color")
        first = _solo(ffr, tc, 200_000, 3)
        a = c.submit(t2, 2_000_000, 11)
        b = c.submit(t3, 1_000_000, 12)
        d = c.submit(tc, 300_000, 13, init=first)
        e = c.continue_(a, 500_000, 14)
        rsp, buf = c.wait(b, with_buffer=True)
        assert rsp["state"] == ffr.JOB_DONE
        assert buf == _solo(ffr, t3, 1_000_000, 12)
        # a second connection waits on the first's job
        c2 = ffr.RemoteServer("127.0.0.1", port)
        c2.wait(e)
        c2.close()
        c.wait(a)
        got = np.frombuffer(c.read(a), dtype=np.uint64)
        want = np.frombuffer(_solo(ffr, t2, 2_000_000, 11), dtype=np.uint64) \
            + np.frombuffer(_solo(ffr, t2, 500_000, 14), dtype=np.uint64)
        np.testing.assert_array_equal(got, want)
        rsp, buf = c.wait(d, with_buffer=True)
        gd = np.frombuffer(buf, dtype=np.uint64).reshape(-1, 4)
        wd = np.frombuffer(_solo(ffr, tc, 300_000, 13), dtype=np.uint64).reshape(-1, 4)
        fd = np.frombuffer(first, dtype=np.uint64).reshape(-1, 4)
        np.testing.assert_array_equal(gd[:, 0], wd[:, 0] + fd[:, 0])
        np.testing.assert_allclose(gd[:, 1:].copy().view(np.float64),
                                   wd[:, 1:].copy().view(np.float64)
                                   + fd[:, 1:].copy().view(np.float64), rtol=1e-12, atol=1e-9)
        with pytest.raises(ffr.FfrError) as err:
            c.submit('{"dimensions": 2', 10, 1)
        assert err.value.status == ffr.FFR_ERR_PARSE
        for j in (a, b, d, e):
            c.release(j)
        c.shutdown()
        c.close()
        assert p.wait(timeout=60) == 0
    finally:
        if p.poll() is None:
            p.kill()
            p.wait()
