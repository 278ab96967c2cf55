"""Upstream's per-shot stdout lines.

CPU: the upstream library built from its sources (oracle/_ref) decodes CSS shots
with and without supplied errors, prob-ordered CSS shots and DEM shots (uniform,
prob, ML) with its stdout captured; grand_format_result, which the decoders print
with GRAND_VERBOSE=1, must reproduce every line byte for byte from the result
records upstream returned (grand_decoder.cu:1230-1238, 1373-1380, 1651-1653 and
the matching lines of the other entry points).

GPU: the CUDA decoder run with GRAND_VERBOSE=1 in a child process prints, for a
golden fixture's shots, the lines upstream printed, timing fields masked (they
are measured times)."""
import contextlib
import ctypes
import os
import re
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import oracle as O
from conftest import ROOT, load_golden
from library_s_grand_gb300 import build as B
from library_s_grand_gb300 import capi, synth

CSS_SYN, CSS_ERR, DEM = 0, 1, 2
TIMES = re.compile(r"(time_sum_ms|total_time_search_ms|transfer_time_ms|total_to_find_ms)=[-0-9.e+inf]+")


@pytest.fixture(scope="module")
def lib():
    B.build()
    L = capi.load_library()
    L.grand_format_result.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p,
                                      ctypes.c_int]
    L.grand_format_result.restype = ctypes.c_int
    return L


def format_lines(L, kind, res):
    buf = ctypes.create_string_buffer(512)
    out = []
    for i in range(len(res)):
        n = L.grand_format_result(kind, res[i:i + 1].ctypes.data, i + 1, buf, 512)
        assert 0 < n < 512
        out.append(buf.value.decode())
    return out


@contextlib.contextmanager
def captured_stdout():
    """fd 1 into a temporary file for the duration; yields a list that receives its lines."""
    libc = ctypes.CDLL(None)
    sys.stdout.flush()
    saved = os.dup(1)
    lines = []
    with tempfile.TemporaryFile(mode="w+b") as f:
        os.dup2(f.fileno(), 1)
        try:
            yield lines
        finally:
            libc.fflush(None)
            os.dup2(saved, 1)
            os.close(saved)
            f.seek(0)
            lines.extend(f.read().decode().splitlines(keepends=True))


class _Upstream(O.Reference):
    """The upstream library with its stdout left in place (not sent to /dev/null)."""

    def run(self, call):
        saved = O.silence_stdout
        O.silence_stdout = contextlib.nullcontext
        try:
            return call()
        finally:
            O.silence_stdout = saved


@pytest.mark.skipif(not O.Reference.available(), reason="upstream library not built here")
def test_format_reproduces_upstream_stdout(lib, tmp_path):
    up = _Upstream()
    bb72 = synth.BB_CODES[72]()
    errors, syndromes = synth.css_shots(bb72.hz, 300, 0.03, seed=3)
    pf = synth.write_phase_file(str(tmp_path / "p.txt"), [(300, 0, 1, 2, 1.0, 0.0, 0.0)])
    dem = synth.random_dem(4, detectors=50, mechanisms=200, logicals=6, p_range=(2e-3, 2e-2))
    det, log, _ = synth.dem_shots(dem, 300, 5)
    lf = synth.write_llr_file(str(tmp_path / "l.txt"), dem.llr)
    cfg = O.make_config(3, cap=40)
    cases = [
        ("cc errors", CSS_ERR, lambda: up.css(O.UNIFORM, bb72.hx, bb72.hz, errors, None, cfg, "x")),
        ("cc syndromes", CSS_SYN, lambda: up.css(O.UNIFORM, bb72.hx, bb72.hz, None, syndromes, cfg, "x")),
        ("prob_cc errors", CSS_ERR, lambda: up.css(O.PROB, bb72.hx, bb72.hz, errors, None, cfg, "x", pf)),
        ("prob_cc syndromes", CSS_SYN, lambda: up.css(O.PROB, bb72.hx, bb72.hz, None, syndromes, cfg, "x", pf)),
        ("cln", DEM, lambda: up.dem(O.UNIFORM, dem.h, dem.l, det, log, cfg)),
        ("prob_cln", DEM, lambda: up.dem(O.PROB, dem.h, dem.l, det, log, O.make_config(6, cap=40), pf)),
        ("ML_cln", DEM, lambda: up.dem(O.ML, dem.h, dem.l, det, log, cfg, lf)),
    ]
    for what, kind, call in cases:
        with captured_stdout() as printed:
            rc, res = up.run(call)
        assert rc == 0, what
        printed = [ln for ln in printed if ln.startswith("shot ")]
        assert len(printed) == len(res), (what, len(printed))
        ours = format_lines(lib, kind, res)
        for i, (a, b) in enumerate(zip(ours, printed)):
            assert a == b, f"{what}, shot {i + 1}:\n ours     {a!r}\n upstream {b!r}"


CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from library_s_grand_gb300 import capi
g = dict(np.load(sys.argv[2], allow_pickle=False))
lib = capi.load_library()
cfg = capi.GrandDecoderConfig(*[int(v) for v in g["cfg"]])
if str(g["kind"]) == "css":
    rc, _ = capi.run_grand_shots_cc(lib, g["hx"], g["hz"], g.get("errors"), g.get("syndromes"),
                                    cfg, str(g["type"]).encode())
else:
    rc, _ = capi.run_grand_shots_cln(lib, g["h"], g["l"], g["detectors"], g["logicals"],
                                     int(g["l"].shape[1]), cfg)
sys.stdout.flush()
sys.exit(rc)
"""


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cc_bb72_x_err_w3", "cc_bb108_x_syn_w3", "cln_dem60_w3_cap20"])
def test_gpu_verbose_lines_match_upstream(lib, name):
    g = load_golden(name)
    kind = DEM if str(g["kind"]) == "dem" else (CSS_ERR if "errors" in g else CSS_SYN)
    want = [TIMES.sub(r"\1=T", ln) for ln in format_lines(lib, kind, g["res"])]
    env = dict(os.environ, GRAND_VERBOSE="1")
    out = subprocess.run([sys.executable, "-c", CHILD, ROOT,
                          os.path.join(ROOT, "tests", "golden", name + ".npz")],
                         capture_output=True, text=True, env=env, timeout=600)
    assert out.returncode == 0, out.stderr
    got = [TIMES.sub(r"\1=T", ln + "\n") for ln in out.stdout.splitlines() if ln.startswith("shot ")]
    assert len(got) == len(want)
    for i, (a, b) in enumerate(zip(got, want)):
        assert a == b, f"{name}, shot {i + 1}:\n GPU      {a!r}\n upstream {b!r}"
