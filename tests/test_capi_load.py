"""The C ABI library loads and exports what include/*.h declares (no GPU calls),
and every validation failure upstream reports before touching the GPU returns
the same code here, also without a GPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from library_s_grand_gb300 import build as B
from library_s_grand_gb300 import capi
from library_s_grand_gb300 import synth as S


@pytest.fixture(scope="module")
def lib():
    B.build()
    return capi.load_library()


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h, encoding="utf-8").read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text):
            name = m.group(1)
            if name.startswith("grand_"):
                names.add(name)
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "grand_decode_cc" in names and "grand_decode_ML_cln" in names
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"


def test_struct_layout_matches_upstream_ctypes_mirror():
    # Examples/auxilary_functions.py:9-35 declares these exact field lists.
    cfg_fields = [f for f, _ in capi.GrandDecoderConfig._fields_]
    assert cfg_fields == ["max_error_weight", "threads_per_block", "use_gpu_sum",
                          "max_size_active_positions", "threshold_for_hybrid", "mode_of_search"]
    offs = {f: getattr(capi.GrandDecoderResult, f).offset for f, _ in capi.GrandDecoderResult._fields_}
    assert offs["total_tested_combinations"] == 24 and offs["hibrido"] == 32
    assert offs["time_sum_ms"] == 40 and offs["total_to_find_ms"] == 64
    assert ctypes.sizeof(capi.GrandDecoderResult) == 72


def test_upstream_argtypes_contract(lib):
    """The upstream load_library argtypes (auxilary_functions.py:175-251) bind."""
    IP = ctypes.POINTER(ctypes.c_int)
    lib2 = ctypes.CDLL(lib._name)
    lib2.grand_decode_cc.argtypes = [IP, IP, ctypes.c_int, ctypes.c_int, IP, IP, ctypes.c_int,
                                     ctypes.POINTER(capi.GrandDecoderConfig),
                                     ctypes.POINTER(capi.GrandDecoderResult), ctypes.c_char]
    lib2.grand_decode_cc.restype = ctypes.c_int
    c = S.BB_CODES[72]()
    e = np.zeros((2, 72), dtype=np.int32)
    cfg = capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1)
    rc, res = capi.run_grand_shots_cc(lib2, c.hx, c.hz, e, None, cfg, b"q")
    assert rc == -1  # invalid type_of_error is rejected before any GPU work


def _cfg(W, mode=-1):
    return capi.GrandDecoderConfig(W, 256, 0, 64, 10, mode)


@pytest.mark.parametrize("W", [0, 8, -1])
def test_invalid_weight_rejected_without_gpu(lib, W, capfd):
    c = S.BB_CODES[72]()
    e = np.zeros((1, 72), dtype=np.int32)
    rc, _ = capi.run_grand_shots_cc(lib, c.hx, c.hz, e, None, _cfg(W), b"x")
    assert rc == -1
    assert "Invalid max_error_weight" in capfd.readouterr().err
    dem = S.random_dem(0, 10, 30, 2)
    det = np.zeros((1, 10), dtype=np.int32)
    log = np.zeros((1, 2), dtype=np.int32)
    rc, _ = capi.run_grand_shots_cln(lib, dem.h, dem.l, det, log, 2, _cfg(W))
    assert rc == -1


def test_prob_weight_message_matches_upstream(lib, tmp_path, capfd):
    c = S.BB_CODES[72]()
    pf = S.write_phase_file(str(tmp_path / "p.txt"), [(300, 0, 1, 2, 1, 0, 0)])
    e = np.zeros((1, 72), dtype=np.int32)
    rc, _ = capi.run_grand_prob_shots_cc(lib, c.hx, c.hz, e, None, _cfg(9), pf, b"x")
    assert rc == -1
    assert "Must be 6 or 7" in capfd.readouterr().err


def test_missing_files_rejected(lib, tmp_path, capfd):
    c = S.BB_CODES[72]()
    e = np.zeros((1, 72), dtype=np.int32)
    rc, _ = capi.run_grand_prob_shots_cc(lib, c.hx, c.hz, e, None, _cfg(3),
                                         str(tmp_path / "none.txt"), b"x")
    assert rc == -1
    err = capfd.readouterr().err
    assert "Error opening probability file" in err and "No phase order masks" in err
    dem = S.random_dem(0, 10, 30, 2)
    det = np.zeros((1, 10), dtype=np.int32)
    log = np.zeros((1, 2), dtype=np.int32)
    rc, _ = capi.run_grand_prob_shots_cln(lib, dem.h, dem.l, det, log, 2, _cfg(3),
                                          str(tmp_path / "none.txt"))
    assert rc == -1
    rc, _ = capi.run_grand_ML_shots_cln(lib, dem.h, dem.l, det, log, 2, _cfg(3),
                                        str(tmp_path / "none.txt"))
    assert rc == -1
    assert "Error opening LLR file" in capfd.readouterr().err
    short = tmp_path / "short.txt"
    short.write_text("1.0\n2.0\n")
    rc, _ = capi.run_grand_ML_shots_cln(lib, dem.h, dem.l, det, log, 2, _cfg(3), str(short))
    assert rc == -1
    assert "expected 30 values" in capfd.readouterr().err
    bad = tmp_path / "nan.txt"
    bad.write_text("nan\n" + "1.0\n" * 29)
    rc, _ = capi.run_grand_ML_shots_cln(lib, dem.h, dem.l, det, log, 2, _cfg(3), str(bad))
    assert rc == -1


def test_zero_shots_returns_zero_without_gpu(lib):
    c = S.BB_CODES[72]()
    e = np.zeros((0, 72), dtype=np.int32)
    cfg = _cfg(3)
    res = (capi.GrandDecoderResult * 1)()
    rc = lib.grand_decode_cc(c.hx.ctypes.data_as(capi.IP), c.hz.ctypes.data_as(capi.IP), 36, 72,
                             e.ctypes.data_as(capi.IP), capi.IP(), 0, ctypes.byref(cfg), res,
                             ctypes.c_char(b"x"))
    assert rc == 0


def test_version_string(lib):
    assert b"sm_103a" in lib.grand_version()


def test_packed_kind_rejected_without_gpu(lib, capfd):
    c = S.BB_CODES[72]()
    words = np.zeros((2, 2), dtype=np.uint32)
    rc, _ = capi.decode_css_packed(lib, c.hx, c.hz, words, 7, _cfg(3), b"x")
    assert rc == -1
    assert "packed record kind" in capfd.readouterr().err


def test_pack_bits_layout():
    a = (np.random.default_rng(0).random((6, 70)) < 0.3).astype(np.int32)
    w = capi.pack_bits(a)
    assert w.shape == (6, 3) and w.dtype == np.uint32
    for i in range(6):
        for j in range(70):
            assert (int(w[i, j // 32]) >> (j % 32)) & 1 == a[i, j]
