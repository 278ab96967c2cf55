"""TEST INFRASTRUCTURE ONLY: ctypes access to the two CPU checkers.

* ``Port``      -- oracle/liboracle_port.so, the C restatement of the upstream CPU
                   search mode (grand_oracle.c), which also returns the decoded
                   patterns, logical flips and ML costs;
* ``Reference`` -- oracle/_ref/libgranddecoder_ref.so, the upstream library
                   compiled unmodified from its sources (present only where the
                   upstream sources were available to build it).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product library never does.
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle_port.so")
REF_SO = os.path.join(HERE, "_ref", "libgranddecoder_ref.so")

RESULT_DTYPE = np.dtype([
    ("found", "<i4"), ("found_weight", "<i4"), ("original_weight", "<i4"),
    ("degenerate", "<i4"), ("is_equal", "<i4"), ("tam", "<i4"),
    ("total_tested_combinations", "<u8"), ("hibrido", "<i4"), ("iteration", "<i4"),
    ("time_sum_ms", "<f8"), ("total_time_search_ms", "<f8"),
    ("transfer_time_ms", "<f8"), ("total_to_find_ms", "<f8"),
], align=True)
assert RESULT_DTYPE.itemsize == 72

#: Result fields that do not depend on timing.
DETERMINISTIC_FIELDS = ("found", "found_weight", "original_weight", "degenerate", "is_equal",
                        "tam", "total_tested_combinations", "hibrido", "iteration")

UNIFORM, PROB, ML = 0, 1, 2


class Config(ctypes.Structure):
    _fields_ = [("max_error_weight", ctypes.c_int), ("threads_per_block", ctypes.c_int),
                ("use_gpu_sum", ctypes.c_int), ("max_size_active_positions", ctypes.c_int),
                ("threshold_for_hybrid", ctypes.c_int), ("mode_of_search", ctypes.c_int)]


def make_config(W, mode=-1, cap=300, thr=10, tpb=256, use_gpu_sum=0) -> Config:
    return Config(W, tpb, use_gpu_sum, cap, thr, mode)


def build(quiet: bool = True, ref_dir: str | None = None) -> None:
    """Compile the port, and the upstream library when ref_dir (default: the
    GRAND_REFERENCE_DIR environment variable) holds its sources."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-C", HERE, "port"], stdout=out)
    ref_dir = ref_dir or os.environ.get("GRAND_REFERENCE_DIR")
    if ref_dir:
        subprocess.call(["make", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], stdout=out, stderr=out)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a, ctype=ctypes.c_int):
    if a is None:
        return ctypes.POINTER(ctype)()
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _cstr(s):
    return None if s is None else os.fsencode(s)


@contextlib.contextmanager
def silence_stdout():
    """The upstream library prints one line per shot; send fd 1 to /dev/null."""
    import sys
    libc = ctypes.CDLL(None)
    sys.stdout.flush()
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(devnull, 1)
        yield
    finally:
        libc.fflush(None)
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)


class Port:
    """C restatement of the upstream CPU search mode."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        ip = ctypes.POINTER(ctypes.c_int)
        up = ctypes.POINTER(ctypes.c_ubyte)
        fp = ctypes.POINTER(ctypes.c_float)
        L.oracle_decode_css.argtypes = [ctypes.c_int, ip, ip, ctypes.c_int, ctypes.c_int, ip, ip,
                                        ctypes.c_int, ctypes.POINTER(Config), ctypes.c_void_p,
                                        ctypes.c_char, ctypes.c_char_p, up]
        L.oracle_decode_css.restype = ctypes.c_int
        L.oracle_decode_dem.argtypes = [ctypes.c_int, ip, ip, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ip, ip, ctypes.c_int,
                                        ctypes.POINTER(Config), ctypes.c_void_p, ctypes.c_char_p,
                                        up, up, fp]
        L.oracle_decode_dem.restype = ctypes.c_int
        L.oracle_ncr.argtypes = [ctypes.c_int, ctypes.c_int]
        L.oracle_ncr.restype = ctypes.c_ulonglong
        L.oracle_unrank.argtypes = [ctypes.c_ulonglong, ctypes.c_int, ctypes.c_int, ip]
        L.oracle_unrank.restype = None

    def css(self, variant, hx, hz, errors, syndromes, cfg, type_of_error="x", prob_file=None):
        hx, hz = _i32(hx), _i32(hz)
        n, m = hx.shape
        errors, syndromes = _i32(errors), _i32(syndromes)
        shots = (errors if errors is not None else syndromes).shape[0]
        res = np.zeros(shots, dtype=RESULT_DTYPE)
        dec = np.zeros((shots, m), dtype=np.uint8)
        rc = self.lib.oracle_decode_css(variant, _ptr(hx), _ptr(hz), n, m, _ptr(errors),
                                        _ptr(syndromes), shots, ctypes.byref(cfg),
                                        res.ctypes.data, type_of_error.encode()[:1],
                                        _cstr(prob_file), _ptr(dec, ctypes.c_ubyte))
        return rc, res, dec

    def dem(self, variant, h, l, detectors, logicals, cfg, file=None):
        h, l = _i32(h), _i32(l)
        n, m = h.shape
        nl = l.shape[1]
        detectors, logicals = _i32(detectors), _i32(logicals)
        shots = detectors.shape[0]
        res = np.zeros(shots, dtype=RESULT_DTYPE)
        dec = np.zeros((shots, m), dtype=np.uint8)
        dlog = np.zeros((shots, max(nl, 1)), dtype=np.uint8)
        cost = np.zeros(shots, dtype=np.float32)
        rc = self.lib.oracle_decode_dem(variant, _ptr(h), _ptr(l), n, m, nl, _ptr(detectors),
                                        _ptr(logicals), shots, ctypes.byref(cfg), res.ctypes.data,
                                        _cstr(file), _ptr(dec, ctypes.c_ubyte),
                                        _ptr(dlog, ctypes.c_ubyte), _ptr(cost, ctypes.c_float))
        return rc, res, dec, dlog[:, :nl], cost

    def ncr(self, n, k):
        return int(self.lib.oracle_ncr(n, k))

    def unrank(self, rank, n, k):
        out = (ctypes.c_int * max(k, 1))()
        self.lib.oracle_unrank(rank, n, k, out)
        return list(out)[:k]


class Reference:
    """The upstream library built from its own sources (CPU search mode only here)."""

    def __init__(self, path: str = REF_SO):
        self.lib = ctypes.CDLL(path)
        L = self.lib
        ip = ctypes.POINTER(ctypes.c_int)
        css = [ip, ip, ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_int, ctypes.POINTER(Config),
               ctypes.c_void_p, ctypes.c_char]
        dem = [ip, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_int,
               ctypes.POINTER(Config), ctypes.c_void_p]
        L.grand_decode_cc.argtypes = css
        L.grand_decode_prob_cc.argtypes = css + [ctypes.c_char_p]
        L.grand_decode_cln.argtypes = dem
        L.grand_decode_prob_cln.argtypes = dem + [ctypes.c_char_p]
        L.grand_decode_ML_cln.argtypes = dem + [ctypes.c_char_p]
        for f in ("grand_decode_cc", "grand_decode_prob_cc", "grand_decode_cln",
                  "grand_decode_prob_cln", "grand_decode_ML_cln"):
            getattr(L, f).restype = ctypes.c_int

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    def css(self, variant, hx, hz, errors, syndromes, cfg, type_of_error="x", prob_file=None):
        hx, hz = _i32(hx), _i32(hz)
        n, m = hx.shape
        errors, syndromes = _i32(errors), _i32(syndromes)
        shots = (errors if errors is not None else syndromes).shape[0]
        res = np.zeros(shots, dtype=RESULT_DTYPE)
        args = [_ptr(hx), _ptr(hz), n, m, _ptr(errors), _ptr(syndromes), shots,
                ctypes.byref(cfg), res.ctypes.data, type_of_error.encode()[:1]]
        with silence_stdout():
            if variant == PROB:
                rc = self.lib.grand_decode_prob_cc(*args, _cstr(prob_file))
            else:
                rc = self.lib.grand_decode_cc(*args)
        return rc, res

    def dem(self, variant, h, l, detectors, logicals, cfg, file=None):
        h, l = _i32(h), _i32(l)
        n, m = h.shape
        nl = l.shape[1]
        detectors, logicals = _i32(detectors), _i32(logicals)
        shots = detectors.shape[0]
        res = np.zeros(shots, dtype=RESULT_DTYPE)
        args = [_ptr(h), _ptr(l), n, m, nl, _ptr(detectors), _ptr(logicals), shots,
                ctypes.byref(cfg), res.ctypes.data]
        with silence_stdout():
            if variant == PROB:
                rc = self.lib.grand_decode_prob_cln(*args, _cstr(file))
            elif variant == ML:
                rc = self.lib.grand_decode_ML_cln(*args, _cstr(file))
            else:
                rc = self.lib.grand_decode_cln(*args)
        return rc, res


def fields_equal(a, b, fields=DETERMINISTIC_FIELDS):
    """Index list of shots whose deterministic fields differ."""
    bad = np.zeros(len(a), dtype=bool)
    for f in fields:
        bad |= a[f] != b[f]
    return np.nonzero(bad)[0]
