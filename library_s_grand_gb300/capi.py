"""ctypes binding of libgranddecoder.so.

Mirrors the upstream Python interface (Examples/auxilary_functions.py:9-35 for
the structs, :172-253 for ``load_library`` and its argtypes, :255-394 for the
``run_grand_*`` wrappers): same names, same argument meaning, same
``(rc, results)`` return values, so code written against the upstream library
runs unchanged.  The ``*_ex`` wrappers additionally return the decoded error
patterns, decoded logical flips and ML costs.

The library is the in-tree CUDA build; there is no CPU fallback: loading
fails loudly when it has not been built.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_LIB = os.path.join(HERE, "libgranddecoder.so")


class GrandDecoderConfig(ctypes.Structure):
    _fields_ = [
        ("max_error_weight", ctypes.c_int),
        ("threads_per_block", ctypes.c_int),
        ("use_gpu_sum", ctypes.c_int),
        ("max_size_active_positions", ctypes.c_int),
        ("threshold_for_hybrid", ctypes.c_int),
        ("mode_of_search", ctypes.c_int),
    ]


class GrandDecoderResult(ctypes.Structure):
    _fields_ = [
        ("found", ctypes.c_int),
        ("found_weight", ctypes.c_int),
        ("original_weight", ctypes.c_int),
        ("degenerate", ctypes.c_int),
        ("is_equal", ctypes.c_int),
        ("tam", ctypes.c_int),
        ("total_tested_combinations", ctypes.c_ulonglong),
        ("hibrido", ctypes.c_int),
        ("iteration", ctypes.c_int),
        ("time_sum_ms", ctypes.c_double),
        ("total_time_search_ms", ctypes.c_double),
        ("transfer_time_ms", ctypes.c_double),
        ("total_to_find_ms", ctypes.c_double),
    ]


class GrandDecodeOutputs(ctypes.Structure):
    _fields_ = [
        ("decoded_errors", ctypes.POINTER(ctypes.c_ubyte)),
        ("decoded_logicals", ctypes.POINTER(ctypes.c_ubyte)),
        ("ml_cost", ctypes.POINTER(ctypes.c_float)),
    ]


assert ctypes.sizeof(GrandDecoderConfig) == 24
assert ctypes.sizeof(GrandDecoderResult) == 72

RESULT_DTYPE = np.dtype([
    ("found", "<i4"), ("found_weight", "<i4"), ("original_weight", "<i4"),
    ("degenerate", "<i4"), ("is_equal", "<i4"), ("tam", "<i4"),
    ("total_tested_combinations", "<u8"), ("hibrido", "<i4"), ("iteration", "<i4"),
    ("time_sum_ms", "<f8"), ("total_time_search_ms", "<f8"),
    ("transfer_time_ms", "<f8"), ("total_to_find_ms", "<f8"),
], align=True)

IP = ctypes.POINTER(ctypes.c_int)
_CSS = [IP, IP, ctypes.c_int, ctypes.c_int, IP, IP, ctypes.c_int,
        ctypes.POINTER(GrandDecoderConfig), ctypes.POINTER(GrandDecoderResult), ctypes.c_char]
_DEM = [IP, IP, ctypes.c_int, ctypes.c_int, ctypes.c_int, IP, IP, ctypes.c_int,
        ctypes.POINTER(GrandDecoderConfig), ctypes.POINTER(GrandDecoderResult)]
_OUT = ctypes.POINTER(GrandDecodeOutputs)

#: Every symbol include/grand_decoder.h declares, with its argtypes.
SIGNATURES = {
    "grand_decode_cc": (_CSS, ctypes.c_int),
    "grand_decode_prob_cc": (_CSS + [ctypes.c_char_p], ctypes.c_int),
    "grand_decode_cln": (_DEM, ctypes.c_int),
    "grand_decode_prob_cln": (_DEM + [ctypes.c_char_p], ctypes.c_int),
    "grand_decode_ML_cln": (_DEM + [ctypes.c_char_p], ctypes.c_int),
    "grand_decode_cc_ex": (_CSS + [_OUT], ctypes.c_int),
    "grand_decode_prob_cc_ex": (_CSS + [ctypes.c_char_p, _OUT], ctypes.c_int),
    "grand_decode_cln_ex": (_DEM + [_OUT], ctypes.c_int),
    "grand_decode_prob_cln_ex": (_DEM + [ctypes.c_char_p, _OUT], ctypes.c_int),
    "grand_decode_ML_cln_ex": (_DEM + [ctypes.c_char_p, _OUT], ctypes.c_int),
    "grand_decode_cc_noalloc": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_int, ctypes.POINTER(GrandDecoderConfig),
                                 ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "grand_decode_cc_packed": ([IP, IP, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                ctypes.c_int, ctypes.POINTER(GrandDecoderConfig),
                                ctypes.POINTER(GrandDecoderResult), ctypes.c_char, ctypes.c_char_p],
                               ctypes.c_int),
    "grand_decode_cln_packed": ([IP, IP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(GrandDecoderConfig),
                                 ctypes.POINTER(GrandDecoderResult), ctypes.c_int, ctypes.c_char_p],
                                ctypes.c_int),
    "grand_version": ([], ctypes.c_char_p),
    "grand_last_error": ([], ctypes.c_char_p),
}


def load_library(lib_path: str | None = None):
    """Load libgranddecoder.so and declare every entry point (upstream
    load_library, Examples/auxilary_functions.py:172-253)."""
    path = lib_path or os.environ.get("GRAND_LIB") or DEFAULT_LIB
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} not found: build it with `python -m library_s_grand_gb300.build`")
    lib = ctypes.CDLL(path)
    for name, (argtypes, restype) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = argtypes
        fn.restype = restype
    return lib


def _flat(a):
    return np.ascontiguousarray(np.asarray(a).ravel(), dtype=np.int32)


def _p(a):
    return a.ctypes.data_as(IP)


def _outputs(shots, m, nl, ml):
    dec = np.zeros((shots, m), dtype=np.uint8)
    dlog = np.zeros((shots, max(nl, 1)), dtype=np.uint8)
    cost = np.zeros(shots, dtype=np.float32)
    o = GrandDecodeOutputs(dec.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
                           dlog.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)) if nl else None,
                           cost.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if ml else None)
    return o, dec, dlog[:, :nl], cost


def results_array(results) -> np.ndarray:
    """Copy a ctypes GrandDecoderResult array into a numpy structured array."""
    n = len(results)
    buf = np.frombuffer((ctypes.c_char * (72 * n)).from_address(ctypes.addressof(results)),
                        dtype=RESULT_DTYPE, count=n)
    return buf.copy()


def _css_args(Hx, Hz, errors, syndromes):
    n_rows, n_cols = np.asarray(Hx).shape
    hx, hz = _flat(Hx), _flat(Hz)
    null = IP()
    if errors is not None:
        shots = np.asarray(errors).shape[0]
        e = _flat(errors)
        return (hx, hz, e), [_p(hx), _p(hz), n_rows, n_cols, _p(e), null, shots], shots, n_cols
    shots = np.asarray(syndromes).shape[0]
    s = _flat(syndromes)
    return (hx, hz, s), [_p(hx), _p(hz), n_rows, n_cols, null, _p(s), shots], shots, n_cols


def run_grand_shots_cc(lib, Hx, Hz, errors, syndromes, cfg, error_type):
    keep, args, shots, _ = _css_args(Hx, Hz, errors, syndromes)
    results = (GrandDecoderResult * shots)()
    rc = lib.grand_decode_cc(*args, ctypes.byref(cfg), results, ctypes.c_char(error_type))
    return rc, results


def run_grand_prob_shots_cc(lib, Hx, Hz, errors, syndromes, cfg, prob_file_path, error_type):
    keep, args, shots, _ = _css_args(Hx, Hz, errors, syndromes)
    results = (GrandDecoderResult * shots)()
    rc = lib.grand_decode_prob_cc(*args, ctypes.byref(cfg), results, ctypes.c_char(error_type),
                                  prob_file_path.encode("utf-8"))
    return rc, results


def _dem_args(H_dem, L_dem, detectors, logicals, n_logicos):
    n_rows, n_cols = np.asarray(H_dem).shape
    h, l = _flat(H_dem), _flat(L_dem)
    d, g = _flat(detectors), _flat(logicals)
    shots = np.asarray(detectors).shape[0]
    return (h, l, d, g), [_p(h), _p(l), n_rows, n_cols, n_logicos, _p(d), _p(g), shots], shots, n_cols


def run_grand_shots_cln(lib, H_dem, L_dem, detectors, logicals, n_logicos, cfg):
    keep, args, shots, _ = _dem_args(H_dem, L_dem, detectors, logicals, n_logicos)
    results = (GrandDecoderResult * shots)()
    rc = lib.grand_decode_cln(*args, ctypes.byref(cfg), results)
    return rc, results


def run_grand_prob_shots_cln(lib, H_dem, L_dem, detectors, logicals, n_logicos, cfg,
                             prob_file_path):
    keep, args, shots, _ = _dem_args(H_dem, L_dem, detectors, logicals, n_logicos)
    results = (GrandDecoderResult * shots)()
    rc = lib.grand_decode_prob_cln(*args, ctypes.byref(cfg), results,
                                   prob_file_path.encode("utf-8"))
    return rc, results


def run_grand_ML_shots_cln(lib, H_dem, L_dem, detectors, logicals, n_logicos, cfg, llr_file_path):
    keep, args, shots, _ = _dem_args(H_dem, L_dem, detectors, logicals, n_logicos)
    results = (GrandDecoderResult * shots)()
    rc = lib.grand_decode_ML_cln(*args, ctypes.byref(cfg), results, llr_file_path.encode("utf-8"))
    return rc, results


# ---- extensions: decoded patterns, logical flips, ML costs -------------------

def decode_css_ex(lib, variant, Hx, Hz, errors, syndromes, cfg, error_type, prob_file=None):
    """variant: "uniform" or "prob".  Returns (rc, results ndarray, decoded errors)."""
    keep, args, shots, m = _css_args(Hx, Hz, errors, syndromes)
    results = (GrandDecoderResult * shots)()
    out, dec, _, _ = _outputs(shots, m, 0, False)
    et = ctypes.c_char(error_type if isinstance(error_type, bytes) else error_type.encode())
    if variant == "prob":
        rc = lib.grand_decode_prob_cc_ex(*args, ctypes.byref(cfg), results, et,
                                         os.fsencode(prob_file), ctypes.byref(out))
    else:
        rc = lib.grand_decode_cc_ex(*args, ctypes.byref(cfg), results, et, ctypes.byref(out))
    return rc, results_array(results), dec


def decode_dem_ex(lib, variant, H_dem, L_dem, detectors, logicals, cfg, file=None):
    """variant: "uniform", "prob" or "ml".  Returns (rc, results ndarray,
    decoded errors, decoded logical flips, ML costs)."""
    nl = int(np.asarray(L_dem).shape[1])
    keep, args, shots, m = _dem_args(H_dem, L_dem, detectors, logicals, nl)
    results = (GrandDecoderResult * shots)()
    out, dec, dlog, cost = _outputs(shots, m, nl, variant == "ml")
    if variant == "prob":
        rc = lib.grand_decode_prob_cln_ex(*args, ctypes.byref(cfg), results, os.fsencode(file),
                                          ctypes.byref(out))
    elif variant == "ml":
        rc = lib.grand_decode_ML_cln_ex(*args, ctypes.byref(cfg), results, os.fsencode(file),
                                        ctypes.byref(out))
    else:
        rc = lib.grand_decode_cln_ex(*args, ctypes.byref(cfg), results, ctypes.byref(out))
    return rc, results_array(results), dec, dlog, cost


PACKED_SYNDROMES, PACKED_ERRORS = 0, 1


def pack_bits(rows) -> np.ndarray:
    """(shots, entries) 0/1 array -> (shots, ceil(entries/32)) uint32 words, LSB-first:
    bit i of word k is entry 32k + i (the layout of the *_packed entry points)."""
    a = (np.asarray(rows) != 0).astype(np.uint8)
    shots, n = a.shape
    words = (n + 31) // 32
    pad = np.zeros((shots, words * 32), dtype=np.uint8)
    pad[:, :n] = a
    b = np.packbits(pad.reshape(shots, words * 4, 8), axis=2, bitorder="little")
    return np.ascontiguousarray(b.reshape(shots, words * 4)).view("<u4").reshape(shots, words)


def _type_byte(error_type) -> bytes:
    return error_type if isinstance(error_type, bytes) else str(error_type).encode()


def run_grand_shots_cc_packed(lib, Hx, Hz, words, kind, cfg, error_type, prob_file=None):
    """Bit-packed CSS records in the style of the run_grand_* helpers: returns
    (rc, ctypes GrandDecoderResult array) without converting the results."""
    n_rows, n_cols = np.asarray(Hx).shape
    hx, hz = _flat(Hx), _flat(Hz)
    w = np.ascontiguousarray(words, dtype=np.uint32)
    shots = w.shape[0]
    results = (GrandDecoderResult * shots)()
    rc = lib.grand_decode_cc_packed(_p(hx), _p(hz), n_rows, n_cols, w.ctypes.data, kind, shots,
                                    ctypes.byref(cfg), results, ctypes.c_char(_type_byte(error_type)),
                                    os.fsencode(prob_file) if prob_file else None)
    return rc, results


def decode_css_packed(lib, Hx, Hz, words, kind, cfg, error_type, prob_file=None):
    """Bit-packed CSS records (pack_bits layout).  kind: PACKED_SYNDROMES or
    PACKED_ERRORS; prob_file None searches as grand_decode_cc, otherwise as
    grand_decode_prob_cc.  Returns (rc, results ndarray)."""
    n_rows, n_cols = np.asarray(Hx).shape
    hx, hz = _flat(Hx), _flat(Hz)
    w = np.ascontiguousarray(words, dtype=np.uint32)
    shots = w.shape[0]
    results = (GrandDecoderResult * shots)()
    rc = lib.grand_decode_cc_packed(_p(hx), _p(hz), n_rows, n_cols, w.ctypes.data, kind, shots,
                                    ctypes.byref(cfg), results, ctypes.c_char(_type_byte(error_type)),
                                    os.fsencode(prob_file) if prob_file else None)
    return rc, results_array(results)


def decode_dem_packed(lib, variant, H_dem, L_dem, det_words, log_words, cfg, file=None):
    """Bit-packed DEM records (pack_bits layout); variant "uniform", "prob" or "ml".
    Returns (rc, results ndarray)."""
    n_rows, n_cols = np.asarray(H_dem).shape
    nl = int(np.asarray(L_dem).shape[1])
    h, l = _flat(H_dem), _flat(L_dem)
    d = np.ascontiguousarray(det_words, dtype=np.uint32)
    g = np.ascontiguousarray(log_words, dtype=np.uint32)
    shots = d.shape[0]
    results = (GrandDecoderResult * shots)()
    v = {"uniform": 0, "prob": 1, "ml": 2}[variant]
    rc = lib.grand_decode_cln_packed(_p(h), _p(l), n_rows, n_cols, nl, d.ctypes.data, g.ctypes.data,
                                     shots, ctypes.byref(cfg), results, v,
                                     os.fsencode(file) if file else None)
    return rc, results_array(results)
