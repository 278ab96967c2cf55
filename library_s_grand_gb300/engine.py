"""Python handle on the batched engine (include/grand_engine.h)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import capi

VP = ctypes.c_void_p
IP = capi.IP

_SIGS = {
    "grand_engine_create": ([ctypes.POINTER(VP)], ctypes.c_int),
    "grand_engine_destroy": ([VP], None),
    "grand_engine_add_css": ([VP, IP, IP, ctypes.c_int, ctypes.c_int, ctypes.c_char, ctypes.c_int,
                              ctypes.POINTER(capi.GrandDecoderConfig), ctypes.c_char_p,
                              ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "grand_engine_add_dem": ([VP, IP, IP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.POINTER(capi.GrandDecoderConfig), ctypes.c_int,
                              ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "grand_engine_record_len": ([VP, ctypes.c_int], ctypes.c_int),
    "grand_engine_decode": ([VP, ctypes.c_int, IP, IP, VP, ctypes.POINTER(capi.GrandDecodeOutputs)],
                            ctypes.c_int),
    "grand_engine_decode_device": ([VP, ctypes.c_int, VP, VP, VP, VP, VP, ctypes.c_int],
                                   ctypes.c_int),
    "grand_engine_sync_status": ([VP, VP], ctypes.c_int),
    "grand_engine_decode_plain": ([VP, ctypes.c_int, IP, IP, VP], ctypes.c_int),
    "grand_engine_set_tuning": ([VP, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "grand_engine_kernel_times": ([VP, VP, ctypes.POINTER(ctypes.c_float),
                                   ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "grand_engine_batch_times": ([VP] + [ctypes.POINTER(ctypes.c_float)] * 4, ctypes.c_int),
    "grand_engine_launch_stats": ([VP, VP, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "grand_engine_sample": ([VP, ctypes.c_int, VP, ctypes.c_ulonglong, ctypes.c_ulonglong,
                             ctypes.c_int, VP, VP], ctypes.c_int),
    "grand_measure_int_peak": ([], ctypes.c_double),
    "grand_device_info": ([ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
}
capi.SIGNATURES.update(_SIGS)

UNIFORM, PROB, ML = 0, 1, 2


def declare(lib):
    for name, (a, r) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = a
        fn.restype = r
    return lib


class Engine:
    """Registered codes stay resident on the GPU; batches may mix codes."""

    def __init__(self, lib=None):
        self.lib = declare(lib or capi.load_library())
        h = VP()
        rc = self.lib.grand_engine_create(ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"grand_engine_create failed ({rc})")
        self.h = h
        self.rec_lens = []
        self.widths = []

    def close(self):
        if self.h:
            self.lib.grand_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_css(self, hx, hz, type_of_error, records_are_errors, cfg, prob_file=None) -> int:
        hx = np.ascontiguousarray(hx, dtype=np.int32)
        hz = np.ascontiguousarray(hz, dtype=np.int32)
        cid = ctypes.c_int(-1)
        rc = self.lib.grand_engine_add_css(
            self.h, hx.ctypes.data_as(IP), hz.ctypes.data_as(IP), hx.shape[0], hx.shape[1],
            ctypes.c_char(type_of_error.encode() if isinstance(type_of_error, str) else type_of_error),
            int(bool(records_are_errors)), ctypes.byref(cfg),
            os.fsencode(prob_file) if prob_file else None, ctypes.byref(cid))
        if rc != 0:
            raise RuntimeError(f"grand_engine_add_css failed ({rc})")
        self.rec_lens.append(self.lib.grand_engine_record_len(self.h, cid.value))
        self.widths.append(hx.shape[1])
        return cid.value

    def add_dem(self, h, l, cfg, variant=UNIFORM, file=None) -> int:
        h = np.ascontiguousarray(h, dtype=np.int32)
        l = np.ascontiguousarray(l, dtype=np.int32)
        cid = ctypes.c_int(-1)
        rc = self.lib.grand_engine_add_dem(self.h, h.ctypes.data_as(IP), l.ctypes.data_as(IP),
                                           h.shape[0], h.shape[1], l.shape[1], ctypes.byref(cfg),
                                           variant, os.fsencode(file) if file else None,
                                           ctypes.byref(cid))
        if rc != 0:
            raise RuntimeError(f"grand_engine_add_dem failed ({rc})")
        self.rec_lens.append(self.lib.grand_engine_record_len(self.h, cid.value))
        self.widths.append(h.shape[1])
        return cid.value

    def set_tuning(self, light_log2=10, tile_k=4, search_ctas_per_sm=0):
        rc = self.lib.grand_engine_set_tuning(self.h, light_log2, tile_k, search_ctas_per_sm)
        if rc != 0:
            raise ValueError("bad tuning")

    def decode(self, records, shot_code=None, num_shots=None, decoded=False):
        """records: flat int32 array of concatenated shot records."""
        rec = np.ascontiguousarray(records, dtype=np.int32).ravel()
        sc = None if shot_code is None else np.ascontiguousarray(shot_code, dtype=np.int32)
        n = len(sc) if sc is not None else (num_shots or len(rec) // self.rec_lens[0])
        res = np.zeros(n, dtype=capi.RESULT_DTYPE)
        out = None
        dec = None
        if decoded:
            dec = np.zeros((n, self.widths[0]), dtype=np.uint8)
            out = capi.GrandDecodeOutputs(dec.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
                                          None, None)
        rc = self.lib.grand_engine_decode(self.h, n, sc.ctypes.data_as(IP) if sc is not None else None,
                                          rec.ctypes.data_as(IP), res.ctypes.data,
                                          ctypes.byref(out) if out is not None else None)
        return (rc, res, dec) if decoded else (rc, res)

    def decode_plain(self, records, shot_code=None, num_shots=None):
        rec = np.ascontiguousarray(records, dtype=np.int32).ravel()
        sc = None if shot_code is None else np.ascontiguousarray(shot_code, dtype=np.int32)
        n = len(sc) if sc is not None else (num_shots or len(rec) // self.rec_lens[0])
        res = np.zeros(n, dtype=capi.RESULT_DTYPE)
        rc = self.lib.grand_engine_decode_plain(self.h, n, sc.ctypes.data_as(IP) if sc is not None else None,
                                                rec.ctypes.data_as(IP), res.ctypes.data)
        return rc, res

    def decode_device(self, num_shots, d_records, d_results, stream=0, d_shot_code=0,
                      d_offsets=0, use_graph=True):
        return self.lib.grand_engine_decode_device(self.h, num_shots, d_shot_code or None,
                                                   d_offsets or None, d_records, d_results,
                                                   stream or None, int(bool(use_graph)))

    def sync_status(self, stream=0):
        return self.lib.grand_engine_sync_status(self.h, stream or None)

    def kernel_times(self, stream=0):
        a, b = ctypes.c_float(), ctypes.c_float()
        rc = self.lib.grand_engine_kernel_times(self.h, stream or None, ctypes.byref(a), ctypes.byref(b))
        return (a.value, b.value) if rc == 0 else (None, None)

    def sample(self, code_id, d_p, seed, first_shot, num_shots, d_records, stream=0):
        """Draw shots of a registered code on the device (device pointers d_p: m FP32
        flip probabilities, d_records: num_shots * record_len int32)."""
        return self.lib.grand_engine_sample(self.h, code_id, d_p, seed, first_shot, num_shots,
                                            d_records, stream or None)

    def launch_stats(self, stream=0):
        """(settled by classification, per-shot path, Jobs, tiles, scratch words) of the
        last device decode on `stream`."""
        out = (ctypes.c_longlong * 31)()
        rc = self.lib.grand_engine_launch_stats(self.h, stream or None, out)
        return tuple(out[:5]) if rc == 0 else None

    def launch_profile(self, stream=0):
        """Phase profile of the last device decode on `stream` (the engine created
        with GRAND_PROFILE=1): warp-ns per kind of work, when the last of each kind
        ended (ns after the first warp started) and the number of work steps."""
        out = (ctypes.c_longlong * 31)()
        rc = self.lib.grand_engine_launch_stats(self.h, stream or None, out)
        if rc != 0:
            return None
        kinds = ("chunks", "shots", "tiles", "wait")
        parts = ("chunk_read", "chunk_test", "chunk_write", "shot_pack", "shot_counts",
                 "shot_light", "shot_publish", "shot_finish", "tile_setup", "tile_finish")
        return {"warp_ns": dict(zip(kinds, out[5:9])), "last_end_ns": dict(zip(kinds, out[9:13])),
                "steps": out[13], "split_warp_ns": dict(zip(parts, out[14:24])),
                "publish_warp_ns": dict(zip(("reserve", "stage", "write", "ready"), out[24:28])),
                "last_shot_start_ns": out[28], "longest_shot_ns": out[29],
                "longest_tile_draw_ns": out[30]}

    def batch_times(self):
        """(h2d, control reset, decode kernel, d2h) ms of the last host-buffer decode."""
        v = [ctypes.c_float() for _ in range(4)]
        rc = self.lib.grand_engine_batch_times(self.h, *[ctypes.byref(x) for x in v])
        return tuple(x.value for x in v) if rc == 0 else None

    def int_peak(self):
        return self.lib.grand_measure_int_peak()

    def device_info(self) -> str:
        buf = ctypes.create_string_buffer(256)
        self.lib.grand_device_info(buf, 256)
        return buf.value.decode()


def offsets_for(rec_lens, shot_code):
    """int64 record offsets for a shot-code sequence."""
    lens = np.asarray(rec_lens, dtype=np.int64)[np.asarray(shot_code)]
    off = np.zeros(len(lens), dtype=np.int64)
    if len(lens) > 1:
        np.cumsum(lens[:-1], out=off[1:])
    return off
