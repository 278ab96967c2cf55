"""Python handle on the continuous-batching server (include/grand_server.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from .engine import Engine

VP = ctypes.c_void_p
IP = capi.IP
DP = ctypes.POINTER(ctypes.c_double)

_SIGS = {
    "grand_server_create": ([VP, ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(VP)],
                            ctypes.c_int),
    "grand_server_destroy": ([VP], None),
    "grand_server_info": ([VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t)],
                          ctypes.c_int),
    "grand_server_submit": ([VP, ctypes.c_int, IP, IP, VP, ctypes.POINTER(ctypes.c_ulonglong)],
                            ctypes.c_int),
    "grand_server_wait": ([VP, ctypes.c_ulonglong, ctypes.c_int, DP], ctypes.c_int),
    "grand_server_replay": ([VP, ctypes.c_int, DP, IP, IP, IP, VP, DP, DP], ctypes.c_int),
}
capi.SIGNATURES.update(_SIGS)


class Server:
    """Continuous batching over `slots` micro-batches in flight on one GPU."""

    def __init__(self, engine: Engine, slots=4, max_shots_per_batch=4096, hbm_budget_bytes=0):
        self.engine = engine
        self.lib = engine.lib
        for name, (a, r) in _SIGS.items():
            fn = getattr(self.lib, name)
            fn.argtypes = a
            fn.restype = r
        h = VP()
        rc = self.lib.grand_server_create(engine.h, slots, max_shots_per_batch, hbm_budget_bytes,
                                          ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"grand_server_create failed ({rc})")
        self.h = h
        self.max_shots = max_shots_per_batch
        self._pending = {}

    def info(self):
        s, b = ctypes.c_int(), ctypes.c_size_t()
        self.lib.grand_server_info(self.h, ctypes.byref(s), ctypes.byref(b))
        return s.value, b.value

    def submit(self, records, shot_code=None, num_shots=None) -> int:
        rec = np.ascontiguousarray(records, dtype=np.int32).ravel()
        sc = None if shot_code is None else np.ascontiguousarray(shot_code, dtype=np.int32)
        n = len(sc) if sc is not None else (num_shots or len(rec) // self.engine.rec_lens[0])
        res = np.zeros(n, dtype=capi.RESULT_DTYPE)
        rid = ctypes.c_ulonglong()
        rc = self.lib.grand_server_submit(self.h, n, sc.ctypes.data_as(IP) if sc is not None else None,
                                          rec.ctypes.data_as(IP), res.ctypes.data, ctypes.byref(rid))
        if rc != 0:
            raise RuntimeError(f"grand_server_submit failed ({rc})")
        self._pending[rid.value] = (rec, sc, res)  # keep the buffers alive
        return rid.value

    def wait(self, rid, timeout_ms=-1):
        lat = ctypes.c_double()
        rc = self.lib.grand_server_wait(self.h, rid, timeout_ms, ctypes.byref(lat))
        if rc == 1:
            return 1, None, None
        _, _, res = self._pending.pop(rid)
        return rc, res, lat.value

    def replay(self, arrival_s, num_shots, records, shot_code=None):
        arr = np.ascontiguousarray(arrival_s, dtype=np.float64)
        ns = np.ascontiguousarray(num_shots, dtype=np.int32)
        rec = np.ascontiguousarray(records, dtype=np.int32).ravel()
        sc = None if shot_code is None else np.ascontiguousarray(shot_code, dtype=np.int32)
        res = np.zeros(int(ns.sum()), dtype=capi.RESULT_DTYPE)
        lat = np.zeros(len(ns), dtype=np.float64)
        wall = ctypes.c_double()
        rc = self.lib.grand_server_replay(self.h, len(ns), arr.ctypes.data_as(DP), ns.ctypes.data_as(IP),
                                          sc.ctypes.data_as(IP) if sc is not None else None,
                                          rec.ctypes.data_as(IP), res.ctypes.data,
                                          lat.ctypes.data_as(DP), ctypes.byref(wall))
        return rc, res, lat, wall.value

    def close(self):
        if self.h:
            self.lib.grand_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
