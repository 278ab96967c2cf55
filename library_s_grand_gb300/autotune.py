"""Autotuner for the engine's launch parameters.

Three knobs shape a launch and none of them changes a result:
  light_log2          largest per-iteration search (2^x candidates) finished by
                      the warp that triages the shot instead of becoming a Job
                      that every warp searches;
  tile_k              prefixes per lane in the masked colex tiles (weights 1-2,
                      and every weight when R > 256);
  search_ctas_per_sm  resident CTAs per SM of the persistent decode kernel (0:
                      the occupancy maximum).
The tuner times a workload's device decode (CUDA events around the control
reset and the decode kernel) over a small grid, keeps the fastest setting on the engine and
caches it in a JSON file keyed by the workload's name and the GPU.
"""
from __future__ import annotations

import json
import os

import numpy as np

DEFAULT_GRID = [(l, k, c) for l in (8, 10, 12, 14) for k in (2, 4) for c in (0, 2)]


def _cache_path():
    return os.environ.get("GRAND_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "grand_gb300_tune.json"))


def tune(engine, key, num_shots, d_records, d_results, stream, d_shot_code=0, d_offsets=0,
         grid=None, reps=3, use_cache=True):
    """Return (best (light_log2, tile_k, ctas), table of (setting, ms)) and apply it."""
    path = _cache_path()
    gpu = engine.device_info()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path, encoding="utf-8") as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    ck = f"{key}|{gpu}"
    if use_cache and ck in cache:
        best = tuple(cache[ck]["best"])
        engine.set_tuning(*best)
        return best, cache[ck]["table"]
    table = []
    for setting in (grid or DEFAULT_GRID):
        engine.set_tuning(*setting)
        times = []
        for _ in range(reps + 1):
            rc = engine.decode_device(num_shots, d_records, d_results, stream, d_shot_code,
                                      d_offsets, use_graph=False)
            if rc != 0 or engine.sync_status(stream) != 0:
                raise RuntimeError(f"decode failed under tuning {setting}")
            reset_ms, decode_ms = engine.kernel_times(stream)
            times.append(reset_ms + decode_ms)
        table.append((list(setting), float(np.median(times[1:]))))
    best = tuple(min(table, key=lambda t: t[1])[0])
    engine.set_tuning(*best)
    if use_cache:
        cache[ck] = {"best": list(best), "table": table}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w", encoding="utf-8") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return best, table
