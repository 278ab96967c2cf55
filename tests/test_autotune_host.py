"""The autotuner's host logic (library_s_grand_gb300.autotune) against a fake
engine whose kernel times are a known function of the setting: the fastest
setting is chosen from medians that drop the first (warm-up) run, applied to
the engine, written to the cache under the workload and GPU, and read back
from the cache without timing again; a failing decode raises."""
import json

import pytest

from library_s_grand_gb300 import autotune


class FakeEngine:
    def __init__(self, cost, gpu="GB300 sm_103", fail=None):
        self.cost, self.gpu, self.fail = cost, gpu, fail
        self.setting = None
        self.applied = []
        self.decodes = 0
        self._runs = {}

    def device_info(self):
        return self.gpu

    def set_tuning(self, light, tile_k, ctas):
        self.setting = (light, tile_k, ctas)
        self.applied.append(self.setting)

    def decode_device(self, n, rec, res, stream, shot_code=0, offsets=0, use_graph=True):
        self.decodes += 1
        return -1 if self.setting == self.fail else 0

    def sync_status(self, stream):
        return 0

    def kernel_times(self, stream):
        k = self._runs.get(self.setting, 0)
        self._runs[self.setting] = k + 1
        t = self.cost(self.setting)
        # the first run of a setting is slow (warm-up); the tuner must drop it
        return (t * (50.0 if k == 0 else 1.0), 0.01)


def _cost(setting):
    light, tile_k, ctas = setting
    return 0.05 + 0.001 * abs(light - 10) + 0.002 * (tile_k != 4) + 0.003 * (ctas != 0)


def test_picks_fastest_and_caches(tmp_path, monkeypatch):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("GRAND_TUNE_CACHE", str(cache))
    eng = FakeEngine(_cost)
    best, table = autotune.tune(eng, "mixed-100k", 1000, 0, 0, 0)
    assert best == (10, 4, 0)
    assert eng.setting == best  # applied last
    assert len(table) == len(autotune.DEFAULT_GRID)
    for setting, ms in table:
        assert ms == pytest.approx(_cost(tuple(setting)) + 0.01)  # warm-up run dropped
    stored = json.loads(cache.read_text())
    assert stored["mixed-100k|GB300 sm_103"]["best"] == [10, 4, 0]

    # second call: from the cache, no decode
    eng2 = FakeEngine(lambda s: 1.0)
    best2, table2 = autotune.tune(eng2, "mixed-100k", 1000, 0, 0, 0)
    assert best2 == (10, 4, 0) and eng2.decodes == 0 and eng2.setting == (10, 4, 0)
    assert table2 == stored["mixed-100k|GB300 sm_103"]["table"]

    # another GPU or workload name is a separate entry
    eng3 = FakeEngine(lambda s: 0.05 + 0.001 * abs(s[0] - 14), gpu="other")
    best3, _ = autotune.tune(eng3, "mixed-100k", 1000, 0, 0, 0, grid=[(8, 4, 0), (14, 4, 0)])
    assert best3 == (14, 4, 0) and eng3.decodes > 0
    assert set(json.loads(cache.read_text())) == {"mixed-100k|GB300 sm_103", "mixed-100k|other"}


def test_no_cache_and_failure(tmp_path, monkeypatch):
    monkeypatch.setenv("GRAND_TUNE_CACHE", str(tmp_path / "t.json"))
    eng = FakeEngine(_cost)
    best, _ = autotune.tune(eng, "w", 10, 0, 0, 0, grid=[(12, 2, 2), (10, 2, 2)], reps=2,
                            use_cache=False)
    assert best == (10, 2, 2) and not (tmp_path / "t.json").exists()
    bad = FakeEngine(_cost, fail=(12, 4, 0))
    with pytest.raises(RuntimeError):
        autotune.tune(bad, "w", 10, 0, 0, 0, grid=[(10, 4, 0), (12, 4, 0)], use_cache=False)
