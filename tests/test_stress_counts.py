"""The candidate counts the roofline lines divide by (bench.stress_ops for the
exhaustive [[144]] shots, bench.dem_stress_ops for the capped DEM stress) equal
the oracle's total_tested_combinations on unmatched shots of the same workloads,
and upstream's own count where its library was built here (CPU).  The GPU runs
of both workloads assert their totals against these functions, so these pin the
full-size counts to upstream."""
import numpy as np
import pytest

import oracle as O
import bench
from library_s_grand_gb300 import workloads


def _ref():
    return O.Reference() if O.Reference.available() else None


def test_dem_stress_counts(port):
    wl = workloads.stress_dem(40)
    cfg = O.Config(*wl.config)
    rc, res, _, _, _ = port.dem(O.UNIFORM, wl.dem.h, wl.dem.l, wl.detectors, wl.logicals, cfg)
    assert rc == 0
    assert int(res["found"].sum()) == 0
    per_shot = [bench.dem_stress_ops(wl.dem.h, wl.detectors[i:i + 1], wl.W, wl.cap)[0]
                for i in range(len(wl.detectors))]
    assert per_shot == [int(v) for v in res["total_tested_combinations"]]
    # the workload's point: sizable capped searches, some shots above the cap throughout
    assert max(per_shot) > 3 * 20000 and min(per_shot) == 0 and np.mean(per_shot) > 25000
    ref = _ref()
    if ref is not None:
        rc, rres = ref.dem(O.UNIFORM, wl.dem.h, wl.dem.l, wl.detectors, wl.logicals, cfg)
        assert rc == 0
        assert [int(v) for v in rres["total_tested_combinations"]] == per_shot


def test_css_stress_counts(port):
    code, syn = workloads.stress_bb144(2)
    cfg = O.Config(4, 256, 0, 300, 10, -1)
    rc, res, _ = port.css(O.UNIFORM, code.hx, code.hz, None, syn, cfg, "x")
    assert rc == 0
    assert int(res["found"].sum()) == 0
    per_shot = [bench.stress_ops(code.hz, syn[i:i + 1], 4)[0] for i in range(len(syn))]
    assert per_shot == [int(v) for v in res["total_tested_combinations"]]
    ref = _ref()
    if ref is not None:
        rc, rres = ref.css(O.UNIFORM, code.hx, code.hz, None, syn, cfg, "x")
        assert rc == 0
        assert [int(v) for v in rres["total_tested_combinations"]] == per_shot


@pytest.mark.parametrize("cap", [0, 20, 64])
def test_dem_cap_rule(port, cap):
    """Tighter caps: more iterations fall back to the last set within the cap."""
    wl = workloads.stress_dem(12, seed=5)
    cfg = O.Config(wl.W, 256, 0, cap, 10, -1)
    rc, res, _, _, _ = port.dem(O.UNIFORM, wl.dem.h, wl.dem.l, wl.detectors, wl.logicals, cfg)
    assert rc == 0
    assert int(res["found"].sum()) == 0
    per_shot = [bench.dem_stress_ops(wl.dem.h, wl.detectors[i:i + 1], wl.W, cap)[0]
                for i in range(len(wl.detectors))]
    assert per_shot == [int(v) for v in res["total_tested_combinations"]]


@pytest.mark.gpu
def test_dem_stress_gpu(port, gpulib):
    """The capped DEM stress on a GB300, through the engine's device path (as the
    bench decodes it) and through grand_decode_cln: every deterministic field
    equals the oracle's, and the totals equal dem_stress_ops."""
    import torch
    from library_s_grand_gb300 import capi
    from library_s_grand_gb300.engine import UNIFORM, Engine
    n = 512
    wl = workloads.stress_dem(n, seed=3)
    rc, want, _, _, _ = port.dem(O.UNIFORM, wl.dem.h, wl.dem.l, wl.detectors, wl.logicals,
                                 O.Config(*wl.config))
    assert rc == 0
    cfg = capi.GrandDecoderConfig(*wl.config)
    eng = Engine(gpulib)
    eng.add_dem(wl.dem.h, wl.dem.l, cfg, UNIFORM)
    dev = torch.device("cuda", 0)
    sp = torch.cuda.current_stream(dev).cuda_stream
    d_rec = torch.from_numpy(wl.records.ravel()).to(dev)
    d_res = torch.empty(n * 72, dtype=torch.uint8, device=dev)
    assert eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=False) == 0
    assert eng.sync_status(sp) == 0
    got = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    bad = O.fields_equal(got, want)
    assert len(bad) == 0, (bad[:5], got[bad[:3]], want[bad[:3]])
    assert eng.launch_stats(sp)[2] > 0  # the shots' searches ran as Jobs
    assert int(got["total_tested_combinations"].sum()) == \
        bench.dem_stress_ops(wl.dem.h, wl.detectors, wl.W, wl.cap)[0]
    rc, res = capi.run_grand_shots_cln(gpulib, wl.dem.h, wl.dem.l, wl.detectors, wl.logicals,
                                       wl.dem.l.shape[1], cfg)
    assert rc == 0
    bad = O.fields_equal(capi.results_array(res), want)
    assert len(bad) == 0, bad[:5]
