"""GPU parity on shots whose threshold iterations have small-to-medium active
sets (the light path enumerates sets of at most 14 positions as bit masks and
larger ones weight block by weight block).  Shots are drawn at error rates that
put many iterations on both sides of that limit; every deterministic result
field, the decoded patterns, the logical flips and the ML costs must equal the
oracle's."""
import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _tam_spread(res):
    tam = res["tam"]
    return int(((tam >= 6) & (tam <= 14)).sum()), int(((tam >= 15) & (tam <= 40)).sum())


def _compare(res, pres, dec, pdec):
    bad = O.fields_equal(res, pres)
    assert len(bad) == 0, f"shots {bad[:5]}\nGPU {res[bad[:3]]}\noracle {pres[bad[:3]]}"
    diff = np.nonzero((dec != pdec).any(axis=1))[0]
    assert len(diff) == 0, f"decoded patterns differ on shots {diff[:5]}"


# mode 1 skips iterations above the cap (bounded oracle time at W = 5, 6);
# mode -1 and mode 0 search every iteration
@pytest.mark.parametrize("W,mode,thr,cap", [(4, -1, 10, 64), (6, 1, 10, 24), (5, 1, 8, 20),
                                            (3, 0, 10, 64)])
def test_uniform_css_small_sets(gpulib, port, W, mode, thr, cap):
    code = synth.BB_CODES[72]()
    errors = np.concatenate([synth.css_shots(code.hz, 400, p, seed=100 + i)[0]
                             for i, p in enumerate((0.02, 0.045, 0.07))])
    cfg = (W, 256, 0, cap, thr, mode)
    rc, res, dec = capi.decode_css_ex(gpulib, "uniform", code.hx, code.hz, errors, None,
                                      capi.GrandDecoderConfig(*cfg), "x")
    assert rc == 0
    prc, pres, pdec = port.css(O.UNIFORM, code.hx, code.hz, errors, None, O.Config(*cfg), "x")
    assert prc == 0
    small, medium = _tam_spread(pres)
    assert small >= 20 and medium >= 5, (small, medium)
    _compare(res, pres, dec, pdec)


def test_prob_css_small_sets_with_repeated_phases(gpulib, port, tmp_path):
    # sets up to 9 positions search phases 0, 1, 2; larger ones list phase 0
    # twice, so weights 1..5 appear twice and the second listing never wins
    phase = synth.write_phase_file(str(tmp_path / "phase.txt"),
                                   [(9, 0, 1, 2, 0.5, 0.3, 0.2), (300, 0, 0, 1, 0.6, 0.3, 0.1)])
    code = synth.BB_CODES[108]()
    errors = np.concatenate([synth.css_shots(code.hz, 500, p, seed=200 + i)[0]
                             for i, p in enumerate((0.015, 0.03, 0.05))])
    cfg = (7, 256, 0, 24, 10, 1)
    rc, res, dec = capi.decode_css_ex(gpulib, "prob", code.hx, code.hz, errors, None,
                                      capi.GrandDecoderConfig(*cfg), "x", phase)
    assert rc == 0
    prc, pres, pdec = port.css(O.PROB, code.hx, code.hz, errors, None, O.Config(*cfg), "x", phase)
    assert prc == 0
    small, medium = _tam_spread(pres)
    assert small >= 20 and medium >= 5, (small, medium)
    _compare(res, pres, dec, pdec)


@pytest.mark.parametrize("W", [3, 4])
def test_ml_dem_small_sets(gpulib, port, tmp_path, W):
    dem = synth.random_dem(5, detectors=60, mechanisms=240, logicals=6, p_range=(4e-3, 3e-2))
    llr = synth.write_llr_file(str(tmp_path / "llr.txt"), dem.llr)
    det, log, _ = synth.dem_shots(dem, 1500, seed=300 + W)
    cfg = (W, 256, 0, 24, 10, -1)
    rc, res, dec, dlog, cost = capi.decode_dem_ex(gpulib, "ml", dem.h, dem.l, det, log,
                                                  capi.GrandDecoderConfig(*cfg), llr)
    assert rc == 0
    prc, pres, pdec, pdlog, pcost = port.dem(O.ML, dem.h, dem.l, det, log, O.Config(*cfg), llr)
    assert prc == 0
    small, medium = _tam_spread(pres)
    assert small >= 20 and medium >= 5, (small, medium)
    _compare(res, pres, dec, pdec)
    assert np.array_equal(dlog, pdlog)
    assert np.array_equal(cost.view(np.uint32), pcost.view(np.uint32))
