"""Full-size parity on the benchmark workloads: every shot of each batch the
benchmark decodes, compared with the oracle (the C restatement of upstream's CPU
search mode) in every deterministic result field and in the decoded patterns.

* BB[[72,12,6]], grand_decode_cc, p = 0.005, 1024 shots, seed 0, W = 3 (errors
  given, so is_equal and degeneracy are compared too);
* the headline batch: BB[[144,12,12]], grand_decode_prob_cc, 16384 shots, W = 4,
  phase mask "300 0 1 2" -- through the C ABI and through the engine's
  device-resident, graph-replayed path that the benchmark times;
* the ML DEM: 120 x 720, 65536 shots, W = 3 -- FP32 costs bit-exact against the
  oracle and within 1e-5 relative of an FP64 sum of the FP64 LLRs;
* the 100k-shot mixed batch (BB72/108 at W = 3, BB144/288 at W = 4, shuffled):
  the persistent mixed-code decode against each code's shots decoded by the
  oracle, shot by shot.

Upstream references: grand_decoder.cu:1117-1396 (cc), :790-1115 (prob_cc),
:1996-2277 (ML_cln)."""
import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, workloads
from library_s_grand_gb300.engine import Engine, offsets_for

pytestmark = pytest.mark.gpu


def _assert_fields(got, want, what):
    bad = O.fields_equal(got, want)
    assert len(bad) == 0, f"{what}: shots {bad[:5]}\nGPU    {got[bad[:2]]}\noracle {want[bad[:2]]}"


def _assert_patterns(dec, pdec, what):
    diff = np.nonzero((dec != pdec).any(axis=1))[0]
    assert len(diff) == 0, f"{what}: decoded patterns differ on shots {diff[:5]}"


def test_uniform_bb72_1024_shots(gpulib, port):
    w = workloads.uniform_bb72()
    cfg = capi.GrandDecoderConfig(*w.config)
    rc, res, dec = capi.decode_css_ex(gpulib, "uniform", w.code.hx, w.code.hz, w.errors, None,
                                      cfg, "x")
    assert rc == 0
    prc, pres, pdec = port.css(O.UNIFORM, w.code.hx, w.code.hz, w.errors, None,
                               O.Config(*w.config), "x")
    assert prc == 0
    _assert_fields(res, pres, "BB72 cc")
    _assert_patterns(dec, pdec, "BB72 cc")
    assert res["found"].sum() > 100 and res["is_equal"].sum() > 100


def test_prob_bb144_headline_batch(gpulib, port, tmp_path):
    import torch
    w = workloads.prob_bb144()
    pf = w.phase_file(str(tmp_path))
    cfg = capi.GrandDecoderConfig(*w.config)
    prc, pres, pdec = port.css(O.PROB, w.code.hx, w.code.hz, w.errors, None, O.Config(*w.config),
                               "x", pf)
    assert prc == 0
    rc, res, dec = capi.decode_css_ex(gpulib, "prob", w.code.hx, w.code.hz, w.errors, None, cfg,
                                      "x", pf)
    assert rc == 0
    _assert_fields(res, pres, "headline, C ABI")
    _assert_patterns(dec, pdec, "headline, C ABI")
    # the benchmark's timed path: records resident on the device, graph replay
    eng = Engine(gpulib)
    eng.add_css(w.code.hx, w.code.hz, "x", True, cfg, pf)
    d_rec = torch.from_numpy(np.ascontiguousarray(w.errors.ravel())).cuda()
    d_res = torch.empty(len(w.errors) * 72, dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    for _ in range(3):  # capture, then replays
        assert eng.decode_device(len(w.errors), d_rec.data_ptr(), d_res.data_ptr(), sp,
                                 use_graph=True) == 0
    assert eng.sync_status(sp) == 0
    got = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    _assert_fields(got, pres, "headline, device-resident graph replay")
    assert pres["total_tested_combinations"].max() > 1_000_000  # heavy shots are in the batch


def test_ml_dem_65536_shots(gpulib, port, tmp_path):
    w = workloads.ml_dem()
    lf = w.llr_file(str(tmp_path))
    cfg = capi.GrandDecoderConfig(*w.config)
    rc, res, dec, dlog, cost = capi.decode_dem_ex(gpulib, "ml", w.dem.h, w.dem.l, w.detectors,
                                                  w.logicals, cfg, lf)
    assert rc == 0
    prc, pres, pdec, pdlog, pcost = port.dem(O.ML, w.dem.h, w.dem.l, w.detectors, w.logicals,
                                             O.Config(*w.config), lf)
    assert prc == 0
    _assert_fields(res, pres, "ML DEM")
    _assert_patterns(dec, pdec, "ML DEM")
    assert np.array_equal(dlog, pdlog)
    assert np.array_equal(cost.view(np.uint32), pcost.view(np.uint32)), "ML costs differ"
    found = res["found"] == 1
    ref = (dec[found].astype(np.float64) * w.dem.llr[None, :]).sum(axis=1)
    rel = np.abs(cost[found].astype(np.float64) - ref) / np.abs(ref)
    assert rel.max() <= 1e-5, float(rel.max())
    assert found.sum() > 10000


def test_mixed_100k_batch(gpulib, port):
    import torch
    w = workloads.bb_mix()
    eng = Engine(gpulib)
    want_parts = []
    for c, W, s in zip(w.codes, w.Ws, w.syndromes):
        cfg = capi.GrandDecoderConfig(*workloads.config_tuple(W))
        eng.add_css(c.hx, c.hz, "x", False, cfg)
        rc, r, _ = port.css(O.UNIFORM, c.hx, c.hz, None, s, O.Config(*workloads.config_tuple(W)),
                            "x")
        assert rc == 0
        want_parts.append(r)
    want = np.concatenate(want_parts)[w.order]
    rec = w.records()
    rc, got = eng.decode(rec, w.shot_code)
    assert rc == 0
    _assert_fields(got, want, "100k mix, persistent engine")
    # the graph-replayed device path the benchmark times
    off = offsets_for(eng.rec_lens, w.shot_code)
    d_rec = torch.from_numpy(rec).cuda()
    d_sc = torch.from_numpy(np.ascontiguousarray(w.shot_code)).cuda()
    d_off = torch.from_numpy(off).cuda()
    d_res = torch.empty(w.num_shots * 72, dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    for _ in range(3):
        assert eng.decode_device(w.num_shots, d_rec.data_ptr(), d_res.data_ptr(), sp,
                                 d_sc.data_ptr(), d_off.data_ptr(), True) == 0
    assert eng.sync_status(sp) == 0
    got_dev = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    _assert_fields(got_dev, want, "100k mix, device-resident graph replay")
