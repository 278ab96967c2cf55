"""Batched engine on the GPU: a shuffled mixed-code batch (CSS uniform / prob,
syndrome and error records, DEM uniform / ML) decoded in one launch must give
every shot exactly the result the oracle gives it alone; the device-resident
graph path and the one-launch-per-call path must agree with it."""
import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth
from library_s_grand_gb300.engine import Engine, offsets_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("mix")
    pf = synth.write_phase_file(str(tmp / "p.txt"), [(300, 0, 1, 2, 1, 0, 0)])
    dem = synth.random_dem(5, 60, 240, 6, p_range=(2e-3, 2e-2))
    lf = synth.write_llr_file(str(tmp / "l.txt"), dem.llr)
    c72, c108, c144 = synth.BB_CODES[72](), synth.BB_CODES[108](), synth.BB_CODES[144]()
    codes = [
        ("css", c72, 3, False, True, None),     # uniform, error records
        ("css", c108, 3, False, False, None),   # uniform, syndrome records
        ("css", c144, 4, True, True, pf),       # prob, error records
        ("dem", dem, 3, "uniform", None, None),
        ("dem", dem, 3, "ml", None, lf),
    ]
    rng = np.random.default_rng(9)
    per_code = 160
    shots = []
    for ci, (kind, c, W, var, rec_err, f) in enumerate(codes):
        if kind == "css":
            e, s = synth.css_shots(c.hz, per_code, 0.02, seed=100 + ci)
            recs = e if rec_err else s
            shots += [(ci, r) for r in recs]
        else:
            det, log, _ = synth.dem_shots(dem, per_code, 200 + ci)
            shots += [(ci, np.concatenate([d, l])) for d, l in zip(det, log)]
    order = rng.permutation(len(shots))
    shots = [shots[i] for i in order]
    return codes, shots, pf, lf, dem


def expected(codes, shots):
    """Each shot decoded alone by the oracle."""
    port = O.Port()
    out = np.zeros(len(shots), dtype=O.RESULT_DTYPE)
    for i, (ci, rec) in enumerate(shots):
        kind, c, W, var, rec_err, f = codes[ci]
        cap = 64
        cfg = O.make_config(W, mode=-1, cap=cap)
        if kind == "css":
            v = O.PROB if var is True else O.UNIFORM
            e = rec[None] if rec_err else None
            s = None if rec_err else rec[None]
            _, r, _ = port.css(v, c.hx, c.hz, e, s, cfg, "x", f)
        else:
            v = O.ML if var == "ml" else O.UNIFORM
            det, log = rec[None, :c.n], rec[None, c.n:]
            _, r, *_ = port.dem(v, c.h, c.l, det, log, cfg, f)
        out[i] = r[0]
    return out


def build_engine(gpulib, codes):
    eng = Engine(gpulib)
    for kind, c, W, var, rec_err, f in codes:
        cfg = capi.GrandDecoderConfig(W, 256, 0, 64, 10, -1)
        if kind == "css":
            eng.add_css(c.hx, c.hz, "x", rec_err, cfg, f)
        else:
            eng.add_dem(c.h, c.l, cfg, 2 if var == "ml" else 0, f)
    return eng


def test_mixed_batch_equals_each_shot_alone(gpulib, mix):
    codes, shots, *_ = mix
    eng = build_engine(gpulib, codes)
    sc = np.array([ci for ci, _ in shots], dtype=np.int32)
    recs = np.concatenate([r for _, r in shots]).astype(np.int32)
    rc, res = eng.decode(recs, sc)
    assert rc == 0
    exp = expected(codes, shots)
    bad = O.fields_equal(res, exp)
    assert len(bad) == 0, (bad[:5], res[bad[:3]], exp[bad[:3]])
    assert res["found"].sum() > 200
    # the call's event times are reported; the decode kernel ran and took time
    h2d, reset, dec, d2h = eng.batch_times()
    assert dec > 0.0 and min(h2d, reset, d2h) >= 0.0
    # per-shot timers come from the GPU timer: finite, non-negative
    for f in ("time_sum_ms", "total_time_search_ms", "transfer_time_ms", "total_to_find_ms"):
        assert np.isfinite(res[f]).all() and (res[f] >= 0.0).all(), f


def test_device_graph_path_and_plain_path_agree(gpulib, mix):
    import torch
    codes, shots, *_ = mix
    eng = build_engine(gpulib, codes)
    sc = np.array([ci for ci, _ in shots], dtype=np.int32)
    recs = np.concatenate([r for _, r in shots]).astype(np.int32)
    rc, ref = eng.decode(recs, sc)
    assert rc == 0
    off = offsets_for(eng.rec_lens, sc)
    d_rec = torch.from_numpy(recs).cuda()
    d_sc = torch.from_numpy(sc).cuda()
    d_off = torch.from_numpy(off).cuda()
    n = len(sc)
    d_res = torch.zeros(n * 72, dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    for use_graph in (False, True, True):
        d_res.zero_()
        rc = eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, d_sc.data_ptr(),
                               d_off.data_ptr(), use_graph=use_graph)
        assert rc == 0
        assert eng.sync_status(sp) == 0
        got = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
        assert len(O.fields_equal(got, ref)) == 0
    rc, plain = eng.decode_plain(recs, sc)
    assert rc == 0
    assert len(O.fields_equal(plain, ref)) == 0


@pytest.mark.parametrize("tile_k,light", [(1, 0), (2, 6), (8, 20), (4, 12)])
def test_tuning_does_not_change_results(gpulib, mix, tile_k, light):
    codes, shots, *_ = mix
    eng = build_engine(gpulib, codes)
    sc = np.array([ci for ci, _ in shots], dtype=np.int32)
    recs = np.concatenate([r for _, r in shots]).astype(np.int32)
    rc, ref = eng.decode(recs, sc)
    eng.set_tuning(light, tile_k, 0)
    rc2, got = eng.decode(recs, sc)
    assert rc == rc2 == 0
    assert len(O.fields_equal(got, ref)) == 0


def test_zero_copy_and_copy_paths_agree(gpulib, tmp_path):
    """The C ABI reads records / writes results in host memory directly when the
    GPU can access pageable memory; GRAND_ZERO_COPY=0 forces staged copies.
    Both must give identical results, decoded patterns and ML costs."""
    import os
    import subprocess
    import sys
    from conftest import ROOT, load_golden, write_aux
    script = tmp_path / "run.py"
    script.write_text(
        "import sys, numpy as np\n"
        f"sys.path.insert(0, {ROOT!r}); sys.path.insert(0, {os.path.join(ROOT, 'tests')!r})\n"
        "from conftest import load_golden\n"
        "from library_s_grand_gb300 import capi\n"
        "lib = capi.load_library()\n"
        "out = {}\n"
        "for name, aux in [('cc_bb72_x_err_w3', None), ('ml_dem60_w3_cap20', sys.argv[2])]:\n"
        "    g = load_golden(name)\n"
        "    cfg = capi.GrandDecoderConfig(*[int(v) for v in g['cfg']])\n"
        "    if str(g['kind']) == 'css':\n"
        "        rc, res, dec = capi.decode_css_ex(lib, 'uniform', g['hx'], g['hz'], g['errors'], None, cfg, 'x')\n"
        "        cost = np.zeros(1, np.float32)\n"
        "    else:\n"
        "        rc, res, dec, dlog, cost = capi.decode_dem_ex(lib, 'ml', g['h'], g['l'], g['detectors'], g['logicals'], cfg, aux)\n"
        "    assert rc == 0\n"
        "    out[name + '_res'] = res; out[name + '_dec'] = dec; out[name + '_cost'] = cost\n"
        "np.savez(sys.argv[1], **out)\n")
    g = load_golden("ml_dem60_w3_cap20")
    aux = write_aux(tmp_path, g)
    outs = []
    for zc in ("1", "0"):
        path = tmp_path / f"out{zc}.npz"
        env = dict(os.environ, GRAND_ZERO_COPY=zc)
        subprocess.check_call([sys.executable, str(script), str(path), aux], env=env)
        outs.append(np.load(path))
    for k in outs[0].files:
        a, b = outs[0][k], outs[1][k]
        if a.dtype.names:
            for f in ("found", "found_weight", "tam", "total_tested_combinations", "iteration",
                      "degenerate", "is_equal", "hibrido"):
                assert np.array_equal(a[f], b[f]), (k, f)
        else:
            assert np.array_equal(a, b), k
