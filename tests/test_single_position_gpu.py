"""GPU parity on iterations with one active position.  Such an iteration has a
single candidate (that column, weight 1), and the triage warp tests it without
staging the iteration.  The shots here put many first iterations at one
position: single-column errors, where the one fully flagged column is the
answer, and pairs of errors, where a lone fully flagged column can fail to
match so that the search moves on to the next iteration.  Every deterministic
result field and the decoded patterns must equal the oracle's across the
branch rules (mode -1, 0 and 1 with the iteration under or over the threshold),
the prob phases and the DEM active-set cap."""
import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _compare(res, pres, dec, pdec):
    bad = O.fields_equal(res, pres)
    assert len(bad) == 0, f"shots {bad[:5]}\nGPU {res[bad[:3]]}\noracle {pres[bad[:3]]}"
    diff = np.nonzero((dec != pdec).any(axis=1))[0]
    assert len(diff) == 0, f"decoded patterns differ on shots {diff[:5]}"


def _css_errors(m, seed):
    rng = np.random.default_rng(seed)
    single = np.eye(m, dtype=np.int32)                    # every column once
    pairs = np.zeros((3 * m, m), dtype=np.int32)
    for row in pairs:
        row[rng.choice(m, 2, replace=False)] = 1
    return np.concatenate([single, pairs])


def _one_position_share(pres):
    found = pres["found"] == 1
    return int((found & (pres["tam"] == 1)).sum()), int((pres["iteration"] >= 2).sum())


# mode 1 with thr 10: one position is under the threshold (CPU-branch counts);
# mode 0 puts every iteration on the GPU branch; mode -1 on the CPU branch
@pytest.mark.parametrize("W,mode,thr,cap", [(4, -1, 10, 64), (3, 0, 10, 64), (4, 1, 10, 64),
                                            (1, 1, 0, 64)])
def test_uniform_css_one_position(gpulib, port, W, mode, thr, cap):
    code = synth.BB_CODES[144]()
    errors = _css_errors(code.m, 11 + W)
    cfg = (W, 256, 0, cap, thr, mode)
    rc, res, dec = capi.decode_css_ex(gpulib, "uniform", code.hx, code.hz, errors, None,
                                      capi.GrandDecoderConfig(*cfg), "x")
    assert rc == 0
    prc, pres, pdec = port.css(O.UNIFORM, code.hx, code.hz, errors, None, O.Config(*cfg), "x")
    assert prc == 0
    one, later = _one_position_share(pres)
    assert one >= code.m // 2 and later >= 10, (one, later)
    _compare(res, pres, dec, pdec)


@pytest.mark.parametrize("first_group_order", [(0, 1, 2), (1, 0, 2)])
def test_prob_css_one_position(gpulib, port, tmp_path, first_group_order):
    # W = 4 searches one phase.  With phase 0 first, a one-position iteration
    # has its weight-1 block; with phase 1 (weight 6) first it has no block at
    # all, and every such shot moves on to its next iteration.
    phase = synth.write_phase_file(str(tmp_path / "phase.txt"),
                                   [(1, *first_group_order, 0.3, 0.6, 0.1),
                                    (300, 0, 1, 2, 0.8, 0.1, 0.1)])
    code = synth.BB_CODES[108]()
    errors = _css_errors(code.m, 23)
    for mode in (-1, 1):
        cfg = (4, 256, 0, 64, 10, mode)
        rc, res, dec = capi.decode_css_ex(gpulib, "prob", code.hx, code.hz, errors, None,
                                          capi.GrandDecoderConfig(*cfg), "x", phase)
        assert rc == 0
        prc, pres, pdec = port.css(O.PROB, code.hx, code.hz, errors, None, O.Config(*cfg), "x",
                                   phase)
        assert prc == 0
        one, later = _one_position_share(pres)
        if first_group_order[0] == 0:
            assert one >= code.m // 2, one
        else:
            assert one == 0 and later >= code.m // 2, (one, later)
        _compare(res, pres, dec, pdec)


@pytest.mark.parametrize("variant", ["uniform", "prob"])
def test_dem_one_position_with_cap(gpulib, port, tmp_path, variant):
    # cap 2: an iteration over the cap falls back to the previous active-set
    # size, which can be one position
    dem = synth.random_dem(9, detectors=48, mechanisms=160, logicals=5)
    m = dem.h.shape[1]
    f = np.concatenate([np.eye(m, dtype=np.int64), synth.dem_shots(dem, 400, seed=41)[2]])
    det = (f @ dem.h.T % 2).astype(np.int32)
    log = (f @ dem.l % 2).astype(np.int32)
    phase = None
    if variant == "prob":
        phase = synth.write_phase_file(str(tmp_path / "p.txt"), [(300, 0, 1, 2, 0.9, 0.05, 0.05)])
    for cap in (2, 64):
        cfg = (3, 256, 0, cap, 10, -1)
        rc, res, dec, dlog, _ = capi.decode_dem_ex(gpulib, variant, dem.h, dem.l, det, log,
                                                   capi.GrandDecoderConfig(*cfg), phase)
        assert rc == 0
        pv = O.UNIFORM if variant == "uniform" else O.PROB
        prc, pres, pdec, pdlog, _ = port.dem(pv, dem.h, dem.l, det, log, O.Config(*cfg), phase)
        assert prc == 0
        assert int(((pres["found"] == 1) & (pres["tam"] == 1)).sum()) >= 20
        _compare(res, pres, dec, pdec)
        assert np.array_equal(dlog, pdlog)
