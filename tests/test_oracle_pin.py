"""Pin the CPU oracle: every golden fixture (upstream results, CPU search mode)
must be reproduced field for field by the C restatement in oracle/."""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
from conftest import golden_index, golden_names, load_golden, write_aux
from library_s_grand_gb300 import synth as S


def _digest(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    h = hashlib.sha256()
    h.update(np.asarray(a.shape, dtype=np.int64).tobytes())
    h.update(a.tobytes())
    return h.hexdigest()


def run_port(port, g, aux):
    cfg = O.Config(*[int(v) for v in g["cfg"]])
    variant = int(g["variant"])
    if str(g["kind"]) == "css":
        errors = g.get("errors")
        syn = g.get("syndromes")
        rc, res, dec = port.css(variant, g["hx"], g["hz"], errors, syn, cfg, str(g["type"]), aux)
        return rc, res, dec, None, None
    rc, res, dec, dlog, cost = port.dem(variant, g["h"], g["l"], g["detectors"], g["logicals"],
                                        cfg, aux)
    return rc, res, dec, dlog, cost


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_upstream(name, port, tmp_path):
    g = load_golden(name)
    rc, res, *_ = run_port(port, g, write_aux(tmp_path, g))
    assert rc == 0
    bad = O.fields_equal(res, g["res"])
    assert len(bad) == 0, f"{name}: shots {bad[:5]} differ:\n{res[bad[:3]]}\n{g['res'][bad[:3]]}"


def test_bb_construction_matches_upstream_matrices():
    dig = golden_index()["matrix_sha256"]
    for n in (72, 108, 144, 288):
        c = S.BB_CODES[n]()
        assert _digest(c.hx) == dig[f"hx_{n}"]
        assert _digest(c.hz) == dig[f"hz_{n}"]


def test_bb_code_parameters():
    # [[n, k]]: k = n - rank(Hx) - rank(Hz) over GF(2)
    def rank2(a):
        a = a.copy() % 2
        r = 0
        for c in range(a.shape[1]):
            piv = np.nonzero(a[r:, c])[0]
            if len(piv) == 0:
                continue
            p = r + piv[0]
            a[[r, p]] = a[[p, r]]
            rows = np.nonzero(a[:, c])[0]
            for i in rows:
                if i != r:
                    a[i] ^= a[r]
            r += 1
            if r == a.shape[0]:
                break
        return r
    for n, k in ((72, 12), (108, 8), (144, 12), (288, 12)):
        c = S.BB_CODES[n]()
        assert c.m == n
        assert n - rank2(c.hx) - rank2(c.hz) == k
        assert (c.hx @ c.hz.T % 2 == 0).all()  # CSS commutation
        assert (c.hz.sum(axis=0) == 3).all() and (c.hz.sum(axis=1) == 6).all()


def test_known_answer_low_weight_patterns_decode_exactly():
    """Upstream's fixture patterns of weight <= 2 all decode to themselves."""
    for name in ("kat_patterns72_cc_w3", "kat_patterns144_cc_w4"):
        g = load_golden(name)
        w = g["errors"].sum(axis=1)
        r = g["res"][w <= 2]
        assert len(r) > 40
        assert (r["found"] == 1).all() and (r["is_equal"] == 1).all()


def test_syndrome_kat_is_hz_times_patterns():
    g = load_golden("kat_syndromes72_cc_w6")
    assert g["syndromes"].shape == (30, 36)
    r = g["res"]
    assert (r["found"] == 1).all() and (r["found_weight"] == 1).all()


def test_unrank_is_lexicographic(port):
    import itertools
    for n, k in ((7, 3), (9, 4), (6, 6), (12, 2)):
        combos = list(itertools.combinations(range(n), k))
        assert port.ncr(n, k) == len(combos)
        for r, c in enumerate(combos):
            assert tuple(port.unrank(r, n, k)) == c


def test_ml_costs_match_fp64_oracle(port, tmp_path):
    g = load_golden("ml_dem120_w3_cap64")
    aux = write_aux(tmp_path, g)
    rc, res, dec, dlog, cost = run_port(port, g, aux)
    found = np.nonzero(res["found"])[0]
    assert len(found) > 100
    for i in found:
        # FP32 sum in upstream's order vs FP64 sum of the FP64 LLRs: 1e-5 relative
        ref = float(np.sum(g["llr64"][dec[i] == 1]))
        assert abs(float(cost[i]) - ref) <= 1e-5 * abs(ref)


def test_decoded_patterns_satisfy_syndrome(port, tmp_path):
    for name in ("cc_bb72_x_err_w3", "cln_dem60_w3_cap20", "prob_cc_bb72_w6_masks"):
        g = load_golden(name)
        rc, res, dec, *_ = run_port(port, g, write_aux(tmp_path, g))
        if str(g["kind"]) == "css":
            H = g["hz"] if str(g["type"]).lower() == "x" else g["hx"]
            s = g["errors"].astype(np.int64) @ H.T.astype(np.int64) % 2
        else:
            H = g["h"]
            s = g["detectors"].astype(np.int64)
        f = res["found"] == 1
        got = dec[f].astype(np.int64) @ H.T.astype(np.int64) % 2
        assert (got == s[f]).all()
        assert (dec[f].sum(axis=1) == res["found_weight"][f]).all()


@pytest.mark.skipif(not O.Reference.available(), reason="upstream library not built here")
def test_port_matches_live_upstream_random(port, tmp_path):
    """Fresh seeds, every entry point, against the upstream library itself."""
    ref = O.Reference()
    c = S.BB_CODES[108]()
    pf = S.write_phase_file(str(tmp_path / "p.txt"), [(6, 1, 0, 2, 0, 0, 0), (300, 0, 1, 2, 0, 0, 0)])
    for seed in range(3):
        e, s = S.css_shots(c.hz, 120, 0.02, seed=1000 + seed)
        for W in (2, 3):
            cfg = O.make_config(W, mode=-1)
            for var, f in ((O.UNIFORM, None), (O.PROB, pf)):
                _, a, _ = port.css(var, c.hx, c.hz, e, None, cfg, "x", f)
                _, b = ref.css(var, c.hx, c.hz, e, None, cfg, "x", f)
                assert len(O.fields_equal(a, b)) == 0
    dem = S.random_dem(77, 50, 200, 6, p_range=(3e-3, 3e-2))
    det, log, _ = S.dem_shots(dem, 200, 78)
    lf = S.write_llr_file(str(tmp_path / "l.txt"), dem.llr)
    for var, f in ((O.UNIFORM, None), (O.PROB, pf), (O.ML, lf)):
        cfg = O.make_config(3, cap=18)
        _, a, *_ = port.dem(var, dem.h, dem.l, det, log, cfg, f)
        _, b = ref.dem(var, dem.h, dem.l, det, log, cfg, f)
        assert len(O.fields_equal(a, b)) == 0
