"""Bit-packed record entry points on the GPU: every deterministic result field
equals the int32 entry points' and the oracle's on the same shots (CSS syndromes
and errors, uniform and prob; DEM uniform, prob and ML), with junk bits set past
the last entry of each shot's final word to check that they are ignored."""
import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _junk(words, n):
    """Set every bit past entry n-1 in the last word (they must be ignored)."""
    w = words.copy()
    if n % 32:
        w[:, -1] |= np.uint32((0xFFFFFFFF << (n % 32)) & 0xFFFFFFFF)
    return w


@pytest.mark.parametrize("records", ["syndromes", "errors"])
@pytest.mark.parametrize("prob", [False, True])
def test_css_packed_equals_int32_and_oracle(gpulib, port, tmp_path, records, prob):
    code = synth.BB_CODES[72]()
    errors, syndromes = synth.css_shots(code.hz, 700, 0.03, seed=41)
    pf = synth.write_phase_file(str(tmp_path / "p.txt"), [(300, 0, 1, 2, 1, 0, 0)]) if prob else None
    cfg = capi.GrandDecoderConfig(7 if prob else 4, 256, 0, 64, 10, -1)
    variant = "prob" if prob else "uniform"
    if records == "errors":
        rc, ref, _ = capi.decode_css_ex(gpulib, variant, code.hx, code.hz, errors, None, cfg, "x", pf)
        words = _junk(capi.pack_bits(errors), code.m)
        kind = capi.PACKED_ERRORS
    else:
        rc, ref, _ = capi.decode_css_ex(gpulib, variant, code.hx, code.hz, None, syndromes, cfg, "x", pf)
        words = _junk(capi.pack_bits(syndromes), code.n)
        kind = capi.PACKED_SYNDROMES
    assert rc == 0
    rc, res = capi.decode_css_packed(gpulib, code.hx, code.hz, words, kind, cfg, "x", pf)
    assert rc == 0
    assert len(O.fields_equal(res, ref)) == 0
    prc, pres, _ = port.css(O.PROB if prob else O.UNIFORM, code.hx, code.hz,
                            errors if records == "errors" else None,
                            syndromes if records == "syndromes" else None,
                            O.Config(*[getattr(cfg, f) for f, _ in cfg._fields_]), "x", pf)
    assert prc == 0
    assert len(O.fields_equal(res, pres)) == 0
    assert res["found"].sum() > 100


@pytest.mark.parametrize("variant", ["uniform", "prob", "ml"])
def test_dem_packed_equals_int32_and_oracle(gpulib, port, tmp_path, variant):
    dem = synth.random_dem(7, detectors=70, mechanisms=260, logicals=5, p_range=(2e-3, 2e-2))
    det, log, _ = synth.dem_shots(dem, 700, seed=43)
    f = None
    if variant == "prob":
        f = synth.write_phase_file(str(tmp_path / "p.txt"), [(300, 0, 1, 2, 1, 0, 0)])
    elif variant == "ml":
        f = synth.write_llr_file(str(tmp_path / "l.txt"), dem.llr)
    cfg = capi.GrandDecoderConfig(3, 256, 0, 48, 10, -1)
    rc, ref, *_ = capi.decode_dem_ex(gpulib, variant, dem.h, dem.l, det, log, cfg, f)
    assert rc == 0
    rc, res = capi.decode_dem_packed(gpulib, variant, dem.h, dem.l,
                                     _junk(capi.pack_bits(det), dem.n),
                                     _junk(capi.pack_bits(log), dem.n_logicos), cfg, f)
    assert rc == 0
    assert len(O.fields_equal(res, ref)) == 0
    v = {"uniform": O.UNIFORM, "prob": O.PROB, "ml": O.ML}[variant]
    prc, pres, *_ = port.dem(v, dem.h, dem.l, det, log,
                             O.Config(*[getattr(cfg, f) for f, _ in cfg._fields_]), f)
    assert prc == 0
    assert len(O.fields_equal(res, pres)) == 0
    assert res["found"].sum() > 100

