"""GPU parity: the CUDA decoder, called through the C ABI, against the upstream
results stored in the golden fixtures (every deterministic result field) and
against the oracle's decoded patterns, logical flips and ML costs (bit-exact;
ML costs also within 1e-5 relative of an FP64 sum)."""
import numpy as np
import pytest

import oracle as O
from conftest import golden_names, load_golden, write_aux
from library_s_grand_gb300 import capi

pytestmark = pytest.mark.gpu

VARIANTS = {0: "uniform", 1: "prob", 2: "ml"}


def run_gpu(lib, g, aux):
    cfg = capi.GrandDecoderConfig(*[int(v) for v in g["cfg"]])
    v = VARIANTS[int(g["variant"])]
    if str(g["kind"]) == "css":
        rc, res, dec = capi.decode_css_ex(lib, v, g["hx"], g["hz"], g.get("errors"),
                                          g.get("syndromes"), cfg, str(g["type"]), aux)
        return rc, res, dec, None, None
    return capi.decode_dem_ex(lib, v, g["h"], g["l"], g["detectors"], g["logicals"], cfg, aux)


def run_port(port, g, aux):
    cfg = O.Config(*[int(v) for v in g["cfg"]])
    variant = int(g["variant"])
    if str(g["kind"]) == "css":
        rc, res, dec = port.css(variant, g["hx"], g["hz"], g.get("errors"), g.get("syndromes"),
                                cfg, str(g["type"]), aux)
        return rc, res, dec, None, None
    return port.dem(variant, g["h"], g["l"], g["detectors"], g["logicals"], cfg, aux)


@pytest.mark.parametrize("name", golden_names())
def test_gpu_matches_upstream_and_oracle(name, gpulib, port, tmp_path):
    g = load_golden(name)
    aux = write_aux(tmp_path, g)
    rc, res, dec, dlog, cost = run_gpu(gpulib, g, aux)
    assert rc == 0
    bad = O.fields_equal(res, g["res"])
    assert len(bad) == 0, f"{name}: shots {bad[:5]}\nGPU {res[bad[:3]]}\nupstream {g['res'][bad[:3]]}"
    prc, pres, pdec, pdlog, pcost = run_port(port, g, aux)
    assert prc == 0
    diff = np.nonzero((dec != pdec).any(axis=1))[0]
    assert len(diff) == 0, f"{name}: decoded patterns differ on shots {diff[:5]}"
    if dlog is not None:
        assert np.array_equal(dlog, pdlog)
    if int(g["variant"]) == 2:
        assert np.array_equal(cost.view(np.uint32), pcost.view(np.uint32))
        llr64 = g["llr64"]
        for i in np.nonzero(res["found"])[0]:
            ref = float(np.sum(llr64[dec[i] == 1]))
            assert abs(float(cost[i]) - ref) <= 1e-5 * abs(ref), (i, cost[i], ref)
