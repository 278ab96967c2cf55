"""Phase-mask generation from decoded statistics (library_s_grand_gb300.phases):
the table on hand-computed cases, the file format, and (GPU) a file generated from
decoded shots driving the prob search exactly as the oracle does with it."""
import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, phases, synth


def _results(pairs, unfound=0):
    r = np.zeros(len(pairs) + unfound, dtype=capi.RESULT_DTYPE)
    for i, (tam, w) in enumerate(pairs):
        r[i]["found"], r[i]["tam"], r[i]["found_weight"] = 1, tam, w
    for i in range(len(pairs), len(r)):
        r[i]["tam"], r[i]["found_weight"] = 3, 6  # not found: ignored
    return r


def test_table_groups_weights_and_orders():
    # tam 1 -> group 1; tams 3, 4 -> group "3-5"; tams 8, 9 -> "6-10"; 97 -> "96+"
    pairs = [(1, 1)] * 4 + [(3, 1), (3, 2), (4, 2), (4, 3)] + [(8, 6)] * 3 + [(9, 2)] + \
            [(97, 7)] * 2 + [(97, 6)]
    rows = phases.phase_table(_results(pairs, unfound=5))
    assert [r[0] for r in rows] == [1, 5, 10, 96]
    assert rows[0] == (1, 0, 1, 2, 1.0, 0.0, 0.0)
    assert rows[1] == (5, 0, 1, 2, 1.0, 0.0, 0.0)
    up, o0, o1, o2, p0, p1, p2 = rows[2]  # 3 of 4 at weight 6, feasible up to 7
    assert (o0, o1, o2) == (1, 0, 2) and (p0, p1, p2) == (0.25, 0.75, 0.0)
    up, o0, o1, o2, p0, p1, p2 = rows[3]
    assert (o0, o1, o2) == (2, 1, 0) and abs(p2 - 2 / 3) < 1e-12 and abs(p1 - 1 / 3) < 1e-12


def test_infeasible_weights_do_not_count():
    # group "3-5" has upper bound 5: weight-6 finds there do not enter its probabilities
    rows = phases.phase_table(_results([(5, 6), (5, 1)]), max_weight_decoder=7)
    assert rows[0][4:] == (0.5, 0.0, 0.0)
    rows = phases.phase_table(_results([(8, 7), (8, 6)]), max_weight_decoder=6)
    assert rows[0][4:] == (0.0, 0.5, 0.0)


def test_file_format(tmp_path):
    rows = phases.phase_table(_results([(2, 1), (9, 6), (9, 6), (9, 1)]))
    path = phases.write_phase_file(str(tmp_path / "p.txt"), rows)
    lines = open(path).read().splitlines()
    assert lines[0] == "2 0 1 2 1.000000 0.000000 0.000000"
    assert lines[1] == "10 1 0 2 0.333333 0.666667 0.000000"


@pytest.mark.gpu
def test_generated_file_drives_prob_search_like_the_oracle(gpulib, port, tmp_path):
    code = synth.BB_CODES[108]()
    errors, _ = synth.css_shots(code.hz, 1500, 0.04, seed=61)
    cfg = (7, 256, 0, 24, 10, 1)
    first = synth.write_phase_file(str(tmp_path / "p0.txt"), [(300, 0, 1, 2, 1, 0, 0)])
    rc, res, _ = capi.decode_css_ex(gpulib, "prob", code.hx, code.hz, errors, None,
                                    capi.GrandDecoderConfig(*cfg), "x", first)
    assert rc == 0
    rows = phases.phase_table(res)
    assert len(rows) >= 3
    tuned = phases.write_phase_file(str(tmp_path / "p1.txt"), rows)
    rc, res2, dec = capi.decode_css_ex(gpulib, "prob", code.hx, code.hz, errors, None,
                                       capi.GrandDecoderConfig(*cfg), "x", tuned)
    assert rc == 0
    prc, pres, pdec = port.css(O.PROB, code.hx, code.hz, errors, None, O.Config(*cfg), "x", tuned)
    assert prc == 0
    assert len(O.fields_equal(res2, pres)) == 0
    assert np.array_equal(dec, pdec)
