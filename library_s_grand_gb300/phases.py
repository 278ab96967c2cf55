"""Phase-mask files from decoded statistics (the prob-mode tuning step).

Upstream builds the phase-mask file of grand_decode_prob_cc / _prob_cln with a
pandas notebook (Create_Files/create_prob_files.ipynb, cells 8-10): from the
decoded shots that were found, the distribution of the found weight per active
set size, pooled into size groups, gives each group's probability of phase 0
(weights 1..5), phase 1 (weight 6) and phase 2 (weight 7); the phases are then
ordered by that probability.  This module computes the same table with numpy
from a results array (GrandDecoderResult fields `found`, `found_weight`, `tam`)
and writes it in the format the decoders read.
"""
from __future__ import annotations

import numpy as np

# Upper bounds of the active-set size groups: 1, 2, 3-5, 6-10, ..., 91-95, 96+
# (create_prob_files.ipynb cell 8, assign_tam_group / tam_group_to_upper_bound).
GROUP_UPPER = [1, 2, 5] + list(range(10, 100, 5)) + [96]


def _group_upper(tam: int) -> int:
    for u in GROUP_UPPER[:-1]:
        if tam <= u:
            return u
    return GROUP_UPPER[-1]  # "96+"


def phase_table(results, max_weight_decoder: int = 7):
    """Rows (size_upper, order0, order1, order2, p0, p1, p2), one per active-set
    size group that has found shots, in ascending size order.

    Per group the weight probabilities are the found shots' weight counts over
    the group's found shots (the notebook's count-weighted mean of per-size
    probabilities); p0 = sum of p_w for w = 1..5, p1 = p_6, p2 = p_7, each only
    for weights up to min(max_weight_decoder, size_upper); the order lists the
    phases by decreasing probability, ties in phase order."""
    r = np.asarray(results)
    found = r["found"] == 1
    tam = np.asarray(r["tam"])[found].astype(np.int64)
    w = np.asarray(r["found_weight"])[found].astype(np.int64)
    rows = []
    groups: dict[int, list[int]] = {}
    for t in np.unique(tam):
        groups.setdefault(_group_upper(int(t)), []).append(int(t))
    for upper in sorted(groups, key=lambda u: min(groups[u])):
        sel = np.isin(tam, groups[upper])
        total = int(sel.sum())
        counts = np.bincount(w[sel], minlength=8)
        feasible = min(max_weight_decoder, upper)

        def p(k):
            return counts[k] / total if k <= feasible else 0.0

        probs = [sum(p(k) for k in range(1, 6)), p(6), p(7)]
        order = sorted(range(3), key=lambda i: -probs[i])  # stable: ties keep phase order
        rows.append((upper, order[0], order[1], order[2], float(probs[0]), float(probs[1]),
                     float(probs[2])))
    return rows


def write_phase_file(path: str, rows) -> str:
    """One line per row: the three integers, then the probabilities as %.6f
    (create_prob_files.ipynb cell 10)."""
    with open(path, "w", encoding="utf-8") as f:
        for row in rows:
            f.write(" ".join(f"{x:.6f}" if isinstance(x, float) else str(int(x)) for x in row) + "\n")
    return str(path)
