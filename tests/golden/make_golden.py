"""Regenerate the golden fixtures in this directory.

Each fixture is one decoding call: its inputs, its configuration, the text of
any phase-mask / LLR file, and the result fields the upstream library returned
for it in its CPU search mode (mode_of_search = -1, or mode 1 where every
iteration stays on upstream's CPU branch).  The upstream library is the one
oracle/Makefile builds unmodified from the upstream sources; the error-pattern
and syndrome known-answer sets are rows of the upstream fixture files
Errors/patterns_{72,144}.txt and Syndromes/syndromes_72.txt.  The upstream
matrices in H_Matrix/ are recorded by SHA-256 of their parsed content, so the
bivariate-bicycle construction can be checked against them without the files.

Run from the repository root, with the upstream sources at REF_DIR (the argument,
or the GRAND_REFERENCE_DIR environment variable):

    python tests/golden/make_golden.py REF_DIR
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from library_s_grand_gb300 import synth as S  # noqa: E402
from library_s_grand_gb300 import workloads as W_  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def matrix_digest(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a, dtype=np.int32)
    h = hashlib.sha256()
    h.update(np.asarray(a.shape, dtype=np.int64).tobytes())
    h.update(a.tobytes())
    return h.hexdigest()


def read_bits_file(path, n_cols, rows=None):
    out = []
    with open(path, encoding="utf-8") as f:
        for i, line in enumerate(f):
            line = line.strip()
            if not line:
                continue
            parts = line.split()
            if len(parts) == n_cols:
                v = [int(x) for x in parts]
            else:
                v = [int(ch) for ch in parts[0]]
            out.append(v)
    a = np.asarray(out, dtype=np.int32)
    return a if rows is None else a[rows]


class Writer:
    def __init__(self, ref):
        self.ref = ref
        self.index = []

    def css(self, name, variant, code, errors, syndromes, cfg, t="x", phase_lines=None,
            keep=None):
        pf = None
        if phase_lines is not None:
            pf = S.write_phase_file(os.path.join(OUT, "_tmp_phase.txt"), phase_lines)
        rc, res = self.ref.css(variant, code.hx, code.hz, errors, syndromes, cfg, t, pf)
        assert rc == 0, (name, rc)
        sel = np.arange(len(res)) if keep is None else keep(res)
        data = dict(kind="css", variant=variant, hx=code.hx.astype(np.uint8),
                    hz=code.hz.astype(np.uint8), type=t, cfg=np.asarray(list_cfg(cfg)),
                    res=res[sel])
        if errors is not None:
            data["errors"] = errors[sel].astype(np.uint8)
        else:
            data["syndromes"] = syndromes[sel].astype(np.uint8)
        if phase_lines is not None:
            data["phase_text"] = open(pf, encoding="utf-8").read()
            os.remove(pf)
        self.save(name, data)

    def dem(self, name, variant, dem, det, log, cfg, phase_lines=None, llr=None, keep=None):
        f = None
        if phase_lines is not None:
            f = S.write_phase_file(os.path.join(OUT, "_tmp_phase.txt"), phase_lines)
        if llr is not None:
            f = S.write_llr_file(os.path.join(OUT, "_tmp_llr.txt"), llr)
        rc, res = self.ref.dem(variant, dem.h, dem.l, det, log, cfg, f)
        assert rc == 0, (name, rc)
        sel = np.arange(len(res)) if keep is None else keep(res)
        data = dict(kind="dem", variant=variant, h=dem.h.astype(np.uint8),
                    l=dem.l.astype(np.uint8), cfg=np.asarray(list_cfg(cfg)),
                    detectors=det[sel].astype(np.uint8), logicals=log[sel].astype(np.uint8),
                    res=res[sel])
        if f is not None:
            data["file_text"] = open(f, encoding="utf-8").read()
            os.remove(f)
        if llr is not None:
            data["llr64"] = np.asarray(llr, dtype=np.float64)
        self.save(name, data)

    def save(self, name, data):
        path = os.path.join(OUT, name + ".npz")
        np.savez_compressed(path, **data)
        res = data["res"]
        self.index.append(dict(name=name, shots=int(len(res)), found=int(res["found"].sum()),
                               tested=int(res["total_tested_combinations"].sum())))
        print(f"{name}: {len(res)} shots, found {int(res['found'].sum())}, "
              f"tested {int(res['total_tested_combinations'].sum())}")


def list_cfg(c):
    return [c.max_error_weight, c.threads_per_block, c.use_gpu_sum,
            c.max_size_active_positions, c.threshold_for_hybrid, c.mode_of_search]


def cpu_branch_only(res):
    """Keep shots on which upstream never took its GPU branch (no GPU here)."""
    return np.nonzero(res["hibrido"] < 0)[0]


def main(ref_dir):
    O.build(ref_dir=ref_dir)
    ref = O.Reference()
    w = Writer(ref)
    mk = O.make_config

    # --- matrix digests of the upstream fixtures -------------------------------
    digests = {}
    for n in (72, 108, 144, 288):
        for k in ("hx", "hz"):
            a = np.loadtxt(os.path.join(ref_dir, "H_Matrix", f"{k}_ibm_{n}.txt"), dtype=np.int32)
            digests[f"{k}_{n}"] = matrix_digest(a)

    bb72, bb144, bb288 = S.BB_CODES[72](), S.BB_CODES[144](), S.BB_CODES[288]()
    bb108 = S.BB_CODES[108]()

    # --- known-answer sets from the upstream fixture files ---------------------
    p72 = read_bits_file(os.path.join(ref_dir, "Errors", "patterns_72.txt"), 72)
    rng = np.random.default_rng(7)
    rows = np.concatenate([np.arange(72), 72 + rng.choice(len(p72) - 72, 400, replace=False)])
    w.css("kat_patterns72_cc_w3", O.UNIFORM, bb72, p72[rows], None, mk(3))
    p144 = read_bits_file(os.path.join(ref_dir, "Errors", "patterns_144.txt"), 144)
    rows = np.concatenate([np.arange(0, 144, 3), 144 + rng.choice(len(p144) - 144, 150, replace=False)])
    w.css("kat_patterns144_cc_w4", O.UNIFORM, bb144, p144[rows], None, mk(4))
    s72 = read_bits_file(os.path.join(ref_dir, "Syndromes", "syndromes_72.txt"), 36)
    w.css("kat_syndromes72_cc_w6", O.UNIFORM, bb72, None, s72, mk(6))

    # --- seeded synthetic CSS --------------------------------------------------
    for W in (1, 2, 3, 4):
        e, _ = S.css_shots(bb72.hz, 400, 0.02, seed=100 + W)
        w.css(f"cc_bb72_x_err_w{W}", O.UNIFORM, bb72, e, None, mk(W))
    e, _ = S.css_shots(bb72.hx, 400, 0.02, seed=111)
    w.css("cc_bb72_z_err_w3", O.UNIFORM, bb72, e, None, mk(3), t="z")
    _, s = S.css_shots(bb108.hz, 300, 0.015, seed=112)
    w.css("cc_bb108_x_syn_w3", O.UNIFORM, bb108, None, s, mk(3))
    e, _ = S.css_shots(bb288.hz, 200, 0.006, seed=113)
    w.css("cc_bb288_x_err_w3", O.UNIFORM, bb288, e, None, mk(3))
    e, _ = S.css_shots(bb72.hz, 300, 0.03, seed=114)
    w.css("cc_bb72_w7", O.UNIFORM, bb72, e, None, mk(7))
    # hard shots: random syndromes force exhaustive enumeration
    rs = (np.random.default_rng(1).random((6, 72)) < 0.5).astype(np.int32)
    w.css("cc_bb144_randsyn_w2", O.UNIFORM, bb144, None, rs, mk(2))
    rs = (np.random.default_rng(2).random((3, 72)) < 0.5).astype(np.int32)
    w.css("cc_bb144_randsyn_w3", O.UNIFORM, bb144, None, rs, mk(3))
    rs = (np.random.default_rng(3).random((40, 36)) < 0.15).astype(np.int32)
    w.css("cc_bb72_sparse_randsyn_w4", O.UNIFORM, bb72, None, rs, mk(4))
    # mode 1: small iterations on the CPU branch, large ones skipped by the cap
    e, _ = S.css_shots(bb72.hz, 400, 0.04, seed=115)
    w.css("cc_bb72_mode1_cap", O.UNIFORM, bb72, e, None, mk(3, mode=1, cap=4, thr=12),
          keep=cpu_branch_only)
    # an unknown mode runs no branch at all
    w.css("cc_bb72_mode5", O.UNIFORM, bb72, e[:50], None, mk(2, mode=5))

    # --- probability-ordered CSS -----------------------------------------------
    p = np.exp(np.random.default_rng(0).uniform(np.log(1e-3), np.log(1e-2), 144))
    e, _ = S.css_shots(bb144.hz, 600, 3 * p, seed=120)
    w.css("prob_cc_bb144_w4_phase012", O.PROB, bb144, e, None, mk(4, cap=64),
          phase_lines=[(300, 0, 1, 2, 1.0, 0.0, 0.0)])
    e, _ = S.css_shots(bb72.hz, 300, 0.03, seed=121)
    masks = [(3, 1, 0, 2, 0.2, 0.8, 0.0), (8, 0, 1, 2, 0.9, 0.1, 0.0), (40, 0, 0, 1, 0.5, 0.5, 0.0)]
    w.css("prob_cc_bb72_w6_masks", O.PROB, bb72, e, None, mk(6), phase_lines=masks)
    w.css("prob_cc_bb72_w2_masks", O.PROB, bb72, e, None, mk(2), phase_lines=masks)
    w.css("prob_cc_bb72_w7_masks", O.PROB, bb72, e[:120], None, mk(7),
          phase_lines=[(300, 2, 1, 0, 0.1, 0.1, 0.8)])
    w.css("prob_cc_bb72_z_w3_order1", O.PROB, bb72, e[:200], None, mk(3), t="Z",
          phase_lines=[(300, 1, 0, 2, 0.1, 0.1, 0.8)])

    # --- DEM family ------------------------------------------------------------
    dem = S.random_dem(11, detectors=60, mechanisms=240, logicals=8, p_range=(2e-3, 2e-2))
    det, log, _ = S.dem_shots(dem, 400, 12)
    for W, cap in ((1, 300), (2, 10), (3, 20), (3, 300), (4, 16)):
        w.dem(f"cln_dem60_w{W}_cap{cap}", O.UNIFORM, dem, det, log, mk(W, cap=cap))
        w.dem(f"ml_dem60_w{W}_cap{cap}", O.ML, dem, det, log, mk(W, cap=cap), llr=dem.llr)
    masks = [(4, 1, 0, 2, 0.0, 1.0, 0.0), (300, 0, 1, 2, 1.0, 0.0, 0.0)]
    for W, cap in ((2, 12), (5, 20), (6, 10)):
        w.dem(f"prob_cln_dem60_w{W}_cap{cap}", O.PROB, dem, det, log, mk(W, cap=cap),
              phase_lines=masks)
    # irregular DEM with empty columns and duplicated columns
    dem2 = S.random_dem(21, detectors=40, mechanisms=160, logicals=5, col_weights=(1, 5),
                        p_range=(3e-3, 3e-2))
    dem2.h[:, 7] = 0
    dem2.h[:, 9] = dem2.h[:, 8]
    det, log, _ = S.dem_shots(dem2, 300, 22)
    w.dem("cln_dem40_irregular_w3", O.UNIFORM, dem2, det, log, mk(3, cap=25))
    w.dem("ml_dem40_irregular_w3", O.ML, dem2, det, log, mk(3, cap=25), llr=dem2.llr)
    # ML with some negative LLRs (p > 1/2): exercises the prefix-bound break
    llr_neg = dem2.llr.copy()
    llr_neg[::11] *= -0.25
    w.dem("ml_dem40_negllr_w3", O.ML, dem2, det, log, mk(3, cap=25), llr=llr_neg)
    # ML with tied LLRs: ties are broken by enumeration order
    llr_tie = np.round(dem2.llr)
    w.dem("ml_dem40_ties_w3", O.ML, dem2, det, log, mk(3, cap=25), llr=llr_tie)
    # the benchmark-shaped DEM (120 x 720, 12 logicals), small slices
    dem3 = S.random_dem(0)
    det, log, _ = S.dem_shots(dem3, 1000, 1)
    w.dem("ml_dem120_w3_cap64", O.ML, dem3, det, log, mk(3, cap=64), llr=dem3.llr)
    w.dem("cln_dem120_w3_cap64", O.UNIFORM, dem3, det, log, mk(3, cap=64))
    # heavier DEM shots
    det, log, _ = S.dem_shots(S.Dem(dem3.h, dem3.l, dem3.p * 6, dem3.llr), 200, 2)
    w.dem("ml_dem120_w3_cap40_dense", O.ML, dem3, det, log, mk(3, cap=40), llr=dem3.llr)
    w.dem("cln_dem120_w4_cap40_dense", O.UNIFORM, dem3, det, log, mk(4, cap=40))
    # mode 1 for the DEM family with every search on upstream's CPU branch
    w.dem("cln_dem120_mode1", O.UNIFORM, dem3, det, log, mk(3, mode=1, cap=30, thr=30),
          keep=cpu_branch_only)
    # more than 256 detectors: columns wider than 8 words (runtime-width kernels)
    dem4 = S.random_dem(31, detectors=300, mechanisms=600, logicals=10, p_range=(3e-3, 2e-2))
    det, log, _ = S.dem_shots(dem4, 250, 32)
    w.dem("cln_dem300_w3_cap24", O.UNIFORM, dem4, det, log, mk(3, cap=24))
    w.dem("ml_dem300_w3_cap24", O.ML, dem4, det, log, mk(3, cap=24), llr=dem4.llr)
    # ML at weight 5 and 6: sub-prefixes of 3-4 elements inside the register-blocked tiles
    det, log, _ = S.dem_shots(dem, 150, 33)
    w.dem("ml_dem60_w5_cap24", O.ML, dem, det, log, mk(5, cap=24), llr=dem.llr)
    w.dem("cln_dem60_w6_cap20", O.UNIFORM, dem, det, log, mk(6, cap=20))
    # BB[[288]] (5-word columns) random syndromes: exhaustive heavy searches
    rs = (np.random.default_rng(4).random((2, 144)) < 0.5).astype(np.int32)
    w.css("cc_bb288_randsyn_w3", O.UNIFORM, bb288, None, rs, mk(3))
    # the first shots of the integer-roofline stress input (BB[[144]] random
    # syndromes, seed 1, W = 4, cap 300): ~1.2e7 candidates each, all tested
    _, rs = W_.stress_bb144(3, seed=1)
    w.css("cc_bb144_randsyn_w4", O.UNIFORM, bb144, None, rs, mk(4, cap=300))

    with open(os.path.join(OUT, "index.json"), "w", encoding="utf-8") as f:
        json.dump(dict(matrix_sha256=digests, fixtures=w.index), f, indent=1, sort_keys=True)
    print("wrote", len(w.index), "fixtures")


if __name__ == "__main__":
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GRAND_REFERENCE_DIR")
    if not ref_dir:
        sys.exit("usage: make_golden.py REF_DIR  (or set GRAND_REFERENCE_DIR): the directory "
                 "holding the upstream grand_decoder.cu, H_Matrix/, Errors/ and Syndromes/")
    main(ref_dir)
