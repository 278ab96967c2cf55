"""Seeded synthetic codes and shots for the GRAND decoder.

The upstream library ships a handful of fixed matrices and builds its decoding
inputs offline with stim / qldpc / qiskit (Create_Files/stim_matrix_generation.py:30-77,
Create_Files/create_syndrome_file_cc.py:21-31), none of which exist here.  This
module produces the same kinds of inputs from numpy's PCG64 generator:

* bivariate-bicycle CSS codes: x = S_l (x) I_m, y = I_l (x) S_m with S the cyclic
  shift, A and B sums of monomials, Hx = [A|B], Hz = [B^T|A^T];
* random sparse detector error models (H_dem detectors x mechanisms, L_dem
  mechanisms x logicals, per-mechanism probabilities and FP64 LLRs);
* i.i.d. X-error shots for CSS codes and independent mechanism flips for DEMs;
* the phase-mask and LLR text files read by the prob / ML entry points.

All arrays are int32 0/1, row-major, as the C ABI expects.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

__all__ = [
    "BB_CODES", "bb_code", "CssCode", "Dem", "random_dem", "css_shots", "dem_shots",
    "write_phase_file", "write_llr_file", "llr_from_p",
]


def _shift(n: int) -> np.ndarray:
    return np.roll(np.eye(n, dtype=np.int64), 1, axis=1)


@dataclasses.dataclass
class CssCode:
    name: str
    hx: np.ndarray  # (n_checks, n_qubits) int32
    hz: np.ndarray

    @property
    def n(self) -> int:
        return int(self.hx.shape[0])

    @property
    def m(self) -> int:
        return int(self.hx.shape[1])


def bb_code(l: int, m: int, a_terms, b_terms, name: str = "") -> CssCode:
    """Bivariate-bicycle code.  Terms are ("x", k) or ("y", k) monomials."""
    x = np.kron(_shift(l), np.eye(m, dtype=np.int64))
    y = np.kron(np.eye(l, dtype=np.int64), _shift(m))

    def poly(terms):
        acc = np.zeros((l * m, l * m), dtype=np.int64)
        for var, k in terms:
            base = x if var == "x" else y
            acc = acc + np.linalg.matrix_power(base, k)
        return acc % 2

    A, B = poly(a_terms), poly(b_terms)
    hx = np.hstack([A, B]).astype(np.int32)
    hz = np.hstack([B.T, A.T]).astype(np.int32)
    return CssCode(name or f"bb_{2 * l * m}", hx, hz)


_AB = ([("x", 3), ("y", 1), ("y", 2)], [("y", 3), ("x", 1), ("x", 2)])
_AB288 = ([("x", 3), ("y", 2), ("y", 7)], [("y", 3), ("x", 1), ("x", 2)])

#: The four bivariate-bicycle codes of the benchmark mix: [[72,12,6]],
#: [[108,8,10]], [[144,12,12]] and [[288,12,18]].
BB_CODES = {
    72: lambda: bb_code(6, 6, *_AB, name="bb72"),
    108: lambda: bb_code(9, 6, *_AB, name="bb108"),
    144: lambda: bb_code(12, 6, *_AB, name="bb144"),
    288: lambda: bb_code(12, 12, *_AB288, name="bb288"),
}


@dataclasses.dataclass
class Dem:
    h: np.ndarray      # (detectors, mechanisms) int32
    l: np.ndarray      # (mechanisms, logicals) int32
    p: np.ndarray      # (mechanisms,) float64
    llr: np.ndarray    # (mechanisms,) float64, log((1-p)/p)

    @property
    def n(self) -> int:
        return int(self.h.shape[0])

    @property
    def m(self) -> int:
        return int(self.h.shape[1])

    @property
    def n_logicos(self) -> int:
        return int(self.l.shape[1])


def llr_from_p(p: np.ndarray) -> np.ndarray:
    """Per-position LLR computed once in FP64."""
    p = np.asarray(p, dtype=np.float64)
    return np.log((1.0 - p) / p)


def random_dem(seed: int, detectors: int = 120, mechanisms: int = 720, logicals: int = 12,
               col_weights=(2, 3, 4), p_logical: float = 0.1,
               p_range=(1e-4, 5e-3)) -> Dem:
    """Random sparse DEM: each mechanism flips a uniform-weight set of distinct
    detectors and each logical with probability p_logical; mechanism
    probabilities are log-uniform in p_range."""
    rng = np.random.default_rng(seed)
    h = np.zeros((detectors, mechanisms), dtype=np.int32)
    lo, hi = min(col_weights), max(col_weights)
    for c in range(mechanisms):
        w = int(rng.integers(lo, hi + 1))
        rows = rng.choice(detectors, size=w, replace=False)
        h[rows, c] = 1
    lmat = (rng.random((mechanisms, logicals)) < p_logical).astype(np.int32)
    p = np.exp(rng.uniform(np.log(p_range[0]), np.log(p_range[1]), size=mechanisms))
    return Dem(h, lmat, p, llr_from_p(p))


def css_shots(code_h: np.ndarray, num_shots: int, p, seed: int):
    """i.i.d. errors (scalar p or per-qubit p array) and their syndromes H.e."""
    rng = np.random.default_rng(seed)
    m = code_h.shape[1]
    p = np.broadcast_to(np.asarray(p, dtype=np.float64), (m,))
    errors = (rng.random((num_shots, m)) < p).astype(np.int32)
    syndromes = (errors.astype(np.int64) @ code_h.T.astype(np.int64) % 2).astype(np.int32)
    return errors, syndromes


def dem_shots(dem: Dem, num_shots: int, seed: int):
    """Independent mechanism flips -> (detectors, true logical flips, flips)."""
    rng = np.random.default_rng(seed)
    flips = (rng.random((num_shots, dem.m)) < dem.p).astype(np.int64)
    det = (flips @ dem.h.T.astype(np.int64) % 2).astype(np.int32)
    log = (flips @ dem.l.astype(np.int64) % 2).astype(np.int32)
    return det, log, flips.astype(np.int32)


def write_phase_file(path: str, lines) -> str:
    """lines: iterable of (tam_upper, o0, o1, o2, p0, p1, p2)."""
    with open(path, "w", encoding="utf-8") as f:
        for t in lines:
            f.write("%d %d %d %d %r %r %r\n" % (int(t[0]), int(t[1]), int(t[2]), int(t[3]),
                                                float(t[4]), float(t[5]), float(t[6])))
    return os.fspath(path)


def write_llr_file(path: str, llr: np.ndarray) -> str:
    """One value per line, %.17g, so that "%f" parsing yields float32(llr)."""
    with open(path, "w", encoding="utf-8") as f:
        for v in np.asarray(llr, dtype=np.float64):
            f.write("%.17g\n" % v)
    return os.fspath(path)
