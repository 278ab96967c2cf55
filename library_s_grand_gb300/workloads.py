"""The benchmark workloads as concrete seeded inputs.

Each builder returns the exact arrays the benchmark and the full-size parity
tests decode, so that both work on the same shots:

* ``uniform_bb72``   -- grand_decode_cc on BB[[72,12,6]] (Hz 36 x 72): X errors,
  p = 0.005, 1024 shots, seed 0, max_error_weight 3, cap 64, mode -1;
* ``prob_bb144``     -- grand_decode_prob_cc on BB[[144,12,12]] (Hz 72 x 144): per-qubit
  p log-uniform in [1e-3, 1e-2] (drawn from seed 0), X errors, 16384 shots,
  max_error_weight 4, cap 64, phase mask "300 0 1 2" (phase 0 = weights 1..5);
* ``ml_dem``         -- grand_decode_ML_cln on a random 120 x 720 DEM (column weight
  2-4, 12 logicals, p log-uniform in [1e-4, 5e-3]), 65536 shots, max_error_weight 3,
  cap 64; LLRs log((1-p)/p) in FP64, written with %.17g;
* ``bb_mix``         -- 100k syndrome records mixing BB[[72]], [[108]] (W = 3),
  [[144]] and [[288]] (W = 4) at p = 0.003, 25k each, shuffled with seed 0, cap 64;
* ``stress_bb144``   -- random syndromes (Bernoulli 1/2) of BB[[144,12,12]], W = 4:
  nothing matches, so every candidate of the three threshold iterations is tested;
* ``stress_dem``     -- random detectors (Bernoulli 0.36) of the ``ml_dem`` matrix,
  grand_decode_cln, W = 3, cap 64: first active sets of ~40 columns (up to 64),
  later iterations above the cap repeat that set (the DEM family's cap rule), and
  nothing matches, so every candidate is tested (at most C(64,3) + C(64,2) + 64 =
  43,744 per iteration).

The upstream library builds its inputs with stim / qldpc (not available); these
are numpy PCG64 stand-ins with the shapes and distributions of those workloads.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from . import synth

PHASE_300_012 = [(300, 0, 1, 2, 1.0, 0.0, 0.0)]

# (n, max_error_weight) of the four codes of the mixed batch
MIX_SPEC = [(72, 3), (108, 3), (144, 4), (288, 4)]
MIX_PER_CODE = 25000
MIX_P = 0.003


def config_tuple(W, cap=64, mode=-1, thr=10, tpb=256, use_gpu_sum=0):
    """GrandDecoderConfig fields in declaration order."""
    return (W, tpb, use_gpu_sum, cap, thr, mode)


@dataclasses.dataclass
class CssWorkload:
    code: synth.CssCode
    errors: np.ndarray | None
    syndromes: np.ndarray
    W: int
    cap: int
    variant: str                  # "uniform" or "prob"
    phase_lines: list | None = None

    def phase_file(self, directory: str) -> str | None:
        if self.phase_lines is None:
            return None
        return synth.write_phase_file(os.path.join(directory, "phase.txt"), self.phase_lines)

    @property
    def config(self):
        return config_tuple(self.W, self.cap)


def uniform_bb72() -> CssWorkload:
    code = synth.BB_CODES[72]()
    errors, syn = synth.css_shots(code.hz, 1024, 0.005, seed=0)
    return CssWorkload(code, errors, syn, 3, 64, "uniform")


def prob_bb144(seed: int = 0, shots: int = 16384) -> CssWorkload:
    """The headline batch (seed 0); other seeds draw other error shots with the same p."""
    code = synth.BB_CODES[144]()
    rng = np.random.default_rng(0)
    p = np.exp(rng.uniform(np.log(1e-3), np.log(1e-2), code.m))
    errors, syn = synth.css_shots(code.hz, shots, p, seed=1 + seed)
    return CssWorkload(code, errors, syn, 4, 64, "prob", PHASE_300_012)


@dataclasses.dataclass
class DemWorkload:
    dem: synth.Dem
    detectors: np.ndarray
    logicals: np.ndarray
    W: int
    cap: int

    def llr_file(self, directory: str) -> str:
        return synth.write_llr_file(os.path.join(directory, "llr.txt"), self.dem.llr)

    @property
    def config(self):
        return config_tuple(self.W, self.cap)

    @property
    def records(self) -> np.ndarray:
        """Detector bits followed by the true logical flips, one row per shot."""
        return np.ascontiguousarray(np.concatenate([self.detectors, self.logicals], axis=1),
                                    dtype=np.int32)


def ml_dem(shots: int = 65536) -> DemWorkload:
    dem = synth.random_dem(0)
    det, log, _ = synth.dem_shots(dem, shots, 1)
    return DemWorkload(dem, det, log, 3, 64)


@dataclasses.dataclass
class MixWorkload:
    codes: list          # synth.CssCode per code index
    Ws: list             # max_error_weight per code index
    syndromes: list      # per code: (MIX_PER_CODE, n) int32
    order: np.ndarray    # batch position -> index into the per-code concatenation
    shot_code: np.ndarray  # per batch position: code index

    @property
    def num_shots(self) -> int:
        return len(self.order)

    def records(self) -> np.ndarray:
        """The shuffled batch's records back to back (flat int32)."""
        rows = [r for s in self.syndromes for r in s]
        return np.concatenate([rows[i] for i in self.order]).astype(np.int32)


def bb_mix(per_code: int = MIX_PER_CODE) -> MixWorkload:
    codes, Ws, syns = [], [], []
    for ci, (n, W) in enumerate(MIX_SPEC):
        c = synth.BB_CODES[n]()
        _, s = synth.css_shots(c.hz, per_code, MIX_P, seed=40 + ci)
        codes.append(c)
        Ws.append(W)
        syns.append(s)
    N = per_code * len(MIX_SPEC)
    order = np.random.default_rng(0).permutation(N)
    sc = np.concatenate([np.full(per_code, ci, np.int32) for ci in range(len(MIX_SPEC))])[order]
    return MixWorkload(codes, Ws, syns, order, sc)


def stress_bb144(shots: int, seed: int = 1):
    """(code, random syndromes) of BB[[144,12,12]]."""
    code = synth.BB_CODES[144]()
    syn = (np.random.default_rng(seed).random((shots, code.n)) < 0.5).astype(np.int32)
    return code, syn


STRESS_DEM_DENSITY = 0.36


def stress_dem(shots: int, seed: int = 1) -> DemWorkload:
    """Random detector records of the ml_dem matrix (logical flips all zero),
    W = 3, cap 64, for a uniform (grand_decode_cln) search."""
    dem = synth.random_dem(0)
    rng = np.random.default_rng(seed)
    det = (rng.random((shots, dem.n)) < STRESS_DEM_DENSITY).astype(np.int32)
    log = np.zeros((shots, dem.l.shape[1]), dtype=np.int32)
    return DemWorkload(dem, det, log, 3, 64)
