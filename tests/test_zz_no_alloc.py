"""The allocation-free decode entry point, checked against the regular one and the oracle.

grand_decode_cc_noalloc is for callers that may not allocate device memory
while they run: a real-time decoding loop in a quantum-control stack that
reserves its memory at start-up and must never wait in the allocator during an
experiment, or a process whose device memory already belongs to another
framework's pool.  It keeps all of its working memory in one fixed device array
that every call reuses, so the test calls it several times in a row with
different codes and batch sizes -- each call must ignore what the previous one
left behind -- and compares every deterministic result field with
grand_decode_cc on the same syndromes and with the oracle (integers: exact
equality).  The batches span more than one internal 2048-shot chunk and include
random syndromes, so the persistent search kernel and its job table run too; a
256 x 1024 code (the entry point's size limit) with hundreds of random
syndromes per chunk fills the fixed search arena, so its re-run rounds run as
well.  Free device memory is the same before and after a call.

This file is collected last on purpose: if it fails, every other test has
already run.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth

pytestmark = pytest.mark.gpu

FIELDS = ("found", "found_weight", "original_weight", "degenerate", "is_equal", "tam",
          "total_tested_combinations", "hibrido", "iteration")


def _syndromes(code, shots, p, rand, seed):
    _, syn = synth.css_shots(code.hz, shots, p, seed=seed)
    noise = (np.random.default_rng(seed + 1).random((rand, code.n)) < 0.5).astype(np.int32)
    out = np.concatenate([syn, noise])
    out = out[np.random.default_rng(seed + 2).permutation(len(out))]
    return np.ascontiguousarray(out, dtype=np.int32)


def _sparse_code(n, m, colw, seed):
    """A random CSS-shaped pair: Hz with colw ones per column, Hx its row-shifted copy."""
    rng = np.random.default_rng(seed)
    hz = np.zeros((n, m), dtype=np.int32)
    for c in range(m):
        hz[rng.choice(n, size=colw, replace=False), c] = 1
    return synth.CssCode(f"sparse{n}x{m}", np.roll(hz, 1, axis=0), hz)


def _regular(lib, code, syn, cfg):
    rc, results = capi.run_grand_shots_cc(lib, code.hx, code.hz, None, syn, cfg, b"x")
    assert rc == 0
    return capi.results_array(results)


def _noalloc(lib, code, syn, cfg):
    """Two calls in a row on the same inputs (the second into a fresh result
    buffer); returns the second call's results and the free device memory seen
    just before and just after it."""
    import torch
    d_h = torch.from_numpy(np.ascontiguousarray(code.hz, dtype=np.int32)).cuda()
    d_s = torch.from_numpy(syn).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    out, free = None, None
    for rep in range(2):
        d_r = torch.full((len(syn) * 72,), 0xAB, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info()[0]
        rc = lib.grand_decode_cc_noalloc(d_h.data_ptr(), code.n, code.m, d_s.data_ptr(), len(syn),
                                         ctypes.byref(cfg), d_r.data_ptr(), stream)
        after = torch.cuda.mem_get_info()[0]
        assert rc == 0
        out = np.frombuffer(d_r.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE).copy()
        free = (before, after)
    return out, free


def _check(got, want, what):
    for f in FIELDS:
        bad = np.nonzero(got[f] != want[f])[0]
        assert len(bad) == 0, f"{what}: field {f} differs at {bad[:5]}"


def test_noalloc_equals_regular_entry_point_and_oracle_on_consecutive_calls(gpulib, port):
    bb72, bb144 = synth.BB_CODES[72](), synth.BB_CODES[144]()
    big = _sparse_code(256, 1024, 3, 5)
    # (code, syndromes, config, whether some shot needs the persistent search
    # kernel, how many shots the oracle checks)
    cases = [
        (bb72, _syndromes(bb72, 3000, 0.03, 40, 11), capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1), True, None),
        (big, _syndromes(big, 1500, 0.0015, 600, 14), capi.GrandDecoderConfig(2, 256, 0, 64, 10, -1), True, 160),
        (bb144, _syndromes(bb144, 2500, 0.01, 16, 12), capi.GrandDecoderConfig(4, 256, 0, 64, 10, 0), True, None),
        (bb72, _syndromes(bb72, 700, 0.05, 8, 13), capi.GrandDecoderConfig(2, 256, 0, 64, 10, -1), False, None),
    ]
    for code, syn, cfg, heavy, n_oracle in cases:
        what = f"{code.name} W={cfg.max_error_weight} mode={cfg.mode_of_search}"
        want = _regular(gpulib, code, syn, cfg)
        got, (free_before, free_after) = _noalloc(gpulib, code, syn, cfg)
        _check(got, want, what + " vs grand_decode_cc")
        sl = slice(None) if n_oracle is None else slice(0, n_oracle)
        o_cfg = O.make_config(cfg.max_error_weight, mode=cfg.mode_of_search,
                              cap=cfg.max_size_active_positions, thr=cfg.threshold_for_hybrid)
        rc, ref, _ = port.css(O.UNIFORM, code.hx, code.hz, None, syn[sl], o_cfg, "x")
        assert rc == 0
        _check(got[sl], ref, what + " vs oracle")
        assert free_after == free_before, f"{what}: free device memory changed during the call"
        assert want["found"].sum() > 100
        if heavy:  # beyond the 4096-candidate budget of the triage warp
            assert want["total_tested_combinations"].max() > 4096


def test_noalloc_rejects_sizes_beyond_its_limit(gpulib, capfd):
    import torch
    big = torch.zeros(300 * 64, dtype=torch.int32, device="cuda")
    syn = torch.zeros(300, dtype=torch.int32, device="cuda")
    res = torch.zeros(72, dtype=torch.uint8, device="cuda")
    cfg = capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1)
    rc = gpulib.grand_decode_cc_noalloc(big.data_ptr(), 300, 64, syn.data_ptr(), 1,
                                        ctypes.byref(cfg), res.data_ptr(), None)
    assert rc == -3
    assert "at most 256 rows" in capfd.readouterr().err
