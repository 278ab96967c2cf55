"""The allocation-free decode entry point, checked against the regular one.

grand_decode_cc_noalloc is for callers that may not allocate device memory
while they run: a real-time decoding loop in a quantum-control stack that
reserves its memory at start-up and must never wait in the allocator during an
experiment, or a process whose device memory already belongs to another
framework's pool.  It keeps all of its working memory in one fixed device array
that every call reuses, so the test calls it several times in a row with
different codes and batch sizes -- each call must ignore what the previous one
left behind -- and compares every deterministic result field with
grand_decode_cc on the same syndromes (integers: exact equality).  The batches
span more than one internal 2048-shot chunk and include random syndromes, so
the persistent search kernel and its job table run too.

This file is collected last on purpose: if it fails, every other test has
already run.
"""
import ctypes

import numpy as np
import pytest

from library_s_grand_gb300 import capi, synth

pytestmark = pytest.mark.gpu

FIELDS = ("found", "found_weight", "original_weight", "degenerate", "is_equal", "tam",
          "total_tested_combinations", "hibrido", "iteration")


def _syndromes(code, shots, p, rand, seed):
    _, syn = synth.css_shots(code.hz, shots, p, seed=seed)
    noise = (np.random.default_rng(seed + 1).random((rand, code.n)) < 0.5).astype(np.int32)
    return np.ascontiguousarray(np.concatenate([syn, noise]), dtype=np.int32)


def _regular(lib, code, syn, cfg):
    rc, results = capi.run_grand_shots_cc(lib, code.hx, code.hz, None, syn, cfg, b"x")
    assert rc == 0
    return capi.results_array(results)


def _noalloc(lib, code, syn, cfg):
    import torch
    d_h = torch.from_numpy(np.ascontiguousarray(code.hz, dtype=np.int32)).cuda()
    d_s = torch.from_numpy(syn).cuda()
    d_r = torch.full((len(syn) * 72,), 0xAB, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.grand_decode_cc_noalloc(d_h.data_ptr(), code.n, code.m, d_s.data_ptr(), len(syn),
                                     ctypes.byref(cfg), d_r.data_ptr(), stream)
    assert rc == 0
    return np.frombuffer(d_r.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE).copy()


def test_noalloc_equals_regular_entry_point_on_consecutive_calls(gpulib):
    bb72, bb144 = synth.BB_CODES[72](), synth.BB_CODES[144]()
    # (code, syndromes, config, whether some shot needs the persistent search kernel)
    cases = [
        (bb72, _syndromes(bb72, 3000, 0.03, 40, 11), capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1), True),
        (bb144, _syndromes(bb144, 2500, 0.01, 16, 12), capi.GrandDecoderConfig(4, 256, 0, 64, 10, 0), True),
        (bb72, _syndromes(bb72, 700, 0.05, 8, 13), capi.GrandDecoderConfig(2, 256, 0, 64, 10, -1), False),
    ]
    for code, syn, cfg, heavy in cases:
        want = _regular(gpulib, code, syn, cfg)
        got = _noalloc(gpulib, code, syn, cfg)
        for f in FIELDS:
            bad = np.nonzero(got[f] != want[f])[0]
            assert len(bad) == 0, f"{code.name} W={cfg.max_error_weight}: field {f} differs at {bad[:5]}"
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
