"""On-device shot generation (grand_engine_sample).

CPU: the host restatement of Philox4x32-10 against the generator's published
known-answer vectors, and the host sampler's consistency.  GPU: the device
sampler writes exactly the host restatement's records (CSS errors, CSS
syndromes, DEM detectors + logicals), its flip rate matches p, and decoding the
sampled records on the device equals decoding them through the C ABI."""
import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth
from library_s_grand_gb300 import sample as SM


# Philox4x32-10 known-answer vectors (Salmon et al., SC 2011; Random123 kat_vectors):
# counter words, key words -> output words
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(ctr, key, want):
    got = SM.philox4x32_10(*ctr, *key)
    assert tuple(int(x) for x in got) == want


def test_host_sampler_rate_and_shot_offsets():
    p = np.full(300, 0.02, dtype=np.float32)
    f = SM.flips(p, 99, 0, 8000)
    assert abs(f.mean() - 0.02) < 0.002
    assert (SM.flips(p, 99, 500, 40) == f[500:540]).all()
    assert not (SM.flips(p, 100, 0, 40) == f[:40]).all()
    assert SM.flips(np.zeros(10, np.float32), 1, 0, 100).sum() == 0
    assert SM.flips(np.ones(10, np.float32), 1, 0, 100).mean() > 0.999


def _engine_css(gpulib, code, errors):
    from library_s_grand_gb300.engine import Engine
    eng = Engine(gpulib)
    eng.add_css(code.hx, code.hz, "x", errors, capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1))
    return eng


@pytest.mark.gpu
@pytest.mark.parametrize("errors", [True, False])
def test_device_css_records_equal_host_restatement(gpulib, errors):
    import torch
    code = synth.BB_CODES[144]()
    eng = _engine_css(gpulib, code, errors)
    rng = np.random.default_rng(3)
    p = np.exp(rng.uniform(np.log(1e-3), np.log(3e-2), code.m)).astype(np.float32)
    n, seed, first = 600, 0x1234_5678_9ABC, 1000
    L = eng.rec_lens[0]
    d_p = torch.from_numpy(p).cuda()
    d_rec = torch.full((n * L,), -7, dtype=torch.int32, device="cuda")
    assert eng.sample(0, d_p.data_ptr(), seed, first, n, d_rec.data_ptr()) == 0
    torch.cuda.synchronize()
    got = d_rec.cpu().numpy().reshape(n, L)
    want = SM.css_records(code.hz, p, seed, first, n, errors)
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_device_dem_records_equal_host_restatement(gpulib):
    import torch
    from library_s_grand_gb300.engine import Engine
    dem = synth.random_dem(2, detectors=90, mechanisms=300, logicals=7)
    eng = Engine(gpulib)
    eng.add_dem(dem.h, dem.l, capi.GrandDecoderConfig(3, 256, 0, 48, 10, -1), 0, None)
    n, seed = 500, 77
    L = eng.rec_lens[0]
    p = dem.p.astype(np.float32)
    d_p = torch.from_numpy(p).cuda()
    d_rec = torch.zeros(n * L, dtype=torch.int32, device="cuda")
    assert eng.sample(0, d_p.data_ptr(), seed, 0, n, d_rec.data_ptr()) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_rec.cpu().numpy().reshape(n, L), SM.dem_records(dem.h, dem.l, p, seed, 0, n))


@pytest.mark.gpu
def test_device_sampled_batch_decodes_like_the_c_abi(gpulib):
    import torch
    code = synth.BB_CODES[72]()
    eng = _engine_css(gpulib, code, True)
    n = 4096
    p = np.full(code.m, 0.01, dtype=np.float32)
    d_p = torch.from_numpy(p).cuda()
    d_rec = torch.zeros(n * code.m, dtype=torch.int32, device="cuda")
    d_res = torch.zeros(n * 72, dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    assert eng.sample(0, d_p.data_ptr(), 5, 0, n, d_rec.data_ptr(), sp) == 0
    assert eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=False) == 0
    assert eng.sync_status(sp) == 0
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    rec = d_rec.cpu().numpy().reshape(n, code.m)
    assert abs(rec.mean() - 0.01) < 0.002
    rc, ref, _ = capi.decode_css_ex(gpulib, "uniform", code.hx, code.hz, rec, None,
                                    capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1), "x")
    assert rc == 0
    assert len(O.fields_equal(res, ref)) == 0
