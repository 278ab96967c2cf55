"""Continuous-batching server on the GPU.  Requests of 1-256 shots over the
serving mix (four bivariate-bicycle codes with syndrome records, W = 3, and the
120 x 720 random DEM in ML mode) are submitted concurrently from several threads
and replayed as a Poisson trace; every request's results must equal those of
decoding that request alone and the oracle's for each of its shots."""
import threading

import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth
from library_s_grand_gb300.engine import Engine
from library_s_grand_gb300.server import Server

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serving(gpulib, tmp_path_factory):
    tmp = tmp_path_factory.mktemp("srv")
    dem = synth.random_dem(0)
    lf = synth.write_llr_file(str(tmp / "llr.txt"), dem.llr)
    eng = Engine(gpulib)
    codes = []
    for n in (72, 108, 144, 288):
        c = synth.BB_CODES[n]()
        eng.add_css(c.hx, c.hz, "x", False, capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1))
        codes.append(("css", c))
    eng.add_dem(dem.h, dem.l, capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1), 2, lf)
    codes.append(("dem", dem))
    return eng, codes, lf


def make_requests(codes, count, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        n = int(rng.integers(1, 257))
        cid = rng.integers(0, len(codes), size=n).astype(np.int32)
        recs = []
        for j, c in enumerate(cid):
            kind, code = codes[c]
            if kind == "css":
                _, s = synth.css_shots(code.hz, 1, 0.01, seed=seed * 100003 + i * 517 + j)
                recs.append(s[0])
            else:
                det, log, _ = synth.dem_shots(code, 1, seed * 100003 + i * 517 + j)
                recs.append(np.concatenate([det[0], log[0]]))
        reqs.append((cid, np.concatenate(recs).astype(np.int32)))
    return reqs


def by_oracle(codes, cid, rec, lf):
    """Each shot decoded by the oracle (shots of one code decoded together, in order)."""
    port = O.Port()
    lens = np.array([codes[c][1].n + (codes[c][1].n_logicos if codes[c][0] == "dem" else 0)
                     for c in range(len(codes))])
    starts = np.concatenate([[0], np.cumsum(lens[cid])[:-1]])
    out = np.zeros(len(cid), dtype=O.RESULT_DTYPE)
    cfg = O.make_config(3, cap=64)
    for c, (kind, code) in enumerate(codes):
        idx = np.nonzero(cid == c)[0]
        if len(idx) == 0:
            continue
        rows = np.stack([rec[starts[i]:starts[i] + lens[c]] for i in idx])
        if kind == "css":
            rc, r, _ = port.css(O.UNIFORM, code.hx, code.hz, None, rows, cfg, "x")
        else:
            rc, r, *_ = port.dem(O.ML, code.h, code.l, rows[:, :code.n], rows[:, code.n:], cfg, lf)
        assert rc == 0
        out[idx] = r
    return out


def alone(eng, req):
    cid, rec = req
    rc, res = eng.decode(rec, cid)
    assert rc == 0
    return res


def test_concurrent_requests_equal_alone_and_oracle(serving):
    eng, codes, lf = serving
    srv = Server(eng, slots=3, max_shots_per_batch=1024)
    slots, nbytes = srv.info()
    assert slots == 3 and nbytes > 0
    reqs = make_requests(codes, 60, 1)
    got = [None] * len(reqs)
    lock = threading.Lock()

    def worker(idx):
        for i in idx:
            cid, rec = reqs[i]
            with lock:
                rid = srv.submit(rec, cid)
            rc, res, lat = srv.wait(rid)
            assert rc == 0 and lat >= 0.0
            got[i] = res

    threads = [threading.Thread(target=worker, args=(range(k, len(reqs), 4),)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i, req in enumerate(reqs):
        assert len(O.fields_equal(got[i], alone(eng, req))) == 0, i
        assert len(O.fields_equal(got[i], by_oracle(codes, *req, lf))) == 0, i
    srv.close()


def test_poisson_replay_equals_alone_and_oracle(serving):
    eng, codes, lf = serving
    srv = Server(eng, slots=4, max_shots_per_batch=2048)
    reqs = make_requests(codes, 200, 2)
    rng = np.random.default_rng(3)
    arrival = np.cumsum(rng.exponential(1.0 / 4000.0, size=len(reqs)))
    ns = np.array([len(c) for c, _ in reqs], dtype=np.int32)
    sc = np.concatenate([c for c, _ in reqs])
    rec = np.concatenate([r for _, r in reqs])
    rc, res, lat, wall = srv.replay(arrival, ns, rec, sc)
    assert rc == 0
    assert (lat > 0).all() and wall > 0
    rc2, ref = eng.decode(rec, sc)
    assert rc2 == 0
    assert len(O.fields_equal(res, ref)) == 0
    assert len(O.fields_equal(res, by_oracle(codes, sc, rec, lf))) == 0
    srv.close()


def test_admission_by_memory(serving):
    eng, _, _ = serving
    srv = Server(eng, slots=8, max_shots_per_batch=1024, hbm_budget_bytes=2 * 45 * (1 << 20))
    slots, nbytes = srv.info()
    assert 1 <= slots < 8 and nbytes <= 2 * 45 * (1 << 20)
    srv.close()
    with pytest.raises(RuntimeError):
        Server(eng, slots=2, max_shots_per_batch=1024, hbm_budget_bytes=1 << 20)
