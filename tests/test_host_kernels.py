"""CPU parity of the decode kernel itself: grand_decode.cuh (classification,
per-shot path, prefix-lookup search) compiled for the host (tests/host_kernels.cpp: one thread block
per kernel, one host thread per lane, warp collectives at a barrier) and run on
CSS and DEM shots (uniform, prob and ML searches) whose results must equal the
oracle's in every deterministic field, decoded pattern, logical flip and ML
cost.  A small light budget sends most iterations through the Jobs' lookup
search (lookup tiles, bucket walks, the Job finisher) as well as the per-shot
paths (classification, one-position iterations, bit-mask enumeration, run
tiles).
Runs without a GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from library_s_grand_gb300 import capi, synth

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    return None


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    cxx, inc = shutil.which("g++"), _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("hk") / "host_kernels")
    subprocess.run([cxx, "-std=c++20", "-O2", "-pthread",
                    "-I", os.path.join(ROOT, "library_s_grand_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), "-I", inc,
                    os.path.join(HERE, "host_kernels.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def _num_phases(W):  # upstream's phase count per max weight
    return {6: 2, 7: 3}.get(W, 1 if 0 < W < 6 else 0)


def _run(exe, d, H, Ho, records, errors_input, variant, cfg, masks, light, tile_k=4,
         L=None, logicals=None, llr_path=None, packed=False, fast=True):
    """CSS when L is None (Ho: the other check matrix), else DEM (L: m x n_logicos,
    logicals: the true flips).  Returns results, decoded errors, the emulator's
    log line and, for a DEM, decoded logical flips and ML costs."""
    W, _, _, cap, thr, mode = cfg
    n, m = H.shape
    N = records.shape[0]
    dem = L is not None
    nl = int(L.shape[1]) if dem else 0
    kind = 2 if dem else (1 if errors_input else 0)
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write(f"{1 if dem else 0} {variant} {kind} {n} {m} {N} {W} {mode} {thr} {cap} "
                f"{_num_phases(W) if variant == 1 else 0} {len(masks)} {light} {tile_k} {nl} "
                f"{1 if packed else 0}\n")
        for row in masks:
            f.write(" ".join(str(int(v)) for v in row[:4]) + "\n")
    np.ascontiguousarray(H, dtype=np.int32).tofile(os.path.join(d, "H.bin"))
    pack = (lambda a: capi.pack_bits(a)) if packed else (lambda a: np.asarray(a, dtype=np.int32))
    np.ascontiguousarray(pack(records)).tofile(os.path.join(d, "rec.bin"))
    if dem:
        np.ascontiguousarray(L, dtype=np.int32).tofile(os.path.join(d, "L.bin"))
        np.ascontiguousarray(pack(logicals)).tofile(os.path.join(d, "log.bin"))
        if llr_path:
            shutil.copy(llr_path, os.path.join(d, "llr.txt"))
    else:
        np.ascontiguousarray(Ho, dtype=np.int32).tofile(os.path.join(d, "Hother.bin"))
    env = dict(os.environ, GRAND_EMU_FAST="1" if fast else "0")
    out = subprocess.run([exe, d], capture_output=True, text=True, timeout=600, env=env)
    assert out.returncode == 0, out.stderr + out.stdout
    res = np.fromfile(os.path.join(d, "res.bin"), dtype=capi.RESULT_DTYPE)
    dec = np.fromfile(os.path.join(d, "dec.bin"), dtype=np.uint8).reshape(N, m)
    if not dem:
        return res, dec, out.stdout
    dlog = np.fromfile(os.path.join(d, "declog.bin"), dtype=np.uint8).reshape(N, nl)
    cost = np.fromfile(os.path.join(d, "cost.bin"), dtype=np.float32)
    return res, dec, out.stdout, dlog, cost


def _compare(res, dec, pres, pdec):
    bad = O.fields_equal(res, pres)
    assert len(bad) == 0, f"shots {bad[:5]}\nemulated {res[bad[:3]]}\noracle {pres[bad[:3]]}"
    diff = np.nonzero((dec != pdec).any(axis=1))[0]
    assert len(diff) == 0, f"decoded patterns differ on shots {diff[:5]}"


@pytest.mark.parametrize("W,mode,thr,cap,light,packed", [(4, -1, 10, 64, 3, False),
                                                         (4, -1, 10, 64, 3, True),
                                                         (3, 0, 10, 64, 5, False),
                                                         (4, 1, 8, 24, 12, False),
                                                         (5, -1, 10, 64, 4, False)])
def test_uniform_errors(emulator, port, tmp_path, W, mode, thr, cap, light, packed):
    code = synth.BB_CODES[72]()
    errors = np.concatenate([synth.css_shots(code.hz, 60, p, seed=900 + i)[0]
                             for i, p in enumerate((0.01, 0.03, 0.06))])
    cfg = (W, 256, 0, cap, thr, mode)
    res, dec, log = _run(emulator, str(tmp_path), code.hz, code.hx, errors, True, 0, cfg, [], light,
                         packed=packed)
    prc, pres, pdec = port.css(O.UNIFORM, code.hx, code.hz, errors, None, O.Config(*cfg), "x")
    assert prc == 0
    _compare(res, dec, pres, pdec)
    assert int(log.split()[3]) > 0 or light >= 12, log  # the launch had Jobs


@pytest.mark.parametrize("packed", [False, True])
def test_prob_syndromes(emulator, port, tmp_path, packed):
    code = synth.BB_CODES[108]()
    errors = np.concatenate([synth.css_shots(code.hz, 60, p, seed=950 + i)[0]
                             for i, p in enumerate((0.01, 0.03))])
    syn = (errors.astype(np.int64) @ code.hz.T.astype(np.int64) % 2).astype(np.int32)
    masks = [(9, 0, 1, 2, 0.5, 0.3, 0.2), (300, 1, 0, 2, 0.6, 0.3, 0.1)]
    phase = synth.write_phase_file(str(tmp_path / "phase.txt"), masks)
    cfg = (4, 256, 0, 30, 8, 1)  # mode 1: sets above 30 positions are skipped
    d = tmp_path / "run"
    d.mkdir()
    res, dec, log = _run(emulator, str(d), code.hz, code.hx, syn, False, 1, cfg, masks, 4,
                         packed=packed)
    prc, pres, pdec = port.css(O.PROB, code.hx, code.hz, None, syn, O.Config(*cfg), "x", phase)
    assert prc == 0
    _compare(res, dec, pres, pdec)
    assert int(log.split()[3]) > 0, log  # the launch had Jobs


@pytest.mark.parametrize("variant,packed", [("uniform", False), ("prob", False), ("ml", False),
                                            ("ml", True)])
def test_dem(emulator, port, tmp_path, variant, packed):
    dem = synth.random_dem(8, detectors=48, mechanisms=200, logicals=6, p_range=(4e-3, 3e-2))
    det, log, _ = synth.dem_shots(dem, 160, seed=990)
    cfg = (3, 256, 0, 24, 10, -1)
    masks, path, v, pv = [], None, 0, O.UNIFORM
    if variant == "prob":
        masks = [(5, 0, 1, 2, 0.7, 0.2, 0.1), (300, 0, 1, 2, 0.6, 0.3, 0.1)]
        path, v, pv = synth.write_phase_file(str(tmp_path / "phase.txt"), masks), 1, O.PROB
    elif variant == "ml":
        path, v, pv = synth.write_llr_file(str(tmp_path / "llr.txt"), dem.llr), 2, O.ML
    d = tmp_path / "run"
    d.mkdir()
    res, dec, out, dlog, cost = _run(emulator, str(d), dem.h, None, det, False, v, cfg, masks, 3,
                                     L=dem.l, logicals=log, llr_path=path if v == 2 else None,
                                     packed=packed)
    prc, pres, pdec, pdlog, pcost = port.dem(pv, dem.h, dem.l, det, log, O.Config(*cfg), path)
    assert prc == 0
    _compare(res, dec, pres, pdec)
    assert np.array_equal(dlog, pdlog)
    if variant == "ml":
        assert np.array_equal(cost.view(np.uint32), np.asarray(pcost, np.float32).view(np.uint32))
    assert int(out.split()[3]) > 0, out  # the launch had Jobs


def test_wide_rows_and_weight_six(emulator, port, tmp_path):
    # BB[[288]]: 144 check rows, so a column spans 5 words (8 with padding) and the
    # flagged-check counts take their general path; prob with W = 7 lists phase 1
    # (weight 6) and phase 2, in orders that differ by active-set size
    code = synth.BB_CODES[288]()
    errors = np.concatenate([synth.css_shots(code.hz, 40, p, seed=970 + i)[0]
                             for i, p in enumerate((0.004, 0.01))])
    masks = [(6, 1, 0, 2, 0.2, 0.7, 0.1), (300, 0, 2, 1, 0.8, 0.1, 0.1)]
    phase = synth.write_phase_file(str(tmp_path / "phase.txt"), masks)
    cfg = (7, 256, 0, 12, 6, 1)  # mode 1 and cap 12 keep the weight-6 blocks small
    d = tmp_path / "run"
    d.mkdir()
    res, dec, log = _run(emulator, str(d), code.hz, code.hx, errors, True, 1, cfg, masks, 3)
    prc, pres, pdec = port.css(O.PROB, code.hx, code.hz, errors, None, O.Config(*cfg), "x", phase)
    assert prc == 0
    _compare(res, dec, pres, pdec)


def _write_code(d, H, variant, kind, cfg, masks, Ho=None, L=None, llr_path=None):
    os.makedirs(d)
    W, _, _, cap, thr, mode = cfg
    n, m = H.shape
    nl = 0 if L is None else int(L.shape[1])
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write(f"{0 if L is None else 1} {variant} {kind} {n} {m} 0 {W} {mode} {thr} {cap} "
                f"{_num_phases(W) if variant == 1 else 0} {len(masks)} 0 0 {nl} 0\n")
        for row in masks:
            f.write(" ".join(str(int(v)) for v in row[:4]) + "\n")
    np.ascontiguousarray(H, dtype=np.int32).tofile(os.path.join(d, "H.bin"))
    if L is None:
        np.ascontiguousarray(Ho, dtype=np.int32).tofile(os.path.join(d, "Hother.bin"))
    else:
        np.ascontiguousarray(L, dtype=np.int32).tofile(os.path.join(d, "L.bin"))
    if llr_path:
        shutil.copy(llr_path, os.path.join(d, "llr.txt"))


@pytest.mark.parametrize("layout", ["slot_order", "code_order"])
def test_mixed_codes_in_one_batch(emulator, port, tmp_path, layout):
    """Three codes in one shuffled batch (per-shot code and record offsets, as the
    engine launches them): each shot's result equals the oracle's for its code.
    slot_order: the records lie back to back in launch-slot order (as the engine
    packs them); code_order: they stay in per-code order while the slots are
    shuffled, so the records of a chunk's lanes form many separate runs (as the
    server reads requests' buffers in place)."""
    c72, c108 = synth.BB_CODES[72](), synth.BB_CODES[108]()
    dem = synth.random_dem(4, detectors=40, mechanisms=160, logicals=5, p_range=(4e-3, 3e-2))
    e72 = synth.css_shots(c72.hz, 70, 0.03, seed=31)[0]
    e108 = synth.css_shots(c108.hz, 70, 0.02, seed=32)[0]
    s108 = (e108.astype(np.int64) @ c108.hz.T.astype(np.int64) % 2).astype(np.int32)
    det, log, _ = synth.dem_shots(dem, 70, seed=33)
    masks = [(8, 0, 1, 2, 0.6, 0.3, 0.1), (300, 0, 1, 2, 0.6, 0.3, 0.1)]
    phase = synth.write_phase_file(str(tmp_path / "phase.txt"), masks)
    llr = synth.write_llr_file(str(tmp_path / "llr.txt"), dem.llr)
    cfg72, cfg108, cfgd = (3, 256, 0, 64, 10, -1), (4, 256, 0, 30, 8, 1), (3, 256, 0, 24, 10, -1)
    d = tmp_path / "mix"
    _write_code(str(d / "code0"), c72.hz, 0, 1, cfg72, [], Ho=c72.hx)
    _write_code(str(d / "code1"), c108.hz, 1, 0, cfg108, masks, Ho=c108.hx)
    _write_code(str(d / "code2"), dem.h, 2, 2, cfgd, [], L=dem.l, llr_path=llr)
    records = [list(r) for r in e72] + [list(r) for r in s108] + \
              [list(a) + list(b) for a, b in zip(det, log)]  # DEM: detectors, then logicals
    codes = [0] * 70 + [1] * 70 + [2] * 70
    order = np.random.default_rng(34).permutation(len(records))
    flat, off = [], []
    if layout == "slot_order":
        for i in order:
            off.append(len(flat))
            flat.extend(records[i])
    else:
        start = []
        for r in records:
            start.append(len(flat))
            flat.extend(r)
        off = [start[i] for i in order]
    N = len(order)
    with open(d / "mixed.txt", "w") as f:
        f.write(f"3 {N} 3 4\n")
    np.asarray(flat, dtype=np.int32).tofile(d / "rec.bin")
    np.asarray(off, dtype=np.int64).tofile(d / "off.bin")
    np.asarray([codes[i] for i in order], dtype=np.int32).tofile(d / "code.bin")
    out = subprocess.run([emulator, str(d)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr + out.stdout
    # "ok N shots, J jobs, S slow": shots settled by the chunk step in either layout
    assert int(out.stdout.split()[5]) < N, out.stdout
    res = np.fromfile(d / "res.bin", dtype=capi.RESULT_DTYPE)
    assert int(out.stdout.split()[3]) > 0, out.stdout  # the launch had Jobs
    got = np.empty(N, dtype=capi.RESULT_DTYPE)
    got[order] = res  # back to the per-code order
    _, p72, _ = port.css(O.UNIFORM, c72.hx, c72.hz, e72, None, O.Config(*cfg72), "x")
    _, p108, _ = port.css(O.PROB, c108.hx, c108.hz, None, s108, O.Config(*cfg108), "x", phase)
    _, pd, _, _, _ = port.dem(O.ML, dem.h, dem.l, det, log, O.Config(*cfgd), llr)
    for part, want in ((got[:70], p72), (got[70:140], p108), (got[140:], pd)):
        bad = O.fields_equal(part, want)
        assert len(bad) == 0, f"shots {bad[:5]}\nemulated {part[bad[:3]]}\noracle {want[bad[:3]]}"


def test_largest_code_shapes(emulator, port, tmp_path):
    """The kernels' size limits: 1024 check rows (every lane of the warp holds a
    syndrome word) and 4000 columns (125 mask words per threshold iteration);
    syndromes of one or two columns, empty ones and random dense ones, with
    mode 1 and a cap that skip the dense shots' large active sets; three- and
    four-column syndromes (beyond W = 2) become Jobs for the lookup search."""
    rng = np.random.default_rng(77)
    n, m = 1024, 4000
    hz = np.zeros((n, m), dtype=np.int32)
    for c in range(m):
        hz[rng.choice(n, 3, replace=False), c] = 1
    hx = np.zeros((n, m), dtype=np.int32)  # unused by syndrome records
    syn = np.zeros((100, n), dtype=np.int32)
    for i in range(80):  # 1-2 columns (found), then 3-4 (beyond W: searched to the end)
        for c in rng.choice(m, 1 + i % 2 if i < 60 else 3 + i % 2, replace=False):
            syn[i] ^= hz[:, c]
    syn[90:] = rng.integers(0, 2, size=(10, n))
    cfg = (2, 256, 0, 40, 10, 1)
    d = tmp_path / "run"
    d.mkdir()
    res, dec, log = _run(emulator, str(d), hz, hx, syn, False, 0, cfg, [], 3)
    prc, pres, pdec = port.css(O.UNIFORM, hx, hz, None, syn, O.Config(*cfg), "x")
    assert prc == 0
    _compare(res, dec, pres, pdec)
    assert int((pres["found"] == 1).sum()) >= 55
    assert int(log.split()[3]) > 0, log  # the launch had Jobs


def _slow(log):
    """Shots the emulated launch sent through the per-shot path."""
    return int(log.split()[5])


@pytest.mark.parametrize("name,variant,cfg,masks", [
    ("mode -1", 0, (3, 256, 0, 64, 10, -1), []),
    ("mode 0", 0, (3, 256, 0, 64, 10, 0), []),
    ("mode 1, one position above thr", 0, (3, 256, 0, 64, 0, 1), []),
    ("mode 1, cap 0", 0, (3, 256, 0, 0, 0, 1), []),
    ("mode 5", 0, (3, 256, 0, 64, 10, 5), []),
    ("prob, small sets skip weight 1", 1, (3, 256, 0, 64, 10, -1),
     [(1, 1, 2, 2, 0.5, 0.5, 0.0), (300, 0, 1, 2, 1.0, 0.0, 0.0)]),
    ("prob, phase 0 listed second", 1, (3, 256, 0, 64, 10, 0),
     [(2, 1, 0, 2, 0.5, 0.5, 0.0), (300, 0, 1, 2, 1.0, 0.0, 0.0)]),
])
@pytest.mark.parametrize("fast", [True, False])
def test_classification_rules(emulator, port, tmp_path, name, variant, cfg, masks, fast):
    """Shots settled 32 at a time (empty syndromes, weight-1 matches of a
    one-position first iteration) get the per-shot path's results under every
    rule that decides whether that iteration is searched: the mode / threshold /
    cap branches and phase masks whose order for one position lists no weight 1
    or lists it after another phase.  Errors are supplied, so a match that
    differs from the supplied error (a stabilizer away) takes the per-shot path
    for its degeneracy test; fast=False sends every shot there."""
    code = synth.BB_CODES[72]()
    errors = np.concatenate([synth.css_shots(code.hz, 70, p, seed=1000 + i)[0]
                             for i, p in enumerate((0.005, 0.02))])
    errors[3] = code.hx[0]          # a stabilizer: empty syndrome, nonzero error
    errors[4] = 0
    errors[4, 5] = 1
    errors[4] ^= code.hx[1]         # single-column syndrome, error one stabilizer away
    phase = synth.write_phase_file(str(tmp_path / "phase.txt"), masks) if masks else None
    d = tmp_path / "run"
    d.mkdir()
    res, dec, log = _run(emulator, str(d), code.hz, code.hx, errors, True, variant, cfg, masks, 12,
                         fast=fast)
    prc, pres, pdec = port.css(O.PROB if variant else O.UNIFORM, code.hx, code.hz, errors, None,
                               O.Config(*cfg), "x", phase)
    assert prc == 0
    _compare(res, dec, pres, pdec)
    if not fast:
        assert _slow(log) == len(errors), log
    else:
        assert _slow(log) < len(errors), log  # empty syndromes at least were settled


@pytest.mark.parametrize("fast", [True, False])
def test_dem_classification(emulator, port, tmp_path, fast):
    """DEM records with the true logicals in their own array (the C ABI's layout):
    one-position matches compare the mechanism's logical flips with the truth;
    cap 0 skips every first iteration (upstream's cap keeps the last accepted
    set, here none)."""
    dem = synth.random_dem(12, detectors=40, mechanisms=160, logicals=5, p_range=(2e-3, 1e-2))
    det, log, _ = synth.dem_shots(dem, 150, seed=44)
    for cap in (24, 0):
        cfg = (3, 256, 0, cap, 10, -1)
        d = tmp_path / f"run{cap}"
        d.mkdir()
        res, dec, out, dlog, _ = _run(emulator, str(d), dem.h, None, det, False, 0, cfg, [], 12,
                                      L=dem.l, logicals=log, fast=fast)
        prc, pres, pdec, pdlog, _ = port.dem(O.UNIFORM, dem.h, dem.l, det, log, O.Config(*cfg))
        assert prc == 0
        _compare(res, dec, pres, pdec)
        assert np.array_equal(dlog, pdlog)


def test_capped_dem_stress(emulator, port, tmp_path):
    """Shots of the capped DEM stress (random detectors of the 120 x 720 DEM, W = 3,
    cap 64): first active sets of up to 64 columns searched as Jobs, later
    iterations above the cap repeating that set, nothing matched."""
    from library_s_grand_gb300 import workloads
    wl = workloads.stress_dem(6, seed=11)  # one shot's sets all exceed the cap: nothing searched
    cfg = wl.config
    res, dec, out, dlog, _ = _run(emulator, str(tmp_path), wl.dem.h, None, wl.detectors, False, 0,
                                  cfg, [], 10, L=wl.dem.l, logicals=wl.logicals)
    prc, pres, pdec, pdlog, _ = port.dem(O.UNIFORM, wl.dem.h, wl.dem.l, wl.detectors, wl.logicals,
                                         O.Config(*cfg))
    assert prc == 0
    tot = pres["total_tested_combinations"]
    assert int(pres["found"].sum()) == 0 and int(tot.max()) > 60000 and int(tot.min()) == 0
    _compare(res, dec, pres, pdec)
    assert np.array_equal(dlog, pdlog)
    assert int(out.split()[3]) > 0, out  # the launch had Jobs


@pytest.mark.parametrize("variant", ["uniform", "ml"])
def test_dem_empty_and_duplicate_columns(emulator, port, tmp_path, variant):
    """An irregular DEM with empty mechanisms (never active), duplicated columns
    (equal sketches: the bucket walk and the exact test must keep the lower
    rank) and columns of weight 1 beside weight 4 (the offset lifts them)."""
    dem = synth.random_dem(13, detectors=36, mechanisms=150, logicals=4, col_weights=(1, 4),
                           p_range=(5e-3, 3e-2))
    h = dem.h.copy()
    h[:, 7] = 0
    h[:, 90] = 0
    h[:, 31] = h[:, 30]
    h[:, 120] = h[:, 5]
    dem = synth.Dem(h, dem.l, dem.p, dem.llr)
    det, log, _ = synth.dem_shots(dem, 120, seed=61)
    cfg = (3, 256, 0, 40, 10, -1)
    path, v, pv = None, 0, O.UNIFORM
    if variant == "ml":
        path, v, pv = synth.write_llr_file(str(tmp_path / "llr.txt"), dem.llr), 2, O.ML
    d = tmp_path / "run"
    d.mkdir()
    res, dec, out, dlog, cost = _run(emulator, str(d), dem.h, None, det, False, v, cfg, [], 3,
                                     L=dem.l, logicals=log, llr_path=path)
    prc, pres, pdec, pdlog, pcost = port.dem(pv, dem.h, dem.l, det, log, O.Config(*cfg), path)
    assert prc == 0
    _compare(res, dec, pres, pdec)
    assert np.array_equal(dlog, pdlog)
    if variant == "ml":
        assert np.array_equal(cost.view(np.uint32), np.asarray(pcost, np.float32).view(np.uint32))
    assert int(out.split()[3]) > 0, out
