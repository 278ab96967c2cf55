#!/usr/bin/env python
"""GRAND decoder benchmark on GB300.

Workload (one step = one batch): grand_decode_prob_cc on the bivariate-bicycle
code [[144,12,12]] (Hz 72 x 144), X errors with per-qubit probabilities
log-uniform in [1e-3, 1e-2], 16384 shots, max_error_weight 4, active-position
cap 64, phase mask "300 0 1 2" (upstream: phase 0 = weights 1..5).  Seeded
synthetic data (numpy PCG64); no dataset exists for this workload.

Reported (one JSON line, rank 0):
  value      shots/s of the persistent batched decoder, records resident in HBM,
             graph-replayed decode launches (one persistent kernel per batch), L2
             flushed between steps;
  e2e        shots/s through the upstream-compatible C ABI (grand_decode_prob_cc)
             from host buffers, the records' trip to the GPU and the results' trip
             back included (read and written in place over NVLink-C2C where the
             GPU can access pageable memory, else copied);
  roofline   the decode kernel on the stress input the integer roofline is
             defined on (random syndromes, W = 4, exhaustive enumeration):
             candidates at 1.5 integer ops each against the measured lop3 issue
             rate, and beside it the prefix probes the lookup search executes
             against the shared-memory bound of two words per probe;
  roofline_dem  the same conventions on the capped DEM stress (random detectors
             of the 120 x 720 DEM, W = 3, cap 64), at the default and at a tuned
             light budget;
  cpu_baseline  the upstream CPU search algorithm (its C restatement in oracle/,
             or the upstream library itself where it was built) on all host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "shots/s & candidates/s, BB n=144 w≤4, plain vs persistent; p50/p99 latency"
SHOTS = 16384
W_MAX = 4
CAP = 64
PHASE = [(300, 0, 1, 2, 1.0, 0.0, 0.0)]
FLUSH_BYTES = 256 << 20


def workload(seed: int):
    """The headline batch for one rank (seed 0 on rank 0; other ranks draw other shots)."""
    from library_s_grand_gb300 import workloads
    w = workloads.prob_bb144(seed)
    return w.code, w.errors


def workload_config():
    return {"workload": "grand_decode_prob_cc BB[[144,12,12]] Hz 72x144, X errors p_i log-uniform "
                        "[1e-3,1e-2], 16384 shots, W=4, cap 64, phase mask '300 0 1 2'",
            "shots_per_step": SHOTS, "max_error_weight": W_MAX, "active_cap": CAP,
            "mode_of_search": -1, "records": "int32 errors (144 per shot)",
            "l2": "flushed between timed steps (256 MiB write)"}


# ---------------------------------------------------------------------------
# CPU side: the upstream CPU search algorithm on host cores
# ---------------------------------------------------------------------------
_W = {}
CPU_CHUNK = 128  # shots per task: small, so that the few hard shots do not pin one core


def _worker_init(kind):
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)  # upstream prints one line per shot
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from library_s_grand_gb300 import workloads
    w = workloads.prob_bb144()
    _W["lib"] = O.Reference() if kind == "reference" else O.Port()
    _W["O"] = O
    _W["w"] = w
    _W["phase"] = w.phase_file(tempfile.mkdtemp())


def _worker_chunk(span):
    """Decode shots [lo, hi) of the headline batch; (shots, candidates tested)."""
    lo, hi = span
    O, w = _W["O"], _W["w"]
    r = _W["lib"].css(O.PROB, w.code.hx, w.code.hz, w.errors[lo:hi], None, O.Config(*w.config),
                      "x", _W["phase"])
    assert r[0] == 0
    return hi - lo, int(r[1]["total_tested_combinations"].sum())


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


class CpuPool:
    """Worker processes fed from one shared task queue of 128-shot chunks.

    Passes over the batch are queued together, so while one core works through
    a pass's few hard shots (one shot of the headline batch tests 8.3e6
    candidates, 60 % of the pass's work) the others take chunks of the next
    passes: the figure is a throughput with every core kept busy."""

    def __init__(self, cores=None):
        import multiprocessing as mp
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        self.kind = "reference" if O.Reference.available() else "port"
        self.cores = cores or os.cpu_count() or 1
        self.pool = mp.get_context("spawn").Pool(self.cores, initializer=_worker_init,
                                                 initargs=(self.kind,))
        self.pool.map(_worker_chunk, [(0, 1)] * self.cores, chunksize=1)  # imports, library load

    def passes(self, k):
        """Decode the batch k times; (wall seconds, shots, candidates)."""
        spans = [(lo, min(lo + CPU_CHUNK, SHOTS)) for _ in range(k)
                 for lo in range(0, SHOTS, CPU_CHUNK)]
        t0 = time.perf_counter()
        shots = cands = 0
        for s, c in self.pool.imap_unordered(_worker_chunk, spans, chunksize=1):
            shots += s
            cands += c
        return time.perf_counter() - t0, shots, cands

    def close(self):
        self.pool.terminate()
        self.pool.join()


def cpu_baseline(seconds=12.0):
    """The upstream CPU algorithm on this host: one core (whole passes) and all cores."""
    one = CpuPool(cores=1)
    try:
        t1, s1, c1 = one.passes(1)
        passes1 = 1
        while t1 < 0.25 * seconds and passes1 < 50:
            dt, s, c = one.passes(1)
            t1, s1, c1, passes1 = t1 + dt, s1 + s, c1 + c, passes1 + 1
    finally:
        one.close()
    pool = CpuPool()
    try:
        pool.passes(1)  # warm-up
        k = max(2, int(round(0.75 * seconds / max(t1 / passes1, 1e-3) * pool.cores)))
        k = min(k, 400)
        t_all, shots, cands = pool.passes(k)
    finally:
        pool.close()
    return {"value": shots / t_all, "unit": "shots/s", "cores": pool.cores, "kind": pool.kind,
            "candidates_per_s": cands / t_all,
            "value_1core": s1 / t1, "candidates_per_s_1core": c1 / t1,
            "all_cores_vs_1core": (shots / t_all) / (s1 / t1), "cpu_model": cpu_model(),
            "sample": f"all cores: {k} passes over the 16384-shot batch as {CPU_CHUNK}-shot tasks "
                      f"on {pool.cores} processes ({t_all:.1f} s wall); 1 core: {passes1} "
                      f"pass(es) ({t1:.1f} s); upstream CPU search algorithm, mode -1"}


# ---------------------------------------------------------------------------
# Clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.path = tempfile.mktemp(suffix=".csv")
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def stress_ops(code_h, syndromes, W):
    """Exhaustive search work of random-syndrome shots, iteration sets as upstream:
    (candidates, ops, prefixes) with ops = (w+1)*ceil(R/32) per weight-w
    candidate and prefixes = the C(tam-1, w-1) (w-1)-prefixes a weight-w block
    is split into (one probe each in the lookup search)."""
    R = code_h.shape[0]
    words = math.ceil(R / 32)
    colw = code_h.sum(axis=0)
    max_soma = int(colw.max())
    sums = syndromes.astype(np.int64) @ code_h.astype(np.int64)
    cands = ops = prefixes = 0
    for s in sums:
        for it in range(min(max_soma, 3)):
            tam = int((s >= max_soma - it).sum())
            for w in range(1, min(W, 6) + 1):
                c = math.comb(tam, w)
                cands += c
                ops += c * (w + 1) * words
                prefixes += math.comb(tam - 1, w - 1) if tam >= w else 0
    return cands, ops, prefixes


def dem_stress_ops(h, detectors, W, cap):
    """Exhaustive search work of unmatched DEM shots under the uniform search (mode -1),
    iteration sets as upstream's DEM family (grand_decoder.cu:1542-1607): flagged-check
    counts with the irregular offset (:376-416), and an iteration whose active set exceeds
    the cap searches the last set within it instead (:1550-1554).  Returns (candidates,
    ops, prefixes) as stress_ops."""
    R = h.shape[0]
    words = math.ceil(R / 32)
    colw = h.sum(axis=0)
    max_soma = int(colw.max())
    sums = detectors.astype(np.int64) @ h.astype(np.int64) + np.where(colw > 0, max_soma - colw, 0)
    sums[:, colw == 0] = 0
    cands = ops = prefixes = 0
    for s in sums:
        tam_old = 0
        for it in range(min(max_soma, 3)):
            tam = int((s >= max_soma - it).sum())
            if tam > cap:
                tam = tam_old
            else:
                tam_old = tam
            for w in range(1, min(W, 6) + 1):
                if tam >= w:
                    c = math.comb(tam, w)
                    cands += c
                    ops += c * (w + 1) * words
                    prefixes += math.comb(tam - 1, w - 1)
    return cands, ops, prefixes


def run_ours(args):
    import torch
    from library_s_grand_gb300 import launch
    rank, world, local = launch.env_ranks()
    if world > 1 and world != args.gpus:
        raise SystemExit(f"bench.py: WORLD_SIZE={world} but --gpus {args.gpus}")
    torch.cuda.set_device(local)
    dist = launch.init_from_env("nccl", torch.device("cuda", local))
    from library_s_grand_gb300 import build as B
    from library_s_grand_gb300 import capi, synth
    from library_s_grand_gb300.engine import Engine

    B.build()
    lib = capi.load_library()
    eng = Engine(lib)
    tmp = tempfile.mkdtemp()
    phase = synth.write_phase_file(os.path.join(tmp, "phase.txt"), PHASE)
    code, errors = workload(rank)
    cfg = capi.GrandDecoderConfig(W_MAX, 256, 0, CAP, 10, -1)
    eng.add_css(code.hx, code.hz, "x", True, cfg, phase)

    dev = torch.device("cuda", local)
    d_rec = torch.from_numpy(np.ascontiguousarray(errors.ravel())).to(dev)
    d_res = torch.empty(SHOTS * 72, dtype=torch.uint8, device=dev)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def step():
        rc = eng.decode_device(SHOTS, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=True)
        if rc != 0:
            raise RuntimeError(f"device decode failed ({rc})")

    for _ in range(args.warmup):
        flush.fill_(1)
        step()
    if eng.sync_status(sp) != 0:
        raise RuntimeError("device decode status error")
    # one checked pass: device results equal the C ABI's
    res_dev = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    rc, res_c, _ = capi.decode_css_ex(lib, "prob", code.hx, code.hz, errors, None, cfg, "x", phase)
    assert rc == 0
    for f in ("found", "found_weight", "tam", "total_tested_combinations", "iteration", "degenerate"):
        assert np.array_equal(res_dev[f], res_c[f]), f
    cands_step = int(res_c["total_tested_combinations"].sum())

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    for i in range(args.steps):
        flush.fill_(i & 255)
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    time.sleep(0.2)
    clk = clocks.stop()
    if dist:
        dist.barrier()
    if eng.sync_status(sp) != 0:
        raise RuntimeError("device decode status error")
    per = np.array([a.elapsed_time(b) for a, b in ev])
    total_ms = launch.max_over_ranks(dist, float(per.sum()), dev)
    value = world * SHOTS * args.steps / (total_ms * 1e-3)
    if world > 1:
        sys.stderr.write(f"rank {rank}: n_gpus {world}, {SHOTS * args.steps} shots in "
                         f"{per.sum():.3f} ms (max over ranks {total_ms:.3f} ms)\n")

    # kernel split (non-graph launches with events; median of 5)
    split = []
    for _ in range(5):
        flush.fill_(7)
        eng.decode_device(SHOTS, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=False)
        eng.sync_status(sp)
        split.append(eng.kernel_times(sp))
    reset_ms, dec_ms = (float(np.median([x[i] for x in split])) for i in range(2))
    hbm = hbm_streaming(code, dec_ms)

    out = None
    if rank == 0:
        # e2e through the upstream-compatible C ABI, host buffers in and out
        e_flat = np.ascontiguousarray(errors, dtype=np.int32)
        hx = np.ascontiguousarray(code.hx, dtype=np.int32)
        hz = np.ascontiguousarray(code.hz, dtype=np.int32)
        k_e2e = max(3, min(args.steps, 200))
        for _ in range(3):
            rc, _ = capi.run_grand_prob_shots_cc(lib, hx, hz, e_flat, None, cfg, phase, b"x")
        torch.cuda.synchronize()
        lat = []
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            a = time.perf_counter()
            rc, _ = capi.run_grand_prob_shots_cc(lib, hx, hz, e_flat, None, cfg, phase, b"x")
            lat.append(time.perf_counter() - a)
            assert rc == 0
        e2e_s = time.perf_counter() - t0
        e2e = {"value": SHOTS * k_e2e / e2e_s, "unit": "shots/s",
               "h2d_bytes_per_step": SHOTS * code.m * 4, "d2h_bytes_per_step": SHOTS * 72,
               "steps": k_e2e, "p50_ms": float(np.percentile(lat, 50) * 1e3),
               "p99_ms": float(np.percentile(lat, 99) * 1e3)}

        # the same batch as bit-packed error records (grand_decode_cc_packed):
        # 5 words per shot instead of 144 int32 entries
        words = capi.pack_bits(errors)
        for _ in range(3):
            rc, _ = capi.run_grand_shots_cc_packed(lib, hx, hz, words, capi.PACKED_ERRORS, cfg, "x",
                                                   phase)
        lat_p = []
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            a = time.perf_counter()
            rc, _ = capi.run_grand_shots_cc_packed(lib, hx, hz, words, capi.PACKED_ERRORS, cfg, "x",
                                                   phase)
            lat_p.append(time.perf_counter() - a)
            assert rc == 0
        e2e_p = time.perf_counter() - t0
        e2e_packed = {"value": SHOTS * k_e2e / e2e_p, "unit": "shots/s",
                      "h2d_bytes_per_step": int(words.nbytes), "d2h_bytes_per_step": SHOTS * 72,
                      "steps": k_e2e, "p50_ms": float(np.percentile(lat_p, 50) * 1e3),
                      "what": "grand_decode_cc_packed with the phase file: bit-packed error "
                              "records (LSB-first uint32 words), host buffers"}

        # plain one-launch-per-call path (per shot), on a 1024-shot slice
        n_plain = 1024
        rc, _ = eng.decode_plain(errors[:64].ravel(), num_shots=64)
        t0 = time.perf_counter()
        rc, res_plain = eng.decode_plain(errors[:n_plain].ravel(), num_shots=n_plain)
        plain_s = time.perf_counter() - t0
        assert rc == 0
        assert np.array_equal(res_plain["total_tested_combinations"],
                              res_c["total_tested_combinations"][:n_plain])

        roof = stress_roofline(torch, lib, dev, sp)
        extra = {}
        if not args.headline_only:
            extra["batching"] = bench_batching(torch, lib, dev, sp, flush)
            extra["ml_dem"] = bench_ml(torch, lib, dev, sp, flush)
            extra["sampling"] = bench_sampling(torch, lib, dev, sp)
            extra["serving"] = bench_serving(lib)
            extra["roofline_dem"] = dem_stress_roofline(torch, lib, dev, sp)
        cpu = cpu_baseline(seconds=args.cpu_seconds) if args.cpu_seconds > 0 else None

        out = {
            "metric": METRIC, "value": value, "unit": "shots/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded numpy PCG64)", "config": workload_config(),
            "candidates_per_s": world * cands_step * args.steps / (total_ms * 1e-3),
            "candidates_per_step": cands_step,
            "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99)),
                           "what": "per 16384-shot batch, device-resident, graph replay"},
            "plain_shots_per_s": n_plain / plain_s,
            "plain_what": "one call per shot: H2D record, decode launch, sync, D2H",
            "persistent_vs_plain": value / world / (n_plain / plain_s),
            "kernel_ms": {"decode": dec_ms, "control_reset": reset_ms},
            "e2e": e2e, "e2e_packed": e2e_packed, "roofline": roof, "hbm_streaming": hbm,
            "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": args.steps,
        }
        out.update(extra)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return out


# DRAM bytes (read + write) of one decode_kernel launch on the headline batch, from an ncu
# --set full capture (profiles/decode_kernel_prob_cc_bb144_16384.md).
HEADLINE_TRAFFIC = 9.694976e6 + 768.0


def hbm_peak():
    """Measured copy bandwidth of the GB300s (MEASURED_PEAKS.json), else the fallback."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path, encoding="utf-8") as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def hbm_streaming(code, dec_ms):
    """Record streaming of the decode kernel on the headline batch: int32 error records in
    (4m bytes per shot) and 72-byte results out, per launch, over the kernel's event time."""
    peak, src = hbm_peak()
    per_shot = 4 * code.m + 72
    gbs = SHOTS * per_shot / (dec_ms * 1e-3) / 1e9
    return {"kernel": "decode_kernel", "achieved": gbs, "peak": peak, "unit": "GB/s",
            "frac": gbs / peak, "peak_source": src + " copy bandwidth (MEASURED_PEAKS.json)",
            "algorithmic_bytes_per_launch": SHOTS * per_shot, "traffic": HEADLINE_TRAFFIC,
            "traffic_unit": "bytes per launch (ncu)", "decode_ms": dec_ms,
            "what": "bytes per launch: int32 error records (4m per shot) + 72-byte results"}


STRESS_SHOTS = 192
SKETCH_OPS_PER_CANDIDATE = 1.5
# DRAM bytes (read + write) of one decode_kernel launch on the 192 stress shots, from an
# ncu --set full capture (profiles/decode_kernel_stress_bb144_w4.md), per shot.
STRESS_TRAFFIC_PER_SHOT = (317184.0 + 6656.0) / 192
# The lookup search's bound per prefix probe: two shared-memory words (the last
# element's sketch and one filter word) at 32 words per SM per clock.
PROBE_WORDS = 2
SMEM_WORDS_PER_SM_CLOCK = 32
SM_CLOCK_HZ = 2.07e9  # the GB300's maximum SM clock (the runs' median clock, bench `clocks`)


def stress_case(torch, lib, dev, n=STRESS_SHOTS):
    """Engine + device buffers for exhaustive random-syndrome shots of [[144,12,12]], W=4."""
    from library_s_grand_gb300 import capi, synth
    from library_s_grand_gb300.engine import Engine
    code = synth.BB_CODES[144]()
    syn = (np.random.default_rng(1).random((n, code.n)) < 0.5).astype(np.int32)
    eng = Engine(lib)
    eng.add_css(code.hx, code.hz, "x", False, capi.GrandDecoderConfig(4, 256, 0, 300, 10, -1))
    d_rec = torch.from_numpy(syn.ravel()).to(dev)
    d_res = torch.empty(n * 72, dtype=torch.uint8, device=dev)
    return code, syn, eng, d_rec, d_res


def stress_roofline(torch, lib, dev, sp):
    """Decode kernel on exhaustive random-syndrome shots of [[144,12,12]], W=4.

    Candidate convention (comparable across versions of the search): a candidate
    tested by a sketch scan costs one XOR (its last column's sketch against the
    prefix sketch) and half a 3-way minimum, 1.5 integer ops whatever R, against
    the lop3 issue rate measured on this GPU; the word-compare count ceil(R/32)+1
    and the fixed count (w+1)*ceil(R/32) are reported beside it.  The lookup
    search tests a prefix's candidates with one probe, so it also gets a probe
    convention: prefix probes per second against the shared-memory bound of two
    words per probe (the fraction of the machine the search itself uses)."""
    from library_s_grand_gb300 import capi
    n = STRESS_SHOTS
    code, syn, eng, d_rec, d_res = stress_case(torch, lib, dev, n)
    cands, ops_fixed, prefixes = stress_ops(code.hz, syn, 4)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    probe_peak = sms * SMEM_WORDS_PER_SM_CLOCK / PROBE_WORDS * SM_CLOCK_HZ
    words = math.ceil(code.n / 32)
    times = []
    for rep in range(4):
        eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=False)
        if eng.sync_status(sp) != 0:
            raise RuntimeError("stress decode failed")
        times.append(eng.kernel_times(sp)[1])
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    assert int(res["found"].sum()) == 0
    assert int(res["total_tested_combinations"].sum()) == cands, "count mismatch"
    search_ms = float(np.median(times[1:]))
    peak = eng.int_peak()
    rate = cands / (search_ms * 1e-3)
    achieved = rate * SKETCH_OPS_PER_CANDIDATE
    return {"bound": "int_alu", "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "Gop/s",
            "frac": achieved / peak, "traffic": STRESS_TRAFFIC_PER_SHOT * n,
            "traffic_unit": "bytes per launch (ncu capture of the same 192 shots)",
            "kernel": "decode_kernel",
            "workload": f"{n} random-syndrome shots of BB[[144,12,12]], W=4, exhaustive "
                        f"({cands} candidates, 3 threshold iterations)",
            "ops_per_candidate": "1.5 (sketch XOR + half a 3-way min)",
            "search_ms": search_ms, "candidates_per_s": rate,
            "frac_word_convention": rate * (words + 1) / peak,
            "word_convention": f"ceil(R/32)+1 = {words + 1} ops per candidate (XOR-OR words + min)",
            "frac_fixed_convention": ops_fixed / (search_ms * 1e-3) / peak,
            "fixed_convention": "(w+1)*ceil(R/32) ops per candidate",
            "peak_source": "lop3.b32 issue rate measured on this GPU (grand_measure_int_peak)",
            "prefix_probes": prefixes, "probes_per_s": prefixes / (search_ms * 1e-3),
            "probe_peak_per_s": probe_peak,
            "frac_probe_convention": prefixes / (search_ms * 1e-3) / probe_peak,
            "probe_convention": "one prefix probe = 2 shared-memory words (sketch, filter word); "
                                "peak = SMs x 32 words/clock / 2 x 2.07 GHz"}


STRESS_DEM_SHOTS = 8192


def dem_stress_case(torch, lib, dev, n=STRESS_DEM_SHOTS):
    """Engine + device buffers for the capped DEM stress (random detectors of the 120 x 720
    DEM, grand_decode_cln, W = 3, cap 64)."""
    from library_s_grand_gb300 import capi, workloads
    from library_s_grand_gb300.engine import UNIFORM, Engine
    wl = workloads.stress_dem(n)
    eng = Engine(lib)
    eng.add_dem(wl.dem.h, wl.dem.l, capi.GrandDecoderConfig(*wl.config), UNIFORM)
    d_rec = torch.from_numpy(wl.records.ravel()).to(dev)
    d_res = torch.empty(n * 72, dtype=torch.uint8, device=dev)
    return wl, eng, d_rec, d_res


def dem_stress_roofline(torch, lib, dev, sp):
    """Decode kernel on the capped DEM stress, in the conventions of stress_roofline.  Each
    shot's search is small (at most 43,744 candidates per iteration), so the figure covers
    the whole per-shot pipeline (record, counts, planning, Job publication) as much as
    the scan."""
    from library_s_grand_gb300 import autotune, capi
    n = STRESS_DEM_SHOTS
    wl, eng, d_rec, d_res = dem_stress_case(torch, lib, dev, n)
    cands, ops_fixed, prefixes = dem_stress_ops(wl.dem.h, wl.detectors, wl.W, wl.cap)

    def timed():
        times = []
        for rep in range(4):
            eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=False)
            if eng.sync_status(sp) != 0:
                raise RuntimeError("DEM stress decode failed")
            times.append(eng.kernel_times(sp)[1])
        res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
        assert int(res["found"].sum()) == 0
        assert int(res["total_tested_combinations"].sum()) == cands, "count mismatch"
        return float(np.median(times[1:])), eng.launch_stats(sp)

    search_ms, stats = timed()
    # the same shots with the light budget tuned for them (larger budgets keep these
    # small searches in the warp that triages the shot instead of publishing Jobs)
    best, table = autotune.tune(eng, "dem-stress", n, d_rec.data_ptr(), d_res.data_ptr(), sp,
                                use_cache=False, grid=[(l, 4, 0) for l in (10, 12, 14, 16)])
    tuned_ms, tuned_stats = timed()
    eng.set_tuning()
    peak = eng.int_peak()
    rate = cands / (search_ms * 1e-3)
    words = math.ceil(wl.dem.n / 32)
    return {"bound": "int_alu", "achieved": rate * SKETCH_OPS_PER_CANDIDATE / 1e9,
            "peak": peak / 1e9, "unit": "Gop/s", "frac": rate * SKETCH_OPS_PER_CANDIDATE / peak,
            "kernel": "decode_kernel",
            "workload": f"{n} random-detector shots (Bernoulli 0.36) of the 120 x 720 DEM, "
                        f"grand_decode_cln, W=3, cap 64, exhaustive ({cands} candidates)",
            "ops_per_candidate": "1.5 (sketch XOR + half a 3-way min)",
            "search_ms": search_ms, "candidates_per_s": rate, "shots_per_s": n / (search_ms * 1e-3),
            "jobs": int(stats[2]), "lookup_tiles": int(stats[3]),
            "frac_word_convention": rate * (words + 1) / peak,
            "frac_fixed_convention": ops_fixed / (search_ms * 1e-3) / peak,
            "prefix_probes": prefixes, "probes_per_s": prefixes / (search_ms * 1e-3),
            "peak_source": "lop3.b32 issue rate measured on this GPU (grand_measure_int_peak)",
            "tuned": {"light_log2": best[0], "search_ms": tuned_ms,
                      "candidates_per_s": cands / (tuned_ms * 1e-3),
                      "frac": cands / (tuned_ms * 1e-3) * SKETCH_OPS_PER_CANDIDATE / peak,
                      "jobs": int(tuned_stats[2]), "table_ms": table}}


def _time_device(torch, eng, n, d_rec, d_res, sp, flush, steps, warmup, d_sc=0, d_off=0):
    """Graph-replayed device decode: per-step CUDA-event times with an L2 flush between."""
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        flush.fill_(1)
        if eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, d_sc, d_off, True) != 0:
            raise RuntimeError("device decode failed")
    if eng.sync_status(sp) != 0:
        raise RuntimeError("device decode status error")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for i in range(steps):
        flush.fill_(i & 255)
        ev[i][0].record(stream)
        eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, d_sc, d_off, True)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    if eng.sync_status(sp) != 0:
        raise RuntimeError("device decode status error")
    return np.array([a.elapsed_time(b) for a, b in ev])


def bench_batching(torch, lib, dev, sp, flush):
    """Mixed-code batch: 100k shots mixing BB[[72]], [[108]] (W=3), [[144]], [[288]] (W=4) at
    p = 0.003, shuffled, in one persistent launch (tuned, graph-replayed) vs the plain
    paths: one C ABI call per code, and one call (one launch pair) per shot."""
    from library_s_grand_gb300 import autotune, capi, synth
    from library_s_grand_gb300.engine import Engine, offsets_for
    spec = [(72, 3), (108, 3), (144, 4), (288, 4)]
    per = 25000
    eng = Engine(lib)
    codes, syns, cfgs = [], [], []
    for ci, (n, W) in enumerate(spec):
        c = synth.BB_CODES[n]()
        cfg = capi.GrandDecoderConfig(W, 256, 0, 64, 10, -1)
        eng.add_css(c.hx, c.hz, "x", False, cfg)
        _, s = synth.css_shots(c.hz, per, 0.003, seed=40 + ci)
        codes.append(c)
        syns.append(s)
        cfgs.append(cfg)
    N = per * len(spec)
    order = np.random.default_rng(0).permutation(N)
    sc = np.concatenate([np.full(per, ci, np.int32) for ci in range(len(spec))])[order]
    rows = [r for s in syns for r in s]
    rec = np.concatenate([rows[i] for i in order]).astype(np.int32)
    off = offsets_for(eng.rec_lens, sc)
    d_rec = torch.from_numpy(rec).to(dev)
    d_sc = torch.from_numpy(sc).to(dev)
    d_off = torch.from_numpy(off).to(dev)
    d_res = torch.empty(N * 72, dtype=torch.uint8, device=dev)
    best, table = autotune.tune(eng, "bb-mix-100k", N, d_rec.data_ptr(), d_res.data_ptr(), sp,
                                d_sc.data_ptr(), d_off.data_ptr(), use_cache=False,
                                grid=[(l, 4, c) for l in (8, 10, 12, 14) for c in (0, 2)])
    per_step = _time_device(torch, eng, N, d_rec, d_res, sp, flush, 50, 5, d_sc.data_ptr(),
                            d_off.data_ptr())
    dev_rate = N / (per_step.mean() * 1e-3)
    # persistent, host buffers in and out (the engine's public call)
    eng.decode(rec, sc)
    t0 = time.perf_counter()
    reps = 10
    for _ in range(reps):
        rc, res_e = eng.decode(rec, sc)
    e2e_rate = N * reps / (time.perf_counter() - t0)
    # plain: one upstream-API call per code (one warm pass, then 3 timed passes)
    for c, s, cfg in zip(codes, syns, cfgs):
        capi.run_grand_shots_cc(lib, c.hx, c.hz, None, s, cfg, b"x")
    t0 = time.perf_counter()
    for _ in range(3):
        raw = [capi.run_grand_shots_cc(lib, c.hx, c.hz, None, s, cfg, b"x")[1]
               for c, s, cfg in zip(codes, syns, cfgs)]
    per_code_rate = 3 * N / (time.perf_counter() - t0)
    ref = np.concatenate([capi.results_array(r) for r in raw])[order]
    for f in ("found", "found_weight", "tam", "total_tested_combinations", "iteration"):
        assert np.array_equal(res_e[f], ref[f]), f
    # plain: one call per shot, on a sample
    k = 2000
    t0 = time.perf_counter()
    rc, res_p = eng.decode_plain(rec[:int(off[k])], sc[:k])
    per_shot_rate = k / (time.perf_counter() - t0)
    assert np.array_equal(res_p["total_tested_combinations"], ref["total_tested_combinations"][:k])
    return {"workload": "100k shots: BB72/BB108 W=3, BB144/BB288 W=4, p=0.003, shuffled, "
                        "syndrome records", "shots": N,
            "persistent_shots_per_s": dev_rate, "persistent_ms_per_batch": float(per_step.mean()),
            "persistent_e2e_shots_per_s": e2e_rate,
            "plain_per_code_call_shots_per_s": per_code_rate,
            "plain_per_shot_call_shots_per_s": per_shot_rate,
            "persistent_vs_plain_per_code": dev_rate / per_code_rate,
            "persistent_vs_plain_per_shot": dev_rate / per_shot_rate,
            "autotune": {"best": {"light_log2": best[0], "tile_k": best[1],
                                  "search_ctas_per_sm": best[2]},
                         "table_ms": [[s, round(t, 4)] for s, t in table]},
            "candidates_per_batch": int(ref["total_tested_combinations"].sum())}


def bench_ml(torch, lib, dev, sp, flush):
    """ML DEM batch: grand_decode_ML_cln on the 120 x 720 random DEM, 65536 shots, W=3."""
    from library_s_grand_gb300 import capi, synth
    from library_s_grand_gb300.engine import Engine
    dem = synth.random_dem(0)
    tmp = tempfile.mkdtemp()
    lf = synth.write_llr_file(os.path.join(tmp, "llr.txt"), dem.llr)
    n = 65536
    det, log, _ = synth.dem_shots(dem, n, 1)
    cfg = capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1)
    eng = Engine(lib)
    eng.add_dem(dem.h, dem.l, cfg, 2, lf)
    rec = np.ascontiguousarray(np.concatenate([det, log], axis=1), dtype=np.int32)
    d_rec = torch.from_numpy(rec.ravel()).to(dev)
    d_res = torch.empty(n * 72, dtype=torch.uint8, device=dev)
    per_step = _time_device(torch, eng, n, d_rec, d_res, sp, flush, 50, 5)
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    capi.run_grand_ML_shots_cln(lib, dem.h, dem.l, det, log, dem.n_logicos, cfg, lf)
    t0 = time.perf_counter()
    reps = 10
    for _ in range(reps):
        rc, r = capi.run_grand_ML_shots_cln(lib, dem.h, dem.l, det, log, dem.n_logicos, cfg, lf)
        assert rc == 0
    e2e = n * reps / (time.perf_counter() - t0)
    return {"workload": "grand_decode_ML_cln, random DEM 120 x 720 (column weight 2-4, 12 "
                        "logicals), p log-uniform [1e-4, 5e-3], 65536 shots, W=3, cap 64",
            "device_shots_per_s": n / (per_step.mean() * 1e-3),
            "device_ms_per_batch": float(per_step.mean()), "e2e_shots_per_s": e2e,
            "found_fraction": float(res["found"].mean()),
            "logical_success_fraction": float(res["degenerate"].mean()),
            "candidates_per_batch": int(res["total_tested_combinations"].sum())}


def bench_sampling(torch, lib, dev, sp):
    """Statistical run on the device: draw the headline code's shots with the on-device
    sampler (Philox4x32-10, per-qubit p log-uniform in [1e-3, 1e-2]) and decode them in
    place, batch after batch, with no host traffic."""
    from library_s_grand_gb300 import capi, synth
    from library_s_grand_gb300.engine import Engine
    tmp = tempfile.mkdtemp()
    phase = synth.write_phase_file(os.path.join(tmp, "phase.txt"), PHASE)
    code = synth.BB_CODES[144]()
    rng = np.random.default_rng(0)
    p = np.exp(rng.uniform(np.log(1e-3), np.log(1e-2), code.m)).astype(np.float32)
    eng = Engine(lib)
    eng.add_css(code.hx, code.hz, "x", True, capi.GrandDecoderConfig(W_MAX, 256, 0, CAP, 10, -1), phase)
    n, batches = SHOTS, 40
    d_p = torch.from_numpy(p).to(dev)
    d_rec = torch.empty(n * code.m, dtype=torch.int32, device=dev)
    d_res = torch.empty(n * 72, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def batch(k):
        if eng.sample(0, d_p.data_ptr(), 2024, k * n, n, d_rec.data_ptr(), sp) != 0:
            raise RuntimeError("sample failed")
        if eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=True) != 0:
            raise RuntimeError("decode failed")

    for k in range(3):
        batch(k)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for k in range(batches):
        batch(3 + k)
    b.record(stream)
    torch.cuda.synchronize()
    if eng.sync_status(sp) != 0:
        raise RuntimeError("status error")
    ms = a.elapsed_time(b)
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), dtype=capi.RESULT_DTYPE)
    return {"workload": f"BB[[144,12,12]] prob_cc W={W_MAX}: on-device sampling (Philox4x32-10) "
                        f"+ decode, {batches} batches of {n} shots",
            "shots_per_s": n * batches / (ms * 1e-3), "ms_per_batch": ms / batches,
            "found_fraction": float(res["found"].mean()),
            "corrected_fraction": float(((res["degenerate"] == 1) | (res["original_weight"] == 0)).mean()),
            "host_bytes_per_batch": 0}


def bench_serving(lib):
    """Serving: Poisson arrivals of 1-256-shot requests over four BB codes (W=3,
    syndrome records) and the 120 x 720 DEM in ML mode, offered load swept to
    saturation through the continuous-batching server."""
    from library_s_grand_gb300 import capi, synth
    from library_s_grand_gb300.engine import Engine
    from library_s_grand_gb300.server import Server
    tmp = tempfile.mkdtemp()
    dem = synth.random_dem(0)
    lf = synth.write_llr_file(os.path.join(tmp, "llr.txt"), dem.llr)
    eng = Engine(lib)
    pools = []
    for i, nq in enumerate((72, 108, 144, 288)):
        c = synth.BB_CODES[nq]()
        eng.add_css(c.hx, c.hz, "x", False, capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1))
        _, s = synth.css_shots(c.hz, 4096, 0.003, seed=60 + i)
        pools.append(s)
    eng.add_dem(dem.h, dem.l, capi.GrandDecoderConfig(3, 256, 0, 64, 10, -1), 2, lf)
    det, log, _ = synth.dem_shots(dem, 4096, 65)
    pools.append(np.concatenate([det, log], axis=1).astype(np.int32))
    rng = np.random.default_rng(7)
    nreq = 6000
    sizes = rng.integers(1, 257, size=nreq).astype(np.int32)
    cids = rng.integers(0, len(pools), size=nreq)
    recs, scs = [], []
    for s, c in zip(sizes, cids):
        start = int(rng.integers(0, 4096 - s))
        recs.append(pools[c][start:start + s].ravel())
        scs.append(np.full(s, c, np.int32))
    rec = np.concatenate(recs).astype(np.int32)
    sc = np.concatenate(scs)
    # capacity estimate: everything as one batch
    eng.decode(rec, sc)
    t0 = time.perf_counter()
    rc, ref = eng.decode(rec, sc)
    cap_req = nreq / (time.perf_counter() - t0)
    srv = Server(eng, slots=4, max_shots_per_batch=4096)
    points = []
    shot0 = np.concatenate([[0], np.cumsum(sizes)])
    rec0 = np.concatenate([[0], np.cumsum([len(r) for r in recs])])
    for frac in (0.1, 0.25, 0.5, 0.75, 1.0, 1.5):
        rate = cap_req * frac
        k = int(min(nreq, max(400, rate * 0.6)))
        arrival = np.cumsum(rng.exponential(1.0 / rate, size=k))
        rc, res, lat, wall = srv.replay(arrival, sizes[:k], rec[:rec0[k]], sc[:shot0[k]])
        assert rc == 0
        assert np.array_equal(res["total_tested_combinations"],
                              ref["total_tested_combinations"][:shot0[k]])
        points.append({"offered_requests_per_s": rate, "offered_shots_per_s": rate * 128.5,
                       "requests": k, "achieved_shots_per_s": float(shot0[k] / wall),
                       "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                       "p999_ms": float(np.percentile(lat, 99.9))})
    slots, nbytes = srv.info()
    srv.close()
    return {"workload": "Poisson arrivals, requests of U{1..256} shots, code uniform over "
                        "BB72/BB108/BB144/BB288 (W=3, syndrome records) and the 120 x 720 DEM (ML)",
            "slots": slots, "slot_device_bytes": nbytes, "batch_capacity_requests_per_s": cap_req,
            "sweep": points}


def run_case(args):
    """Profiling entry point: run one case a few times, print kernel times only."""
    import torch
    from library_s_grand_gb300 import build as B
    from library_s_grand_gb300 import capi, synth
    from library_s_grand_gb300.engine import Engine
    B.build()
    lib = capi.load_library()
    dev = torch.device("cuda", 0)
    sp = torch.cuda.current_stream(dev).cuda_stream
    if args.case == "stress":
        code, syn, eng, d_rec, d_res = stress_case(torch, lib, dev, args.case_shots or 48)
        n = len(syn)
    elif args.case == "stress_dem":
        wl, eng, d_rec, d_res = dem_stress_case(torch, lib, dev, args.case_shots or STRESS_DEM_SHOTS)
        n = len(wl.detectors)
    else:
        tmp = tempfile.mkdtemp()
        phase = synth.write_phase_file(os.path.join(tmp, "phase.txt"), PHASE)
        code, errors = workload(0)
        eng = Engine(lib)
        eng.add_css(code.hx, code.hz, "x", True, capi.GrandDecoderConfig(W_MAX, 256, 0, CAP, 10, -1),
                    phase)
        n = SHOTS
        d_rec = torch.from_numpy(np.ascontiguousarray(errors.ravel())).to(dev)
        d_res = torch.empty(n * 72, dtype=torch.uint8, device=dev)
    for _ in range(args.case_reps):
        if eng.decode_device(n, d_rec.data_ptr(), d_res.data_ptr(), sp, use_graph=False) != 0:
            raise RuntimeError("decode failed")
        if eng.sync_status(sp) != 0:
            raise RuntimeError("status error")
        rst, dec = eng.kernel_times(sp)
        print(f"case {args.case}: decode kernel {dec:.4f} ms (control reset {rst:.4f} ms)", flush=True)


def run_reference(args):
    """The upstream CPU search algorithm on every host core, on the headline batch: each
    step is one pass over the 16384 shots; the warm-up passes and then the timed passes
    are each queued as one set of 128-shot tasks (every core busy)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    pool = CpuPool()
    try:
        if args.warmup:
            pool.passes(args.warmup)
        t_tot, shots, cands = pool.passes(args.steps)
    finally:
        pool.close()
    value = shots / t_tot
    return {"metric": METRIC, "value": value, "unit": "shots/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_tot * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded numpy PCG64)", "config": workload_config(),
            "impl": "reference", "candidates_per_s": cands / t_tot,
            "cpu_baseline": {"value": value, "unit": "shots/s", "cores": pool.cores,
                             "kind": pool.kind, "cpu_model": cpu_model(),
                             "sample": f"{args.steps} timed passes over the 16384-shot batch, "
                                       f"queued together as {CPU_CHUNK}-shot tasks on "
                                       f"{pool.cores} processes, mode -1"},
            "e2e": {"value": value, "unit": "shots/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def _rank_entry(argd):
    """One rank of a multi-GPU run started by bench.py itself."""
    out = run_ours(argparse.Namespace(**argd))
    if out is not None:
        print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--case", choices=["stress", "stress_dem", "headline"], default=None,
                    help="profiling mode: run one case --case-reps times, print kernel times")
    ap.add_argument("--case-reps", type=int, default=2)
    ap.add_argument("--case-shots", type=int, default=0)
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the batching, ML and serving sections")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.case:
        run_case(args)
        return
    if args.impl == "ours" and args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # no outside launcher: one process per GPU, started here (weak scaling: each rank
        # decodes its own 16384-shot batch)
        import torch
        have = torch.cuda.device_count()
        if have < args.gpus:
            sys.stderr.write(f"bench.py --gpus {args.gpus}: only {have} CUDA device(s) visible; "
                             f"a {args.gpus}-rank run needs one GPU per rank\n")
            sys.exit(2)
        from library_s_grand_gb300 import launch
        codes = launch.spawn_ranks(args.gpus, _rank_entry, (vars(args),))
        sys.exit(0 if all(c == 0 for c in codes) else 1)
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
