"""Multi-rank shot sharding on CPU: two gloo ranks each decode their contiguous
shard (the oracle stands in for each rank's GPU decode) and the gathered results
equal one decode of the whole batch."""
import os
import socket

import numpy as np
import pytest

from library_s_grand_gb300.shard import record_slice, shard_range


def test_shard_ranges_cover_exactly():
    for n in (0, 1, 7, 100, 16384):
        for world in (1, 2, 3, 8):
            spans = [shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_record_slice_mixed_lengths():
    lens = [144, 36, 132]
    sc = np.array([0, 1, 2, 1, 0], dtype=np.int32)
    assert record_slice(lens, sc, 0, 5) == (0, 144 + 36 + 132 + 36 + 144)
    assert record_slice(lens, sc, 1, 3) == (144, 144 + 36 + 132)
    assert record_slice([36], None, 2, 4) == (72, 144)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_path):
    import sys
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import torch.distributed as dist
    import oracle as O
    from library_s_grand_gb300 import synth
    from library_s_grand_gb300.shard import decode_sharded
    dist.init_process_group("gloo", rank=rank, world_size=world)
    code = synth.BB_CODES[72]()
    errors, _ = synth.css_shots(code.hz, 301, 0.03, seed=3)
    port_lib = O.Port()
    cfg = O.make_config(3, mode=-1)

    def decode(rec, sc):
        e = rec.reshape(-1, code.m)
        return port_lib.css(O.UNIFORM, code.hx, code.hz, e, None, cfg, "x")[1]

    res = decode_sharded(decode, errors, [code.m], len(errors))
    if rank == 0:
        np.save(out_path, res)
    dist.destroy_process_group()


def test_two_rank_gloo_sharding_equals_single_decode(tmp_path):
    import multiprocessing as mp
    import oracle as O
    from library_s_grand_gb300 import synth
    port = _free_port()
    out = str(tmp_path / "gathered.npy")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = np.load(out)
    code = synth.BB_CODES[72]()
    errors, _ = synth.css_shots(code.hz, 301, 0.03, seed=3)
    _, want, _ = O.Port().css(O.UNIFORM, code.hx, code.hz, errors, None, O.make_config(3, mode=-1), "x")
    assert len(O.fields_equal(got, want)) == 0
