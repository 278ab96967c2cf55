"""The multi-rank launch path of bench.py on CPU: launch.spawn_ranks starts two
processes with the rendezvous environment torch.distributed.run would give them,
each joins a gloo process group from it, meets the other at a barrier, decodes its
own shard of a batch (the oracle stands in for each rank's GPU) and takes the
max-over-ranks of its time -- the same calls bench.py makes with NCCL, one process
per GPU.  On a machine with fewer GPUs than asked for, `bench.py --gpus 2` stops
with a clear message instead of running one rank."""
import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT
from library_s_grand_gb300 import launch


def _rank(out_dir):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from library_s_grand_gb300 import launch as L
    from library_s_grand_gb300 import synth
    from library_s_grand_gb300.shard import shard_range
    rank, world, local = L.env_ranks()
    dist = L.init_from_env("gloo")
    dist.barrier()
    code = synth.BB_CODES[72]()
    errors, _ = synth.css_shots(code.hz, 257, 0.03, seed=8)
    lo, hi = shard_range(len(errors), rank, world)
    _, res, _ = O.Port().css(O.UNIFORM, code.hx, code.hz, errors[lo:hi], None,
                             O.make_config(3), "x")
    t = L.max_over_ranks(dist, 10.0 + rank)
    np.save(os.path.join(out_dir, f"res{rank}.npy"), res)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": rank, "world": world, "local": local, "max": t,
                   "addr": os.environ["MASTER_ADDR"]}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_spawn_ranks_gloo_two_ranks(tmp_path):
    import oracle as O
    from library_s_grand_gb300 import synth
    codes = launch.spawn_ranks(2, _rank, (str(tmp_path),), timeout=180)
    assert codes == [0, 0]
    info = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert [i["rank"] for i in info] == [0, 1] and all(i["world"] == 2 for i in info)
    assert all(i["max"] == 11.0 for i in info)  # both ranks see the slower rank's time
    assert all(i["addr"] == "127.0.0.1" for i in info)
    got = np.concatenate([np.load(tmp_path / f"res{r}.npy") for r in range(2)])
    code = synth.BB_CODES[72]()
    errors, _ = synth.css_shots(code.hz, 257, 0.03, seed=8)
    _, want, _ = O.Port().css(O.UNIFORM, code.hx, code.hz, errors, None, O.make_config(3), "x")
    assert len(O.fields_equal(got, want)) == 0


def test_bench_refuses_more_ranks_than_gpus():
    import torch
    if torch.cuda.device_count() >= 2:
        return  # a real multi-GPU machine: nothing to refuse
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2",
                          "--steps", "3", "--warmup", "3"], capture_output=True, text=True,
                         env=env, timeout=300)
    assert out.returncode == 2
    assert "needs one GPU per rank" in out.stderr
