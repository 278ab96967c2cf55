"""One process per GPU on one node, without an outside launcher.

``spawn_ranks(n, fn, args)`` starts n processes (the ``spawn`` start method) with
RANK, LOCAL_RANK, WORLD_SIZE, MASTER_ADDR = 127.0.0.1 and a free MASTER_PORT in
their environment -- what ``torch.distributed.run`` would set -- and each calls
``fn(*args)``.  ``init_from_env`` then joins the process group from those
variables (NCCL on GPUs, gloo on CPU) and logs the communicator it made.  Shots
are independent, so the decoder itself needs no collective: ranks only meet at
barriers and in the max-over-ranks reduction of their timings.
"""
from __future__ import annotations

import os
import socket
import sys


def free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _child(rank, world, port, fn, args):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    fn(*args)


def spawn_ranks(world: int, fn, args=(), timeout: float | None = None) -> list:
    """Run fn(*args) in `world` fresh processes; returns their exit codes."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = free_port()
    procs = [ctx.Process(target=_child, args=(r, world, port, fn, tuple(args)))
             for r in range(world)]
    for p in procs:
        p.start()
    codes = []
    for p in procs:
        p.join(timeout)
        if p.exitcode is None:  # still running past the timeout
            p.terminate()
            p.join()
        codes.append(p.exitcode)
    return codes


def env_ranks():
    """(rank, world, local_rank) from the environment (1 process if unset)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init_from_env(backend: str, device=None):
    """Join the process group the environment describes; returns the
    torch.distributed module, or None for a single process."""
    rank, world, _ = env_ranks()
    if world <= 1:
        return None
    import torch.distributed as dist
    if device is not None:
        dist.init_process_group(backend, device_id=device)
    else:
        dist.init_process_group(backend)
    sys.stderr.write(f"rank {rank}/{world}: {backend} process group up "
                     f"({os.environ.get('MASTER_ADDR')}:{os.environ.get('MASTER_PORT')})\n")
    return dist


def max_over_ranks(dist, value: float, device=None) -> float:
    """The largest `value` over all ranks (the value itself for one process)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
