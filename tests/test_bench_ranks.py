"""The multi-process path of bench.py (replicas: one independent filter per
rank, no data-path collective) on CPU with gloo, world size 2: rank
discovery from the torchrun environment, the barrier, the max-over-ranks
time, and the reference arm running on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_init()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    t = bench.max_over_ranks(w, 10.0 + rank, "cpu")
    args = type("A", (), dict(gpus=world, steps=1, warmup=0))()
    ref = bench.run_reference(args, w, r) if r != 0 else "rank0"
    out.put((rank, t, ref))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_gloo_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 11.0, "rank0"), (1, 11.0, None)]
