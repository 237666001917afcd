"""The N>1 path of bench.py on host-only ranks (gloo, world size 2): the
rendering work does not shard (replicas only), so ranks share nothing but
the barrier around the timed region and the max-over-ranks of its time; the
reported value is the units all ranks processed over that max time."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    assert (w, r) == (ws, rank)
    bench.barrier(w)
    t = 10.0 + rank * 5.0  # rank 1 is the slower replica
    q.put((rank, bench.max_over_ranks(w, t)))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_replicas_share_only_barrier_and_max_time():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(ws))
    assert got == {0: 15.0, 1: 15.0}
