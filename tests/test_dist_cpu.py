"""The multi-process path of bench.py on the CPU: two gloo ranks on
127.0.0.1 set up from the torchrun environment variables, meet at the
barrier and take the max of their timings (the replicas contract: every
rank times its own independent replica, rank 0 reports the slowest)."""

import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    m = bench.max_over_ranks(10.0 + rank, w)
    out.put((rank, m))
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 11.0), (1, 11.0)]
