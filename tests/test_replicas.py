"""The multi-process plumbing of bench.py on CPU: two ranks over gloo (the
path shards as replicas only, one process per GPU, no data-path
collective).  The rendezvous, the barrier and the max over ranks that
bench.py takes of its timings, the environment it reads, and the reference
arm, whose non-zero ranks leave without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        env = bench.dist_env()
        bench.barrier(world)
        m = bench.max_over_ranks(1.5 * (rank + 1), world)
        ref = bench.run_reference(None, rank, world) if rank != 0 else "rank0"
        out.put((rank, env, m, ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[1] for g in got] == [(0, 2, 0), (1, 2, 1)]
    assert all(g[2] == 3.0 for g in got)  # max of 1.5 and 3.0 on both ranks
    assert got[1][3] is None  # the reference arm runs on rank 0 only
