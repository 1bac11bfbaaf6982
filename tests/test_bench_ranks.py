"""The multi-GPU path of bench.py on CPU ranks: two gloo processes, each with its own timings,
agree on the element-wise maximum (the slowest replica sets the step time)."""
import os
import socket
import sys

import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        out.put((rank, bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5], "cpu")))
    finally:
        dist.destroy_process_group()


def test_step_times_are_the_maximum_over_two_ranks():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: [2.0, 10.0, 0.5], 1: [2.0, 10.0, 0.5]}
