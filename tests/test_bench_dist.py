"""bench.py's multi-process plumbing with world size 2 on CPU (gloo): the
barrier, the max over ranks that the timed region reports, and the reference
arm, which only rank 0 runs (the others exit without work)."""

import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.init("gloo")
    d.barrier()
    m = d.max(10.0 * rank + 1.5)
    ref = bench.run_reference(None, d) if rank != 0 else "rank0"
    d.barrier()
    out.put((rank, m, ref))
    d.pg.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    out = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(out.get() for _ in range(2))
    # every rank sees the slowest rank's value; rank 1 leaves the reference arm at once
    assert got == [(0, 11.5, "rank0"), (1, 11.5, None)]
