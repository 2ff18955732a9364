"""Multi-rank plumbing of bench.py on CPU ranks (gloo, world size 2): process
group set-up from the launcher's environment, the barrier, the max over ranks of
the timed duration, and the replica rule that only rank 0 runs and prints the
reference arm.  The GPU step itself runs as independent replicas (no exchange)."""
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


def _rank(rank, world, port, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import argparse

    import torch.distributed as dist

    import bench
    args = argparse.Namespace(impl="reference")
    w, r, local = bench.dist_init(args)
    assert (w, r, local) == (world, rank, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    m = bench.max_over_ranks(w, float(10 + rank), "cpu")
    bench.barrier(w)
    dist.destroy_process_group()
    out.put((rank, m))


def test_two_cpu_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 11.0), (1, 11.0)]


def _reference_rank(rank, world, port, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import argparse
    import io
    from contextlib import redirect_stdout

    import bench
    called = []
    class _Pool:
        def close(self):
            pass

        def join(self):
            pass

    bench.reference_setup = lambda: (_Pool(), 1, None, None)
    bench.cpu_step = lambda *a, **k: called.append(1) or 1.0
    args = argparse.Namespace(impl="reference", gpus=world, steps=1, warmup=0)
    w, r, _ = bench.dist_init(args)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_arm(args, w, r)
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((rank, len(called), buf.getvalue().count('"impl": "reference"')))


@pytest.mark.parametrize("world", [2])
def test_reference_arm_runs_on_rank0_only(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_reference_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert got == [(0, 1, 1), (1, 0, 0)]
