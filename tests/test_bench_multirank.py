"""Multi-rank logic of bench.py on CPU (gloo, world size 2): the timed
region is the max over ranks, the whole-job value counts every rank's
steps, and only rank 0 prints the reference arm."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(100.0 + 50.0 * rank)
    rank_, world_, _ = bench.dist_env()
    buf = io.StringIO()

    class A:
        size, warmup, steps = 10, 3, 1
    # the reference arm prints on rank 0 only; skip its (slow) CPU sample here
    orig = bench.run_cpu_baseline
    bench.run_cpu_baseline = lambda case, W, K: {"value": 1.0, "unit": "load steps/s", "cores": 1,
                                                 "kind": "port", "sample": "stub"}
    with redirect_stdout(buf):
        bench.run_reference(A)
    bench.run_cpu_baseline = orig
    dist.destroy_process_group()
    q.put((rank_, world_, ms, buf.getvalue()))


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == 150.0 for o in out)  # max over ranks
    assert '"impl": "reference"' in out[0][3] and out[1][3] == ""
