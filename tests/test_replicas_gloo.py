"""The multi-process bench path on CPU (gloo, world size 2): the path does not
shard -- every rank runs an independent replica of the solve -- so the only
exchanges are the barrier around the timed region and the maximum of the
per-rank step times; the whole-job value is the DOFs of all replicas over that
maximum."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), DGX_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    r, w, _ = bench.dist_init()
    bench.barrier(w)
    ms = 1.0 + r               # rank 1 is the slower replica
    worst = bench.allreduce_max(ms, w)
    dofs = 1000
    q.put((r, w, worst, dofs * w / (worst * 1e-3)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_time_by_the_slowest_rank():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert all(g[2] == 2.0 for g in got)                  # the maximum over ranks
    assert all(abs(g[3] - 2 * 1000 / 2e-3) < 1e-6 for g in got)
