"""The multi-GPU path is replicas only (every rank images its own frames, no
collective on the data path): the host-side pieces bench.py uses under
torchrun -- process-group set-up, the barrier around the timed region and the
max over ranks of the step time -- on two CPU ranks over gloo."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), BENCH_BACKEND="gloo")
    import torch.distributed as dist

    import bench
    ws, r, local = bench.dist_init()
    bench.barrier(ws)
    # each rank's own step time; every rank must report the slowest
    t = bench.max_over_ranks(ws, 10.0 + 5.0 * r, "cpu")
    bench.barrier(ws)
    q.put((r, ws, local, t))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=90) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert got == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_one_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_init() == (1, 0, 0)
    assert bench.max_over_ranks(1, 3.5, "cpu") == 3.5
