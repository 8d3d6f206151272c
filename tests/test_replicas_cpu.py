"""The multi-GPU path is replicas only: bench.py's host-side barrier and
max/sum reductions over gloo, checked with two CPU ranks (no GPU, no
data-path collective)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    # each rank's timed milliseconds and monomer-steps, as run_gpu aggregates them
    ms = 10.0 + 5.0 * rank
    units = 1000.0 * (rank + 1)
    t_max = d.max(ms)
    total = d.sum(units)
    out.put((rank, t_max, total, total / (t_max / 1e3)))
    d.close()


def test_two_gloo_ranks_aggregate_replicas():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, t_max, total, value in res:
        assert t_max == 15.0 and total == 3000.0
        assert abs(value - 3000.0 / 0.015) < 1e-6
