"""bench.py's replica logic across two ranks (CPU, gloo, world size 2).

``bench.py --gpus N`` runs N independent replicas of the workload (one process per GPU): the
path has no data exchange for this metric.  Each replica times its own steps; the job's time is
the slowest replica's (barrier + max all-reduce), and ``value`` counts the units all replicas
processed.  Two spawned CPU ranks exercise exactly those functions with the gloo backend.
"""

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    w, r, local = bench.dist_env()
    assert (w, r, local) == (world, rank, rank)
    dist = bench.replicas_begin(w, backend="gloo")
    bench.replicas_barrier(dist)
    ms = 100.0 + 50.0 * rank  # the second replica is the slow one
    job_ms = bench.replicas_max_ms(dist, ms)
    out.put((rank, job_ms, bench.whole_job_rate(w, 20 * 64, job_ms)))
    bench.replicas_end(dist)


def test_two_replicas_take_the_slowest_time_and_count_all_units():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, job_ms, value in res:
        assert job_ms == 150.0                                # max over ranks
        assert value == pytest.approx(2 * 20 * 64 / 0.150)   # both replicas' units over the slowest time


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replicas_begin(1) is None
    assert bench.replicas_max_ms(None, 12.5) == 12.5
    assert bench.whole_job_rate(1, 64, 1000.0) == 64.0
