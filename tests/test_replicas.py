"""CPU, world_size 2 over gloo: the replica coordination bench.py uses for --gpus N (independent
transforms per rank, no data-path collective; a barrier and max-over-ranks timing; the job total
summed over ranks).  Each rank transforms its own seeded field with the CPU oracle."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import time

    import bench
    import pyoracle
    reps = bench.Replicas()
    assert (reps.rank, reps.world) == (rank, world)
    gd, gd2 = (16, 12, 10), (9, 12, 10)
    x = np.random.default_rng(512 + rank).uniform(-1, 1, (10, 12, 16))
    plan = pyoracle.OraclePlan((5, 9, 9), gd, (0, 1, 2), gd2, (1, 2, 0), -1, 0)
    reps.barrier()
    t0 = time.perf_counter()
    y = plan.exec(x, idir=2, nthreads=1)
    dt = time.perf_counter() - t0 + 0.01 * rank  # rank 1 deliberately slower
    t_max = reps.max(dt)
    units = reps.sum(1.0)
    checksum = float(np.abs(y).sum())
    all_sums = reps.sum(checksum)
    out.put((rank, dt, t_max, units, checksum, all_sums))
    reps.close()


def test_two_replicas_over_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, dt0, tmax0, u0, c0, s0), (r1, dt1, tmax1, u1, c1, s1) = res
    assert tmax0 == tmax1 == pytest.approx(max(dt0, dt1))  # max over ranks, seen by both
    assert u0 == u1 == 2.0  # whole-job units: summed over ranks
    assert c0 != c1  # independent seeded inputs per rank
    assert s0 == s1 == pytest.approx(c0 + c1)
