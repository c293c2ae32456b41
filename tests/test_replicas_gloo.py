"""Multi-rank host logic on CPU: independent replica boxes, one per rank (world size 2, gloo).

The benchmark shards by replicas: each rank owns one box (seed 1 + rank), there
is no collective on the data path, and only the timing is reduced (max over
ranks) to form the whole-job throughput.  Here each rank advances its replica
with the oracle and the reductions are checked.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import time

    import bench
    from oracle import port as oport
    from mdacp_gb300 import lattice

    d = bench.Dist(world)
    q, L = lattice.fcc_cube(5, 0.5)
    p = lattice.maxwell(len(q), 1.0, 1 + d.rank)
    s = oport.System(q, p, L, rc=2.5, margin=0.5)
    s.make_pairlist()
    d.barrier()
    t0 = time.perf_counter()
    s.calculate(20)
    dt = time.perf_counter() - t0
    tmax = d.max(dt)
    e = s.observe()[2]
    out.put((d.rank, dt, tmax, e, len(q)))
    d.close()


def test_replicas_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    (r0, t0, m0, e0, n0), (r1, t1, m1, e1, n1) = res
    assert (r0, r1) == (0, 1)
    assert m0 == m1 == pytest.approx(max(t0, t1))   # both ranks agree on the job time
    assert e0 != e1                                  # independent replicas
    value = 2 * n0 * 20 / m0
    assert np.isfinite(value) and value > 0
