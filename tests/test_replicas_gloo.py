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


def test_bench_starts_its_own_ranks():
    # `bench.py --gpus 2` without torchrun's environment starts two ranks under
    # torch.distributed.run (rendezvous on 127.0.0.1); both join the gloo group
    # and rank 0 alone prints the line.  The reference arm runs on the host
    # cores, so this runs without a GPU.
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR",
                                                             "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--cells", "12", "--cpu-seconds", "0.5", "--cpu-threads", "2", "--steps", "3",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, env=env, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["ranks_joined"] == 2
    assert line["config"]["parallelism"] == "replicas x2" and line["value"] > 0


def test_bench_refuses_a_rank_count_that_differs_from_the_job():
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--cells", "12"], capture_output=True, text=True, timeout=300, env=env, cwd=root)
    assert r.returncode != 0 and "WORLD_SIZE is 1" in r.stderr
