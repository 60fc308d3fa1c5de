"""Multi-rank path of bench.py on CPU (gloo, world size 2).

The lattice does not shard across GPUs here: N ranks run N independent
replicas and the whole-job throughput is all ranks' cell updates over the
slowest rank's time.  These tests run that aggregation with real gloo ranks.
"""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, results):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import bench
    d = bench.Dist(backend="gloo")
    cells = 1000 * (rank + 1)          # ranks may hold different lattices
    seconds = 2.0 if rank == 0 else 4.0  # rank 1 is the slow one
    mlups, t = bench.aggregate_mlups(cells, 10, seconds, d)
    d.barrier()
    results[rank] = (mlups, t)
    d.close()


@pytest.mark.timeout(120)
def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    expected = (1000 + 2000) * 10 / 4.0 / 1e6
    for r in range(2):
        mlups, t = results[r]
        assert t == 4.0
        assert abs(mlups - expected) < 1e-12


def _lattice_worker(rank, world, port, results):
    """Each rank steps its own replica (the oracle's C port stands in for the
    GPU step on a CPU-only host), times it, and the ranks aggregate."""
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import time
    import numpy as np
    import bench
    from oracle import d2q9
    from oracle import port as c_port
    d = bench.Dist(backend="gloo")
    nx, ny, steps = 48 + 16 * rank, 40, 20  # uneven replicas
    f = d2q9.equilibrium(np.ones((nx, ny)), np.zeros((nx, ny)), np.zeros((nx, ny)))
    d.barrier()
    t0 = time.perf_counter()
    c_port.cavity_run(f, 1.7, 0.1, steps, nthreads=1)
    secs = time.perf_counter() - t0
    mlups, t = bench.aggregate_mlups(nx * ny, steps, secs, d)
    ref = d2q9.equilibrium(np.ones((nx, ny)), np.zeros((nx, ny)), np.zeros((nx, ny)))
    for _ in range(steps):
        d2q9.cavity_step(ref, 1.7, 0.1)
    results[rank] = (mlups, t, secs, nx * ny, float(np.abs(f - ref).max()))
    d.close()


@pytest.mark.timeout(120)
def test_replicas_step_their_own_lattices_two_ranks():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_lattice_worker, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    slowest = max(results[r][2] for r in range(2))
    total = sum(results[r][3] * 20 for r in range(2))
    for r in range(2):
        mlups, t, _, _, err = results[r]
        assert t == slowest and abs(mlups - total / slowest / 1e6) < 1e-9 * mlups
        assert err < 1e-12  # each replica's lattice is the oracle's


def test_single_process_needs_no_process_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    d = bench.Dist()
    assert d.world == 1 and d.dist is None
    mlups, t = bench.aggregate_mlups(2_000_000, 5, 0.5, d)
    assert t == 0.5 and abs(mlups - 20.0) < 1e-12


def test_numpy_opt1_baseline_runs_one_process_per_core():
    """The numpy (opt1) CPU baseline: one spawned process per core, each on its
    own strip, reported as an aggregate over all of them."""
    import bench
    mlups, n, sample = bench.numpy_opt1_sample(64, 1.7, 0.1, "cavity", rows=16, steps=2)
    assert n == (os.cpu_count() or 1)
    assert mlups > 0 and "%d processes" % n in sample and "cavity_opt1.py" in sample
