"""The multi-GPU form of the bench (replicas only: the path does not shard within a run, and
the reference's own build has FDPS's MPI decomposition disabled): every rank advances its own
copy of the workload, the ranks enter the timed steps together, the slowest rank's time is the
job's, and the whole-job throughput counts every rank's particles.  Two gloo ranks on the CPU
run that host logic (bench.py's dist_init / replica_barrier / replica_max / replica_throughput)
with no GPU and no data-path collective."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    r, w, dist = bench.dist_init(world)
    try:
        bench.replica_barrier(dist)
        ms = 10.0 + 5.0 * r                      # rank 1 is the slower replica
        worst = bench.replica_max(ms, dist)
        q.put((r, w, worst, bench.replica_throughput(w, 1000, worst / 4)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in procs)
    assert [o[:2] for o in out] == [(0, 2), (1, 2)]
    for _, _, worst, value in out:
        assert worst == 15.0                     # max over ranks, seen by both
        assert value == pytest.approx(2 * 1000 / (15.0 / 4 * 1e-3))


def test_one_process_needs_no_process_group():
    import bench
    assert bench.dist_init(1)[2] is None if "WORLD_SIZE" not in os.environ else True
    assert bench.replica_max(3.5, None) == 3.5
    bench.replica_barrier(None)
    assert bench.replica_throughput(1, 1_000_000, 10.0) == pytest.approx(1e8)
