"""bench.py under torchrun with N > 1: independent replicas, a barrier
around the timed region, the whole-job aggregate (units summed over ranks)
and the slowest rank's time.  Run here as two gloo ranks on the CPU (the
process group and the reductions are the bench's own functions)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    import bench
    dist = bench.dist_setup()
    try:
        bench.barrier(dist)
        units, ms = bench.replica_totals(dist, rank + 1, 10.0 * (rank + 1))
        q.put((rank, units, ms, dist.get_backend()))
    finally:
        dist.destroy_process_group()


def test_replica_totals_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    # daemon ranks: a rank that hangs cannot keep the test process alive
    procs = [ctx.Process(target=_rank, args=(r, port, q), daemon=True) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = [q.get(timeout=120) for _ in procs]
        for p in procs:
            p.join(timeout=60)
            assert p.exitcode == 0
    finally:
        for p in procs:
            if p.is_alive():
                p.terminate()
    assert sorted(got) == [(0, 3.0, 20.0, "gloo"), (1, 3.0, 20.0, "gloo")]


def test_single_process_is_its_own_total(monkeypatch):
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    dist = bench.dist_setup()
    assert dist is None
    bench.barrier(dist)
    assert bench.replica_totals(dist, 4, 12.5) == (4.0, 12.5)
