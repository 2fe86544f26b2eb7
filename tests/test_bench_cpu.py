"""bench.py's multi-GPU replica aggregation (replicas only: independent systems, no exchange),
exercised with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # rank 1 is the slower one: 0.2 ms per step against 0.1
    ms = 0.1 * (rank + 1)
    out = {"value": 86400e-6 / (ms * 1e-3), "ms_per_step": ms, "n_gpus": 1, "config": {"workload": "w"},
           "e2e": {"value": 100.0 * (rank + 1), "unit": "ns/day"}, "gpu_launches": 15}
    single = bench.aggregate_ranks(out, world)
    # replica batches: rank r holds the replicas r, r + world, ... of 5 (3 and 2 here), each at
    # the rank's step time
    nloc = len(bench.replica_partition(5, rank, world))
    rep = {"value": nloc * 86400e-6 / (ms * 1e-3), "ms_per_step": ms, "n_gpus": 1, "config": {"workload": "r"},
           "replicas_this_rank": nloc, "gpu_launches": 10}
    q.put((rank, (single, bench.aggregate_ranks(rep, world))))
    dist.destroy_process_group()


def test_aggregate_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    for r in (0, 1):
        o, b = res[r]
        assert o["n_gpus"] == 2 and o["scaling"] == "weak"
        assert o["ms_per_step"] == pytest.approx(0.2)               # the slowest rank's step
        assert o["value"] == pytest.approx(2 * 86400e-6 / 0.2e-3)   # two replicas at that pace
        assert o["e2e"]["value"] == pytest.approx(2 * 100.0)        # the slowest rank's calls, x2
        assert o["gpu_launches"] == 30
        assert b["replicas_total"] == 5
        assert b["value"] == pytest.approx(5 * 86400e-6 / 0.2e-3)   # all five replicas at the slow pace
        assert b["gpu_launches"] == 20


def test_replica_partition_covers_each_replica_once():
    import bench

    for n, world in ((64, 1), (64, 2), (64, 3), (64, 8), (5, 8)):
        parts = [bench.replica_partition(n, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(n))
        assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1


def test_replica_extra_reports_its_own_failure():
    """The config-4 extra line keeps the arm's compact record, or the arm's error in its own entry,
    so that the headline line is printed either way."""
    import bench

    def failing(args):
        raise RuntimeError("replica batch: no device")

    assert bench.replica_extra(None, failing) == {"error": "RuntimeError: replica batch: no device"}
    keys = ("value", "unit", "ms_per_step", "config", "per_replica_ns_per_day", "sequential",
            "batch_speedup_vs_sequential", "batch_mode", "step_ms_min_median_max", "clocks")
    full = {k: 1 for k in keys}
    full["extra_key"] = 2
    assert bench.replica_extra(None, lambda args: full) == {k: 1 for k in keys}
