"""The N > 1 path on the host, with two gloo ranks on 127.0.0.1: the
partition of one ensemble into whole systems per rank, the gathering of the
results in ensemble order, and bench.py's barrier and max-over-ranks
aggregation.  No data crosses ranks while systems run."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _spawn(fn, world, *args):
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.spawn(fn, args=(world, _free_port(), out, *args), nprocs=world, join=True)
        return dict(out)


def _init(rank, world, port):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return dist


def _rank_aggregate(rank, world, port, out):
    import bench
    dist = _init(rank, world, port)
    try:
        bench.dist_barrier(world)
        # rank r took (r + 1) seconds for its share: the job time is the max
        value, t = bench.aggregate(beads=1000, md_steps=10, steps=5, dev_time_local=float(rank + 1),
                                   world=world)
        out[rank] = (value, t)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate():
    world = 2
    res = _spawn(_rank_aggregate, world)
    for r in range(world):
        value, t = res[r]
        assert t == 2.0
        # 1000 beads on each of the two ranks
        assert value == pytest.approx(1000 * world * 10 * 5 / 2.0)


def test_partition_is_complete_disjoint_and_balanced():
    from opencafemol_gb300 import partition, synth
    sizes = synth.ensemble_sizes(1024, 50, 800, 2024)
    costs = [partition.system_cost(int(n)) for n in sizes]
    for world in (1, 2, 3, 8):
        parts = partition.assign(costs, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(sizes)))
        assert partition.balance(costs, parts) < 1.01
        # deterministic: every rank computes the same assignment
        assert parts == partition.assign(costs, world)
    # more ranks than systems: some ranks idle, nothing lost
    parts = partition.assign([5.0, 1.0], 4)
    assert sorted(k for p in parts for k in p) == [0, 1] and sum(1 for p in parts if not p) == 2
    with pytest.raises(ValueError):
        partition.assign(costs, 0)


def _rank_shard(rank, world, port, out, sizes):
    from opencafemol_gb300 import partition
    dist = _init(rank, world, port)
    try:
        sh = partition.shard(sizes, rank, world)
        # stand-in for a rank's batch: a result that names its system
        local = {k: np.full(3, float(sizes[k] * 10 + k)) for k in sh.indices}
        got = partition.gather_in_order(local, len(sizes), world)
        out[rank] = (sh.indices, None if got is None else [g.tolist() for g in got])
    finally:
        dist.destroy_process_group()


def test_two_ranks_run_disjoint_shares_and_gather_in_order():
    sizes = [800, 50, 333, 120, 640, 77, 410, 95, 260]
    res = _spawn(_rank_shard, 2, sizes)
    a, b = res[0][0], res[1][0]
    assert not set(a) & set(b) and sorted(a + b) == list(range(len(sizes)))
    assert res[1][1] is None
    assert res[0][1] == [[float(n * 10 + k)] * 3 for k, n in enumerate(sizes)]


def _rank_gather_missing(rank, world, port, out):
    from opencafemol_gb300 import partition
    dist = _init(rank, world, port)
    try:
        local = {0: 1.0} if rank == 0 else {}
        try:
            partition.gather_in_order(local, 2, world)
            out[rank] = "ok"
        except RuntimeError as e:
            out[rank] = str(e)
    finally:
        dist.destroy_process_group()


def test_gather_reports_a_missing_system():
    res = _spawn(_rank_gather_missing, 2)
    assert "came back from no rank" in res[0] and res[1] == "ok"
