"""The N > 1 benchmark path on the host: two gloo ranks on 127.0.0.1 run the
barrier and the max-over-ranks aggregation of bench.py (the per-rank work is
an independent replica set, so no data crosses ranks)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
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
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        value, t = res[r]
        assert t == 2.0
        assert value == pytest.approx(1000 * 10 * 5 * world / 2.0)
