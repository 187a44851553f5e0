"""The N > 1 path of bench.py (one process per GPU, independent replicas):
per-rank seeds, max-over-ranks timing and the job throughput, exercised with
two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from flowmc_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 10 + r ms; the job's time is the slowest rank's
        t = replicas.max_over_ranks(10.0 + rank)
        thr = replicas.job_throughput(1000.0, t / 1e3)
        out[rank] = (t, thr, replicas.replica_seed(4, rank), replicas.world_size())
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_seeds_distinct():
    seeds = {replicas.replica_seed(4, r) for r in range(8)}
    assert len(seeds) == 8 and replicas.replica_seed(4, 0) == 4


def test_single_process_is_identity():
    assert replicas.world_size() == 1
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_throughput(100.0, 2.0) == 50.0


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for r in range(world):
        t, thr, seed, ws = res[r]
        assert ws == world
        assert t == pytest.approx(11.0)                      # max over ranks
        assert thr == pytest.approx(1000.0 * world / 0.011)  # all ranks' work over the slowest rank's time
    assert res[0][2] != res[1][2]                            # independent replicas
