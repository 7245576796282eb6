"""Multi-GPU host logic of bench.py (replicas only: MDAS has no exchange step on
1-GPU machines), exercised as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r took 10 + r ms of sampler time, 20 + 3r ms of wall time, and 1000 * (r + 1) samples
    res = bench.reduce_across_ranks(10.0 + rank, 20.0 + 3 * rank, 1000 * (rank + 1), world, "cpu")
    out[rank] = (res, bench.replica_seed(100, rank))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replica_reduction_gloo(world):
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(world):
        (mdas_ms, wall_ms, samples), seed = out[r]
        assert mdas_ms == 10.0 + (world - 1)  # max over ranks
        assert wall_ms == 20.0 + 3 * (world - 1)
        assert samples == sum(1000 * (k + 1) for k in range(world))  # sum of the work
        assert seed == 100 + r  # every replica renders its own scene


def test_single_rank_is_identity():
    import bench
    assert bench.reduce_across_ranks(5.0, 6.0, 7, 1, "cpu") == (5.0, 6.0, 7)
