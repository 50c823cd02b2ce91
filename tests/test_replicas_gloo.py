"""The multi-GPU path of bench.py is replicas only: every rank runs its own
population and the job's rate is all ranks' units over the slowest rank's
time.  Checked here with two gloo ranks on the CPU."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        out[rank] = (ms, bench.whole_job_rate(64 * 100, world, ms))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 15.0
    assert out[0][1] == pytest.approx(2 * 6400 / 0.015)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(7.5, 1, "cpu") == 7.5
