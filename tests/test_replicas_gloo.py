"""The multi-GPU path of the benchmark is replicas only (each GPU runs its own copy of the
frame loop; nothing is exchanged between them).  What the ranks share is the timing: a
barrier, then the slowest rank's time over the whole job's frames.  This checks that
aggregation with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 + 25.0 * rank          # rank 1 is the slow replica
    mx = bench.max_over_ranks(local_ms, dist, "cpu")
    rate = bench.whole_job_rate(300, world, mx)
    dist.barrier()
    out[rank] = (mx, rate)
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    for r in range(world):
        mx, rate = out[r]
        assert mx == 125.0
        assert rate == pytest.approx(300 * 2 / 0.125)
