"""Several GPUs = independent replicas (weak scaling, no data-path
collective): each rank assembles its own copy of the workload, the job's
time per step is the slowest rank's (barrier + MAX all-reduce), and the
job's throughput sums the ranks' elements.  World size 2 on the CPU (gloo,
127.0.0.1), as bench.py runs it under torchrun."""
import os

import pytest
import torch.distributed as dist
import torch.multiprocessing as tmp


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    sec = bench.max_over_ranks(0.010 * (rank + 1), dist)   # rank 1 is the slow one
    value = bench.replica_throughput(1_000_000, sec, world)
    q.put((rank, sec, value))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_time_is_the_max_and_throughput_the_sum():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = 29517
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, sec, value in out:
        assert sec == pytest.approx(0.020)                 # both ranks see the max
        assert value == pytest.approx(2 * 1_000_000 / 0.020 / 1e6)


def test_single_process_needs_no_collective():
    import bench
    assert bench.max_over_ranks(0.5, None) == 0.5
    assert bench.replica_throughput(1_000_000, 0.5, 1) == pytest.approx(2.0)
