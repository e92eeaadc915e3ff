"""The N>1 path of bench.py on CPU: two gloo ranks as independent replicas,
the barrier, the max over ranks of the step time, and the whole-job rate."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup(world, backend="gloo")
    bench.barrier(w)
    # each replica reports its own step time; the slowest rank sets the rate
    ms = 100.0 + 50.0 * r
    slowest = bench.max_over_ranks(ms, w)
    out.put((r, w, local, slowest, bench.aggregate_rate(1e9, w, slowest)))
    bench.barrier(w)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replicas_take_max_over_ranks(world):
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = 100.0 + 50.0 * (world - 1)
    for r, (rank, w, local, got, rate) in enumerate(results):
        assert (rank, w, local) == (r, world, r)
        assert got == slowest
        # world replicas of 1e9 units per step each, at the slowest rank's time
        assert abs(rate - world * 1.0 / (slowest / 1e3)) < 1e-9
