"""Multi-process (world size 2, gloo, CPU) checks of the replica bookkeeping that bench.py and
multi-GPU runs use: max-over-ranks timing, whole-job throughput, cost-balanced sharding."""
import os
import socket

import pytest

from diffrg_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        r, w, lr = replicas.dist_env()
        elapsed = 1.0 + 0.5 * rank  # rank 1 is the slow one
        m = replicas.max_over_ranks(elapsed)
        rate = replicas.aggregate_rate(384, 10, w, m)
        dist.barrier()
        q.put((r, w, lr, m, rate))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_rate_world2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    for _, _, _, m, rate in out:
        assert m == 1.5  # the slowest rank's time
        assert rate == pytest.approx(384 * 10 * 2 / 1.5)


def test_single_process_needs_no_group():
    assert replicas.max_over_ranks(3.25) == 3.25
    assert replicas.aggregate_rate(100, 4, 1, 2.0) == 200.0


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_by_cost_covers_and_balances(world):
    import numpy as np

    rng = np.random.default_rng(world)
    costs = list(np.prod(rng.integers(16, 257, size=(500, 3)), axis=1).astype(float))
    parts = replicas.partition_by_cost(costs, world)
    assert len(parts) == world and parts[0][0] == 0 and parts[-1][1] == len(costs)
    for (a, b), (c, d) in zip(parts, parts[1:]):
        assert b == c and a <= b
    share = [sum(costs[a:b]) for a, b in parts]
    assert max(share) <= sum(costs) / world + max(costs) + 1e-9
