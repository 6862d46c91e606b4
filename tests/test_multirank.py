"""The N>1 path of bench.py on CPU: two gloo ranks each plan their own query
shard (no shared query, no collective on the data path) and agree on the
whole-job rate through one max-reduction of the timed region."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from oracle import oracle as O
        shard = bench.make_workload(rank, n_queries=3)
        shard = [s for s in shard]
        for s in shard:
            s.config = s.config.replace(tree_capacity=3000, max_iterations=12)
        res = O.plan_batch(shard, threads=1)
        local_ms = 100.0 * (rank + 1)  # rank 1 is the slowest
        slowest, rate = bench.whole_job_rate(local_ms, len(shard), 2, world)
        starts = [tuple(s.init[:3].tolist()) for s in shard]
        q.put((rank, slowest, rate, starts, [r["tree_size"] for r in res]))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharding_and_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    (_, s0, r0, st0, t0), (_, s1, r1, st1, t1) = out
    assert s0 == s1 == 200.0
    # 3 queries per rank x 2 ranks x 2 steps / 0.2 s
    assert r0 == r1 == pytest.approx(60.0)
    assert not set(st0) & set(st1), "ranks must plan different scenes"
