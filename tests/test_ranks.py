"""The multi-rank path of bench.py on CPU: two gloo ranks (127.0.0.1).

bench.py runs one process per GPU; a single model runs as replicas and an
ensemble shards its members by rank.  The only collectives are barriers and
the max over ranks of the timed interval.  These tests drive exactly those
helpers with world_size 2 on the gloo backend, no GPU.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # replicas: each rank timed its own steps; the job's rate uses the slowest
        elapsed = [1.5, 2.0][rank]
        bench.rank_barrier(world)
        slowest = bench.rank_max(elapsed, world)
        rate = bench.whole_job_rate(10, world, slowest)
        # ensemble: members shard with no overlap
        mine = bench.shard(range(2 * 7), rank, world)
        # the uneven configuration-3 members: each rank takes its part of a
        # cost-balanced split of 64 per rank, and the ranks' loads are
        # compared through a collective of the test (not of the data path)
        from hmec import synth

        allm = synth.ensemble_members(64 * world)
        costs = [bench.member_cost(o) for o, _, _ in allm]
        part = bench.balanced_split(costs, world)[rank]
        load = torch.tensor([sum(costs[i] for i in part)], dtype=torch.float64)
        loads = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(loads, load)
        q.put((rank, slowest, rate, mine, part, [float(x.item()) for x in loads], sum(costs)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_and_shard():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[1] for r in res] == [2.0, 2.0]  # max over ranks
    assert [r[2] for r in res] == [10.0, 10.0]  # 2 ranks x 10 units / 2.0 s
    members = sorted(m for r in res for m in r[3])
    assert members == list(range(14))  # every member exactly once
    assert res[0][3] == [0, 2, 4, 6, 8, 10, 12] and res[1][3] == [1, 3, 5, 7, 9, 11, 13]
    # balanced members: disjoint, complete, and within 1 % of an even split
    parts = [set(r[4]) for r in res]
    assert not (parts[0] & parts[1]) and len(parts[0] | parts[1]) == 128
    loads, total = res[0][5], res[0][6]
    assert res[1][5] == loads and abs(sum(loads) - total) < 1e-6 * total
    assert max(loads) <= 1.01 * total / world, loads


def test_single_rank_helpers_need_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.rank_max(3.5, 1) == 3.5
    bench.rank_barrier(1)
    assert bench.shard([5, 6, 7], 0, 1) == [5, 6, 7]
    assert bench.whole_job_rate(8, 1, 2.0) == 4.0


def test_balanced_split_beats_round_robin_on_uneven_members():
    """The cost-balanced member split of the ensemble bench against the
    round-robin one, on the 64 uneven configuration-3 members per rank."""
    sys.path.insert(0, ROOT)
    import bench
    from hmec import synth

    for world in (2, 4, 8):
        allm = synth.ensemble_members(64 * world)
        costs = [bench.member_cost(o) for o, _, _ in allm]
        parts = bench.balanced_split(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        bal = max(sum(costs[i] for i in p) for p in parts)
        rr = max(sum(costs[i] for i in bench.shard(range(len(costs)), r, world)) for r in range(world))
        assert bal <= 1.01 * sum(costs) / world and bal <= rr, (world, bal, rr)
