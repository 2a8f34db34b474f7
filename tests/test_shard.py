"""Multi-GPU unit sharding on CPU: two gloo ranks split a swath's bursts,
process them with a stand-in per-unit function, and combine the counts
(SUM) and the times (MAX) -- the only exchange the multi-GPU path has."""
import os
import socket

import pytest

from sentinel1_decode_gb300.shard import assign_units, run_sharded


def test_assign_units_covers_disjoint_and_balances():
    costs = [1500 * 12000, 1460 * 11900, 1550 * 12400, 1480 * 12100, 1520 * 11800, 1500 * 12300, 1490 * 12000,
             1510 * 12200, 1470 * 12500] * 2
    for world in (1, 2, 3, 4, 8):
        plan = assign_units(costs, world)
        flat = sorted(i for p in plan for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in plan]
        # LPT keeps the spread within the largest unit
        assert max(loads) - min(loads) <= max(costs)
    assert assign_units(costs, 2) == assign_units(list(costs), 2)   # deterministic
    with pytest.raises(ValueError):
        assign_units(costs, 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, units, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # stand-in for one burst on this rank's GPU: device ms proportional to size
        done, total, tmax = run_sharded(units, rank, world, lambda s, b: units[[u[:2] for u in units].index((s, b))][2] / 1e6)
        q.put((rank, done, total, tmax))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_and_combine():
    import torch.multiprocessing as mp
    units = [(s, b, (1450 + 13 * b + 7 * s) * (11800 + 50 * b)) for s in range(2) for b in range(9)]
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, units, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    done = [set(r[1]) for r in res]
    assert done[0].isdisjoint(done[1])
    assert done[0] | done[1] == {u[:2] for u in units}
    total = sum(u[2] for u in units)
    for _, _, t, tmax in res:
        assert t == pytest.approx(total)
        per_rank = [sum(u[2] for u in units if u[:2] in d) / 1e6 for d in done]
        assert tmax == pytest.approx(max(per_rank))


def _bench_rank_main(rank, world, port, units, q):
    """One rank of bench.py's multi-GPU path with a stub in place of the GPU:
    the rank's share (rank_bursts) and the job-wide rate (reduce_rate)."""
    import importlib.util
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_rank", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        share = bench.rank_bursts(units, world, rank, 2)
        cost = {(s, b): c for s, b, c in units}
        samples = sum(cost[(s, b)] for s in range(2) for b in share[s])
        seconds = samples / 1e9          # stub: one GPU forms 1e9 samples/s
        total, tmax = bench.reduce_rate(float(samples), seconds)
        q.put((rank, share, total, tmax))
    finally:
        dist.destroy_process_group()


def test_bench_shards_units_over_two_gloo_ranks():
    """bench.py --gpus 2 splits one swath's 18 (stream, burst) units over the
    ranks (disjoint, complete, balanced within one unit) and reports
    all ranks' samples over the slowest rank's time."""
    import torch.multiprocessing as mp
    units = [(s, b, (1450 + 13 * b + 7 * s) * (11800 + 50 * b)) for s in range(2) for b in range(9)]
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_bench_rank_main, args=(r, world, port, units, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got = [{(s, b) for s in range(2) for b in r[1][s]} for r in res]
    assert got[0].isdisjoint(got[1])
    assert got[0] | got[1] == {(s, b) for s, b, _ in units}
    cost = {(s, b): c for s, b, c in units}
    loads = [sum(cost[u] for u in g) for g in got]
    assert max(loads) - min(loads) <= max(cost.values())
    for _, _, total, tmax in res:
        assert total == pytest.approx(sum(loads))
        assert tmax == pytest.approx(max(loads) / 1e9)
