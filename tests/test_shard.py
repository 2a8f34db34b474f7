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
