"""Multi-GPU distribution of independent (stream, burst) units.

Each (polarisation stream, burst) pair goes from raw bytes to SLC without
touching any other burst (the reference also forms bursts one at a time,
s1_decoder.cpp:315-346), so N GPUs share a swath by splitting the units, with
no collective on the data path.  Units are assigned by cost (lines x range
samples) with the longest-processing-time rule; each rank processes its units
on its own GPU and the ranks exchange only two numbers at the end: the SUM of
the samples and the MAX of the device times (the job ends when the slowest
rank does).

One process per GPU (torchrun / torch.distributed): `rank`, `world` from the
environment, any backend (gloo is enough: only host scalars move).
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple


def assign_units(costs: Sequence[float], world: int) -> List[List[int]]:
    """Indices of `costs` per rank, longest first onto the least-loaded rank
    (ties to the lower rank).  Deterministic, so every rank computes the same
    plan without communicating."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    plan: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        plan[r].append(i)
        load[r] += costs[i]
    for p in plan:
        p.sort()
    return plan


def swath_units(decoders, swath: str) -> List[Tuple[int, int, int]]:
    """(stream index, burst index, lines x samples) of every burst of `swath`
    in each decoder, from the packet headers only (no GPU work)."""
    import ctypes
    units = []
    for s, d in enumerate(decoders):
        for b in range(d.num_bursts(swath)):
            r, c = ctypes.c_int64(), ctypes.c_int64()
            d._check(d._lib.s1g_burst_shape(d.handle, swath.encode(), b, 0, ctypes.byref(r), ctypes.byref(c)))
            units.append((s, b, r.value * c.value))
    return units


def combine(samples: float, device_ms: float) -> Tuple[float, float]:
    """(total samples over ranks, max device time over ranks); identity when
    torch.distributed is not initialised."""
    try:
        import torch
        import torch.distributed as dist
    except ImportError:  # pragma: no cover
        return samples, device_ms
    if not (dist.is_available() and dist.is_initialized()):
        return samples, device_ms
    s = torch.tensor([float(samples)], dtype=torch.float64)
    t = torch.tensor([float(device_ms)], dtype=torch.float64)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(s[0]), float(t[0])


def run_sharded(units: Sequence[Tuple[int, int, int]], rank: int, world: int,
                process: Callable[[int, int], float]) -> Tuple[List[Tuple[int, int]], float, float]:
    """Process this rank's share: process(stream, burst) -> device ms for one
    unit.  Returns (units done here, total samples of the job, max device ms
    over ranks)."""
    plan = assign_units([u[2] for u in units], world)
    mine = [units[i] for i in plan[rank]]
    ms = 0.0
    for s, b, _ in mine:
        ms += process(s, b)
    total, tmax = combine(sum(u[2] for u in mine), ms)
    return [(s, b) for s, b, _ in mine], total, tmax
