"""Scenario sharding across GPUs: one process per GPU, replicas of the
topology, no collective inside the Newton loop.

Scenarios are independent (the reference runs them as an embarrassingly
parallel rayon work queue, src/batch.rs:230-281), so N processes each solve
a contiguous, balanced block of the batch on their own GPU with their own
copy of the topology's factorization schedule; the only communication is
the host gather of the per-scenario reports at the end and the max of the
ranks' timings.  Works with any torch.distributed backend (NCCL on GPU
boxes, gloo for the CPU tests).
"""
from __future__ import annotations

from typing import Callable, Optional

import numpy as np


def shard_bounds(n_scen: int, world: int, rank: int) -> tuple[int, int]:
    """[lo, hi) of the scenarios rank `rank` of `world` solves: contiguous
    blocks whose sizes differ by at most one, earlier ranks larger."""
    if world <= 0 or not (0 <= rank < world) or n_scen < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n_scen, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _rows(a, lo, hi):
    a = np.asarray(a)
    return a[lo:hi] if a.ndim == 2 else a


REPORT_KEYS = ("vm", "va", "iters", "status", "max_mismatch")


def solve_replicas(solve: Callable[..., dict], p_spec, q_spec, vm0, va0, outage=None,
                   group=None, **kw) -> dict:
    """Solves this rank's shard with `solve(p, q, vm0, va0, outage=..., **kw)`
    (a dict with the REPORT_KEYS arrays, e.g. Topology.solve via
    report_dict) and gathers every rank's reports in scenario order, on
    every rank.  Without an initialised process group it solves everything
    locally."""
    import torch.distributed as dist

    p_spec = np.atleast_2d(np.asarray(p_spec))
    q_spec = np.atleast_2d(np.asarray(q_spec))
    B = p_spec.shape[0]
    if dist.is_available() and dist.is_initialized():
        world, rank = dist.get_world_size(group), dist.get_rank(group)
    else:
        world, rank = 1, 0
    lo, hi = shard_bounds(B, world, rank)
    out_local = None
    if outage is not None:
        out_local = tuple(np.asarray(o)[lo:hi] for o in outage)
    if hi > lo:
        mine = solve(p_spec[lo:hi], q_spec[lo:hi], _rows(vm0, lo, hi), _rows(va0, lo, hi),
                     outage=out_local, **kw)
        mine = {k: np.asarray(mine[k]) for k in REPORT_KEYS}
    else:
        mine = None
    if world == 1:
        return mine
    parts = [None] * world
    dist.all_gather_object(parts, (lo, hi, mine), group=group)
    parts.sort(key=lambda t: t[0])
    got = [m for (_, _, m) in parts if m is not None]
    return {k: np.concatenate([m[k] for m in got], axis=0) for k in REPORT_KEYS}


def max_over_ranks(value_ms: float, group=None) -> float:
    """The largest of the ranks' timings (a run is as slow as its slowest
    GPU)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value_ms)
    t = torch.tensor([float(value_ms)], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def report_dict(res) -> dict:
    """The REPORT_KEYS view of a solver.BatchResult."""
    return {"vm": res.voltage_mag, "va": res.voltage_ang, "iters": res.iterations,
            "status": res.status, "max_mismatch": res.max_mismatch}


def topology_solver(topology, precision: Optional[int] = None) -> Callable[..., dict]:
    """`solve` for solve_replicas backed by a GPU Topology."""
    def _solve(p, q, vm0, va0, outage=None, **kw):
        if precision is not None:
            kw.setdefault("precision", precision)
        return report_dict(topology.solve(p, q, vm0, va0, outage=outage, **kw))
    return _solve
