"""Several GPUs on independent center-site problems (no data-path
collective): a single problem's matvec is too small to split, so one GPU per
process runs whole problems.  Batches of independent problems are sharded
across ranks by estimated cost (the CostTracker count of one matvec), each
rank solves its shard (``run_sharded``), and the host combines per-rank
timings and results with small control-plane collectives (any
torch.distributed backend: NCCL on GPUs, gloo in the CPU tests).
"""
from __future__ import annotations

import heapq


def shard_by_cost(costs, world):
    """Assign problem indices to `world` ranks, largest cost first, each to the
    rank with the least total so far (ties to the lower rank): a
    deterministic longest-processing-time schedule.  Returns one ascending
    index list per rank."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    heap = [(0, r) for r in range(world)]
    shards = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(s) for s in shards]


def problem_cost(D, chi, terms=9, d=2, nvec=8):
    """CostTracker complex MACs of one block matvec of a (D, chi) center-site
    problem: terms x 2 chi^2 D^6 d per vector."""
    return terms * 2 * chi * chi * D ** 6 * d * nvec


def max_over_ranks(values, dist=None, device=None):
    """Element-wise maximum of a list of floats over all ranks (the slowest
    rank sets a whole-job time); identity without a process group."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def gather_to_root(obj, dist=None, rank=0, world=1):
    """Every rank's object on rank 0 (in rank order); None elsewhere."""
    if dist is None:
        return [obj]
    out = [None] * world if rank == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def run_sharded(specs, cost_of, solve_fn, dist=None, rank=0, world=1, device=None):
    """The sharded batch: this rank takes ``shard_by_cost`` of the problems'
    costs and solves its shard with ``solve_fn(list of specs)``, which
    returns ``dict(energy=[...], iterations=[...], seconds=s)`` in shard
    order; the slowest rank's seconds set the whole-job time.  Rank 0 gets
    every problem's results in the original order, the per-rank loads and
    the whole-job throughput; the other ranks get None."""
    costs = [cost_of(s) for s in specs]
    mine = shard_by_cost(costs, world)[rank]
    if mine:
        res = solve_fn([specs[i] for i in mine])
    else:
        res = dict(energy=[], iterations=[], seconds=0.0)
    seconds = max_over_ranks([res["seconds"]], dist, device)[0]
    part = dict(rank=rank, idx=list(mine), energy=[float(e) for e in res["energy"]],
                iterations=[int(v) for v in res["iterations"]], seconds=float(res["seconds"]),
                cost=sum(costs[i] for i in mine))
    got = gather_to_root(part, dist, rank, world)
    if got is None:
        return None
    n = len(specs)
    energy, iterations = [None] * n, [None] * n
    for g in got:
        for j, i in enumerate(g["idx"]):
            energy[i], iterations[i] = g["energy"][j], g["iterations"][j]
    return dict(problems=n, ranks=world, seconds=seconds, solves_per_s=n / seconds if seconds > 0 else None,
                energy=energy, iterations=iterations,
                per_rank=[dict(rank=g["rank"], problems=len(g["idx"]), seconds=g["seconds"], cost=g["cost"])
                          for g in got])


__all__ = ["shard_by_cost", "problem_cost", "max_over_ranks", "gather_to_root", "run_sharded"]
