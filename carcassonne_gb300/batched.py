"""Many independent center-site problems of uneven shape on one GPU.

Each problem's H_eff is a Stage3Operator applied to a block of Lanczos vectors
on the tensor cores.  Three ways to run a batch of them are provided:

* ``run_loop``   one operator application per problem from the host, in turn
                 (the per-problem launch loop);
* ``capture`` / ``replay``  the same launch sequence captured once into a
                 CUDA graph and replayed as one unit: no host work per kernel;
* ``autotune``   per problem shape, the step-B split-K count of the tensor-core
                 matvec is chosen by timing candidates with CUDA events and
                 stored in the library's autotune cache (carc_tc_autotune_set),
                 which every later launch and capture of that shape uses.

Problems are built and processed in chunks that fit a device-memory budget,
so that a distribution with large members (D=6, chi=96: about 2 GB of stage-2
tensors and packed operands each) never overcommits HBM.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, workloads
from .engine import CDT
from .tensors._2d import sparse as tsp

# chi -> (c_ket, c_bra), chi = c_ket * c_bra
CHI_FACTORS = {16: (4, 4), 24: (6, 4), 32: (8, 4), 40: (8, 5), 48: (8, 6), 56: (8, 7), 64: (8, 8), 72: (9, 8),
               80: (10, 8), 88: (11, 8), 96: (12, 8)}


def sample_problems(count, seed=3, D_choices=(2, 3, 4, 5, 6), chi_choices=tuple(range(16, 97, 8)), h_range=(2.0, 4.0)):
    """(D, chi, h, seed) of each problem: D, chi and h drawn uniformly."""
    rng = np.random.default_rng(seed)
    return [(int(rng.choice(D_choices)), int(rng.choice(chi_choices)), float(rng.uniform(*h_range)), seed * 100003 + i)
            for i in range(count)]


def build_operator(D, chi, h, seed):
    """The transverse-Ising H_eff of one problem (stage-2 tensors built on the device)."""
    ck, cb = CHI_FACTORS[chi]
    ca, sa, oa = workloads.matvec_problem_arrays(D=D, c_ket=ck, c_bra=cb, seed=seed,
                                                 op_arrays=workloads.ti_operator_arrays(h=h))
    corners, sides, op = workloads.to_device(ca, sa, oa)
    H, _ = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    return H.operator


def operator_bytes(op):
    """Device bytes of an operator's stage-2 tensors and packed tensor-core plans."""
    b = sum(t.numel() * t.element_size() for t in op.s2_0 + op.s2_1)
    lib = _lib.load()
    for g in op._groups:
        b += max(lib.carc_stage3_tc_plan_size(g["s0"], g["s1"], g["pt"], len(g["terms"])), 0)
    return b


def _groups_of(g):
    return len({t[1] for t in g["terms"]})


class Batch:
    """A chunk of operators with their Lanczos blocks resident on the device."""

    def __init__(self, ops, nvec=8, seed=0):
        self.ops = ops
        self.nvec = nvec
        g = torch.Generator().manual_seed(seed)
        self.x = [torch.complex(torch.randn((nvec,) + op.in_shape, generator=g, dtype=torch.float64),
                                torch.randn((nvec,) + op.in_shape, generator=g, dtype=torch.float64)).cuda()
                  for op in ops]
        self.y = [torch.empty((nvec,) + op.out_shape, dtype=CDT, device="cuda") for op in ops]
        self.graph = None

    def flops(self):
        return sum(op.cost_of_multiply() * 8 * self.nvec for op in self.ops)

    def run_loop(self):
        for op, x, y in zip(self.ops, self.x, self.y):
            op.apply_tc(x, y, self.nvec)

    def capture(self):
        """Warm up (plans, workspaces at their largest), then capture the
        whole launch sequence into one CUDA graph."""
        self.run_loop()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run_loop()
        s.synchronize()
        with torch.cuda.graph(self.graph, stream=s):
            self.run_loop()
        torch.cuda.synchronize()

    def replay(self):
        self.graph.replay()

    def check_status(self):
        for op in self.ops:
            op.check_status()


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def autotune(op, nvec, candidates=(0, 76, 114, 152, 228, 304), reps=3):
    """Time the tensor-core matvec of one operator for each step-B split-K
    candidate (0 = the one-wave heuristic) and keep the fastest in the
    library's autotune cache; returns {candidate: ms} and the choice."""
    lib = _lib.load()
    x = torch.zeros((nvec,) + op.in_shape, dtype=CDT, device="cuda")
    y = torch.empty((nvec,) + op.out_shape, dtype=CDT, device="cuda")
    results = {}
    for g in op._groups:
        key = (g["s0"], g["s1"], op.d, nvec, _groups_of(g))
        times = {}
        for ks in candidates:
            _lib.check(lib.carc_tc_autotune_set(key[0], key[1], key[2], nvec, key[4], ks))
            times[ks] = _time(lambda: op.apply_tc(x, y, nvec), reps)
        best = min(times, key=times.get)
        _lib.check(lib.carc_tc_autotune_set(key[0], key[1], key[2], nvec, key[4], best))
        results[(tuple(g["shape0"]), tuple(g["shape1"]), key[4])] = dict(ms=times, best=best)
    op.check_status()
    return results


def run(count=32, nvec=8, seed=3, mem_budget=24 << 30, reps=3, tune=True):
    """Build `count` problems of the distribution in memory-bounded chunks; per
    chunk, autotune each new shape, time the per-problem launch loop and the
    graph replay.  Returns the aggregate figures."""
    specs = sample_problems(count, seed)
    totals = dict(flops=0.0, loop_ms=0.0, graph_ms=0.0, problems=0, chunks=0)
    tuned = {}
    pending = list(specs)
    while pending:
        ops, used = [], 0
        while pending:
            D, chi, h, s = pending[0]
            op = build_operator(D, chi, h, s)
            nb = operator_bytes(op)
            if ops and used + nb > mem_budget:
                op = None
                break
            pending.pop(0)
            ops.append(op)
            used += nb
            op = None
        if tune:
            for op in ops:
                k = (op.s0_shape, op.s1_shape, len(op.terms))
                if k not in tuned:
                    tuned[k] = autotune(op, nvec)
            op = None
        batch = Batch(ops, nvec)
        batch.capture()
        totals["loop_ms"] += _time(batch.run_loop, reps)
        totals["graph_ms"] += _time(batch.replay, reps)
        batch.check_status()
        totals["flops"] += batch.flops()
        totals["problems"] += len(ops)
        totals["chunks"] += 1
        del batch, ops
        torch.cuda.empty_cache()
    totals["loop_gflops"] = totals["flops"] / (totals["loop_ms"] * 1e-3) / 1e9
    totals["graph_gflops"] = totals["flops"] / (totals["graph_ms"] * 1e-3) / 1e9
    totals["graph_speedup"] = totals["loop_ms"] / totals["graph_ms"]
    totals["autotuned_shapes"] = len(tuned)
    totals["autotune_choices"] = sorted({v["best"] for r in tuned.values() for v in r.values()})
    return totals


def main(argv=None):
    """Apply one problem's H_eff (transverse Ising, as in the batched
    workload) to a block of centers a few times: on the path the autotune
    cache or the eligibility rule picks, or with ``--ksplit K`` on the
    two-kernel path with step B split K ways.  A small self-contained case for
    timing or profiling one shape."""
    import argparse
    p = argparse.ArgumentParser(prog="python -m carcassonne_gb300.batched")
    p.add_argument("--D", type=int, default=5)
    p.add_argument("--chi", type=int, default=56, choices=sorted(CHI_FACTORS))
    p.add_argument("--h", type=float, default=3.0)
    p.add_argument("--seed", type=int, default=11)
    p.add_argument("--nvec", type=int, default=8)
    p.add_argument("--ksplit", type=int, default=0, help="> 0: pin the two-kernel path with this step-B split")
    p.add_argument("--reps", type=int, default=3)
    a = p.parse_args(argv)
    lib = _lib.load()
    op = build_operator(a.D, a.chi, a.h, a.seed)
    x = torch.zeros((a.nvec,) + op.in_shape, dtype=CDT, device="cuda")
    y = torch.empty((a.nvec,) + op.out_shape, dtype=CDT, device="cuda")
    if a.ksplit > 0:
        for g in op._groups:
            _lib.check(lib.carc_tc_autotune_set(g["s0"], g["s1"], op.d, a.nvec, _groups_of(g), a.ksplit))
    try:
        for _ in range(a.reps):
            op.apply_tc(x, y, a.nvec)
        torch.cuda.synchronize()
        op.check_status()
    finally:
        if a.ksplit > 0:
            _lib.check(lib.carc_tc_autotune_clear())
    print("ok")


__all__ = ["sample_problems", "build_operator", "operator_bytes", "Batch", "autotune", "run", "CHI_FACTORS", "main"]

if __name__ == "__main__":
    main()
