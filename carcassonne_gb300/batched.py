"""Many independent center-site problems of uneven shape on one GPU.

Each problem's H_eff is a Stage3Operator applied to a block of Lanczos vectors
on the tensor cores.  Three ways to run a batch of them are provided:

* ``run_loop``   one operator application per problem from the host, in turn
                 (the per-problem launch loop);
* ``capture`` / ``replay``  the same launch sequence captured once into a
                 CUDA graph and replayed as one unit: no host work per kernel;
* ``autotune``   per problem shape, the tensor-core matvec's path (the
                 compact-operand fused kernel, the first fused kernel, or the
                 two-kernel path with a step-B split-K count) is chosen by
                 timing candidates with CUDA events and stored in the
                 library's autotune cache (carc_tc_autotune_set), which every
                 later launch and capture of that shape uses; the choices are
                 kept in a JSON file (``load_tuning`` / ``save_tuning``) so a
                 later process applies them without re-timing;
* ``run_solves`` the configured solve workload: Hermitian-definite problems
                 (``sample_pencils``), each solved to its lowest eigenpair by
                 the batched block eigensolver (``blocksolve``), all problems
                 of a memory chunk at once against the per-problem loop.

Problems are built and processed in chunks that fit a device-memory budget,
so that a distribution with large members (D=6, chi=96: about 2 GB of stage-2
tensors and packed operands each) never overcommits HBM.
"""
from __future__ import annotations

import json
import os
import time

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


TUNE_CANDIDATES = (0, -1, 76, 114, 152, 228, 304)


def _tune_key(op, g, nvec):
    return dict(s0=[int(v) for v in g["shape0"]], s1=[int(v) for v in g["shape1"]], d=op.d, nvec=nvec,
                groups=_groups_of(g))


def _set_tuning(key, ks, fold=0):
    lib = _lib.load()
    s0, keep0 = _lib.i64_array(key["s0"])
    s1, keep1 = _lib.i64_array(key["s1"])
    _lib.check(lib.carc_tc_autotune_set(s0, s1, key["d"], key["nvec"], key["groups"], int(ks)))
    _lib.check(lib.carc_tc_autotune_set_fold(s0, s1, key["d"], key["nvec"], key["groups"], int(fold)))
    del keep0, keep1


def autotune(op, nvec, candidates=TUNE_CANDIDATES, reps=3):
    """Time the tensor-core matvec of one operator for each path candidate
    (0: the default choice, the compact-operand fused kernel where it takes
    the shape; -1: the first fused kernel where it takes the shape; > 0: the
    two-kernel path with that step-B split-K count), then, where the two-kernel
    path wins, its step-A folding GEMM in the second tile configuration (two
    CTAs per SM, 128-column tiles, two stages); keep the fastest in the
    library's autotune cache.  Returns one entry per term-group shape."""
    x = torch.zeros((nvec,) + op.in_shape, dtype=CDT, device="cuda")
    y = torch.empty((nvec,) + op.out_shape, dtype=CDT, device="cuda")
    results = []
    for g in op._groups:
        key = _tune_key(op, g, nvec)
        times = {}
        for ks in candidates:
            _set_tuning(key, ks)
            times[ks] = _time(lambda: op.apply_tc(x, y, nvec), reps)
        best = min(times, key=times.get)
        fold, fold_ms = 0, None
        if best >= 0:  # the two-kernel path (best > 0), or possibly the default (a shape no fused kernel takes)
            _set_tuning(key, best, 1)
            fold_ms = _time(lambda: op.apply_tc(x, y, nvec), reps)
            if fold_ms < 0.97 * times[best]:  # a margin above timing noise
                fold = 1
        _set_tuning(key, best, fold)
        results.append(dict(key, best=int(best), fold=fold, ms={str(k): round(v, 5) for k, v in times.items()},
                            fold_ms=None if fold_ms is None else round(fold_ms, 5)))
    op.check_status()
    return results


def default_tuning_file():
    """Where the autotune choices are kept: $CARC_TUNE_FILE, else a file in
    the package directory (not under version control)."""
    return os.environ.get("CARC_TUNE_FILE") or os.path.join(os.path.dirname(os.path.abspath(__file__)), ".autotune",
                                                            "stage3_tc.json")


def load_tuning(path=None):
    """Apply the choices of a tuning file to the library's cache; returns the
    entries (empty when the file does not exist)."""
    path = path or default_tuning_file()
    if not os.path.exists(path):
        return []
    with open(path) as f:
        entries = json.load(f)["entries"]
    for e in entries:
        _set_tuning(e, e["best"], e.get("fold", 0))
    return entries


def save_tuning(entries, path=None):
    path = path or default_tuning_file()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    seen, out = set(), []
    for e in entries:
        k = json.dumps({f: e[f] for f in ("s0", "s1", "d", "nvec", "groups")}, sort_keys=True)
        if k not in seen:
            seen.add(k)
            out.append(e)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump({"device": torch.cuda.get_device_name(0) if torch.cuda.is_available() else None,
                   "entries": out}, f, indent=1)
    os.replace(tmp, path)
    return path


def _tune_missing(ops, nvec, entries):
    """Autotune the shapes of ``ops`` that ``entries`` lacks; returns the new entries."""
    have = {json.dumps({f: e[f] for f in ("s0", "s1", "d", "nvec", "groups")}, sort_keys=True) for e in entries}
    new = []
    for op in ops:
        keys = [json.dumps(_tune_key(op, g, nvec), sort_keys=True) for g in op._groups]
        if all(k in have for k in keys):
            continue
        for e in autotune(op, nvec):
            have.add(json.dumps({f: e[f] for f in ("s0", "s1", "d", "nvec", "groups")}, sort_keys=True))
            new.append(e)
    return new


def run(count=32, nvec=8, seed=3, mem_budget=24 << 30, reps=3, tune=True, tune_file=None):
    """Build `count` problems of the distribution in memory-bounded chunks; per
    chunk, autotune each new shape (choices read from and added to the tuning
    file), time the per-problem launch loop and the graph replay.  Returns
    the aggregate figures."""
    specs = sample_problems(count, seed)
    totals = dict(flops=0.0, loop_ms=0.0, graph_ms=0.0, problems=0, chunks=0)
    entries = load_tuning(tune_file) if tune else []
    loaded = len(entries)
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
            entries += _tune_missing(ops, nvec, entries)
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
    if tune and len(entries) > loaded:
        save_tuning(entries, tune_file)
    totals["loop_gflops"] = totals["flops"] / (totals["loop_ms"] * 1e-3) / 1e9
    totals["graph_gflops"] = totals["flops"] / (totals["graph_ms"] * 1e-3) / 1e9
    totals["graph_speedup"] = totals["loop_ms"] / totals["graph_ms"]
    totals["autotuned_shapes"] = len(entries)
    totals["autotune_loaded_from_file"] = loaded
    totals["autotune_choices"] = sorted({e["best"] for e in entries})
    return totals


# -- the solve workload ----------------------------------------------------------
def pencil_c(chi):
    """Layer dimension of a Hermitian-definite problem drawn with boundary
    dimension chi: ket and bra layers of equal dimension c, so chi is rounded
    to the nearest square c^2 (c = 4..10 for chi = 16..96)."""
    return int(np.floor(np.sqrt(chi) + 0.5))


def sample_pencils(count, seed=3, D_choices=(2, 3, 4, 5, 6), chi_choices=tuple(range(16, 97, 8)), h_range=(2.0, 4.0)):
    """(D, c, h, seed) of each Hermitian-definite problem: D, chi and h drawn
    uniformly as in the batched matvec workload, chi then rounded to the
    nearest square c^2 (every physical double-layer boundary has ket and bra
    layers of equal dimension c)."""
    rng = np.random.default_rng(seed)
    return [(int(rng.choice(D_choices)), pencil_c(int(rng.choice(chi_choices))), float(rng.uniform(*h_range)),
             seed * 100003 + i) for i in range(count)]


def build_pencil(D, c, h, seed):
    """The transverse-Ising (H_eff, N_eff) operators of one Hermitian-definite
    problem (stage-2 tensors built on the device)."""
    ca, sa, oa = workloads.hermitian_problem_arrays(D=D, c=c, seed=seed, op_arrays=workloads.ti_operator_arrays(h=h))
    corners, sides, op = workloads.to_device(ca, sa, oa)
    H, N = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    return H.operator, N.operator


def run_solves(count=256, m=8, seed=3, tol=1e-4, mem_budget=48 << 30, tune=True, tune_file=None, loop=True,
               max_iter=150, specs=None, return_problems=False):
    """The batched-solve workload: `count` problems from ``sample_pencils``
    (or the given ``specs``), built in memory-bounded chunks; per chunk all
    problems are solved at once by the batched block eigensolver and then
    (``loop``) one at a time by the same solver, the per-problem loop.  Each
    problem's start block is seeded by its own seed, so a problem's result
    does not depend on the chunk or rank that solves it.  Returns the
    aggregate throughput of both, per-D figures, iteration counts and the
    agreement of the two runs (with ``return_problems``, also every problem's
    energy and iteration count in ``specs`` order)."""
    from . import blocksolve
    specs = sample_pencils(count, seed) if specs is None else list(specs)
    energies, iter_list = [None] * len(specs), [None] * len(specs)
    entries = load_tuning(tune_file) if tune else []
    loaded = len(entries)
    tot = dict(problems=0, chunks=0, batched_s=0.0, loop_s=0.0, build_s=0.0, flops=0.0, iterations=[],
               converged=0, max_energy_diff=0.0, iterations_equal=True, max_verify_residual=0.0, per_D={})
    pending = list(enumerate(specs))
    while pending:
        chunk, used = [], 0
        t0 = time.perf_counter()
        while pending:
            i, (D, c, h, s) = pending[0]
            Hop, Nop = build_pencil(D, c, h, s)
            nb = operator_bytes(Hop) + operator_bytes(Nop)
            if chunk and used + nb > mem_budget:
                Hop = Nop = None
                break
            pending.pop(0)
            chunk.append((i, D, (Hop, Nop)))
            used += nb
            Hop = Nop = None
        if tune:
            entries += _tune_missing([p[0] for _, _, p in chunk] + [p[1] for _, _, p in chunk], m, entries)
        torch.cuda.synchronize()
        tot["build_s"] += time.perf_counter() - t0
        probs = [p for _, _, p in chunk]
        seeds = [specs[i][3] + 1 for i, _, _ in chunk]
        solver = blocksolve.BlockEigensolver(probs, m)
        rb = solver.solve(seeds, tol=tol, max_iter=max_iter)
        ver = solver.verify()
        del solver
        tot["batched_s"] += rb["seconds"]
        tot["flops"] += rb["matvec_flops"]
        tot["iterations"] += [int(v) for v in rb["iterations"]]
        tot["converged"] += int(rb["converged"].sum())
        tot["max_verify_residual"] = max(tot["max_verify_residual"], max(r for _, r in ver))
        if loop:
            rl = blocksolve.solve_each(probs, seeds, m, tol=tol, max_iter=max_iter)
            tot["loop_s"] += rl["seconds"]
            diff = np.abs(rl["energy"] - rb["energy"]) / np.maximum(np.abs(rb["energy"]), 1e-300)
            tot["max_energy_diff"] = max(tot["max_energy_diff"], float(diff.max()))
            tot["iterations_equal"] &= bool(np.array_equal(rl["iterations"], rb["iterations"]))
        for j, (i, D, (Hop, _)) in enumerate(chunk):
            energies[i], iter_list[i] = float(rb["energy"][j]), int(rb["iterations"][j])
            pd = tot["per_D"].setdefault(str(D), dict(problems=0, iterations=0, flops=0.0))
            pd["problems"] += 1
            pd["iterations"] += int(rb["iterations"][j])
        tot["problems"] += len(chunk)
        tot["chunks"] += 1
        del probs, chunk
        torch.cuda.empty_cache()
    if tune and len(entries) > loaded:
        save_tuning(entries, tune_file)
    it = np.asarray(tot.pop("iterations"))
    out = dict(problems=tot["problems"], chunks=tot["chunks"], block=m, tol=tol,
               converged=tot["converged"], iterations_mean=float(it.mean()), iterations_max=int(it.max()),
               batched_seconds=tot["batched_s"], batched_solves_per_s=tot["problems"] / tot["batched_s"],
               matvec_gflops_batched=tot["flops"] / tot["batched_s"] / 1e9,
               max_verify_residual=tot["max_verify_residual"], build_seconds=tot["build_s"],
               autotuned_shapes=len(entries), autotune_loaded_from_file=loaded,
               per_D={k: dict(problems=v["problems"], iterations_mean=v["iterations"] / v["problems"])
                      for k, v in sorted(tot["per_D"].items())})
    if loop:
        out.update(loop_seconds=tot["loop_s"], loop_solves_per_s=tot["problems"] / tot["loop_s"],
                   batched_over_loop=tot["loop_s"] / tot["batched_s"],
                   max_energy_diff_batched_vs_loop=tot["max_energy_diff"],
                   iterations_equal_batched_vs_loop=tot["iterations_equal"])
    if return_problems:
        out.update(energy=energies, iterations=iter_list, seconds=tot["batched_s"])
    return out


def pencil_cost(spec, m=8):
    """Sharding key of a ``sample_pencils`` problem: the CostTracker count of
    one block matvec of its H_eff (chi = c^2)."""
    from .replicas import problem_cost
    D, c = spec[0], spec[1]
    return problem_cost(D, c * c, nvec=m)


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
    p.add_argument("--fold", type=int, default=0, choices=[0, 1],
                   help="step A's folding-GEMM configuration on the two-kernel path (1: two CTAs per SM)")
    p.add_argument("--reps", type=int, default=3)
    a = p.parse_args(argv)
    lib = _lib.load()
    op = build_operator(a.D, a.chi, a.h, a.seed)
    x = torch.zeros((a.nvec,) + op.in_shape, dtype=CDT, device="cuda")
    y = torch.empty((a.nvec,) + op.out_shape, dtype=CDT, device="cuda")
    if a.ksplit > 0:
        for g in op._groups:
            _lib.check(lib.carc_tc_autotune_set(g["s0"], g["s1"], op.d, a.nvec, _groups_of(g), a.ksplit))
            _lib.check(lib.carc_tc_autotune_set_fold(g["s0"], g["s1"], op.d, a.nvec, _groups_of(g), a.fold))
    try:
        for _ in range(a.reps):
            op.apply_tc(x, y, a.nvec)
        torch.cuda.synchronize()
        op.check_status()
    finally:
        if a.ksplit > 0:
            _lib.check(lib.carc_tc_autotune_clear())
    print("ok")


__all__ = ["sample_problems", "build_operator", "operator_bytes", "Batch", "autotune", "run", "CHI_FACTORS", "main",
           "TUNE_CANDIDATES", "load_tuning", "save_tuning", "default_tuning_file", "sample_pencils", "build_pencil",
           "run_solves", "pencil_cost", "pencil_c"]

if __name__ == "__main__":
    main()
