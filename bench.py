#!/usr/bin/env python
"""Benchmark of the center-site matvec (stage-3 operator application).

Workload (the center-site matvec microbenchmark): transverse-field Ising
operator center (d=2, 6 tags), boundaries grown one absorption round
(corners 4 tags, sides 5 tags -> 9 stage-3 terms), state bond D=4, merged
boundary dimension chi=32 (8 ket x 4 bra), entries i.i.d. N(0,1) (seed 1)
scaled to unit Frobenius norm.  One step applies the full expectation
operator H_eff to a block of ``--nvec`` centers of shape (D,D,D,D,d).

value: GFLOP/s of algorithmic work (the reference's CostTracker count of
complex MACs x 8 real flops) with inputs resident in HBM, L2 flushed
between timed steps; e2e: the same metric with the block in pinned host
memory and the result returned to pinned host memory inside the timed
region -- the kernel reads and writes host memory mapped into the device's
address space (NVLink-C2C); the figure with a copy each way
(cudaMemcpyAsync) is reported beside it.
``--impl reference`` times the CPU restatement of the reference's path on
the host cores (the reference itself is pure Python/NumPy and is not
available on the GPU host) for ``--warmup`` untimed and ``--steps`` timed
steps of the same block, rank 0 only.  Under torchrun (N > 1) every rank runs
its own replica of the workload with no data-path collective; the slowest
rank's time sets the whole-job value.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="center-site matvec, TI d=2 (9 terms), D=4, chi=32 (8x4)", D=4, chi=32, c_ket=8,
                c_bra=4, d=2, terms=9, seed=1)
METRIC = "center-site matvec GFLOP/s (CostTracker algorithmic flops), 1 GB300"
UNIT = "GFLOP/s"
L2_FLUSH_BYTES = 512 << 20

# full center-site solve, mixed vs plain FP64 (Heisenberg XXX term structure,
# D=4, chi=64 = 8x8, Hermitian-definite synthetic boundaries, seed 2)
SOLVE = dict(workload="center-site solve, Heisenberg XXX d=2, D=4, chi=64 (8x8)", D=4, c=8, seed=2, reps=3)

# batched uneven problems: transverse Ising, h ~ U[2,4], D ~ U{2..6},
# chi ~ U{16,24,..,96}, a block of 8 vectors each, seed 3
BATCHED = dict(workload="batched center-site matvecs, TI, D in 2..6, chi in 16..96, block 8", nvec=8, seed=3)
# batched solves: Hermitian-definite transverse-Ising problems (ket x bra
# boundary layers of equal dimension c: the drawn chi rounded to the nearest
# square c^2), lowest eigenpair of each by the batched block eigensolver
# (LOBPCG, block 8) to relative residual 1e-4
BATCHED_SOLVES = dict(workload="batched center solves, TI, h in [2,4], D in 2..6, chi in 16..96 rounded to the "
                               "nearest square c^2 (c = 4..10), LOBPCG block 8, relative residual 1e-4", block=8,
                      seed=3, tol=1e-4)

# phases of the tensor-core operator, as numbered by carc_phase_timing_read
PHASE_NAMES = ("pack", "step_a", "step_b", "reduce")
KERNEL_OF_PHASE = dict(pack="pack_vin_kernel", step_a="gemm_bf16_tn_kernel<256,1> (folding epilogue)",
                       step_b="gemm_bf16_tn_kernel<256,0> (split-K)", reduce="reduce_planes_kernel",
                       fused="stage3_fused_kernel (one cooperative launch: Vin packing, step A + fold + step B "
                             "with W on chip, plane reduction)",
                       fused2="stage3_fused2_kernel (one cooperative launch on compact operands: Vin packing, step A "
                              "with hi+lo summed in TMEM, fold to W^T in shared memory, transposed step B, plane "
                              "reduction)")
# DRAM bytes (read + write) per launch from one ncu capture of this workload
# (profiles/ holds the summary and the command that produced it)
NCU_TRAFFIC = {
    ("center-site matvec, TI d=2 (9 terms), D=4, chi=32 (8x4)", "fused2"): dict(
        bytes_per_launch=63.65e6,
        source="profiles/stage3_fused2_matvec_D4_chi32_nvec8.md: one cooperative launch of the compact-operand "
               "kernel, dram read 63.08 MB + write 0.56 MB"),
    ("center-site matvec, TI d=2 (9 terms), D=4, chi=32 (8x4)", "fused"): dict(
        bytes_per_launch=129.9e6,
        source="profiles/stage3_fused_matvec_D4_chi32_nvec8.md: one cooperative fused launch (packing, both "
               "steps, plane reduction), dram read 126.1 MB + write 3.9 MB"),
    ("center-site matvec, TI d=2 (9 terms), D=4, chi=32 (8x4)", "step_a"): dict(
        bytes_per_launch=8.97e6,
        source="profiles/stage3_tc_matvec_D4_chi32_nvec8.md: one step-A launch (1-term group, 41.9 MB "
               "algorithmic), dram read 8.46 MB + write 0.51 MB; the W it writes is still in L2 at kernel exit"),
}


def _round_up(a, b):
    return (a + b - 1) // b * b


def _pad_b_rows(n):
    """Padded rows of step A's B operand, Vin (one power-of-two N tile up to
    256, whole 256-row tiles above), as the library pads them."""
    if n > 256:
        return _round_up(n, 256)
    t = 16
    while t < n:
        t *= 2
    return t


def _gemm_pad_n(n):
    """Padded rows of W, step B's B operand: ceil(n / 256) equal N tiles of
    a multiple of 16, as the library pads it."""
    nt = -(-n // 256)
    return nt * _round_up(-(-n // nt), 16)


def _gemm_tile_n(n):
    """The N tile the plain tensor-core GEMM takes for a B operand of n rows."""
    nt = -(-n // 256)
    if n % nt == 0 and (n // nt) % 16 == 0:
        return n // nt
    return next(b for b in (256, 128, 64, 32, 16) if n % b == 0)


def tc_bytes_per_step(opr, nvec):
    """Algorithmic bytes each tensor-core phase must move per operator
    application, from the packed split-BF16 operand geometry: step A reads
    the packed S2_0 tags of its terms (4 bf16 rows x 4K columns per complex
    row, 2 bytes each) and the packed Vin, and writes W; step B reads the live
    rows of the packed S2_1 tags and W and writes its FP32 split planes."""
    out = dict(step_a=0, step_b=0, launches=dict(step_a=0, step_b=0))
    for g in opr._groups:
        x0, x1, k0, k1, l0, l1 = g["shape0"]
        _, _, k2, k3, l2, l3 = g["shape1"]
        d = opr.d
        terms = g["terms"]
        groups = sorted({t[1] for t in terms})
        nt = len(terms)
        rows_a = _round_up(4 * x0 * x1 * l0 * l1, 128)
        reg_a = _round_up(4 * k0 * k1, 64)
        rows_vin = _pad_b_rows(nvec * k2 * k3 * d)
        reg_b = _round_up(4 * x0 * x1 * k2 * k3, 64)
        rows_w = _gemm_pad_n(nvec * l0 * l1 * d)
        kp_b = reg_b * len(groups)
        out["step_a"] += 2 * (rows_a * reg_a * nt + rows_vin * reg_a * nt + rows_w * kp_b)
        out["launches"]["step_a"] += len(groups)
        live_b = 4 * l2 * l3
        rows_sb = _round_up(live_b, 128)
        bn = _gemm_tile_n(rows_w)
        tiles = (rows_sb // 128) * (rows_w // bn)
        kb = kp_b // 64
        ks_b = max(1, min(1 if tiles >= 152 else 152 // tiles, kb))
        kb_per = -(-kb // ks_b)
        ks_b = -(-kb // kb_per)
        live_rows = live_b if rows_sb == 128 and live_b <= 64 else rows_sb
        out["step_b"] += 2 * (live_rows * kp_b + rows_w * kp_b) + 4 * ks_b * rows_sb * rows_w
        out["launches"]["step_b"] += 1
        # the fused kernel (W on chip): packed S2_0 and Vin of every term, the
        # live rows of the packed S2_1 tags, one FP32 plane of the live rows
        # (rounded to 32) per CTA
        units = (x0 * x1 * l0 * l1 // 32) * len(groups)
        grid = max(1, min(152, units))
        out["fused"] = out.get("fused", 0) + 2 * (rows_a * reg_a * nt + rows_vin * reg_a * nt + live_rows * kp_b) \
            + 4 * grid * _round_up(live_b, 32) * nvec * l0 * l1 * d
        out["launches"]["fused"] = out["launches"].get("fused", 0) + 1
        # the compact-operand kernel: S2_0 as (re/im rows) x 64 columns per term,
        # S2_1 as (j, re/im) rows x [hi | lo] planes per tag, Vin per term, and
        # one FP32 plane (VH x NBB x 128) per CTA written and read back
        f2 = _f2_geo(g, nvec, d)
        if f2:
            vh, nah, nbb = f2
            ma = x0 * x1 * l0 * l1
            kcb = x0 * x1 * k2 * k3
            grid2 = max(1, min(152, ma // 64 * len(groups)))
            out["fused2"] = out.get("fused2", 0) + 2 * (2 * ma * 64 * nt + nbb * 4 * kcb * len(groups)
                                                        + vh * nah * 64 * nt) + 2 * 4 * grid2 * vh * nbb * 128
            out["launches"]["fused2"] = out["launches"].get("fused2", 0) + 1
    return out


def _f2_geo(g, nvec, d):
    """(VH, NAh, NBB) of the compact-operand fused kernel for one S2 shape
    group, or None where the library takes another path (its f2_geo)."""
    x0, x1, k0, k1, l0, l1 = g["shape0"]
    _, _, k2, k3, l2, l3 = g["shape1"]
    L, k23, kc = l0 * l1, k2 * k3, k0 * k1
    wp = _round_up(2 * kc, 16)
    groups = len({t[1] for t in g["terms"]})
    ok = (k23 == L and L % 4 == 0 and 64 % L == 0 and (x0 * x1 * L) % 64 == 0 and 2 * wp <= 64
          and _round_up(2 * l2 * l3, 16) <= 128 and groups <= 8 and d in (1, 2, 4, 8))
    if not ok:
        return None
    na = nvec * k23 * d
    vh = 1 if na <= 128 else 2
    if vh == 2 and nvec % 2:
        return None
    nah = na // vh
    if nah % 16 or nah > 128 or nah < 16:
        return None
    return vh, nah, _round_up(2 * l2 * l3, 16)


def path_bytes_per_step(opr, nvec):
    """Algorithmic bytes of one operator application at the path's operand
    type (split-BF16 complex: hi and lo of re and im, 8 bytes per entry):
    each term's two S2 halves once, the block of centers in and out (complex128)."""
    import numpy as np
    out = 0
    for g in opr._groups:
        x0, x1, k0, k1, l0, l1 = g["shape0"]
        _, _, k2, k3, l2, l3 = g["shape1"]
        out += len(g["terms"]) * 8 * (x0 * x1 * k0 * k1 * l0 * l1 + x0 * x1 * k2 * k3 * l2 * l3)
    return out + 2 * nvec * 16 * int(np.prod(opr.in_shape))


def solve_section():
    """Time-to-energy of one center-site solve: plain FP64 (H_eff, N_eff formed
    on the CUDA cores, Lanczos) against mixed (formed on the tensor cores from
    split-BF16 operands, the same Lanczos, FP64 Rayleigh quotient)."""
    import numpy as np
    import torch
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.solve import solve_center
    from carcassonne_gb300.tensors._2d import sparse as tsp
    cc, ss, oo = workloads.hermitian_problem_arrays(D=SOLVE["D"], c=SOLVE["c"], seed=SOLVE["seed"])
    corners, sides, op = workloads.to_device(cc, ss, oo)
    H, N = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    res = {}
    # mixed: with the Newton correction (FP64-level energy); mixed_rayleigh:
    # the Rayleigh quotient of the tensor-core eigenvector with exact H x, N x
    variants = dict(plain=dict(precision="plain"), mixed=dict(precision="mixed"),
                    mixed_rayleigh=dict(precision="mixed", newton=False))
    for name, kw in variants.items():
        solve_center(H, N, **kw)
        times = []
        for _ in range(SOLVE["reps"]):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = solve_center(H, N, **kw)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        res[name] = dict(seconds=statistics.median(times), energy=out["energy"], lanczos_iterations=out["iterations"],
                         rayleigh_before_correction=out["rayleigh_before_correction"],
                         breakdown_ms={k: round(v, 3) for k, v in out["timing_ms"].items()})
    e0 = res["plain"]["energy"]
    return dict(config=dict(SOLVE, n=int(np.prod(H.operator.in_shape)), terms=len(H.operator.terms)),
                plain=res["plain"], mixed=res["mixed"], mixed_rayleigh=res["mixed_rayleigh"],
                rel_energy_diff=abs(res["mixed"]["energy"] - e0) / abs(e0),
                rel_energy_diff_rayleigh=abs(res["mixed_rayleigh"]["energy"] - e0) / abs(e0),
                speedup=res["plain"]["seconds"] / res["mixed"]["seconds"],
                speedup_rayleigh=res["plain"]["seconds"] / res["mixed_rayleigh"]["seconds"])


# growth runs (time-to-energy per absorption step): operator, D, seed,
# absorptions, per-layer boundary dimension kept by state compression
GROWTH = {
    "ti_h3_D2_c8": dict(workload="growth run, transverse Ising h=3, D=2, chi=64 (c=8), 20 absorptions", kind="ti",
                        D=2, seed=0, steps=20, new_dimension=8),
    "heis_D4_c8": dict(workload="growth run, Heisenberg XXX, D=4, chi=64 (c=8), 40 absorptions", kind="heis",
                       D=4, seed=2, steps=40, new_dimension=8, cpu_step=11),
}


def _sync_time(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def _compress_retry(system, corner, cdir, new_dimension, seed, log, step):
    """compressCornerStateTowards from the seeded random start; where the
    compressor's normal equations end above the reference's GMRES tolerance
    (AssertionError, as the reference's own ``assert info == 0``), the same
    compression is retried from a reseeded start, at most three times, and
    every failed attempt is logged.  Returns the wall time of the attempt
    that succeeded."""
    import numpy as np
    for attempt in range(4):
        np.random.seed(seed + 7919 * attempt)
        try:
            return _sync_time(lambda: system.compressCornerStateTowards(corner, cdir, new_dimension))[1]
        except AssertionError as e:
            log.append(dict(step=step, corner=corner, direction=cdir, attempt=attempt, error=str(e)[:160]))
            if attempt == 3:
                raise


def growth_run(spec, cpu_steps=()):
    """One growth run: at every absorption step the center problem is solved
    twice on the same environment, plain (FP64 H_eff / N_eff on the CUDA
    cores, FP64 Lanczos) and mixed (tensor-core formation, complex64
    Lanczos, one FP64 Newton correction), both from the current center; the
    run then absorbs the step's seeded random unit center
    (workloads.growth_center, as the golden run of the reference does:
    contractTowards(step % 4)), timed in FP64 and, on a copy, with every tag
    pair on the tensor cores, and runs compressCornerStateTowards for every
    corner axis above the kept dimension.  Wall times with the device
    synchronised on both sides.  ``cpu_steps``: steps whose environment is
    also solved, absorbed and compressed by the CPU restatement of the
    reference (numpy/SciPy on the host cores), as the reference's per-step
    time."""
    import numpy as np
    from copy import copy
    from carcassonne_gb300 import compression, workloads
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300.sparse import Identity
    from carcassonne_gb300.solve import solve_center
    from carcassonne_gb300.tensors._2d import dense
    system = workloads.bond_start_system(spec["kind"], spec["D"], spec["seed"])
    steps = []
    reseeds, reseeds_tc = [], []

    def one_step(step):
        (H, N), t_build = _sync_time(system.formExpectationAndNormalizationMultipliers)
        x0 = system.state_center_data
        plain, t_plain = _sync_time(lambda: solve_center(H, N, x0=x0, precision="plain"))
        mixed, t_mixed = _sync_time(lambda: solve_center(H, N, x0=x0, precision="mixed"))
        e_p, e_m = plain["energy"], mixed["energy"]
        hop = getattr(H, "operator", None)  # None when H_eff has no terms (a Heisenberg center's first step)
        rec = dict(step=step, n=int(np.prod(N.operator.in_shape)), terms=len(hop.terms) if hop is not None else 0,
                   energy=e_p, rel_err_mixed=abs(e_m - e_p) / abs(e_p) if e_p != 0 else abs(e_m),
                   build_s=t_build, plain_solve_s=t_plain, mixed_solve_s=t_mixed,
                   plain_fallback=plain.get("fallback"), mixed_fallback=mixed.get("fallback"))
        if step in cpu_steps:
            rec["cpu_reference_s"], rec["cpu_energy"] = _cpu_step(system)
        seed_c = workloads.GROWTH_CENTER_SEED[spec["kind"]] + step
        system.setStateCenter(TorchData(workloads.growth_center(tuple(x0.shape), seed_c)))
        if step in cpu_steps:
            rec["cpu_contract_s"], rec["cpu_compress_s"] = _cpu_contract_compress(system, step % 4,
                                                                                 spec["new_dimension"])
        # the same absorption with every tag pair on the tensor cores, on a copy
        tc_sys = copy(system)
        with dense.absorption_precision("tc"):
            _, t_tc = _sync_time(lambda: tc_sys.contractTowards(step % 4))
        _, t_contract = _sync_time(lambda: system.contractTowards(step % 4))
        tc_err = max(float((tc[t]._t - ref[t]._t).abs().max() / ref[t]._t.abs().max().clamp_min(1e-300))
                     for tc, ref in zip(tc_sys.corners + tc_sys.sides, system.corners + system.sides) for t in ref)
        del tc_sys
        # the same compressions with the normal equations' big contractions on
        # the tensor cores, on a copy (same random starts)
        tc_c = copy(system)
        t_compress_tc = 0.0
        with compression.compression_precision("tc"):
            for corner in range(4):
                for cdir, axis in ((0, 0), (1, 3)):
                    if tc_c.corners[corner][Identity()].shape[axis] > spec["new_dimension"]:
                        t_compress_tc += _compress_retry(tc_c, corner, cdir, spec["new_dimension"],
                                                         1000 * step + 10 * corner + cdir, reseeds_tc, step)
        del tc_c
        t_compress = 0.0
        for corner in range(4):
            for cdir, axis in ((0, 0), (1, 3)):
                if system.corners[corner][Identity()].shape[axis] > spec["new_dimension"]:
                    t_compress += _compress_retry(system, corner, cdir, spec["new_dimension"],
                                                  1000 * step + 10 * corner + cdir, reseeds, step)
        rec.update(contract_s=t_contract, contract_tc_s=t_tc, contract_tc_rel_err=tc_err, compress_s=t_compress,
                   compress_tc_s=t_compress_tc)
        # scale of the grown environment: the largest entry of each corner's and
        # side's Identity tag (log10); N_eff is a product of all eight
        scale = [float(b[Identity()]._t.abs().max()) for b in system.corners + system.sides]
        rec["env_log10_max_abs"] = [round(math.log10(v), 2) if v > 0 and math.isfinite(v) else repr(v) for v in scale]
        if spec.get("rescale"):
            # every tag of a boundary divided by one factor: H_eff and N_eff
            # scale alike and every energy and eigenvector stays the same
            for i, v in enumerate(scale[:4]):
                system.corners[i] = {t: d * (1.0 / v) for t, d in system.corners[i].items()}
            for i, v in enumerate(scale[4:]):
                system.sides[i] = {t: d * (1.0 / v) for t, d in system.sides[i].items()}
        return rec

    failed = None
    for step in range(spec["steps"]):
        try:
            steps.append(one_step(step))
        except Exception as e:  # a step the run cannot complete ends it, reported with the steps before it
            failed = dict(step=step, error="%s: %s" % (type(e).__name__, str(e)[:240]))
            break
    if not steps:
        return dict(spec, failed=failed)
    tot = lambda k: sum(r[k] for r in steps)
    out = dict(spec, steps_detail=[{k: (round(v, 6) if isinstance(v, float) and k.endswith("_s") else v)
                                    for k, v in r.items()} for r in steps])
    out.update(time_to_energy_plain_s=tot("build_s") + tot("plain_solve_s"),
               time_to_energy_mixed_s=tot("build_s") + tot("mixed_solve_s"),
               solve_plain_s=tot("plain_solve_s"), solve_mixed_s=tot("mixed_solve_s"),
               build_s=tot("build_s"), contract_s=tot("contract_s"), contract_tc_s=tot("contract_tc_s"),
               compress_s=tot("compress_s"), compress_tc_s=tot("compress_tc_s"),
               max_rel_err_mixed=max(r["rel_err_mixed"] for r in steps),
               max_contract_tc_rel_err=max(r["contract_tc_rel_err"] for r in steps),
               mixed_fallback_steps=[r["step"] for r in steps if r["mixed_fallback"]],
               plain_fallback_steps=[r["step"] for r in steps if r["plain_fallback"]],
               compress_reseeds=reseeds, compress_tc_reseeds=reseeds_tc,
               completed_steps=len(steps), failed=failed)
    out["speedup_solve"] = out["solve_plain_s"] / out["solve_mixed_s"]
    out["speedup_time_to_energy"] = out["time_to_energy_plain_s"] / out["time_to_energy_mixed_s"]
    # whole steps: build, solve, absorb and compress, all FP64 against the
    # mixed solve with the tensor-core absorption and compression (the latter
    # two timed on copies of the same environments; the run itself continues
    # from the FP64 ones)
    out["step_total_plain_s"] = out["build_s"] + out["solve_plain_s"] + out["contract_s"] + out["compress_s"]
    out["step_total_mixed_tc_s"] = (out["build_s"] + out["solve_mixed_s"] + out["contract_tc_s"] +
                                    out["compress_tc_s"])
    out["speedup_step_total"] = out["step_total_plain_s"] / out["step_total_mixed_tc_s"]
    cpu = [r for r in steps if "cpu_reference_s" in r]
    if cpu:
        out["cpu_reference"] = dict(
            kind="port", cores=os.cpu_count(), steps=[r["step"] for r in cpu],
            seconds_per_step=[round(r["cpu_reference_s"], 4) for r in cpu],
            gpu_plain_seconds_same_steps=[round(r["build_s"] + r["plain_solve_s"], 5) for r in cpu],
            gpu_mixed_seconds_same_steps=[round(r["build_s"] + r["mixed_solve_s"], 5) for r in cpu],
            max_rel_energy_diff_vs_gpu_plain=max(abs(r["cpu_energy"] - r["energy"]) / abs(r["energy"]) for r in cpu),
            contract_seconds=[round(r["cpu_contract_s"], 4) for r in cpu],
            gpu_contract_seconds_same_steps=[round(r["contract_s"], 5) for r in cpu],
            gpu_contract_tc_seconds_same_steps=[round(r["contract_tc_s"], 5) for r in cpu],
            compress_seconds=[round(r["cpu_compress_s"], 4) for r in cpu],
            gpu_compress_seconds_same_steps=[round(r["compress_s"], 5) for r in cpu],
            gpu_compress_tc_seconds_same_steps=[round(r["compress_tc_s"], 5) for r in cpu],
            sample="oracle/carc_oracle.py on host copies of the same environments: multipliers, formMatrix, "
                   "scipy.linalg.eigh; contractTowards; compressCornerStateTowards with a direct least-squares "
                   "solve (numpy/BLAS, all host threads)")
    return out


def _oracle_system(system):
    from oracle import carc_oracle as orc
    from tests.tagrepr import parse_tag
    oc = [{parse_tag(repr(t)): d.toArray() for t, d in c.items()} for c in system.corners]
    osd = [{parse_tag(repr(t)): d.toArray() for t, d in s.items()} for s in system.sides]
    oo = {parse_tag(repr(t)): d.toArray() for t, d in system.operator_center_tensor.items()}
    return orc.OracleSystem(oc, osd, system.state_center_data.toArray(), oo)


def _cpu_step(system):
    """The CPU restatement of the reference on one environment: build the
    multipliers, form H_eff and N_eff, dense generalized eigh (the
    reference's minimizeExpectationUsingFullEigensolver, system/_2d.py:498-502)."""
    from oracle import carc_oracle as orc
    osys = _oracle_system(system)
    t0 = time.perf_counter()
    H, N, _ = osys.multipliers()
    w, _ = orc.lowest_generalized(H.formMatrix(), N.formMatrix())
    return time.perf_counter() - t0, float(w)


def _cpu_contract_compress(system, direction, new_dimension):
    """The CPU restatement of the reference on one environment: contractTowards
    (system/_2d.py:435-439) of the step's center, then compressCornerStateTowards
    (system/_2d.py:191-228, the compressor of compression.py:26-46 with a
    direct least-squares solve) for every corner axis above new_dimension."""
    import numpy as np
    from oracle import carc_oracle as orc
    osys = _oracle_system(system)
    t0 = time.perf_counter()
    osys.contract_towards(direction)
    t1 = time.perf_counter()
    rng = np.random.default_rng(direction)
    for corner in range(4):
        for cdir, axis in ((0, 0), (1, 3)):
            old = osys.corners[corner][orc.I_TAG].shape[axis]
            if old > new_dimension:
                init = rng.standard_normal((old, new_dimension)) + 1j * rng.standard_normal((old, new_dimension))
                osys.compress_corner_state_towards(corner, cdir, new_dimension, init)
    return t1 - t0, time.perf_counter() - t1


def growth_section(cpu=True, heis_steps=None, cpu_step=None, rescale=True):
    """Both configured growth runs; ``heis_steps`` runs the Heisenberg one for
    that many absorptions instead of 40, ``cpu_step`` puts the CPU reference's
    step there instead of the run's own (the Heisenberg run's step 11, the
    transverse-Ising run's last), ``rescale`` divides each boundary by its
    largest entry after every step.  Energies and eigenvectors do not change
    under it (H_eff and N_eff scale alike).  Without it the boundaries' scales
    drift by up to tenfold per absorption, and the unscaled Heisenberg run
    stopped partway at a step whose N_eff had no eigenvalue above 1e-12 of
    its largest magnitude left to solve on."""
    out = {}
    for name, spec in GROWTH.items():
        if heis_steps and spec["kind"] == "heis":
            spec = dict(spec, steps=int(heis_steps),
                        workload="growth run, Heisenberg XXX, D=4, chi=64 (c=8), %d absorptions" % int(heis_steps))
        if rescale:
            spec = dict(spec, rescale=True, workload=spec["workload"] + ", boundaries rescaled after each step")
        last = spec["steps"] - 1
        own = spec.get("cpu_step", last)
        cpu_steps = ((min(cpu_step if cpu_step is not None else own, last)),) if cpu else ()
        out[name] = growth_run(spec, cpu_steps)
    return out


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nvec", type=int, default=8)
    p.add_argument("--mode", default="tc", choices=["tc", "fp64"],
                   help="tc: split-BF16 tensor-core matvec (headline); fp64: plain FP64 CUDA-core matvec")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-solve", dest="solve", action="store_false",
                   help="skip the mixed-vs-plain center-site solve comparison")
    p.add_argument("--no-batched", dest="batched", action="store_false",
                   help="skip the batched uneven-problems comparison (graph replay vs launch loop)")
    p.add_argument("--batched-count", type=int, default=32)
    p.add_argument("--no-batched-solves", dest="batched_solves", action="store_false",
                   help="skip the batched solves (batched block eigensolver vs the per-problem loop; sharded "
                        "over ranks under torchrun)")
    p.add_argument("--solves-count", type=int, default=256)
    p.add_argument("--growth-heis-steps", type=int, default=None,
                   help="absorptions of the Heisenberg growth run (default: the configured 40)")
    p.add_argument("--growth-cpu-step", type=int, default=None,
                   help="step of each growth run also run by the CPU reference (default: the Heisenberg run's 11, the "
                        "transverse-Ising run's last)")
    p.add_argument("--growth-no-rescale", dest="growth_rescale", action="store_false",
                   help="keep the growth runs' boundaries unscaled (by default each boundary is divided by its "
                        "largest entry after every step)")
    p.add_argument("--no-growth", dest="growth", action="store_false",
                   help="skip the growth runs' per-step time-to-energy (plain vs mixed)")
    return p.parse_args()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return dict(hbm_gbs=d["hbm_gbs"], bf16_tflops=d["bf16_tflops"], source="measured")
    return dict(hbm_gbs=6800.0, bf16_tflops=1900.0, source="fallback")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def samples(self):
        return len(self.lines)

    def stop(self):
        if self.proc is None:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["nvidia-smi unavailable"])
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxes.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return dict(sm_mhz=statistics.median(sms) if sms else None, sm_max_mhz=max(maxes) if maxes else None,
                    reasons=sorted(reasons), samples=len(sms))


def host_problem():
    from carcassonne_gb300 import workloads
    return workloads.matvec_problem_arrays(D=WORKLOAD["D"], c_ket=WORKLOAD["c_ket"], c_bra=WORKLOAD["c_bra"],
                                           seed=WORKLOAD["seed"])


def cpu_reference(args, seconds):
    """The CPU restatement of the reference's stage-3 path (numpy/BLAS, all
    host threads): builds the same boundaries and applies H_eff to the same
    block, timing as many centers as fit in ``seconds``."""
    import numpy as np
    from oracle import carc_oracle as orc
    from tests.tagrepr import parse_tag
    corners_a, sides_a, op_a = host_problem()
    oc = [{parse_tag(repr(t)): a for t, a in lst} for lst in corners_a]
    osd = [{parse_tag(repr(t)): a for t, a in lst} for lst in sides_a]
    oo = {parse_tag(repr(t)): a for t, a in op_a}
    H, _, info = orc.expectation_and_normalization_multipliers(oc, osd, oo)
    shape = (WORKLOAD["D"],) * 4 + (WORKLOAD["d"],)
    rng = np.random.default_rng(2)
    v = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    H(v)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while True:
        H(v)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    flops = n * H.cost_of_multiply * 8
    return dict(value=flops / dt / 1e9, unit=UNIT, cores=os.cpu_count(), kind="port",
                sample="%d single-center H_eff applications in %.1f s (numpy/BLAS, oracle/carc_oracle.py)" % (n, dt),
                cost_of_multiply=int(H.cost_of_multiply), seconds_per_vector=dt / n)


def cpu_reference_steps(args):
    """The reference arm: the CPU restatement of the reference's stage-3 path
    (numpy/BLAS on all host threads) run for ``--warmup`` untimed and
    ``--steps`` timed steps, a step being H_eff applied to the same block of
    ``--nvec`` centers as a step of the GPU arm."""
    import numpy as np
    from oracle import carc_oracle as orc
    from tests.tagrepr import parse_tag
    corners_a, sides_a, op_a = host_problem()
    oc = [{parse_tag(repr(t)): a for t, a in lst} for lst in corners_a]
    osd = [{parse_tag(repr(t)): a for t, a in lst} for lst in sides_a]
    oo = {parse_tag(repr(t)): a for t, a in op_a}
    H, _, _ = orc.expectation_and_normalization_multipliers(oc, osd, oo)
    shape = (args.nvec,) + (WORKLOAD["D"],) * 4 + (WORKLOAD["d"],)
    rng = np.random.default_rng(2)
    block = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    def step():
        return [H(block[i]) for i in range(args.nvec)]

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    flops = args.steps * args.nvec * H.cost_of_multiply * 8
    return dict(value=flops / dt / 1e9, unit=UNIT, cores=os.cpu_count(), kind="port",
                sample="%d steps of %d single-center H_eff applications in %.2f s (numpy/BLAS, oracle/carc_oracle.py)"
                       % (args.steps, args.nvec, dt),
                ms_per_step=dt / args.steps * 1e3)


def run_reference_arm(args, rank):
    if rank != 0:
        return
    res = cpu_reference_steps(args)
    line = dict(metric=METRIC, value=res["value"], unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=res["ms_per_step"], higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="complex128", data="synthetic",
                config=dict(WORKLOAD, nvec=args.nvec), parallelism="host threads", impl="reference",
                cpu_baseline=dict(value=res["value"], unit=UNIT, cores=res["cores"], kind=res["kind"],
                                  sample=res["sample"]),
                e2e=dict(value=res["value"], unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def batched_solves_section(args, dist, rank, world, device):
    """The batched-solve workload.  One GPU: every problem, solved by the
    batched block eigensolver and by the per-problem loop.  Under torchrun:
    each rank solves its cost-balanced shard with the batched solver (no
    data-path collective), the slowest rank sets the whole-job time, and
    rank 0 reports every problem's result."""
    from carcassonne_gb300 import batched as batched_mod
    from carcassonne_gb300.replicas import run_sharded
    kw = dict(m=BATCHED_SOLVES["block"], tol=BATCHED_SOLVES["tol"])
    if world == 1:
        out = batched_mod.run_solves(count=args.solves_count, seed=BATCHED_SOLVES["seed"], **kw)
        return dict(BATCHED_SOLVES, count=args.solves_count, ranks=1, **out)
    specs = batched_mod.sample_pencils(args.solves_count, BATCHED_SOLVES["seed"])

    def solve_fn(sub):
        return batched_mod.run_solves(specs=sub, loop=False, return_problems=True, **kw)

    res = run_sharded(specs, batched_mod.pencil_cost, solve_fn, dist, rank, world, device=device)
    if res is None:
        return None
    it = [v for v in res["iterations"] if v is not None]
    return dict(BATCHED_SOLVES, count=args.solves_count, ranks=world, sharding="cost-balanced (LPT), no collective",
                problems=res["problems"], batched_seconds=res["seconds"], batched_solves_per_s=res["solves_per_s"],
                iterations_mean=sum(it) / len(it), per_rank=res["per_rank"])


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return
    import numpy as np
    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        dist = dist_mod
    from carcassonne_gb300 import _lib, workloads
    from carcassonne_gb300.engine import CDT
    from carcassonne_gb300.tensors._2d import sparse as tsp
    lib = _lib.load()

    corners_a, sides_a, op_a = host_problem()
    corners, sides, op = workloads.to_device(corners_a, sides_a, op_a)
    H, _ = tsp.formExpectationAndNormalizationMultipliers(corners, sides, op)
    opr = H.operator
    nvec = args.nvec
    assert len(opr.terms) == WORKLOAD["terms"], len(opr.terms)
    rng = np.random.default_rng(2 + rank)
    xs = rng.standard_normal((nvec,) + opr.in_shape) + 1j * rng.standard_normal((nvec,) + opr.in_shape)
    x = torch.as_tensor(xs).to(CDT).cuda()
    y = torch.empty((nvec,) + opr.out_shape, dtype=CDT, device=x.device)
    flops_per_step = nvec * opr.cost_of_multiply() * 8
    flush = torch.empty(L2_FLUSH_BYTES // 16, dtype=CDT, device=x.device)

    def flush_l2():
        flush.zero_()

    apply = opr.apply_tc if args.mode == "tc" else opr.apply

    def step():
        apply(x, y, nvec)

    # accuracy of the timed path against the FP64 path on the same block
    y_ref = opr.apply(x, None, nvec)
    y_chk = apply(x, None, nvec)
    if args.mode == "tc":
        opr.check_status()
    rel_err = float(((y_chk - y_ref).abs().max() / y_ref.abs().max()).item())
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local_rank)
    sampler.start()

    def load_until(pred, limit_s):
        # untimed steps keep the GPU under the same load while nvidia-smi samples
        t0 = time.perf_counter()
        while not pred() and time.perf_counter() - t0 < limit_s:
            for _ in range(20):
                step()
            torch.cuda.synchronize()

    # the timed region is milliseconds long; the clock samples (every 100 ms)
    # bracket it under the same load: at least two before, two after
    n0 = sampler.samples() if sampler.proc else 0
    load_until(lambda: sampler.proc is None or sampler.samples() >= n0 + 2, 5.0)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = lib.carc_launch_counter()
    launches_in_steps = 0
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush_l2()
        starts[i].record()
        c0 = lib.carc_launch_counter()
        step()
        launches_in_steps += lib.carc_launch_counter() - c0
        ends[i].record()
    torch.cuda.synchronize()
    n1 = sampler.samples() if sampler.proc else 0
    load_until(lambda: sampler.proc is None or sampler.samples() >= n1 + 2, 5.0)
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(times) / len(times)
    del launches0

    # per-phase device times of the tensor-core operator (CUDA event pairs
    # around each phase's launches on the launching stream), same workload
    phases = None
    if args.mode == "tc":
        lib.carc_phase_timing_enable(1)
        for i in range(args.steps):
            flush_l2()
            step()
        torch.cuda.synchronize()
        lib.carc_phase_timing_enable(0)
        phases = {}
        for pid, pname in enumerate(PHASE_NAMES):
            tot, cnt = ctypes.c_double(0.0), ctypes.c_int64(0)
            _lib.check(lib.carc_phase_timing_read(pid, ctypes.byref(tot), ctypes.byref(cnt)))
            phases[pname] = dict(ms_per_step=tot.value / args.steps, intervals_per_step=cnt.value / args.steps)

    # the plain FP64 path on the same workload, for reference
    fp64_ms = None
    if args.mode != "fp64":
        for _ in range(2):
            opr.apply(x, y, nvec)
        torch.cuda.synchronize()
        fs, fe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k64 = max(2, args.steps // 4)
        tot = 0.0
        for _ in range(k64):
            flush_l2()
            fs.record()
            opr.apply(x, y, nvec)
            fe.record()
            torch.cuda.synchronize()
            tot += fs.elapsed_time(fe)
        fp64_ms = tot / k64

    # e2e: host block -> device -> operator -> host, copies inside the timed region
    xh = torch.as_tensor(xs).to(CDT).pin_memory()
    yh = torch.empty(y.shape, dtype=CDT).pin_memory()
    xd = torch.empty_like(x)
    for _ in range(2):
        xd.copy_(xh, non_blocking=True)
        apply(xd, y, nvec)
        yh.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    e_starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    e_ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        flush_l2()
        e_starts[i].record()
        xd.copy_(xh, non_blocking=True)
        apply(xd, y, nvec)
        yh.copy_(y, non_blocking=True)
        e_ends[i].record()
    torch.cuda.synchronize()
    e_ms_copies = sum(s.elapsed_time(e) for s, e in zip(e_starts, e_ends)) / args.steps
    e_ms = e_ms_copies
    e2e_transfer = "cudaMemcpyAsync each way (pinned host block -> device, result -> pinned host)"
    if args.mode == "tc":
        # the block and the result in pinned host memory mapped into the device's
        # address space: the kernel reads the block and writes the result over the
        # host link (NVLink-C2C) inside the call, the same bytes each way per step
        from carcassonne_gb300.hostmem import MappedHostBuffer
        xm = MappedHostBuffer(tuple(x.shape))
        ym = MappedHostBuffer(tuple(y.shape))
        xm.host[...] = xs
        for _ in range(2):
            opr.apply_tc_ptr(xm.device_ptr, ym.device_ptr, nvec)
        torch.cuda.synchronize()
        opr.check_status()
        mapped_ok = bool(np.array_equal(ym.host, y_chk.cpu().numpy()))
        m_starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        m_ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        for i in range(args.steps):
            flush_l2()
            m_starts[i].record()
            opr.apply_tc_ptr(xm.device_ptr, ym.device_ptr, nvec)
            m_ends[i].record()
        torch.cuda.synchronize()
        opr.check_status()
        if not mapped_ok:
            raise RuntimeError("the mapped-host matvec differs from the device one")
        e_ms = sum(s.elapsed_time(e) for s, e in zip(m_starts, m_ends)) / args.steps
        e2e_transfer = ("pinned host memory mapped into the device's address space: the kernel reads the block "
                        "and writes the result on the host over NVLink-C2C (result equal to the device path's)")
        xm.close()
        ym.close()

    from carcassonne_gb300.replicas import max_over_ranks
    ms, e_ms, e_ms_copies = max_over_ranks([ms, e_ms, e_ms_copies], dist, device=x.device)
    value = world * flops_per_step / (ms * 1e-3) / 1e9
    e2e_value = world * flops_per_step / (e_ms * 1e-3) / 1e9
    e2e_copies_value = world * flops_per_step / (e_ms_copies * 1e-3) / 1e9
    solves = batched_solves_section(args, dist, rank, world, x.device) if args.batched_solves else None
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks = measured_peaks()
    achieved_tflops = flops_per_step / (ms * 1e-3) / 1e12
    roofline = dict(bound="tensor", achieved=achieved_tflops, peak=peaks["bf16_tflops"], unit="TFLOP/s",
                    frac=achieved_tflops / peaks["bf16_tflops"], traffic=None,
                    peak_source=peaks["source"] + " bf16 dense",
                    note="whole operator: algorithmic (CostTracker) flops per step / step time")
    if phases:
        geo = tc_bytes_per_step(opr, nvec)
        fused = phases["step_b"]["intervals_per_step"] == 0
        if fused:
            # the step-A interval brackets the fused kernel, which does both steps
            # (the compact-operand one wherever it takes the shape)
            name = "fused2" if all(_f2_geo(g, nvec, opr.d) for g in opr._groups) else "fused"
            phases[name] = phases.pop("step_a")
            phases.pop("step_b")
        for pname, ph in phases.items():
            ph["share"] = ph["ms_per_step"] / ms
            if pname in geo:
                ph["algorithmic_bytes_per_step"] = geo[pname]
                ph["achieved_gbs"] = geo[pname] / (ph["ms_per_step"] * 1e-3) / 1e9 if ph["ms_per_step"] else None
        top = max((p for p in phases if p in geo), key=lambda p: phases[p]["ms_per_step"])
        ph = phases[top]
        launches = geo["launches"][top]
        traffic = NCU_TRAFFIC.get((WORKLOAD["workload"], top))
        common = dict(kernel=KERNEL_OF_PHASE[top], traffic=None if traffic is None else traffic["bytes_per_launch"],
                      algorithmic_bytes_per_launch=geo[top] / launches, launch_ms=ph["ms_per_step"] / launches,
                      launches_per_step=launches, traffic_source=None if traffic is None else traffic["source"],
                      whole_operator_tflops=achieved_tflops,
                      whole_operator_frac_of_bf16=achieved_tflops / peaks["bf16_tflops"])
        if top in ("fused", "fused2"):
            # algorithmic flops per launch (CostTracker, the whole operator) over the kernel's time;
            # the split-BF16 tensor work is 4x (first kernel) or 3x (compact kernel: no lo x lo) that
            kt = flops_per_step / (ph["ms_per_step"] * 1e-3) / 1e12
            alg_bytes = path_bytes_per_step(opr, nvec)
            alg_gbs = alg_bytes / (ph["ms_per_step"] * 1e-3) / 1e9
            roofline = dict(bound="tensor", achieved=kt, peak=peaks["bf16_tflops"], unit="TFLOP/s",
                            frac=kt / peaks["bf16_tflops"],
                            tensor_executed_tflops=(3 if top == "fused2" else 4) * kt,
                            path_bytes_per_launch=alg_bytes, hbm_achieved_gbs=alg_gbs,
                            hbm_frac=alg_gbs / peaks["hbm_gbs"],
                            packed_operand_gbs=ph["achieved_gbs"],
                            peak_source=peaks["source"] + " bf16 dense", **common)
        else:
            roofline = dict(bound="hbm", achieved=ph["achieved_gbs"], peak=peaks["hbm_gbs"], unit="GB/s",
                            frac=ph["achieved_gbs"] / peaks["hbm_gbs"], peak_source=peaks["source"] + " HBM copy",
                            **common)
    cpu = cpu_reference(args, args.cpu_seconds) if world == 1 else None
    solve = solve_section() if args.solve else None
    if solve is not None and args.growth and world == 1:
        # single-GPU workloads: under torchrun every rank would repeat them
        solve["growth"] = growth_section(cpu=True, heis_steps=args.growth_heis_steps,
                                         cpu_step=args.growth_cpu_step, rescale=args.growth_rescale)
    batched = None
    if args.batched and world == 1:
        from carcassonne_gb300 import batched as batched_mod
        batched = dict(BATCHED, count=args.batched_count,
                       **batched_mod.run(count=args.batched_count, nvec=BATCHED["nvec"], seed=BATCHED["seed"]))
    if solves is not None:
        batched = dict(batched or {}, solves=solves)
    line = dict(
        metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
        ms_per_step=ms, higher_is_better=True, scaling="weak", vs_baseline=None,
        dtype="bf16 hi+lo split of complex128 operands, fp32 accumulate, fp64 reductions" if args.mode == "tc"
        else "complex128 (fp64)",
        rel_err_vs_fp64=rel_err,
        fp64_path=None if fp64_ms is None else dict(ms_per_step=fp64_ms,
                                                    value=world * flops_per_step / (fp64_ms * 1e-3) / 1e9),
        data="synthetic: i.i.d. N(0,1) seed 1, unit Frobenius norm per tensor",
        config=dict(WORKLOAD, nvec=nvec), mode=args.mode, l2="flushed between timed steps (512 MB write)",
        parallelism="replicas" if world > 1 else "single GPU",
        e2e=dict(value=e2e_value, unit=UNIT, h2d_bytes_per_step=int(xh.numel() * 16),
                 d2h_bytes_per_step=int(yh.numel() * 16), ms_per_step=e_ms, transfer=e2e_transfer,
                 copies_value=e2e_copies_value, copies_ms_per_step=e_ms_copies),
        gpu_launches=int(launches_in_steps),
        roofline=roofline, phases=phases, solve=solve, batched=batched,
        cpu_baseline=None if cpu is None else dict(value=cpu["value"], unit=UNIT, cores=cpu["cores"],
                                                   kind=cpu["kind"], sample=cpu["sample"]),
        clocks=clocks, step_ms=dict(min=min(times), max=max(times)),
    )
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
