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
between timed steps; e2e: the same metric with the block copied from pinned
host memory and the result copied back inside the timed region.
``--impl reference`` times the CPU restatement of the reference's path on
the host cores (the reference itself is pure Python/NumPy and is not
available on the GPU host).
"""
from __future__ import annotations

import argparse
import json
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


def run_reference_arm(args, rank):
    if rank != 0:
        return
    res = cpu_reference(args, args.cpu_seconds)
    line = dict(metric=METRIC, value=res["value"], unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=res["seconds_per_vector"] * 1e3 * args.nvec, higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="complex128", data="synthetic",
                config=dict(WORKLOAD, nvec=args.nvec, parallelism="host threads"), impl="reference",
                cpu_baseline=dict(res, value=res["value"]),
                e2e=dict(value=res["value"], unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


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
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(times) / len(times)
    del launches0

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
    e_ms = sum(s.elapsed_time(e) for s, e in zip(e_starts, e_ends)) / args.steps

    if dist:
        t = torch.tensor([ms, e_ms], dtype=torch.float64, device=x.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, e_ms = float(t[0]), float(t[1])
    value = world * flops_per_step / (ms * 1e-3) / 1e9
    e2e_value = world * flops_per_step / (e_ms * 1e-3) / 1e9
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks = measured_peaks()
    achieved_tflops = flops_per_step / (ms * 1e-3) / 1e12
    cpu = cpu_reference(args, args.cpu_seconds) if world == 1 else None
    line = dict(
        metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
        ms_per_step=ms, higher_is_better=True, scaling="weak", vs_baseline=None,
        dtype="bf16 hi+lo split of complex128 operands, fp32 accumulate, fp64 reductions" if args.mode == "tc"
        else "complex128 (fp64)",
        rel_err_vs_fp64=rel_err,
        fp64_path=None if fp64_ms is None else dict(ms_per_step=fp64_ms,
                                                    value=world * flops_per_step / (fp64_ms * 1e-3) / 1e9),
        data="synthetic: i.i.d. N(0,1) seed 1, unit Frobenius norm per tensor",
        config=dict(WORKLOAD, nvec=nvec, mode=args.mode, l2="flushed between timed steps (512 MB write)",
                    parallelism="replicas" if world > 1 else "single GPU"),
        e2e=dict(value=e2e_value, unit=UNIT, h2d_bytes_per_step=int(xh.numel() * 16),
                 d2h_bytes_per_step=int(yh.numel() * 16)),
        gpu_launches=int(launches_in_steps),
        roofline=dict(bound="tensor", achieved=achieved_tflops, peak=peaks["bf16_tflops"], unit="TFLOP/s",
                      frac=achieved_tflops / peaks["bf16_tflops"], traffic=None,
                      peak_source=peaks["source"] + " bf16 dense",
                      note="achieved = algorithmic (CostTracker) flops per step / step time; the split-BF16 "
                           "path executes 16 real tensor MACs per complex MAC"),
        cpu_baseline=None if cpu is None else dict(value=cpu["value"], unit=UNIT, cores=cpu["cores"],
                                                   kind=cpu["kind"], sample=cpu["sample"]),
        clocks=clocks, step_ms=dict(min=min(times), max=max(times)),
    )
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
