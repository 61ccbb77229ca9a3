"""Benchmark of the GB300 hot path (one JSON line on rank 0).

Modes
  hac   : H_AC applies (ApplyHAvec, VUMPS_helpers.hpp:55-88) on XXZ D=512; a step is one
          Lanczos cycle's worth of applies (20 independent input vectors).
The reference arm (--impl reference) times the CPU restatement of the same path on the host
cores (the reference itself cannot be built: armadillo/ARPACK are not available).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "VUMPS sweeps/s + H_AC TFLOP/s, mixed vs FP64 on one GB300 at |dE|<=1e-9"
APPLIES_PER_STEP = 20
L2_FLUSH_BYTES = 512 << 20


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _fp64_peak_tflops(torch):
    """Dense FP64 matmul throughput measured on this GPU (no FP64 figure is recorded)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    return 2 * n ** 3 / best / 1e12


# ------------------------------------------------------------------------------------------------
# CPU restatement timing (oracle port) -- the reference arm and the cpu_baseline leg
# ------------------------------------------------------------------------------------------------

def _oracle_hac_operands(w):
    """Oracle dict structures for the same operands as the GPU workload."""
    from oracle import imps_oracle as O
    d = w.d
    host = w.host_copies()
    EHL = O.bd_from_vec(host["EHL"], [(b[1], b[3]) for b in w.lehl.blocks])
    EHR = O.bd_from_vec(host["EHR"], [(b[1], b[3]) for b in w.lehr.blocks])

    def redop(vec, lay):
        R = [[dict() for _ in range(d)] for _ in range(d)]
        for (g, qi, qo, r, c), o in zip(lay.blocks, lay.offsets):
            R[g // d][g % d][qi] = (qo, vec[o:o + r * c].reshape(c, r).T.copy())
        return R

    HL, HR = redop(host["HL"], w.lhl), redop(host["HR"], w.lhr)
    sizes = [[(b[1], b[2], b[3], b[4]) for b in w.lac.blocks if b[0] == s] for s in range(d)]
    return O, sizes, EHL, EHR, HL, HR


def cpu_hac_rate(w, budget_s=12.0):
    """Time the oracle's ApplyHAvec (numpy/OpenBLAS on all host cores) on a bounded sample."""
    O, sizes, EHL, EHR, HL, HR = _oracle_hac_operands(w)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(w.n)
    O.ApplyHAvec(x, sizes, EHL, EHR, HL, HR)  # warm-up
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        O.ApplyHAvec(x, sizes, EHL, EHR, HL, HR)
        n += 1
    dt = time.perf_counter() - t0
    return n, dt


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import torch
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300.workload import HacWorkload
    # operands are generated with the product path on the GPU only to share the exact inputs
    ctx = B.Context(0)
    ctx.set_stream(torch.cuda.current_stream())
    w = HacWorkload(ctx, args.workload)
    torch.cuda.synchronize()
    per_step = []
    for i in range(args.warmup + args.steps):
        n, dt = cpu_hac_rate(w, budget_s=max(2.0, 60.0 / max(args.steps + args.warmup, 1)))
        if i >= args.warmup:
            per_step.append(dt / n * APPLIES_PER_STEP)
    ms = 1e3 * float(np.mean(per_step))
    tflops = w.flops * APPLIES_PER_STEP / (ms * 1e-3) / 1e12
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": tflops, "unit": "H_AC TFLOP/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload + " H_AC apply (ApplyHAvec)", "applies_per_step": APPLIES_PER_STEP},
            "cpu_baseline": {"value": tflops, "unit": "H_AC TFLOP/s", "cores": cores, "kind": "port",
                             "sample": f"{APPLIES_PER_STEP}-apply steps timed on a wall-clock budget"},
            "e2e": {"value": tflops, "unit": "H_AC TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------

def run_hac(args):
    import torch
    import torch.distributed as dist
    from imps_cpp_tools_gb300 import _native as N
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300.workload import HacWorkload

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    ctx = B.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    w = HacWorkload(ctx, args.workload)
    if args.precision == "bf16x6":
        w.plan.set_precision(N.PREC_BF16X6)
    X = torch.randn(APPLIES_PER_STEP, w.n, dtype=torch.float64, device="cuda")
    Y = torch.empty_like(X)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    lib = N.load()
    ph = w.plan.handle
    xs = [X[j].data_ptr() for j in range(APPLIES_PER_STEP)]
    ys = [Y[j].data_ptr() for j in range(APPLIES_PER_STEP)]

    def step():
        for j in range(APPLIES_PER_STEP):
            st = lib.imps_hac_apply(ph, xs[j], ys[j], N.MEM_DEVICE)
            if st < 0:
                raise N.ImpsError(st, "imps_hac_apply")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()  # L2 flush between timed steps (outside the events)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    clk = clocks.stop()
    t_step = float(np.mean(times))
    if ws > 1:
        tt = torch.tensor([t_step], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
    total_flops = w.flops * APPLIES_PER_STEP * ws
    value = total_flops / t_step / 1e12

    # e2e: the reference-facing functor with HOST buffers (H2D of the input, D2H of the output
    # inside every call), as ARPACK would call ApplyHAvec through the C ABI
    hx = torch.randn(APPLIES_PER_STEP, w.n, dtype=torch.float64).pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    hxs = [hx[j].data_ptr() for j in range(APPLIES_PER_STEP)]
    hys = [hy[j].data_ptr() for j in range(APPLIES_PER_STEP)]

    def step_host():
        for j in range(APPLIES_PER_STEP):
            st = lib.imps_hac_apply(ph, hxs[j], hys[j], N.MEM_HOST)
            if st < 0:
                raise N.ImpsError(st, "imps_hac_apply(host)")

    for _ in range(max(1, args.warmup)):
        step_host()
    torch.cuda.synchronize()
    et = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step_host()
        et.append(time.perf_counter() - t0)
    e2e_t = float(np.mean(et))
    e2e = {"value": w.flops * APPLIES_PER_STEP * ws / e2e_t / 1e12, "unit": "H_AC TFLOP/s",
           "h2d_bytes_per_step": APPLIES_PER_STEP * w.n * 8, "d2h_bytes_per_step": APPLIES_PER_STEP * w.n * 8,
           "ms_per_step": e2e_t * 1e3}

    peaks = _peaks()
    if args.precision == "bf16x6":
        peak, peak_src = peaks.get("bf16_tflops", 1893.6), "MEASURED_PEAKS.json bf16_tflops (burst)"
        achieved_flops = w.flops * 6  # six BF16 split products per useful FP64-equivalent flop
    else:
        peak, peak_src = _fp64_peak_tflops(torch), "dense FP64 matmul measured in this run"
        achieved_flops = w.flops
    t_apply = t_step / APPLIES_PER_STEP
    achieved = achieved_flops / t_apply / 1e12
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": None, "peak_source": peak_src, "kernel": "grouped_gemm (H_AC apply)",
            "algorithmic_bytes_per_launch": w.bytes_per_apply(),
            "achieved_gbs": w.bytes_per_apply() / t_apply / 1e9}

    cpu = None
    if rank == 0 and not args.no_cpu:
        n, dt = cpu_hac_rate(w, budget_s=args.cpu_budget)
        cpu = {"value": w.flops * n / dt / 1e12, "unit": "H_AC TFLOP/s", "cores": os.cpu_count(),
               "kind": "port", "sample": f"{n} ApplyHAvec calls of the numpy restatement in {dt:.1f} s"}
    nst = w.plan.info()["nstages"]
    line = {"metric": METRIC, "value": value, "unit": "H_AC TFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "bf16x6->f32",
            "data": "synthetic",
            "config": {"workload": f"{args.workload} H_AC apply (ApplyHAvec), {APPLIES_PER_STEP} applies/step",
                       "n": w.n, "flops_per_apply": w.flops, "precision": args.precision,
                       "l2": "flushed between steps (512 MB write)", "parallelism": f"replicas x{ws}"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": args.steps * APPLIES_PER_STEP * nst, "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="hac", choices=["hac"])
    ap.add_argument("--workload", default="xxz_d512")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "bf16x6"])
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return
    run_hac(args)


if __name__ == "__main__":
    main()
