"""Benchmark of the GB300 hot path; rank 0 prints one JSON line.

Workload (default): XXZ spin-1/2 chain, J=1, Delta=1 (antiferromagnet; --Delta=-1 in the
reference's sign convention), two-site unit cell, U(1) Sz sectors q=-10..10 with dims
~exp(-q^2/18) summing to D=512, bond expansion off.  The timed sweeps start from a warmed
state (the committed tests/golden/warm_<workload>.npz: 20 sweeps of the reference's tolerance
schedule from seed 1; workloads without one warm up on the device the same way) and run at the
fixed eigensolver tolerance 1e-12 of the configuration and GMRES tolerance 1e-8 (TIMED_TOLS).
A step is one VUMPS sweep (both site updates of VUMPS_main.cpp:165-354); W warm-up sweeps are
run before the K timed ones.  The headline value is the FP64 path (--precision fp64, the
default); the split-BF16 (tcgen05) path runs the same sweeps from the same state and is reported
beside it, with the energy difference of the two after the last sweep.  Rank 0 also runs one
sweep of the CPU restatement from the same start state (cpu_baseline) and reports its energies
beside the GPU's first sweep (parity_vs_oracle).  Under torchrun every rank runs its own replica
of the sweeps (the path does not shard); the step time is the maximum over ranks and the value
N / that time.

--mode hac times H_AC applies only (ApplyHAvec; a step = 20 applies).
--mode excitations grows the XXZ D=256 ground state by bond expansion and times the 4 lowest Sz = +1
excitation energies at 32 momenta in one batched run, beside the per-momentum path on --steps
of them.
--mode expand times one bond expansion (ExpandFromH, dmmax 20) at the XXZ D=512 and Hubbard
D=1024 starts against the oracle on the same state.
--mode cpp runs the same timed sweeps through the C++ host driver (include/imps_vumps.hpp) beside
the Python driver.
--mode trace runs the timed FP64 sweeps under torch.profiler: summed kernel time against wall time,
kernels by share.
--mode krylov times one bounded thick-restart Lanczos solve (eigs_rs, ncv 64, at most 8 restart
cycles; FP64 at an unreachable tolerance, split-BF16 at its 2e-7 floor) on the synthetic H_AC,
next to the same number of bare applies: the difference is the per-iteration
orthogonalisation, convergence-check and launch cost.
The reference arm (--impl reference) times site updates of the CPU restatement of the same
sweeps from the same start state (the reference itself cannot be built: armadillo/ARPACK are not
available).
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
# DRAM bytes (read + write) of one H_AC apply from one ncu capture of `bench.py --mode hac`
# (profiles/tc_gemm_hac_xxz_d512.md: tc_gemm 5.26 MB + pack 0.40 MB;
# profiles/grouped_gemm_f64_hac_xxz_d512.md, autotuned shape 16x16 split 2: 2.38 + 0.03 MB)
NCU_TRAFFIC_BYTES = {"bf16x6": 5.66e6, "fp64": 2.41e6}
# tolerances of the timed sweeps: the eigensolver tolerance of the configuration (1e-12); GMRES
# 1e-8, because the environment systems of these states do not reach 1e-12 in floating point:
# measured at XXZ D=512 from the warmed state, the relative residual of the left-environment
# solves floors at 2e-11 (site 0) and 1e-9 (site 1, warm start of norm 3e5) after ~200
# iterations, where the reference's unrestarted GMRES then runs on towards maxit = 24,368
TIMED_TOLS = {"eig": 1e-12, "gmres": 1e-8}
# wall-clock bounds of the CPU restatement: the reference arm (warm-up and timed site updates
# together) and the cpu_baseline sample of the GPU arm (one sweep)
REF_BUDGET_S = 360.0
CPU_SAMPLE_BUDGET_S = 90.0
_TIMED = ("2-site VUMPS sweep from a warmed state (20/30 sweeps of the tolerance schedule "
          "min(max(prec/100, 1e-12), 1e-6), VUMPS_main.cpp:177, from seed 1), then fixed eigensolver tol 1e-12 and "
          "GMRES tol 1e-8, expansion off")
WORKLOAD_DESCS = {
    "xxz_d512": "XXZ D=512 (21 U(1) sectors, dims ~exp(-q^2/18)), " + _TIMED,
    "hubbard_d1024": "Fermi-Hubbard t=1, U=4, half filling, D=1024 (60 U(1)xU(1) (N, Sz) sectors, dims "
                     "~exp(-(dN^2+4Sz^2)/8)), " + _TIMED,
}
_WORKLOAD = ["xxz_d512"]  # the VUMPS workload of this run (--workload)


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
        self.index, self.proc, self.lines = index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

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
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def _max_over_ranks(dist, values, device):
    """Element-wise maximum of `values` over all ranks: the slowest replica sets the step time."""
    import torch
    t = torch.tensor([float(x) for x in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def _fp64_peak_tflops(torch):
    """Dense FP64 matmul throughput of this GPU (no FP64 figure is recorded for the pool)."""
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


def _workload_desc():
    return WORKLOAD_DESCS.get(_WORKLOAD[0], _WORKLOAD[0] + ", " + _TIMED)


# ------------------------------------------------------------------------------------------------
# CPU restatement (oracle port): the reference arm and the cpu_baseline leg
# ------------------------------------------------------------------------------------------------

def _oracle_state(name, state):
    """(ALvec, ARvec, Cvec) in the arrangement of the oracle's randMPS_LR (Cvec[n] = the C right
    of site n) from a flat host state (workload.load_warm_state / VumpsGPU.host_state)."""
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300.workload import bond_layouts
    from oracle import imps_oracle as O
    model, d, I2K, h, dimvec = bond_layouts(name)

    def sizes(n):
        lay = B.Layout.mps(I2K, dimvec[n], dimvec[1 - n])
        return [[(qi, qo, r, c) for (g, qi, qo, r, c) in lay.blocks if g == s] for s in range(d)]
    AL = [O.mps_from_vec(state["AL"][n], sizes(n)) for n in range(2)]
    AR = [O.mps_from_vec(state["AR"][n], sizes(n)) for n in range(2)]
    C = [O.bd_from_vec(state["C"][1], sorted(dimvec[1].items())),
         O.bd_from_vec(state["C"][0], sorted(dimvec[0].items()))]
    return AL, AR, C


def _oracle_vumps(name, state):
    """The oracle's VUMPS (VUMPS_main.cpp restated: ARPACK eigs_rs at ncv 20, the reference's
    unrestarted MGS GMRES, per-sector LAPACK decompositions on the host) at the timed
    tolerances, started from `state`; its constructor solves the initial environments."""
    from imps_cpp_tools_gb300 import models
    from imps_cpp_tools_gb300.workload import bond_layouts
    from oracle import imps_oracle as O
    model, d, I2K, h, dimvec = bond_layouts(name)
    return O.VUMPS(h, d, I2K, dimvec[0], dimvec=dimvec, init=_oracle_state(name, state),
                   fixed_tol=TIMED_TOLS["eig"], InvETol=TIMED_TOLS["gmres"])


class _Deadline(Exception):
    """The CPU restatement ran past its time budget (raised from inside an operator apply)."""


_DEADLINE = [None]
_PATCHED = [False]


def _install_deadline():
    """Every operator apply of the oracle checks the wall-clock budget first, so a solve that
    would run for hours (ARPACK's maxit is the problem size, eigs.cpp:386; the reference's GMRES
    runs to maxit = dimension on a system whose residual floors above the tolerance) ends the
    CPU measurement instead."""
    if _PATCHED[0]:
        return
    from oracle import imps_oracle as O
    for name in ("ApplyHAvec", "ApplyHCvec", "ApplyTMLeftUC", "ApplyTMRightUC"):
        f = getattr(O, name)

        def w(*a, _f=f, **k):
            if _DEADLINE[0] is not None and time.perf_counter() > _DEADLINE[0]:
                raise _Deadline()
            return _f(*a, **k)
        setattr(O, name, w)
    _PATCHED[0] = True


def cpu_site_updates(name, state, warmup, steps, budget_s=None):
    """Time `steps` site updates (VUMPS_main.cpp:171-313, one half of a sweep each) of the
    oracle's VUMPS after `warmup` untimed ones, from `state`, on the host's cores (numpy's
    BLAS threads), within `budget_s` seconds of wall time for the whole call (None: no bound).
    Returns (seconds per completed timed site update, the energies after the first full sweep or
    None, threads, whether the budget cut the run short)."""
    ora = _oracle_vumps(name, state)
    times, E, cut = [], None, False
    if budget_s is not None:
        _install_deadline()
        _DEADLINE[0] = time.perf_counter() + budget_s
    try:
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            ora.site_update(i % 2)
            dt = time.perf_counter() - t0
            if i >= warmup:
                times.append(dt)
            if i == 1:
                E = _oracle_sweep_energy(ora)
    except _Deadline:
        cut = True
    finally:
        _DEADLINE[0] = None
    return times, E, os.cpu_count(), cut


def _oracle_sweep_energy(ora):
    """The energies the oracle's sweep() reports after its two site updates."""
    from oracle import imps_oracle as O
    if not hasattr(ora, "C"):
        return None
    for n in range(ora.N):
        ora.L[(n - 1) % ora.N] = O.bd_mul(O.bd_t(ora.C[n]), ora.C[n])
    return O.energy_right(ora.hnnz, ora.AR, ora.L)


def ref_site_update_cycle(name, state, warmup, steps, budget_s):
    """The reference arm's steps: site updates of the oracle's VUMPS in cycles that each start
    from `state` (the constructor's environment solves untimed) and run site 0 then site 1 (one
    sweep), so that every step is the same bounded piece of the workload; the first `warmup`
    site updates are untimed.  Later sweeps are not used: some of their eigensolves ask ARPACK for
    a Ritz residual below what FP64 resolves for the operator, which it then pursues for up to N
    restart cycles (eigs.cpp:386).  Returns (seconds per timed site update, threads, whether the
    wall-clock budget ended the run early)."""
    _install_deadline()
    _DEADLINE[0] = time.perf_counter() + budget_s
    times, done, cut = [], 0, False
    try:
        while done < warmup + steps:
            ora = _oracle_vumps(name, state)
            for nn in range(2):
                if done >= warmup + steps:
                    break
                t0 = time.perf_counter()
                ora.site_update(nn)
                dt = time.perf_counter() - t0
                if done >= warmup:
                    times.append(dt)
                done += 1
    except _Deadline:
        cut = True
    finally:
        _DEADLINE[0] = None
    return times, os.cpu_count(), cut


def run_reference(args):
    """--impl reference: the CPU restatement of the reference's VUMPS (the reference itself cannot
    be built: armadillo and ARPACK are absent) timed on the host's cores.  A step is one site
    update (half a sweep) of the first sweep from the committed warmed state, at the same fixed
    tolerances as the GPU arm; sweeps/s = 1 / (2 x mean site-update time)."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from imps_cpp_tools_gb300 import workload as W
    state = W.load_warm_state(_WORKLOAD[0])
    if state is None:
        print(json.dumps({"impl": "reference", "unavailable": f"no committed warmed start state for {_WORKLOAD[0]} "
                          "(tests/golden/warm_<workload>.npz); the CPU restatement from a random start does not "
                          "finish its first sweeps in minutes"}), flush=True)
        return
    t0 = time.perf_counter()
    times, cores, cut = ref_site_update_cycle(_WORKLOAD[0], state, args.warmup, args.steps, REF_BUDGET_S)
    if not times:
        print(json.dumps({"impl": "reference", "unavailable": f"no timed site update of the CPU restatement finished "
                          f"within {REF_BUDGET_S:.0f} s"}), flush=True)
        return
    # site 0 and site 1 alternate; an unequal count would tilt the mean
    t_site = float(np.mean(times[: len(times) - len(times) % 2])) if len(times) > 1 else float(times[0])
    value = 1.0 / (2.0 * t_site)
    sample = (f"{len(times)} timed site updates (after {args.warmup} untimed) of the numpy/ARPACK restatement of "
              f"VUMPS_main.cpp on {_WORKLOAD[0]}, each cycle of two (site 0, site 1: one sweep) starting from the "
              f"committed warmed state, {cores} host threads; sweeps/s = 1 / (2 x mean site update); wall "
              f"{time.perf_counter() - t0:.1f} s incl. the untimed environment solves"
              + (f"; the {REF_BUDGET_S:.0f} s budget ended the run after {len(times)} of {args.steps} timed steps"
                 if cut else ""))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": ws,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": 1e3 * t_site,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": _workload_desc(), "implementation": "CPU restatement of the reference (oracle)",
                       "step": "one site update of the first sweep from the warmed state (half a sweep)",
                       "budget_s": REF_BUDGET_S, "truncated_by_budget": cut,
                       "ms_per_site_update": [round(1e3 * t, 1) for t in times[:4]],
                       # per site (the two site updates of a sweep differ several-fold), the median
                       "median_s_per_site": [float(np.median(times[k::2])) if len(times) > k else None
                                             for k in (0, 1)],
                       "sweeps_per_s_from_medians": (1.0 / (float(np.median(times[0::2]))
                                                            + float(np.median(times[1::2]))))
                       if len(times) > 1 else None},
            "cpu_baseline": {"value": value, "unit": "sweeps/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------

def _time_hac_applies(torch, plan, n, stream, reps=APPLIES_PER_STEP):
    """Average duration of one H_AC apply (one grouped-GEMM launch, or pack + tcgen05
    launches in mixed mode), CUDA events on the launching stream, L2 flushed before."""
    from imps_cpp_tools_gb300 import _native as N
    lib = N.load()
    X = torch.randn(reps, n, dtype=torch.float64, device="cuda")
    Y = torch.empty_like(X)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for j in range(3):
        lib.imps_hac_apply(plan.handle, X[j].data_ptr(), Y[j].data_ptr(), N.MEM_DEVICE)
    times = []
    for _ in range(5):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for j in range(reps):
            st = lib.imps_hac_apply(plan.handle, X[j].data_ptr(), Y[j].data_ptr(), N.MEM_DEVICE)
            if st < 0:
                raise N.ImpsError(st, "imps_hac_apply")
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3 / reps)
    return float(np.median(times))


_CTX = [None]


def _start_state():
    """The start state of the timed sweeps: the committed warmed state of the workload if there
    is one, else the same warm-up computed on the device (seed 1, WARM_SWEEPS sweeps of the
    tolerance schedule).  Returns (host state, description)."""
    from imps_cpp_tools_gb300 import workload as W
    st = W.load_warm_state(_WORKLOAD[0])
    if st is not None:
        return st, f"tests/golden/warm_{_WORKLOAD[0]}.npz ({W.WARM_SWEEPS[_WORKLOAD[0]]} schedule sweeps from seed 1)"
    st, _, _ = W.warm_on_device(_CTX[0], _WORKLOAD[0])
    return st, f"{W.WARM_SWEEPS[_WORKLOAD[0]]} schedule sweeps from seed 1 on the device"


_MIXED_TM = [False]
_NCV = [126]
_AUTOTUNE = [True]
_CONCURRENT = [True]


def _new_vumps(precision, state):
    import torch
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    model, fn, params = configs.WORKLOADS[_WORKLOAD[0]]
    init = {k: [torch.from_numpy(np.ascontiguousarray(a)).to("cuda") for a in state[k]] for k in ("AL", "AR", "C")}
    # eig_margin 1: the device Lanczos stops at the configured tolerance itself, as ARPACK does
    return VumpsGPU(_CTX[0], model, dims0=fn(), init_state=init, fixed_tol=TIMED_TOLS["eig"],
                    InvETol=TIMED_TOLS["gmres"], eig_margin=1.0, precision=precision,
                    mixed_tm=_MIXED_TM[0] and precision != "fp64", lanczos_ncv=_NCV[0], autotune=_AUTOTUNE[0],
                    concurrent=_CONCURRENT[0], verbose=True, **params)


def _run_vumps(torch, precision, state, steps, warmup, stream, clocks=None, e2e=False, per_sweep=False):
    """W warm-up sweeps, then K device-timed sweeps (CUDA events on the launching stream), from
    `state`.  With e2e, every timed step also uploads the MPS state from pinned host memory
    before the sweep and reads the state and the energies back after it (wall clock around all
    three)."""
    from imps_cpp_tools_gb300 import _native as N
    v = _new_vumps(precision, state)
    E_first = None
    for i in range(warmup):
        E, _, _ = v.sweep()
        if i == 0:
            E_first = E.copy()
    torch.cuda.synchronize()
    lib = N.load()
    host = {k: [t.detach().cpu().pin_memory() for t in getattr(v, k)] for k in ("AL", "AR", "C")} if e2e else None
    h2d = sum(t.numel() * 8 for k in host for t in host[k]) if e2e else 0
    l0 = lib.imps_launch_count()
    s0 = dict(v.stats)
    if clocks:
        clocks.start()
    times, walls, applies_each = [], [], []
    torch.cuda.nvtx.range_push(f"timed_sweeps_{precision}")  # ncu --nvtx-include selects these
    for _ in range(steps):
        a0 = v.stats["lanczos_applies"]
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        if e2e:
            for k in ("AL", "AR", "C"):
                for j, t in enumerate(host[k]):
                    getattr(v, k)[j].copy_(t, non_blocking=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        E, F, prec = v.sweep()
        e1.record(stream)
        if e2e:
            for k in ("AL", "AR", "C"):
                for j, t in enumerate(getattr(v, k)):
                    host[k][j].copy_(t, non_blocking=True)
        torch.cuda.synchronize()
        walls.append(time.perf_counter() - w0)
        times.append(e0.elapsed_time(e1) * 1e-3)
        applies_each.append(v.stats["lanczos_applies"] - a0)
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop() if clocks else None
    launches = lib.imps_launch_count() - l0
    counts = {k: v.stats[k] - s0.get(k, 0) for k in v.stats}
    return {"v": v, "times": times, "walls": walls, "E": E, "F": F, "prec": prec, "launches": launches,
            "counts": counts, "clocks": clk, "h2d": h2d, "E_first": E_first, "applies_each": applies_each}


def run_vumps(args):
    import torch
    import torch.distributed as dist
    from imps_cpp_tools_gb300 import blocks as B

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    ctx = B.Context(local)
    _CTX[0] = ctx
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    state, state_src = _start_state()

    # the headline precision (timed with clocks and end to end) and the other one for comparison,
    # from the same start state
    other = "bf16x6" if args.precision == "fp64" else "fp64"
    _MIXED_TM[0] = bool(getattr(args, "mixed_tm", False))
    _NCV[0] = int(getattr(args, "ncv", 126))
    _AUTOTUNE[0] = not getattr(args, "no_autotune", False)
    roth = None if getattr(args, "headline_only", False) else _run_vumps(torch, other, state, args.steps, args.warmup,
                                                                            stream)
    if ws > 1:
        dist.barrier()
    rmx = _run_vumps(torch, args.precision, state, args.steps, args.warmup, stream, ClockSampler(local), e2e=True)
    if roth is None:
        roth = rmx
    r64, rsp = (rmx, roth) if args.precision == "fp64" else (roth, rmx)
    t_step = float(np.mean(rmx["times"]))
    t_wall = float(np.mean(rmx["walls"]))
    if ws > 1:
        t_step, t_wall = _max_over_ranks(dist, [t_step, t_wall], "cuda")
    value = ws / t_step  # replicas: every rank runs its own sweeps
    E64, Emx = r64["E"], rsp["E"]
    dE = float(abs(Emx.mean() - E64.mean()))

    # H_AC TFLOP/s on the final-state plans (site 0)
    v64, vmx = r64["v"], rsp["v"]
    n = v64.LA[0].nelem
    flops = v64.flops_hac[0]
    t_hac64 = _time_hac_applies(torch, v64.p_hac[0], n, stream)
    t_hacmx = _time_hac_applies(torch, vmx.p_hac[0], n, stream)
    peaks = _peaks()
    bf16_peak = peaks.get("bf16_tflops", 1893.6)
    fp64_peak = _fp64_peak_tflops(torch)
    tile, splits, _ = v64.p_hac[0].stage_shape(0)
    h_ac = {"fp64_tflops": flops / t_hac64 / 1e12, "mixed_tflops": flops / t_hacmx / 1e12,
            "flops_per_apply": flops, "fp64_us": t_hac64 * 1e6, "mixed_us": t_hacmx * 1e6,
            "fp64_launch_shape": {"tile": tile, "splits": splits,
                                  "source": "autotuner" if _AUTOTUNE[0] else "makespan estimate"}}
    fp64_src = ("dense FP64 matmul (torch, cuBLAS DGEMM 4096^3) measured in this run: GB300 has no FP64 tensor "
                "rate, the FP64 pipe bounds this kernel (not in MEASURED_PEAKS.json)")
    if args.precision == "bf16x6":
        achieved = 6 * flops / t_hacmx / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved / bf16_peak, "traffic": NCU_TRAFFIC_BYTES["bf16x6"],
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst), of measured",
                "kernel": "tc_gemm_kernel + pack_kernel (H_AC apply, 6 split-BF16 products per FP64 flop)",
                "achieved_fp64_equivalent_tflops": flops / t_hacmx / 1e12,
                "fp64_engine": {"achieved": flops / t_hac64 / 1e12, "peak": fp64_peak,
                                "frac": flops / t_hac64 / 1e12 / fp64_peak, "peak_source": fp64_src}}
    else:
        achieved = flops / t_hac64 / 1e12
        roof = {"bound": "fp64_pipe", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak, "traffic": NCU_TRAFFIC_BYTES["fp64"], "peak_source": fp64_src,
                "kernel": "grouped_gemm_f64 (H_AC apply; the dominant kernel of the timed sweeps)",
                "split_bf16_engine": {"achieved_fp64_equivalent_tflops": flops / t_hacmx / 1e12,
                                      "tensor_tflops": 6 * flops / t_hacmx / 1e12, "tensor_peak": bf16_peak,
                                      "tensor_frac": 6 * flops / t_hacmx / 1e12 / bf16_peak}}

    e2e = {"value": ws / t_wall, "unit": "sweeps/s", "h2d_bytes_per_step": rmx["h2d"],
           "d2h_bytes_per_step": rmx["h2d"] + 16, "ms_per_step": 1e3 * t_wall,
           "path": "VumpsGPU.sweep (public driver) with the MPS state uploaded from pinned host memory before "
                   "and read back after every timed sweep"}

    cpu, parity = None, None
    if rank == 0 and not args.no_cpu:
        # bounded CPU sample: one sweep (two site updates) of the oracle from the same start state
        times, E_cpu, cores, cut = cpu_site_updates(_WORKLOAD[0], state, 0, 2, CPU_SAMPLE_BUDGET_S)
    if rank == 0 and not args.no_cpu and len(times) == 2:
        t_cpu = float(np.sum(times))
        cpu = {"value": 1.0 / t_cpu, "unit": "sweeps/s", "cores": cores, "kind": "port",
               "sample": f"one sweep (2 site updates, {t_cpu:.1f} s) of the numpy/ARPACK restatement of VUMPS_main.cpp "
                         f"from the start state of the timed sweeps, same tolerances, {cores} host threads"}
        if E_cpu is not None and r64["E_first"] is not None:
            parity = {"what": "energies after the first sweep from the same start state: GPU FP64 vs the oracle",
                      "gpu": [float(x) for x in r64["E_first"]], "oracle": [float(x) for x in E_cpu],
                      "max_abs_diff": float(np.abs(np.asarray(r64["E_first"]) - np.asarray(E_cpu)).max())}
    line = {"metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x6->f32 applies, f64 Krylov/decompositions" if args.precision == "bf16x6"
            else "f64", "data": "synthetic",
            "config": {"workload": _workload_desc(), "precision": args.precision, "start_state": state_src,
                       "lanczos_ncv": _NCV[0], "autotune": _AUTOTUNE[0], "concurrent_solves": _CONCURRENT[0],
                       "l2": "working set (~40 MB) is L2-resident by design; H_AC timing flushes L2 (512 MB write)",
                       "parallelism": f"replicas x{ws}"},
            "fp64": {"sweeps_per_s": 1.0 / float(np.mean(r64["times"])), "ms_per_step": 1e3 * float(np.mean(r64["times"])),
                     "energy": float(E64.mean()), "grad_norm": float(r64["F"].max()), "counts": r64["counts"]},
            "mixed": {"sweeps_per_s": 1.0 / float(np.mean(rsp["times"])), "ms_per_step": 1e3 * float(np.mean(rsp["times"])),
                      "energy": float(Emx.mean()), "grad_norm": float(rsp["F"].max()), "counts": rsp["counts"],
                      "policy": "H_AC/H_C Lanczos on split-BF16 (tcgen05) applies while the tolerance is above "
                                "their 2e-7 floor, FP64 applies below it; GMRES "
                                + ("split-BF16 TM with FP64-residual refinement" if _MIXED_TM[0] else "FP64 TM")
                                + "; Krylov vectors, reorthogonalisation, decompositions, gradient and energy FP64"},
            "dE_mixed_vs_fp64": dE,
            "speedup_mixed_vs_fp64": float(np.mean(r64["times"])) / float(np.mean(rsp["times"])),
            "parity_vs_oracle": parity,
            "h_ac": h_ac, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": rmx["launches"],
            "clocks": rmx["clocks"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def run_trace(args):
    """--mode trace: the timed FP64 sweeps under torch.profiler (CUPTI kernel records): the
    summed duration of every kernel the sweeps launch against the wall time of the sweeps, and
    the kernels by total time.  The difference is what launch gaps, host round trips and the
    Python driver cost; the profiler's own per-launch overhead is part of it."""
    import torch
    from torch.profiler import ProfilerActivity, profile
    from imps_cpp_tools_gb300 import blocks as B
    ctx = B.Context(0)
    _CTX[0] = ctx
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    _NCV[0] = int(args.ncv)
    _AUTOTUNE[0] = not args.no_autotune
    state, src = _start_state()
    v = _new_vumps(args.precision, state)
    for _ in range(args.warmup):
        v.sweep()
    torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            v.sweep()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    per = {}
    for e in prof.key_averages():
        dt = getattr(e, "device_time_total", None)
        if dt is None:
            dt = getattr(e, "cuda_time_total", 0.0)
        if dt and e.count:
            per[e.key] = (per.get(e.key, (0.0, 0))[0] + dt * 1e-6, e.count)
    # kernels only (memcpy/memset records carry "Memcpy"/"Memset" keys)
    kern = {k: t for k, t in per.items() if not k.startswith(("Memcpy", "Memset", "cudaLaunch"))}
    total = sum(t for t, _ in kern.values())
    top = sorted(kern.items(), key=lambda kv: -kv[1][0])[:12]
    print(json.dumps({"mode": "trace", "workload": _WORKLOAD[0], "precision": args.precision, "sweeps": args.steps,
                      "start_state": src, "wall_s_per_sweep": wall / args.steps,
                      "kernel_s_per_sweep": total / args.steps, "wall_over_kernel": wall / max(total, 1e-12),
                      "kernels": [{"name": k[:100], "s_per_sweep": t / args.steps, "launches": c,
                                   "share": t / max(total, 1e-12)} for k, (t, c) in top]}), flush=True)


def _build_cpp_vumps():
    """Compile tests/native/cpp_vumps_check.cpp (the C++ VUMPS driver include/imps_vumps.hpp over
    the C ABI) against the in-tree library."""
    import shutil
    from pathlib import Path
    from imps_cpp_tools_gb300 import _native as N
    gxx, nvcc = shutil.which("g++"), shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = Path(nvcc).resolve().parent.parent
    N.load()
    lib = Path(N.lib_path()).parent
    exe = Path(ROOT) / "imps_cpp_tools_gb300" / "_lib" / "cpp_vumps_check"
    cmd = [gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", str(cuda / "include"),
           os.path.join(ROOT, "tests", "native", "cpp_vumps_check.cpp"), "-L", str(lib), "-limps_gb300",
           "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{lib}", f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def run_cpp(args):
    """--mode cpp: the timed sweeps of the default measurement run by the C++ host driver
    (include/imps_vumps.hpp, no Python in the loop) from the same warmed state and at the same
    tolerances, next to the Python driver: sweeps/s of both and the largest energy difference
    of their sweeps."""
    import torch
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300 import models
    from imps_cpp_tools_gb300 import workload as W
    ctx = B.Context(0)
    _CTX[0] = ctx
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    name = _WORKLOAD[0]
    model, d, I2K, h, dimvec = W.bond_layouts(name)
    hnnz = models.h_nonzeros(h)
    state, src = _start_state()
    nsw = args.warmup + args.steps
    lines = [f"{d} {len(I2K[0])}", " ".join(str(x) for q in I2K for x in q)]
    for b in range(2):
        lines.append(str(len(dimvec[b])))
        lines += [" ".join(str(x) for x in q) + f" {m}" for q, m in sorted(dimvec[b].items())]
    lines.append(str(len(hnnz)))
    lines += [f"{r} {c} {v!r}" for (r, c, v) in hnnz]
    lines.append(f"{nsw} {TIMED_TOLS['eig']!r} {TIMED_TOLS['gmres']!r} 1.0 {0 if args.no_autotune else 1} "
                 f"{0 if args.serial_solves else 1}")
    for k in ("AL", "AR", "C"):
        for n in range(2):
            lines.append(" ".join(repr(float(x)) for x in state[k][n]))
    inp = os.path.join(ROOT, "imps_cpp_tools_gb300", "_lib", f"cpp_vumps_{name}.txt")
    with open(inp, "w") as f:
        f.write("\n".join(lines) + "\n")
    exe = _build_cpp_vumps()
    r = subprocess.run([str(exe), inp], capture_output=True, text=True, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    rows = [list(map(float, ln.split()[2:])) for ln in r.stdout.splitlines() if ln.startswith("sweep ")]
    cpp_ms = [row[6] for row in rows[args.warmup:]]
    cpp_applies = [int(rows[i][7] - (rows[i - 1][7] if i else 0)) for i in range(len(rows))][args.warmup:]
    _AUTOTUNE[0] = not args.no_autotune
    py = _run_vumps(torch, "fp64", state, args.steps, args.warmup, stream, per_sweep=True)
    E_py_last = py["E"]
    dE = float(np.abs(np.array(rows[-1][0:2]) - np.asarray(E_py_last)).max())
    print(json.dumps({"mode": "cpp", "workload": _workload_desc(), "start_state": src, "sweeps_timed": args.steps,
                      "cpp": {"sweeps_per_s": 1e3 / float(np.mean(cpp_ms)), "ms_per_sweep": float(np.mean(cpp_ms)),
                              "ms_each": [round(x, 1) for x in cpp_ms], "lanczos_applies_each": cpp_applies,
                              "energy": float(np.mean(rows[-1][0:2])), "grad_norm": max(rows[-1][2:4]),
                              "timing": "wall clock per sweep, device synchronised before and after"},
                      "python": {"sweeps_per_s": 1.0 / float(np.mean(py["times"])),
                                 "ms_per_sweep": 1e3 * float(np.mean(py["times"])),
                                 "ms_each": [round(1e3 * x, 1) for x in py["times"]],
                                 "lanczos_applies_each": py["applies_each"], "energy": float(E_py_last.mean()),
                                 "grad_norm": float(py["F"].max()), "timing": "CUDA events around each sweep"},
                      "max_abs_dE_last_sweep": dE}), flush=True)


def run_hac(args):
    import torch
    from imps_cpp_tools_gb300 import _native as N
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300.workload import HacWorkload
    ctx = B.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    w = HacWorkload(ctx, args.workload)
    if not args.no_autotune:
        w.plan.autotune()
    if args.precision == "bf16x6":
        w.plan.set_precision(N.PREC_BF16X6)
    t = _time_hac_applies(torch, w.plan, w.n, stream)
    print(json.dumps({"mode": "hac", "workload": args.workload, "precision": args.precision, "us_per_apply": t * 1e6,
                      "tflops": w.flops / t / 1e12, "flops_per_apply": w.flops,
                      "bytes_per_apply": w.bytes_per_apply(), "launch_shape": w.plan.stage_shape(0)[:2]}),
          flush=True)


def run_krylov(args):
    import torch
    from imps_cpp_tools_gb300 import _native as N
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300 import ops
    from imps_cpp_tools_gb300.workload import HacWorkload
    ctx = B.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    w = HacWorkload(ctx, args.workload)
    if args.precision == "bf16x6":
        w.plan.set_precision(N.PREC_BF16X6)
    lib = N.load()
    x0 = torch.randn(w.n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x0)
    res = []
    for rep in range(4):
        x = x0.clone()
        torch.cuda.synchronize()
        l0 = lib.imps_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        # FP64: unreachable tolerance (the full 8 cycles run); split-BF16: its own floor, so that
        # no FP64 finishing phase is timed
        tol = 1e-30 if args.precision == "fp64" else 2e-7
        ev, na, conv = ops.eigs_rs(w.plan, x, tol, ncv=64, maxit=8)
        e1.record(stream)
        torch.cuda.synchronize()
        t_solve = e0.elapsed_time(e1) * 1e-3
        launches = lib.imps_launch_count() - l0
        e0.record(stream)
        for _ in range(na):
            lib.imps_hac_apply(w.plan.handle, x0.data_ptr(), y.data_ptr(), N.MEM_DEVICE)
        e1.record(stream)
        torch.cuda.synchronize()
        t_apply = e0.elapsed_time(e1) * 1e-3
        if rep:
            res.append((t_solve, t_apply, na, launches))
    t_solve, t_apply, na, launches = (float(np.median([r[i] for r in res])) for i in range(4))
    print(json.dumps({"mode": "krylov", "workload": args.workload, "precision": args.precision, "applies": na,
                      "us_per_iteration": 1e6 * t_solve / na, "us_per_apply": 1e6 * t_apply / na,
                      "us_overhead_per_iteration": 1e6 * (t_solve - t_apply) / na,
                      "launches_per_iteration": launches / na}), flush=True)


def run_excitations(args):
    """Excitation energies (Excitations_main.cpp:255-297), configs' excitation workload: the XXZ
    ground state at D=256 grown by bond expansion (ExpandFromH, VUMPS_main.cpp:270-308) from D=32
    and converged to |grad| < 1e-10; then the 4 lowest Sz = +1 energies (charge label K = 2) at 32
    momenta p = pi (k + 1/2) / 32, k = 0..31, all momenta in one batched run (ExcitationsBatchGPU:
    one launch per H_eff program stage and per transfer-matrix stage for every momentum, the
    Lanczos runs in lockstep).  Beside it: the per-momentum path (ExcitationsGPU) on --steps of
    the momenta (time per momentum, energy agreement) and one H_eff apply of the oracle on the
    host (the CPU cost per apply)."""
    import torch
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300.excitations import ExcitationsBatchGPU, ExcitationsGPU, excitation_inputs
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    ctx = B.Context(0)
    ctx.set_stream(torch.cuda.current_stream())
    t0 = time.perf_counter()
    v = VumpsGPU(ctx, "xxz", dims0=configs.xxz_bond_dims(32, 4, 4.0), seed=1, tolmin=1e-12, InvETol=1e-12, mmax=256,
                 dmmax=32, expand_pause=3, J=1.0, Delta=-1.0)
    nsw, F = 0, None
    for nsw in range(1, 201):
        E, F, _ = v.sweep()
        D = sum(v.LB[0].dims().values())
        if nsw % 10 == 0:
            print(f"[excitations] sweep {nsw}: D={D} E={E.mean():.12f} |grad|={F.max():.2e} "
                  f"{time.perf_counter() - t0:.1f}s", file=sys.stderr, flush=True)
        if D >= 256 and F.max() < 1e-10:
            break
    torch.cuda.synchronize()
    t_gs = time.perf_counter() - t0
    inp = excitation_inputs(v, (2,), tol=1e-12)
    args_ = (inp["AL"], inp["AR"], inp["NL"], inp["HLtot"], inp["HRtot"], inp["h"], inp["d"], inp["xdims"])
    print(f"[excitations] ground state: {nsw} sweeps, D={D}, {t_gs:.1f}s", file=sys.stderr, flush=True)
    P = int(args.momenta)
    ps = [np.pi * (k + 0.5) / P for k in range(P)]
    kfs = [np.exp(1j * p) for p in ps]
    tb = time.perf_counter()
    ex = ExcitationsBatchGPU(ctx, *args_, kfs, tol=1e-12, verbose=True)
    t_build = time.perf_counter() - tb
    tb = time.perf_counter()
    ev_b, conv_b, na_b = ex.energies(nev=4, eig_tol=1e-10)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - tb
    print(f"[excitations] batched: {P} momenta, {na_b} applies, {ex.stats['gmres_iters']} GMRES iterations, "
          f"{t_batch:.1f}s", file=sys.stderr, flush=True)
    # the per-momentum path on a sample of the momenta
    single = ExcitationsGPU(ctx, *args_, tol=1e-12)
    sample = [int(round(x)) for x in np.linspace(0, P - 1, max(1, min(args.steps, P)))]
    rows, t_single = [], 0.0
    for k in sample:
        ts = time.perf_counter()
        ev, conv = single.energies(kfs[k], nev=4, eig_tol=1e-10)
        torch.cuda.synchronize()
        dt = time.perf_counter() - ts
        t_single += dt
        rows.append({"p": ps[k], "s": dt, "max_abs_diff_vs_batched": float(np.abs(np.array(ev) - np.array(ev_b[k])).max()),
                     "converged": bool(conv)})
    # CPU: one H_eff apply of the oracle on the same inputs (host copies)
    cpu = None
    if not args.no_cpu:
        from oracle import imps_oracle as O
        rng = np.random.default_rng(1)
        X = [{qi: (qo, rng.standard_normal((ml, mr)) + 1j * rng.standard_normal((ml, mr))) for (qi, qo, ml, mr) in dd}
             for dd in inp["xdims"]]
        tc = time.perf_counter()
        O.ApplyHeff(X, kfs[0], inp["AL"], inp["AR"], inp["NL"], inp["h"], inp["d"], inp["HLtot"], inp["HRtot"], tol=1e-12)
        cpu = {"s_per_heff_apply": time.perf_counter() - tc, "cores": os.cpu_count(), "kind": "port"}
    mtot = sum(r * c for dd in inp["xdims"] for (_, _, r, c) in dd)
    t_per_single = t_single / max(len(rows), 1)
    print(json.dumps({"mode": "excitations", "metric": "excitation energies, %d momenta x 4 bands (s per run)" % P,
                      "workload": "XXZ D=%d ground state (VumpsGPU with ExpandFromH from D=32, %d sweeps, |grad| "
                      "%.1e, E=%.10f), K = Sz +1, 4 lowest states, p = pi (k + 1/2)/%d"
                      % (sum(v.LB[0].dims().values()), nsw, float(F.max()), float(E.mean()), P),
                      "mtot": mtot, "ground_state_s": t_gs, "batched": {
                          "momenta": P, "s": t_batch, "build_s": t_build, "batched_applies": na_b,
                          "gmres_iters": ex.stats["gmres_iters"], "converged": all(conv_b),
                          "energies": [[float(x) for x in e] for e in ev_b], "p": ps},
                      "per_momentum": {"sampled": rows, "s_per_momentum": t_per_single,
                                       "s_for_all_extrapolated": t_per_single * P},
                      "speedup_batched_vs_per_momentum": t_per_single * P / t_batch,
                      "cpu_baseline": cpu, "E0": inp["E0"]}), flush=True)


def run_adjoint(args):
    """The adjoint check's shapes: dE/dA_L and dE/dcouplings of the energy density at the
    left-isometric unit cell of a VUMPS state (a few sweeps from the seeded random start) for
    XXZ D=256 with Delta = 0.5, 1.0, 1.5 (antiferromagnetic sign convention of the reference:
    Delta = -0.5, -1, -1.5) and Hubbard D=256 with U = 2, 4.  Per case: device gradient
    evaluations timed with CUDA events over `steps` repetitions after `warmup`, the gradient's
    difference from the oracle, and the oracle (numpy, all host threads) timed on one evaluation."""
    import torch
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300.adjoint import CouplingGradientGPU, EnergyGradientGPU
    from imps_cpp_tools_gb300.excitations import bd_to_host, mps_to_host
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    from oracle import imps_oracle as O  # the checker and the CPU baseline leg
    ctx = B.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    cases = [("xxz_d256", {"Delta": -0.5}), ("xxz_d256", {"Delta": -1.0}), ("xxz_d256", {"Delta": -1.5}),
             ("hubbard_d256", {"U": 2.0}), ("hubbard_d256", {"U": 4.0})]
    rows = []
    for name, over in cases:
        model, fn, params = configs.WORKLOADS[name]
        params = {**params, **over}
        v = VumpsGPU(ctx, model, dims0=fn(), seed=1, **params)
        for _ in range(3):
            v.sweep()
        R = bd_to_host(v.C[0], v.LB[0])
        R = O.bd_mul(R, O.bd_t(R))
        Rd = torch.from_numpy(O.bd_vec(R)).to("cuda")
        g = EnergyGradientGPU(ctx, v.LA, v.LB, v.hnnz, v.d, tol=1e-11)
        cg = CouplingGradientGPU(ctx, v.LA, v.LB, model, v.d, **params)
        for _ in range(args.warmup):
            g(v.AL[0], v.AL[1], Rd)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        it0 = g.stats["gmres_iters"]
        e0.record(stream)
        for _ in range(max(args.steps, 1)):
            G0, G1, e, _, conv = g(v.AL[0], v.AL[1], Rd)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / max(args.steps, 1)
        dcoup = cg(v.AL[0], v.AL[1], Rd)
        AL = [mps_to_host(v.AL[n], v.LA[n], v.d) for n in range(2)]
        tc = time.perf_counter()
        Gref, eref = O.energy_gradient(AL, R, v.hnnz, tol=1e-11, solver=O.invert_e_proj_scipy)
        t_cpu = time.perf_counter() - tc
        err = max(float(np.linalg.norm(G0.cpu().numpy() - O.mps_vec(Gref[0])) / np.linalg.norm(O.mps_vec(Gref[0]))),
                  float(np.linalg.norm(G1.cpu().numpy() - O.mps_vec(Gref[1])) / np.linalg.norm(O.mps_vec(Gref[1]))))
        rows.append({"workload": name, "params": params, "energy": e, "converged": bool(conv),
                     "ms_per_gradient": ms, "gradients_per_s": 1e3 / ms,
                     "gmres_iters_per_gradient": (g.stats["gmres_iters"] - it0) / max(args.steps, 1),
                     "dE_dcouplings": dcoup, "rel_diff_vs_oracle": err, "oracle_s_per_gradient": t_cpu})
    print(json.dumps({"mode": "adjoint", "metric": "energy-density gradients/s (dE/dA_L via TM/H_AC adjoints + "
                      "transposed-GMRES fixed-point adjoint)", "cpu_cores": os.cpu_count(), "cases": rows}),
          flush=True)


def run_expand(args):
    """ExpandFromH (MPSBlockUtilities.hpp:409-601) at the bond right of site 0 of the seeded
    XXZ D=512 and Hubbard D=1024 starts, dmmax 20 (VUMPS_main.cpp:31): device wall time per
    expansion (host bookkeeping, planning and the device programs, null spaces and SVDs,
    synchronised), the oracle (numpy, all host threads) on the same state, and whether both
    add the same states per charge."""
    import torch
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300 import configs
    from imps_cpp_tools_gb300 import expand as E
    from imps_cpp_tools_gb300.excitations import bd_to_host, mps_to_host
    from imps_cpp_tools_gb300.vumps import VumpsGPU
    from oracle import imps_oracle as O  # the checker and the CPU baseline leg
    ctx = B.Context(0)
    ctx.set_stream(torch.cuda.current_stream())
    rows = []
    for name in ("xxz_d512", "hubbard_d1024"):
        model, fn, params = configs.WORKLOADS[name]
        v = VumpsGPU(ctx, model, dims0=fn(), seed=1, **params)
        call = (ctx, v.I2K, v.hnnz, v.LA[0], v.AL[0], v.LA[1], v.AR[1], v.LB[1], v.C[1], 20)
        for _ in range(args.warmup):
            E.expand_from_h(*call)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(max(args.steps, 1)):
            res = E.expand_from_h(*call)
        torch.cuda.synchronize()
        ms = 1e3 * (time.perf_counter() - t0) / max(args.steps, 1)
        AL = mps_to_host(v.AL[0], v.LA[0], v.d)
        AR = mps_to_host(v.AR[1], v.LA[1], v.d)
        Cb = bd_to_host(v.C[1], v.LB[1])
        tc = time.perf_counter()
        _, _, _, dmo = O.ExpandFromH(v.hnnz, v.I2K, AL, AR, Cb, 20)
        t_cpu = time.perf_counter() - tc
        same = {q: k for q, k in res["dm"].items() if k} == {q: k for q, k in dmo.items() if k}
        rows.append({"workload": name, "bond_dim": sum(v.LB[1].dims().values()), "added": sum(res["dm"].values()),
                     "ms_per_expansion": ms, "oracle_s_per_expansion": t_cpu, "same_states_as_oracle": same,
                     "svd_converged": bool(res["converged"])})
    print(json.dumps({"mode": "expand", "metric": "ExpandFromH wall time per expansion (ms)", "dmmax": 20,
                      "cpu_cores": os.cpu_count(), "cases": rows}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=47)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="vumps", choices=["vumps", "hac", "krylov", "excitations", "adjoint", "expand", "trace", "cpp"])
    ap.add_argument("--workload", default="xxz_d512")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "bf16x6"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--mixed-tm", action="store_true",
                    help="split-BF16 transfer matrices in the mixed arm's GMRES solves (FP64-residual refinement)")
    ap.add_argument("--headline-only", action="store_true", help="skip the other precision's arm (profiling)")
    ap.add_argument("--no-autotune", action="store_true", help="launch shapes from the makespan estimate only")
    ap.add_argument("--momenta", type=int, default=32, help="momenta of --mode excitations")
    ap.add_argument("--serial-solves", action="store_true",
                    help="run the H_C eigensolves after the H_AC eigensolve on one stream")
    ap.add_argument("--ncv", type=int, default=126, help="Krylov dimension of the H_AC / H_C Lanczos solves")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    _CONCURRENT[0] = not args.serial_solves
    if args.mode in ("vumps", "trace", "cpp") or args.impl == "reference":
        if args.workload not in WORKLOAD_DESCS:
            raise SystemExit(f"--workload for the VUMPS bench: one of {sorted(WORKLOAD_DESCS)}")
        _WORKLOAD[0] = args.workload
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "hac":
        run_hac(args)
    elif args.mode == "krylov":
        run_krylov(args)
    elif args.mode == "adjoint":
        run_adjoint(args)
    elif args.mode == "expand":
        run_expand(args)
    elif args.mode == "excitations":
        run_excitations(args)
    elif args.mode == "trace":
        run_trace(args)
    elif args.mode == "cpp":
        run_cpp(args)
    else:
        run_vumps(args)


if __name__ == "__main__":
    main()
