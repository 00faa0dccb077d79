"""Benchmark of the GB300 RK3 duct step (RK_DUCT x 3 with REM_DIV_CURV).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Workload: the stratified Ekman layer 512 x 385 x 257 (NX x NY+2 x NZ+2;
NY = 384 rounded up to MUDPACK form), Re = 1000, Pr = 0.7, Ri = 0.1,
dt = 3e-4, seeded synthetic fields (laminar Ekman spiral + 1% Gaussian
noise), FP64 fields, every per-kx Poisson problem (171 complex ones) driven
to a relative residual of 1e-8 (the singular kx = 0 mode too, after its
right-hand side is projected onto the operator's range).  Prints one JSON line: RK3 steps/s of the batched
mixed-precision projection over K steps after W warm-up steps, timed with
CUDA events on the solver's stream, and beside it the plain FP64 MUDPACK
path on the same workload; the fields are larger than the 126 MB L2, so no
flush is needed between steps.  For N > 1 each rank
runs an independent replica on its own GPU (the path does not shard) and
the value is the sum over ranks.

The line also carries "les": the LES case 1024 x 513 x 385 at Re = 2000,
Ri = 0.15, dt = 1.5e-4 (dynamic Smagorinsky, les_chan / les_chan_th),
timed over one C_DYN period of five steps with the same mixed-precision
method, the plain FP64 path beside it,
the LES kernels' share and roofline, and one oracle LES substep on the host
cores (skip with --no-les), and "ensemble": eight runs on uneven seeded grids
(64..256 points per side) stepped together on the GPU, against the same
members one after another and the plain path's members (skip with
--no-ensemble).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD = "ekman_strat_512x385x257"
MG_TOL = 1e-8
# the mixed method's state path: 1 float-float transforms and ADI, 2 FP32
# transforms and ADI on increments (ek_params.ff_arith)
FF_ARITH = 2
STATE_DTYPE = {
    1: "mixed: f64 spectral state and spectral terms; float-float (~48-bit) physical fields, state transforms "
       "and ADI; f32 nonlinear-term transforms and V-cycles; float-float Poisson residual and update",
    2: "mixed: f64 spectral state and spectral terms; f32 physical fields, with the ADI and the state "
       "transforms in f32 on increments (CU += FFT(increment)); f32 nonlinear-term transforms and V-cycles; "
       "float-float Poisson residual and update",
}
STATE_PRECISION = {
    1: "FP64 spectral fields, spectral right-hand side and projection; physical fields as float-float planes "
       "(~48-bit): state-carrying x-transforms and ADI in float-float; the nonlinear-term transforms and the "
       "transforms of the explicit increment S = R - J phi in FP32; Poisson: float-float residual and update "
       "around FP32 V-cycles",
    2: "FP64 spectral fields, spectral right-hand side and projection; physical fields in FP32; each ADI sweep "
       "solves in FP32 for the increment of its field (the J phi terms cancel algebraically) and the FP32 "
       "transform of the total increment is added to the FP64 spectral state; the nonlinear-term transforms "
       "and the transforms of the explicit increment S = R - J phi in FP32; Poisson: float-float residual "
       "and update around FP32 V-cycles",
}
METRIC = "RK3 steps/s and Poisson solves/s at 1e-8 residual: learned+batched vs plain, 1 GB300"


# DRAM traffic per algorithmic byte of a kernel class, from a committed ncu
# summary of a small case of the same kernel (one kernel, a few launches)
TRAFFIC_PROFILES = {"mg_relax": "profiles/k_f_pline_dram_traffic_512x385x257_nx128.md"}


def profiled_traffic_ratio(kernel_class: str):
    """(measured DRAM bytes / algorithmic bytes, summary path) of a kernel
    class, or (None, None) when no summary covers it."""
    import re
    rel = TRAFFIC_PROFILES.get(kernel_class)
    if rel is None:
        return None, None
    try:
        m = re.search(r"traffic_to_algorithmic:\s*([0-9.]+)", open(os.path.join(ROOT, rel)).read())
        return (float(m.group(1)), rel) if m else (None, None)
    except OSError:
        return None, None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows]
        out["sm_mhz"] = statistics.median(sm)
        out["sm_max_mhz"] = float(rows[0][2])
        out["samples"] = len(rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        out["reasons"] = sorted(reasons)
        return out


# ----------------------------------------------------------------------------
def setup_solver(device_index: int, mg_fast: int = 1, fft_fp32: int = 1, workload=WORKLOAD, ff_arith=None):
    """A solver of a named workload (or a Workload) on its own stream, with
    the initial field projected; returns (w, p, xp, yp, state, solver, stream).
    ff_arith: the state path of the mixed method (default FF_ARITH)."""
    import torch

    from ekman_bl_gb300 import build as ekbuild
    from ekman_bl_gb300.duct import DuctSolver, les_metrics_from_grid, metrics_from_grid
    from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL, WORKLOADS, workload_setup

    ekbuild.build()
    torch.cuda.set_device(device_index)
    w = WORKLOADS[workload] if isinstance(workload, str) else workload
    w.mg_tol = MG_TOL
    p, xp, yp, state = workload_setup(w, EK_MG_STOP_RESIDUAL)
    p.mg_fast = mg_fast
    p.fft_fp32 = fft_fp32
    p.ff_arith = (FF_ARITH if ff_arith is None else ff_arith) if fft_fp32 else 0
    solver = DuctSolver(p, metrics_from_grid(p, xp, yp))
    if p.les:
        solver.set_les_metrics(les_metrics_from_grid(p, xp, yp))
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    solver.upload(*state)
    solver.rem_div_curv()   # CREATE_FLOW_DUCT projects the initial field (duct.F90:3189)
    return w, p, xp, yp, state, solver, stream


def time_steps(solver, stream, steps, warmup, clocks_gpu=None, counts=None):
    """W untimed steps, then exactly `steps` RK3 steps between CUDA events on
    the solver's stream; returns (ms, max MG cycles per substep, launches,
    clock summary or None).  counts (a dict), when given, receives the real
    Poisson problems solved and left above tolerance in the timed steps."""
    import torch

    for _ in range(warmup):
        solver.step(1)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    cycles = []
    sampler = ClockSampler(clocks_gpu) if clocks_gpu is not None else None
    if sampler:
        sampler.__enter__()
    try:
        torch.cuda.synchronize()
        n0 = solver.launch_count()
        c0 = solver.mg_counters()
        with torch.cuda.stream(stream):
            start.record(stream)
            for _ in range(steps):
                solver.step(1)
                cycles.append(solver.mg_stats()["max_cycles"])
            end.record(stream)
        torch.cuda.synchronize()
        launches = solver.launch_count() - n0
        if counts is not None:
            c1 = solver.mg_counters()
            counts["solved"], counts["not_converged"] = c1[0] - c0[0], c1[1] - c0[1]
    finally:
        if sampler:
            sampler.__exit__(None, None, None)
    return start.elapsed_time(end), max(cycles) if cycles else None, launches, sampler.summary() if sampler else None


def time_poisson(solver, stream, p, nrep=3):
    """One batched solve of every active kx (real and imaginary parts together
    = one complex problem) at the tolerance; returns (ms per batch, stats)."""
    import torch

    ncomplex = p.nx // 3 + 1
    kx2 = torch.tensor([(2 * math.pi * (q // 2) / p.lx) ** 2 for q in range(2 * ncomplex)], dtype=torch.float64,
                       device="cuda")
    gen = torch.Generator(device="cpu").manual_seed(7)
    rhs = torch.randn((2 * ncomplex, p.ny + 2, p.nz + 2), generator=gen, dtype=torch.float64)
    rhs[:, 0, :] = 0
    rhs[:, -1, :] = 0
    rhs[:, :, 0] = 0
    rhs[:, :, -1] = 0
    rhs = rhs.cuda()
    phi = torch.zeros_like(rhs)
    torch.cuda.synchronize()
    solver.multigrid_mudpack_device(rhs.data_ptr(), phi.data_ptr(), kx2.data_ptr(), 2 * ncomplex)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(nrep):
            pst, _ = solver.multigrid_mudpack_device(rhs.data_ptr(), phi.data_ptr(), kx2.data_ptr(), 2 * ncomplex)
        e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / nrep, pst, ncomplex


def end_to_end(solver, shape, steps):
    """RK3 steps through the public C ABI with host buffers: every step
    uploads the state from pinned host memory, steps, and downloads the
    state.  Returns (seconds per step, bytes copied each way, steps)."""
    import torch

    pinned = [torch.empty(shape, dtype=torch.complex128, pin_memory=True).numpy() for _ in range(5)]
    cur = solver.download()
    for a, b in zip(pinned, cur):
        a[...] = b
    n = max(2, min(steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        solver.upload(*pinned)
        solver.step(1)
        solver.download(out=pinned)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / n, 5 * int(np.prod(shape)) * 16, n


def replica_throughput(ms: float, steps: int, device: str = "cuda"):
    """Whole-job RK3 steps/s of N independent replicas (the path does not
    shard): the slowest rank's time over the timed steps, all ranks' steps.
    Returns (value, ms_max); without a process group N = 1."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    return world * steps / (ms_max / 1000.0), ms_max


LEARN_FACTOR, LEARN_CHANNELS, LEARN_STEPS, LEARN_ITERS = 4, 32, 3, 300


def run_learned(solver, stream, args):
    """The learned initial guess on the same solver: collect (rhs, solution)
    pairs from LEARN_STEPS steps of its own projections, train the U-Net on
    the GPU, then time the same steps with and without the guess.  Returns
    the measurements (the multigrid tolerance is the same in both)."""
    import torch

    from ekman_bl_gb300.learned import LearnedGuess

    t0 = time.perf_counter()
    lg = LearnedGuess(solver, factor=LEARN_FACTOR, channels=LEARN_CHANNELS, seed=0)
    npairs = lg.collect(LEARN_STEPS)
    collect_s = time.perf_counter() - t0
    rep = lg.train(iters=LEARN_ITERS, batch=16, lr=2e-3)

    def run(on):
        lg.enable(on)
        ms, cyc, _, _ = time_steps(solver, stream, args.steps, 1)
        rho, mcyc = solver.last_guess_stats()
        return ms, cyc, rho, mcyc

    ms_off, cyc_off, _, mc_off = run(False)
    ms_on, cyc_on, rho, mc_on = run(True)
    solver.set_timing(True)
    solver.step(1)
    kt = solver.timing()
    solver.set_timing(False)
    lg.enable(False)
    g_ms, g_cnt, g_flops = kt.get("guess", (0.0, 0, 0.0))
    torch.cuda.synchronize()
    return {"value": round(args.steps / (ms_on / 1000.0), 4), "unit": "RK3 steps/s",
            "ms_per_step": round(ms_on / args.steps, 3),
            "same_steps_without_guess_ms_per_step": round(ms_off / args.steps, 3),
            "mean_corrections_last_substep": {"with": round(mc_on, 3), "without": round(mc_off, 3)},
            "max_corrections": {"with": cyc_on, "without": cyc_off},
            "starting_residual_ratio": round(rho, 4),
            "guess_ms_per_step": round(g_ms, 3),
            "unet_forward_tflops": round(g_flops / (g_ms / 1000.0) / 1e12, 2) if g_ms > 0 else None,
            "network": f"U-Net 4 levels x {LEARN_CHANNELS} channels, 3x3, BF16 tcgen05 tensor cores (direct FP32 first and last layers), FP32 accumulate, on the "
                       f"finest multigrid grid averaged {LEARN_FACTOR}x{LEARN_FACTOR}",
            "training": {"pairs": npairs, "collect_s": round(collect_s, 2), **{k: (round(v, 5) if isinstance(v, float)
                                                                                 else v) for k, v in rep.items()}}}


LES_WORKLOAD = "ekman_les_1024x513x385"
LES_STEPS = 5  # one C_DYN period: RK_STEP 1 of every fifth step recomputes it


def run_les(args, local):
    """The LES case (dynamic Smagorinsky, les_chan / les_chan_th): RK3
    steps/s of the mixed-precision method and of the plain FP64 path over
    one C_DYN period after the FIRST_TIME step, the LES kernels' share and
    roofline, and the oracle's LES substep on the host cores beside it."""
    import torch

    peak, peak_kind = peaks()
    w, p, _, _, _, solver, stream = setup_solver(local, 1, 1, workload=LES_WORKLOAD)
    solver.mg_autotune(reps=2)
    ms, cyc, launches, clocks = time_steps(solver, stream, LES_STEPS, 1, clocks_gpu=local)
    solver.set_timing(True)
    solver.step(LES_STEPS)
    kt = solver.timing()
    solver.set_timing(False)
    solver.close()
    per = {k: (v[0] / LES_STEPS, v[1] / LES_STEPS, v[2] / LES_STEPS) for k, v in kt.items()}
    ktot = sum(v[0] for v in per.values())
    les_ms, les_cnt, les_bytes = per.get("les", (0.0, 0, 0.0))
    roof = None
    if les_ms > 0:
        achieved = les_bytes / (les_ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "kernel": "les (line, scalar-flux and flux-addition kernels)",
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_kind": peak_kind, "share_of_step": round(les_ms / ktot, 4)}
    _, _, _, _, _, plain, pstream = setup_solver(local, 0, 0, workload=LES_WORKLOAD)
    pms, pcyc, _, _ = time_steps(plain, pstream, 2, 1)
    plain.close()
    torch.cuda.synchronize()
    out = {"workload": LES_WORKLOAD, "nx": p.nx, "ny_plus_2": p.ny + 2, "nz_plus_2": p.nz + 2,
           "model": "dynamic Smagorinsky (LES_MODEL_TYPE 2), KAPPA_T = NU_T/PR (LES_MODEL_TYPE_TH 1)",
           "value": round(LES_STEPS / (ms / 1000.0), 4), "unit": "RK3 steps/s",
           "ms_per_step": round(ms / LES_STEPS, 3), "steps": LES_STEPS, "warmup": 1,
           "mg_corrections_per_substep_max": cyc, "gpu_launches": int(launches), "clocks": clocks,
           "plain": {"value": round(2 / (pms / 1000.0), 4), "ms_per_step": round(pms / 2, 3), "steps": 2,
                     "mg_cycles_per_substep_max": pcyc},
           "speedup_vs_plain": round((LES_STEPS / ms) / (2 / pms), 3),
           "kernel_ms_per_step": {k: round(v[0], 3) for k, v in per.items()},
           "roofline": roof}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = les_cpu_baseline()
    return out


ENS_STEPS = 5


def run_ensemble(args, local):
    """The ensemble of eight stratified Ekman-layer runs on uneven grids
    (NX in {64, 128, 256}, NY+2 and NZ+2 drawn from [64, 256] with a fixed
    seed and rounded up to MUDPACK form), each with its own parameters,
    metrics and state.  Times ENS_STEPS RK3 steps of every member with the
    mixed-precision method: all members together (ekgpu_ensemble_step: each
    ensemble step is one CUDA graph launch whose parallel branches are the
    members' step graphs), the same members one after another (each with its
    own step graph), and the plain FP64 path's members together (one stream
    and host thread per member).  Members run concurrently, so the times are
    host wall clock between device-wide synchronisations."""
    import torch

    from ekman_bl_gb300.duct import ensemble_step
    from ekman_bl_gb300.params import ensemble_workloads

    def members(mixed):
        out = []
        for _, w in ensemble_workloads():
            w.mg_tol = MG_TOL
            out.append(setup_solver(local, mixed, mixed, workload=w)[5])
        return out

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    ens = ensemble_workloads()
    pts = [w.nx * w.ny2 * w.nz2 for _, w in ens]
    ms_ = members(1)
    ensemble_step(ms_, 1)  # warm-up (first solves set up their pinned stop flags)
    n0 = sum(m.launch_count() for m in ms_)
    sampler = ClockSampler(local)
    sampler.__enter__()
    try:
        t_together = timed(lambda: ensemble_step(ms_, ENS_STEPS))
    finally:
        sampler.__exit__(None, None, None)
    launches = sum(m.launch_count() for m in ms_) - n0
    t_alone = timed(lambda: [m.step(ENS_STEPS) for m in ms_])
    cyc = max(m.mg_stats()["max_cycles"] for m in ms_)
    divs = [m.divergence() for m in ms_]
    for m in ms_:
        m.close()
    pl = members(0)
    ensemble_step(pl, 1)
    t_plain = timed(lambda: ensemble_step(pl, ENS_STEPS))
    for m in pl:
        m.close()
    nm = len(ens)
    rate = nm * ENS_STEPS / t_together
    return {"members": [w.name for _, w in ens], "drawn_ny2_nz2": [list(d) for d, _ in ens],
            "points_total": int(sum(pts)), "seed": 0,
            "method": "mixed precision as the main line, default line-solve layouts; each ensemble step one CUDA "
                      "graph launch with every member's step graph as a parallel branch (ekgpu_ensemble_step)",
            "value": round(rate, 3), "unit": "member RK3 steps/s", "steps_per_member": ENS_STEPS,
            "ms_per_ensemble_step": round(t_together * 1000.0 / ENS_STEPS, 3),
            "grid_point_steps_per_s": round(sum(pts) * ENS_STEPS / t_together, 1),
            "one_after_another": {"value": round(nm * ENS_STEPS / t_alone, 3),
                                  "ms_per_ensemble_step": round(t_alone * 1000.0 / ENS_STEPS, 3)},
            "speedup_vs_one_after_another": round(t_alone / t_together, 3),
            "plain_together": {"value": round(nm * ENS_STEPS / t_plain, 3),
                               "ms_per_ensemble_step": round(t_plain * 1000.0 / ENS_STEPS, 3)},
            "speedup_vs_plain": round(t_plain / t_together, 3),
            "mg_corrections_per_substep_max": cyc, "max_divergence": max(divs),
            "gpu_launches": int(launches), "clocks": sampler.summary(),
            "timing": "host wall clock between device synchronisations (members run on 8 streams)"}


def les_cpu_baseline():
    """The oracle's LES path on the host cores, bounded sample: one substep
    (RK_STEP 1 of the FIRST_TIME step, C_DYN recomputed) of the LES case."""
    from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL, WORKLOADS, workload_setup
    from oracle import ekref

    cores = os.cpu_count() or 1
    w = WORKLOADS[LES_WORKLOAD]
    w.mg_tol = MG_TOL
    p, xp, yp, state = workload_setup(w, EK_MG_STOP_RESIDUAL)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp), threads=cores)
    o.set_les_metrics(ekref.les_metrics_from_grid(p, xp, yp))
    o.upload(*state)
    o.set_time(0.0, 1)
    t0 = time.perf_counter()
    o.rk_substep(1)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": round(1.0 / (3.0 * dt), 5), "unit": "RK3 steps/s (3 x the substep time)", "cores": cores,
            "kind": "port", "sample": f"1 substep (RK_STEP 1, C_DYN recomputed) of {LES_WORKLOAD}, "
                                      f"{cores} OpenMP threads ({dt:.1f} s)"}


def run_gpu(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    # the method measured: mixed-precision batched projection (mg_fast = 1)
    w, p, xp, yp, state, solver, stream = setup_solver(local, mg_fast=1, fft_fp32=1)
    # the autotuner picks the line solves' problems-per-block layouts (no
    # effect on results: each problem's arithmetic is the same in every layout)
    t_tune = time.perf_counter()
    tuned = solver.mg_autotune(reps=3)
    t_tune = time.perf_counter() - t_tune
    if world > 1:
        dist.barrier()
    counts = {}
    ms, mg_cycles, launches, clocks = time_steps(solver, stream, args.steps, args.warmup, clocks_gpu=local,
                                                 counts=counts)
    if world > 1:
        dist.barrier()
    value, ms_max = replica_throughput(ms, args.steps)
    div = solver.divergence()

    # per-kernel-class timing of one extra step (events around every launch)
    solver.set_timing(True)
    solver.step(1)
    kt = solver.timing()
    solver.set_timing(False)
    ktot = sum(v[0] for v in kt.values())
    pois_ms, pst, ncomplex = time_poisson(solver, stream, p)
    solves_per_s = ncomplex / (pois_ms / 1000.0)

    shape = (p.ny + 2, p.nz + 2, p.nx // 2 + 1)
    e2e_s, bytes_state, n_e2e = end_to_end(solver, shape, args.steps)
    learned = None if args.no_learned else run_learned(solver, stream, args)
    solver.close()

    # the plain FP64 GPU path (MUDPACK's smoother and cycles) at the same
    # tolerance, same workload, for the method-vs-plain ratio
    _, _, _, _, _, plain, pstream = setup_solver(local, mg_fast=0, fft_fp32=0)
    pcounts = {}
    pms, pcyc, _, _ = time_steps(plain, pstream, args.steps, args.warmup, counts=pcounts)
    plain_pois_ms, plain_pst, _ = time_poisson(plain, pstream, p)
    plain_e2e_s, _, plain_n_e2e = end_to_end(plain, shape, 2)
    plain.close()
    les = None if args.no_les else run_les(args, local)
    ensemble = None if args.no_ensemble else run_ensemble(args, local)

    result = None
    if rank == 0:
        peak, peak_kind = peaks()
        # dominant kernel class: achieved = its algorithmic HBM bytes (counted
        # per launch by the library) / its CUDA-event time
        name, (dms, dcnt, dbytes) = max(kt.items(), key=lambda kv: kv[1][0])
        roof = None
        if dcnt > 0 and dms > 0:
            achieved = dbytes / (dms / 1000.0) / 1e9
            ratio, tsrc = profiled_traffic_ratio(name)
            traffic = int(ratio * dbytes / dcnt) if ratio is not None else None
            roof = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
                    "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                    "traffic": traffic, "traffic_source": tsrc,
                    "traffic_note": (f"DRAM bytes per algorithmic byte ({ratio}) of one finest-level sweep of the "
                                     f"class's kernel, measured with ncu on the NX=128 case (fields above L2), "
                                     f"times this class's algorithmic bytes per launch") if ratio else None,
                    "algorithmic_bytes_per_launch": int(dbytes / dcnt),
                    "avg_launch_us": round(dms * 1000.0 / dcnt, 3), "launches_per_step": dcnt,
                    "share_of_step": round(dms / ktot, 4)}
        per_class_gbs = {k: round(v[2] / (v[0] / 1000.0) / 1e9, 1) for k, v in kt.items()
                         if v[0] > 0 and k != "guess"}
        plain_value = args.steps / (pms / 1000.0)
        result = {
            "metric": METRIC,
            "value": round(value, 4),
            "unit": "RK3 steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms_max / args.steps, 3),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": STATE_DTYPE[FF_ARITH],
            "data": "synthetic (seeded laminar Ekman spiral + 1% Gaussian noise; no reference dataset exists)",
            "config": {"workload": WORKLOAD, "nx": p.nx, "ny_plus_2": p.ny + 2, "nz_plus_2": p.nz + 2,
                       "re": w.re, "pr": w.pr, "ri": w.ri, "delta_t": p.delta_t,
                       "method": "batched mixed-precision projection (no learned guess)",
                       "precision": STATE_PRECISION[FF_ARITH],
                       "poisson": f"relative residual {MG_TOL:g} per problem, kx=0 included (its right-hand "
                                  f"side projected onto the operator's range, zero-mean solution)",
                       "mg_corrections_per_substep_max": mg_cycles,
                       "poisson_problems_per_step": counts.get("solved", 0) / args.steps,
                       "poisson_not_converged_per_step": counts.get("not_converged", 0) / args.steps,
                       "line_solve_layouts": {f"L{r['level']}{r['dir']}": f"{r['lanes']}x{r['seg']}" for r in tuned},
                       "autotune_s": round(t_tune, 2),
                       "l2": "fields (407 MB each, ~18 GB resident) exceed the 126 MB L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "plain": {"value": round(plain_value, 4), "unit": "RK3 steps/s", "ms_per_step": round(pms / args.steps, 3),
                      "dtype": "f64",
                      "method": "FP64 MUDPACK FMG + W(2,1), 4-colour GS, every transform and kernel in FP64",
                      "mg_cycles_per_substep_max": pcyc,
                      "poisson_not_converged_per_step": pcounts.get("not_converged", 0) / args.steps,
                      "poisson_solves_per_s": round(ncomplex / (plain_pois_ms / 1000.0), 2),
                      "poisson_max_cycles": plain_pst["max_cycles"],
                      "e2e": {"value": round(world / plain_e2e_s, 4), "unit": "RK3 steps/s",
                              "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
                              "steps": plain_n_e2e}},
            "speedup_vs_plain": round(value / (world * plain_value), 3),
            "poisson_solves_per_s": round(solves_per_s, 2),
            "poisson_batch": {"complex_problems": ncomplex, "ms": round(pois_ms, 3),
                              "max_cycles": pst["max_cycles"], "unit": "complex kx problems/s"},
            "divergence_after_projection": div,
            "clocks": clocks,
            "gpu_launches": int(launches),
            "kernel_ms_per_step": {k: round(v[0], 3) for k, v in kt.items()},
            "kernel_algorithmic_gbs": per_class_gbs,
            "kernel_launches_per_step": {k: v[1] for k, v in kt.items()},
            "e2e": {"value": round(world / e2e_s, 4), "unit": "RK3 steps/s",
                    "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
                    "steps": n_e2e},
            "roofline": roof,
            "learned": learned,
            "les": les,
            "ensemble": ensemble,
        }
        if world == 1 and not args.no_cpu_baseline:
            result["cpu_baseline"] = cpu_baseline(args)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return result


def cpu_baseline(args, nsteps: int = 1):
    """The CPU oracle (a restatement of the reference's Fortran; the Fortran
    itself cannot be built here) on this host's cores, on a bounded sample:
    nsteps RK3 steps of the same workload after the initial projection."""
    from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL, WORKLOADS, workload_setup
    from oracle import ekref

    cores = os.cpu_count() or 1
    w = WORKLOADS[WORKLOAD]
    w.mg_tol = MG_TOL
    p, xp, yp, state = workload_setup(w, EK_MG_STOP_RESIDUAL)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp), threads=cores)
    o.upload(*state)
    o.rem_div()
    t0 = time.perf_counter()
    o.step(nsteps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": round(nsteps / dt, 5), "unit": "RK3 steps/s", "cores": cores, "kind": "port",
            "sample": f"{nsteps} RK3 step(s) of {WORKLOAD} after the initial projection, "
                      f"{cores} OpenMP threads ({dt:.1f} s)"}


def run_reference(args):
    """Reference arm: the oracle (CPU restatement of the reference path) on
    all host cores, same workload/metric; each step a full RK3 step, at most
    3 timed steps and 1 warm-up so the run stays within minutes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL, WORKLOADS, workload_setup
    from oracle import ekref

    ekref.build()
    cores = os.cpu_count() or 1
    w = WORKLOADS[WORKLOAD]
    w.mg_tol = MG_TOL
    p, xp, yp, state = workload_setup(w, EK_MG_STOP_RESIDUAL)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp), threads=cores)
    o.upload(*state)
    o.rem_div()
    for _ in range(min(args.warmup, 1)):
        o.step(1)
    nsteps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    o.step(nsteps)
    dt = time.perf_counter() - t0
    o.close()
    v = nsteps / dt
    sample = f"{nsteps} RK3 step(s) of {WORKLOAD}, {cores} OpenMP threads ({dt:.1f} s)"
    return {
        "metric": METRIC, "value": round(v, 5), "unit": "RK3 steps/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": nsteps, "warmup": min(args.warmup, 1), "ms_per_step": round(1000 * dt / nsteps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded laminar Ekman spiral + 1% Gaussian noise)",
        "config": {"workload": WORKLOAD, "precision": "fp64", "poisson": f"relative residual {MG_TOL:g}"},
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 5), "unit": "RK3 steps/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v, 5), "unit": "RK3 steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip training and timing the learned guess")
    ap.add_argument("--no-les", action="store_true", help="skip the LES case")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the uneven-grid ensemble")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gpu":
        args.warmup = 3
    res = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
