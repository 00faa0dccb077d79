"""Run one RK3 step of a named workload for profiling.

    python -m ekman_bl_gb300.profile_step [--workload NAME] [--warmup W] [--tol T] [--mixed] [--les]

Sets up the workload, runs W warm-up steps, then exactly one RK3 step, and
prints the number of kernel launches issued before that step and inside it,
so that an ncu launch list can bracket the step with -s/-c.  With
--timing it also prints the per-kernel-class CUDA-event times of the step.
"""
from __future__ import annotations

import argparse
import json

from . import build as ekbuild
from .duct import DuctSolver, les_metrics_from_grid, metrics_from_grid
from .params import EK_MG_STOP_RELCHANGE, EK_MG_STOP_RESIDUAL, WORKLOADS, workload_setup


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="ekman_strat_256x257x193", choices=sorted(WORKLOADS))
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--tol", type=float, default=1e-8, help="relative residual; 0 = MUDPACK's own rule")
    ap.add_argument("--timing", action="store_true")
    ap.add_argument("--nx", type=int, default=0, help="override NX (smaller cases for full ncu captures)")
    ap.add_argument("--mixed", action="store_true",
                    help="mixed-precision method: mg_fast = 1, fft_fp32 = 1 (needs --tol > 0)")
    ap.add_argument("--ff", action="store_true", help="float-float state-carrying transforms (ff_arith = 1)")
    ap.add_argument("--ff-arith", type=int, default=-1, help="ff_arith (0, 1, 2); overrides --ff")
    ap.add_argument("--autotune", action="store_true", help="tune the line-solve layouts first, as bench.py does")
    ap.add_argument("--layout", default="", help="LANESxSEG for every line solve (e.g. 8x8) instead of tuning")
    ap.add_argument("--les", action="store_true",
                    help="dynamic-Smagorinsky LES on (CREATE_NEW_FLOW = .FALSE.: subgrid terms from the first step)")
    ap.add_argument("--no-graph", action="store_true",
                    help="issue every launch from the host (no whole-step CUDA graph), for per-kernel profiling")
    ap.add_argument("--guess", action="store_true",
                    help="train the learned initial guess on one warm-up step (50 Adam steps) and use it (needs --mixed)")
    args = ap.parse_args()
    ekbuild.build()
    w = WORKLOADS[args.workload]
    if args.nx:
        w.nx = args.nx

    stop = EK_MG_STOP_RESIDUAL if args.tol > 0 else EK_MG_STOP_RELCHANGE
    if args.tol > 0:
        w.mg_tol = args.tol
    p, xp, yp, state = workload_setup(w, stop)
    if args.mixed:
        p.mg_fast, p.fft_fp32 = 1, 1
    if args.ff:
        p.ff_arith = 1
    if args.ff_arith >= 0:
        p.ff_arith = args.ff_arith
    if args.les:
        p.les, p.create_new_flow = 1, 0
    s = DuctSolver(p, metrics_from_grid(p, xp, yp))
    if args.no_graph:
        s.set_step_graph(False)
    if p.les:
        s.set_les_metrics(les_metrics_from_grid(p, xp, yp))
    s.upload(*state)
    if args.autotune:
        s.mg_autotune(reps=3)
    if args.layout:
        lanes, seg = (int(v) for v in args.layout.split("x"))
        for lev in range(2, len(s.mg_levels()) + 1):
            for d in (0, 1):
                s.mg_set_layout(lev, d, lanes, seg)
    s.rem_div_curv()
    if args.guess:
        from .learned import LearnedGuess
        lg = LearnedGuess(s, factor=4, channels=32, seed=0)
        lg.collect(1)
        lg.train(iters=50, batch=16, lr=2e-3)
        lg.enable()
    s.step(args.warmup)
    before = s.launch_count()
    if args.timing:
        s.set_timing(True)
    s.step(1)
    inside = s.launch_count() - before
    out = {"workload": args.workload, "launches_before_step": before, "launches_in_step": inside,
           "mg": s.mg_stats(), "divergence": s.divergence()}
    if args.timing:
        out["timing"] = {k: {"ms": round(v[0], 3), "launches": v[1], "alg_bytes": v[2]} for k, v in s.timing().items()}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
