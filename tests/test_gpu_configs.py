"""GPU parity at the sizes the bench quotes, the well-posed kx = 0 solve, and
the status of a projection that misses its tolerance.

- The mixed-precision method on the 512 x 385 x 257 stratified workload (the
  bench's headline configuration): one RK3 step from the bench's seeded,
  projected state against the FP64 oracle at the same 1e-8 Poisson residual.
  Velocity and buoyancy within 1e-5 relative L2, the mixed path's bar.
- The plain FP64 path on the 256 x 257 x 193 stratified workload: three RK3
  steps with MUDPACK's own iteration against the oracle, within 1e-10.
- A projection whose problems stop at mg_maxcy above the residual rule's
  tolerance: the substep completes and returns EK_ERR_NOT_CONVERGED (the
  reference's MULTIGRID_MUDPACK drops mud2cr's ierror = -1, mud2cr.f:204-207).
"""
import dataclasses
import math
import os
import warnings

import numpy as np
import pytest

from ekcases import rel_l2, small_case
from ekman_bl_gb300 import build as ekbuild
from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL, WORKLOADS, workload_setup
from oracle import ekref

pytestmark = pytest.mark.gpu

STATE = ("CU1", "CU2", "CU3", "CP", "CTH")


@pytest.fixture(scope="module", autouse=True)
def _build():
    ekbuild.build()


def _oracle(p, xp, yp):
    return ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp), threads=os.cpu_count() or 1)


def test_mixed_method_one_step_at_512x385x257():
    """The bench's method and workload: NX = 512, NY+2 = 385, NZ+2 = 257,
    Re = 1000, Ri = 0.1, dt = 3e-4, every Poisson problem to 1e-8; both
    forms of the state path (ff_arith = 1 float-float, 2 FP32 increments)
    against one step of the oracle."""
    w = dataclasses.replace(WORKLOADS["ekman_strat_512x385x257"], mg_tol=1e-8)
    p, xp, yp, st = workload_setup(w, EK_MG_STOP_RESIDUAL)
    runs = {}
    for ff in (1, 2):
        q = workload_setup(w, EK_MG_STOP_RESIDUAL)[0]
        q.mg_fast, q.fft_fp32, q.ff_arith = 1, 1, ff
        g = DuctSolver(q, metrics_from_grid(q, xp, yp))
        try:
            g.upload(*st)
            assert g.rem_div_curv() == 0
            assert g.step(1) == 0
            runs[ff] = (g.download(), g.divergence(), g.mg_stats())
        finally:
            g.close()
    o = _oracle(p, xp, yp)
    try:
        o.upload(*st)
        o.rem_div()
        o.step(1)
        os_ = o.download()
        odiv = o.divergence()
    finally:
        o.close()
    for ff, (gs, gdiv, gmg) in runs.items():
        errs = {n: rel_l2(a, b) for n, a, b in zip(STATE, gs, os_)}
        print(f"mixed (ff_arith={ff}) vs FP64 oracle after one step at 512x385x257:", errs, "div", gdiv, odiv, gmg)
        for n in ("CU1", "CU2", "CU3", "CTH"):
            assert errs[n] <= 1e-5, (ff, n, errs[n])
        assert gmg["n_not_converged"] == 0 and gmg["max_residual"] <= 1e-8, gmg
        assert np.isfinite(gdiv) and gdiv <= 3.0 * odiv + 1e-12, (gdiv, odiv)


def test_plain_fp64_three_steps_at_256x257x193():
    """The stratified plain-path configuration (NX = 256, NY+2 = 257,
    NZ+2 = 193, Re = 800, Ri = 0.1, dt = 5e-4) with MUDPACK's own iteration
    and stopping rule: three RK3 steps within 1e-10 of the oracle."""
    w = WORKLOADS["ekman_strat_256x257x193"]
    p, xp, yp, st = workload_setup(w)
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        g.rem_div_curv()
        g.step(3)
        gs = g.download()
        gdiv = g.divergence()
    finally:
        g.close()
    o = _oracle(p, xp, yp)
    try:
        o.upload(*st)
        o.rem_div()
        o.step(3)
        os_ = o.download()
        odiv = o.divergence()
    finally:
        o.close()
    errs = {n: rel_l2(a, b) for n, a, b in zip(STATE, gs, os_)}
    print("plain FP64 vs oracle after three steps at 256x257x193:", errs, "div", gdiv, odiv)
    for n in STATE:
        assert errs[n] <= 1e-10, (n, errs[n])
    assert gdiv == pytest.approx(odiv, rel=1e-6, abs=1e-15)


@pytest.mark.parametrize("fast", [1, 0])
def test_capped_projection_reports_not_converged(fast):
    """mg_maxcy = 1 under the residual rule: the substep finishes, returns
    EK_ERR_NOT_CONVERGED and counts the problems; the state stays finite."""
    p, xp, yp, st = small_case()
    p.mg_stop, p.mg_tol, p.mg_maxcy, p.mg_fast = EK_MG_STOP_RESIDUAL, 1e-10, 1, fast
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        with pytest.warns(RuntimeWarning, match="NOT_CONVERGED"):
            code = g.rk_duct(1)
        assert code == 3
        s = g.mg_stats()
        assert s["n_not_converged"] > 0 and s["max_residual"] > 1e-10, s
        solved, nc = g.mg_counters()
        assert solved >= s["nprob"] and nc == s["n_not_converged"]
        assert all(np.isfinite(a).all() for a in g.download())
        # ekgpu_step runs every step before reporting it
        with pytest.warns(RuntimeWarning, match="NOT_CONVERGED"):
            assert g.step(2) == 3
        assert g.get_time()[1] == 2
    finally:
        g.close()


def test_relchange_rule_counts_but_does_not_fail():
    """Under MUDPACK's relative-change rule a capped problem is the
    reference's normal outcome: counted, status EK_OK."""
    p, xp, yp, st = small_case()
    p.mg_maxcy = 1
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        with warnings.catch_warnings():
            warnings.simplefilter("error")
            assert g.rk_duct(1) == 0
        assert g.mg_stats()["n_not_converged"] > 0
        assert g.mg_counters()[1] > 0
    finally:
        g.close()


@pytest.mark.parametrize("fast", [1, 0])
def test_wellposed_kx0_against_oracle(fast):
    """The kx = 0 problems under the residual rule on both GPU solvers: the
    residual against the projected right-hand side b' = b - (z.b) z meets
    the tolerance, phi has zero mean and matches the oracle's solve."""
    p, xp, yp, _ = small_case(nx=16, ny2=33, nz2=17)
    p.mg_stop, p.mg_tol, p.mg_maxcy, p.mg_fast = EK_MG_STOP_RESIDUAL, 1e-10, 200, fast
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    po = small_case(nx=16, ny2=33, nz2=17)[0]
    po.mg_stop, po.mg_tol, po.mg_maxcy = EK_MG_STOP_RESIDUAL, 1e-12, 400
    o = _oracle(po, xp, yp)
    z = o.mg_left_null()
    rng = np.random.default_rng(21)
    kx2 = np.array([0.0, (2 * math.pi / p.lx) ** 2, 0.0])
    rhs = rng.standard_normal((3, p.ny + 2, p.nz + 2))
    try:
        pg, sg, cg = g.multigrid_mudpack(rhs, kx2)
    finally:
        g.close()
    assert cg == 0 and sg["n_not_converged"] == 0, sg
    try:
        po_, so, co = o.poisson(rhs, kx2)
        assert co == 0, so
        for q in (0, 2):
            bp = rhs[q] - (z * rhs[q]).sum() * z
            r = bp - o.mg_apply(0.0, pg[q])
            assert np.linalg.norm(r) <= 1.05e-10 * np.linalg.norm(bp), q
            assert abs(pg[q].mean()) <= 1e-12 * np.abs(pg[q]).max(), q
            assert rel_l2(pg[q], po_[q]) < 1e-8, q
    finally:
        o.close()
