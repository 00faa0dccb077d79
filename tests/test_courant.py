"""COURANT_CURV_MPI (src/duct.F90:3605-3674) under VARIABLE_DT: after the
RK_STEP = 3 ADI the time step becomes min(CFL*DX/|U1|, CFL*J/|U2b|,
CFL*J/|U3b|), capped at DELTA_T_SET, and H_BAR follows it."""
import numpy as np
import pytest

from ekcases import cfl_case, rel_l2, small_case
from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL
from oracle import ekref




def test_oracle_cfl_step_follows_velocity():
    """The oracle's dt after one step equals the formula evaluated on its own
    post-ADI velocity bound: dt <= CFL*DX/max|U1| is the x-term alone."""
    p, xp, yp, st = cfl_case(0.2, 1.0)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    o.upload(*st)
    o.step(1)
    t, n, dt = o.get_time()
    assert n == 1 and 1e-4 < dt < p.delta_t_set
    # the x-term bound: |U1| reaches ~WBULK0 * e^-pi/4 sin(pi/4) > 0.3 in the
    # spiral, so CFL*DX/|U1| < CFL*DX/0.3
    assert dt < 0.2 * (p.lx / p.nx) / 0.3
    p2, xp, yp, st = cfl_case(10.0, 1.0e-3)   # CFL step large: capped at DELTA_T_SET
    o2 = ekref.Oracle(p2, ekref.metrics_from_grid(p2, xp, yp))
    o2.upload(*st)
    o2.step(1)
    assert o2.get_time()[2] == 1.0e-3


@pytest.mark.gpu
@pytest.mark.parametrize("cfl,dtset", [(0.2, 1.0), (10.0, 1.0e-3)])
def test_cfl_steps_match_oracle(cfl, dtset):
    p, xp, yp, st = cfl_case(cfl, dtset)
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    g.upload(*st)
    o.upload(*st)
    for _ in range(3):
        g.step(1)
        o.step(1)
        tg, ng, dg = g.get_time()
        to, no, do = o.get_time()
        assert ng == no and abs(dg - do) <= 1e-12 * do and abs(tg - to) <= 1e-12 * abs(to)
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
        assert rel_l2(x, y) < 1e-10, name


def test_oracle_stops_below_the_dt_bound():
    """REM_DIV_CURV ends with IF (DELTA_T .LT. 1.0E-4) STOP 'DELTA_T is
    zero' (src/duct.F90:2812): a CFL step of ~4e-6 stops the run at the
    projection of the RK_STEP = 3 that set it; a fixed DELTA_T below the
    bound stops the first projection.  The bound is the REAL*4 literal, so
    DELTA_T = 1e-4 itself passes."""
    p, xp, yp, st = cfl_case(2e-3, 1.0)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    o.upload(*st)
    with pytest.raises(RuntimeError, match="status 8: DELTA_T is zero"):
        o.step(1)
    assert 0 < o.get_time()[2] < 1e-4
    for dt, ok in ((5e-5, False), (1e-4, True)):
        p, xp, yp, st = small_case()
        p.delta_t = dt
        o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
        o.upload(*st)
        if ok:
            o.rem_div()
        else:
            with pytest.raises(RuntimeError, match="DELTA_T is zero"):
                o.rem_div()


@pytest.mark.gpu
@pytest.mark.parametrize("fast", [0, 1])
def test_library_stops_below_the_dt_bound(fast):
    """The library returns EK_ERR_DT where the reference stops: after the
    RK_STEP = 3 projection whose CFL step fell below 1.0E-4 (velocity and
    scalar are the ones the oracle holds at its stop; CP has that substep's
    update, which the reference, stopping inside REM_DIV_CURV, never makes),
    and at the first projection of a run whose fixed DELTA_T is below it
    (also where whole-step graphs would otherwise run)."""
    from ekman_bl_gb300.duct import EkError
    p, xp, yp, st = cfl_case(2e-3, 1.0)
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        o.upload(*st)
        with pytest.raises(EkError, match="DELTA_T is zero"):
            g.step(1)
        with pytest.raises(RuntimeError):
            o.step(1)
        assert g.get_time()[2] == pytest.approx(o.get_time()[2], rel=1e-12)
        for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
            if name != "CP":
                assert rel_l2(x, y) < 1e-10, name
    finally:
        g.close()
        o.close()
    p, xp, yp, st = small_case()
    p.delta_t = 5e-5
    if fast:
        p.mg_stop, p.mg_tol, p.mg_maxcy, p.mg_fast, p.fft_fp32, p.ff_arith = EK_MG_STOP_RESIDUAL, 1e-10, 60, 1, 1, 1
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        with pytest.raises(EkError, match="DELTA_T is zero"):
            g.step(2)
        assert g.get_time()[1] == 1
    finally:
        g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ff", [1, 2])
def test_cfl_steps_mixed_path(ff):
    """VARIABLE_DT on the mixed-precision path, whose physical fields are
    float-float planes (ff_arith = 1) or an FP32 field plus its FP32
    increment (ff_arith = 2) when COURANT_CURV_MPI reads them: DELTA_T
    within 1e-6 of the FP64 oracle's over three steps (it follows the mixed
    state's ~1e-7 difference), the state within the mixed bar."""
    p, xp, yp, st = cfl_case(0.2, 1.0)
    q = type(p).from_buffer_copy(p)
    q.mg_stop, q.mg_tol, q.mg_maxcy, q.mg_fast, q.fft_fp32, q.ff_arith = EK_MG_STOP_RESIDUAL, 1e-10, 60, 1, 1, ff
    p.mg_stop, p.mg_tol, p.mg_maxcy = EK_MG_STOP_RESIDUAL, 1e-10, 200
    g = DuctSolver(q, metrics_from_grid(q, xp, yp))
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        o.upload(*st)
        for _ in range(3):
            g.step(1)
            o.step(1)
            assert g.get_time()[2] == pytest.approx(o.get_time()[2], rel=1e-6)
        for name, x, y in zip(("CU1", "CU2", "CU3", "CTH"), *[[a[i] for i in (0, 1, 2, 4)] for a in (g.download(), o.download())]):
            assert rel_l2(x, y) < 1e-5, name
    finally:
        g.close()
        o.close()
