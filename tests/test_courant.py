"""COURANT_CURV_MPI (src/duct.F90:3605-3674) under VARIABLE_DT: after the
RK_STEP = 3 ADI the time step becomes min(CFL*DX/|U1|, CFL*J/|U2b|,
CFL*J/|U3b|), capped at DELTA_T_SET, and H_BAR follows it."""
import numpy as np
import pytest

from ekcases import rel_l2, small_case
from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
from oracle import ekref


def cfl_case(cfl, delta_t_set):
    p, xp, yp, st = small_case()
    p.variable_dt, p.update_dt, p.cfl, p.delta_t_set = 1, 1, cfl, delta_t_set
    return p, xp, yp, st


def test_oracle_cfl_step_follows_velocity():
    """The oracle's dt after one step equals the formula evaluated on its own
    post-ADI velocity bound: dt <= CFL*DX/max|U1| is the x-term alone."""
    p, xp, yp, st = cfl_case(1e-3, 1.0)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    o.upload(*st)
    o.step(1)
    t, n, dt = o.get_time()
    assert n == 1 and 0 < dt < p.delta_t_set
    # the x-term bound: |U1| reaches ~WBULK0 * e^-pi/4 sin(pi/4) > 0.3 in the
    # spiral, so CFL*DX/|U1| < CFL*DX/0.3
    assert dt < 1e-3 * (p.lx / p.nx) / 0.3
    p2, xp, yp, st = cfl_case(10.0, 1.0e-3)   # CFL step large: capped at DELTA_T_SET
    o2 = ekref.Oracle(p2, ekref.metrics_from_grid(p2, xp, yp))
    o2.upload(*st)
    o2.step(1)
    assert o2.get_time()[2] == 1.0e-3


@pytest.mark.gpu
@pytest.mark.parametrize("cfl,dtset", [(2e-3, 1.0), (10.0, 1.0e-3)])
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
