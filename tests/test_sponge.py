"""sponge_th (src/duct.F90:3196-3362) and its profiles (src/diablo.F90:1489-1556).

CPU: the oracle's profiles against the Fortran formulas written out here,
and the library's host routine bit for bit against the oracle.  GPU: RK3
steps with the sponge on, against the oracle, through each branch of
sponge_th: the dynamic mean-flow branch on and off, and the stratified
z-periodic branch with its reset of CU2X(0,:,:) at MOD(2*TIME_STEP,
SAVE_STATS_INT) = 0.
"""
import math

import numpy as np
import pytest

from ekcases import rel_l2, small_case, sponge_case
from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid, sponge_profiles
from oracle import ekref




def formula_profiles(p, xp, yp):
    """diablo.F90:1489-1556 as written (REAL() spans rounded to REAL*4)."""
    NY, NZ = p.ny, p.nz
    so = np.zeros(NZ + 2)
    sg = np.zeros(NY + 2)
    R, L, T = p.nz_s_r, p.nz_s_l, p.ny_s_t
    if p.sponge_type == 1 and R < NZ + 1:
        b = 1.0 / float(np.float32(xp[NY + 1, NZ + 1] - xp[NY + 1, R]))
        for k in range(NZ + 2):
            if k >= R:
                so[k] = ((xp[NY + 1, k] - xp[NY + 1, R]) * b) ** 2
            elif k <= L:
                so[k] = ((xp[NY + 1, L] - xp[NY + 1, k]) * b) ** 2
    elif p.sponge_type == 2 and R < NZ + 1:
        b = math.log(25.0) / float(np.float32(NZ + 1 - R))
        for k in range(NZ + 2):
            if k >= R:
                so[k] = (math.exp(b * abs(k - R)) - 1.0) / 24.0
            elif k <= L:
                so[k] = (math.exp(b * abs(L - k)) - 1.0) / 24.0
    if p.sponge_type == 1:
        b = 1.0 / float(np.float32(yp[NY + 1, NZ + 1] - yp[T, NZ + 1]))
        for j in range(T, NY + 2):
            sg[j] = ((yp[j, NZ + 1] - yp[T, NZ + 1]) * b) ** 2
    elif p.sponge_type == 2:
        b = math.log(30.0) / float(np.float32(NY + 1 - T))
        for j in range(T, NY + 2):
            sg[j] = (math.exp(b * (j - T)) - 1.0) / 29.0
    return sg, so


@pytest.mark.parametrize("sponge_type", [1, 2])
def test_sponge_profiles(sponge_type):
    p, xp, yp, _ = sponge_case(sponge_type)
    sg, so = ekref.sponge_profiles(p, xp, yp)
    fsg, fso = formula_profiles(p, xp, yp)
    np.testing.assert_allclose(sg, fsg, rtol=1e-14, atol=0)
    np.testing.assert_allclose(so, fso, rtol=1e-14, atol=0)
    assert sg[p.ny_s_t] == 0.0 and sg[p.ny + 1] > 0.5
    assert so[p.nz + 1] > 0.5 and so[0] > 0.5 and so[p.nz // 2] == 0.0
    gsg, gso = sponge_profiles(p, xp, yp)
    assert np.array_equal(gsg, sg) and np.array_equal(gso, so)


def test_sponge_profiles_off():
    p, xp, yp, _ = sponge_case(0)
    sg, so = sponge_profiles(p, xp, yp)
    assert not sg.any() and not so.any()


def upper_mean_cu3(p, cu3):
    """The mean sponge_th tests against WBULK0 (velocity ranges of INIT_DUCT
    for the BCs of these cases: J = 1..NY, K = 1..NZ)."""
    nys = (2 * p.ny) // 3 if p.ny_s_t > p.ny else p.ny_s_t
    return cu3[nys:p.ny + 1, 1:p.nz + 1, 0].real.mean()


@pytest.mark.gpu
@pytest.mark.parametrize("dynamic", [True, False])
@pytest.mark.parametrize("sponge_type", [1, 2])
def test_sponge_steps_match_oracle(sponge_type, dynamic):
    p, xp, yp, st = sponge_case(sponge_type, dynamic)
    m = upper_mean_cu3(p, st[2])
    assert (abs(m - p.wbulk0) > p.wbulk0 * 0.001) == dynamic
    sg, so = ekref.sponge_profiles(p, xp, yp)
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    g.set_sponge(sg, so)
    o.set_sponge(sg, so)
    g.upload(*st)
    o.upload(*st)
    # three steps: TIME_STEP = 1, 2, 3; the reset of CU2X(0,:,:) fires at 2
    g.step(3)
    o.step(3)
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
        assert rel_l2(x, y) < 1e-11, name


@pytest.mark.gpu
def test_sponge_changes_the_flow():
    """With SPONGE_TYPE = 2 the step differs from the unsponged one, and the
    fluctuations in the top sponge layer are damped relative to it."""
    p, xp, yp, st = sponge_case(2)
    sg, so = ekref.sponge_profiles(p, xp, yp)
    q = sponge_case(0)[0]
    a = DuctSolver(p, metrics_from_grid(p, xp, yp))
    b = DuctSolver(q, metrics_from_grid(q, xp, yp))
    a.set_sponge(sg, so)
    a.upload(*st)
    b.upload(*st)
    a.step(2)
    b.step(2)
    ua, ub = a.download()[0], b.download()[0]
    top = slice(p.ny - 2, p.ny + 1)
    assert rel_l2(ua, ub) > 1e-6
    assert np.abs(ua[top, 1:-1, 1:]).sum() < np.abs(ub[top, 1:-1, 1:]).sum()


@pytest.mark.gpu
@pytest.mark.parametrize("ff", [1, 2])
def test_sponge_mixed_path_with_reset_matches_oracle(ff):
    """The mixed path (FP32 nonlinear and explicit-increment transforms,
    float-float state transforms, mixed multigrid) through the stratified
    z-periodic branch and its reset of CU2X(0,:,:) at TIME_STEP = 2, from a
    state whose CU2X(0,:,:) is not zero, so that the reset removes a real
    part of the field (a wrong account of it in the explicit-increment
    transform would put half of that part into the ADI right-hand side).
    After three steps velocity and buoyancy are within 1e-6 of the FP64
    oracle, the pressure within 1e-5: CP accumulates phi/h, which carries the
    FP32 nonlinear terms' rounding (measured 2.6e-6)."""
    p, xp, yp, st = sponge_case(2, True)
    rng = np.random.default_rng(9)
    st[1][1:p.ny + 1, 1:p.nz + 1, 0] += 0.01 * rng.standard_normal((p.ny, p.nz))
    sg, so = ekref.sponge_profiles(p, xp, yp)
    p.mg_stop, p.mg_tol, p.mg_maxcy = 1, 1e-10, 200
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    q = sponge_case(2, True)[0]
    q.mg_stop, q.mg_tol, q.mg_maxcy, q.mg_fast, q.fft_fp32, q.ff_arith = 1, 1e-10, 60, 1, 1, ff
    g = DuctSolver(q, metrics_from_grid(q, xp, yp))
    g.set_sponge(sg, so)
    o.set_sponge(sg, so)
    g.upload(*st)
    o.upload(*st)
    g.step(3)
    o.step(3)
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
        assert rel_l2(x, y) < (1e-5 if name == "CP" else 1e-6), name
