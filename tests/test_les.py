"""LES (src/les_chan.F90 LES_MODEL_TYPE 2, src/les_chan_th.F90
LES_MODEL_TYPE_TH 1, and the LES branches of RK_DUCT).

CPU: the library's LES metric helper equals the oracle's bit for bit and
satisfies the identities of its definition; the oracle's dynamic procedure
reproduces an independent numpy evaluation of the model's formulas on a
field whose strain rate is known exactly; the oracle's LES path with a zero
coefficient is the plain path bit for bit.

GPU: the CUDA path through the C ABI against the oracle (states, the
explicit terms, NU_T and C_DYN) over substeps and steps that cover the
C_DYN schedule (FIRST_TIME, every fifth step), the CREATE_NEW_FLOW start,
the restart reset of FIRST_TIME, and the known-answer field.  Tolerances:
relative L2 <= 1e-11 per substep and 1e-10 over ten steps (the FP64 bar).
"""
import math

import numpy as np
import pytest

from ekcases import les_case, rel_l2, refgrid_case, sheared_case, small_case
from ekman_bl_gb300.duct import les_metrics_from_grid, metrics_from_grid
from ekman_bl_gb300.params import EK_F_CF1, EK_F_CF2, EK_F_CF3, EK_F_CFTH, EK_F_CR1, spectral_shape
from oracle import ekref

# les_chan.F90:37 PARAMETER (alpha=2.44950) into a REAL*8: the literal is
# default REAL, so alpha is 2.4495 rounded to single precision
ALPHA = float(np.float32(2.44950))


def oracle_for(p, xp, yp, st):
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    o.set_les_metrics(ekref.les_metrics_from_grid(p, xp, yp))
    o.upload(*st)
    return o


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_les_metrics_match_oracle(case):
    p, xp, yp, _ = les_case(case)
    a = les_metrics_from_grid(p, xp, yp)
    b = ekref.les_metrics_from_grid(p, xp, yp)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_les_metric_identities():
    """GMAT_*_y + GMAT_*_z = 3 GMAT_* on the computed faces; the J=0 row and
    the K=0 column are linear extrapolations; the (0,0) corner averages the
    two for GMAT_11_* and GMAT_22_* and keeps the row value for GMAT_12_*."""
    p, xp, yp, _ = les_case("sheared")
    m = metrics_from_grid(p, xp, yp)
    lm = les_metrics_from_grid(p, xp, yp)
    for t in ("11", "12", "22"):
        s = lm[f"gmat_{t}_y"] + lm[f"gmat_{t}_z"]
        g = m[f"gmat_{t}"]
        sl = (slice(None), slice(1, p.ny + 2), slice(1, p.nz + 2))
        assert np.allclose(s[sl], 3.0 * g[sl], rtol=1e-13, atol=1e-13 * np.abs(g).max())
        for v in ("y", "z"):
            a = lm[f"gmat_{t}_{v}"]
            assert np.allclose(a[:, 1:p.ny + 2, 0], 2 * a[:, 1:p.ny + 2, 1] - a[:, 1:p.ny + 2, 2], rtol=0, atol=0)
            assert np.array_equal(a[:, 0, 1:p.nz + 2], 2 * a[:, 1, 1:p.nz + 2] - a[:, 2, 1:p.nz + 2])
            # a[f, J, K]: the K = 0 column value at J = 0 is overwritten by the row
            if t == "12":
                assert np.array_equal(a[:, 0, 0], 2 * a[:, 1, 0] - a[:, 2, 0])
            else:
                assert np.array_equal(a[:, 0, 0], 0.5 * (2 * a[:, 1, 0] - a[:, 2, 0] + 2 * a[:, 0, 1] - a[:, 0, 2]))
            assert np.array_equal(a[:, p.ny + 2, :p.nz + 2], a[:, p.ny + 1, :p.nz + 2])
            assert np.array_equal(a[:, :p.ny + 2, p.nz + 2], a[:, :p.ny + 2, p.nz + 1])


# U1(x) = sum a cos(k x) + b sin(k x) over these modes m (k = 2 pi m/LX);
# one mode alone gives a Germano coefficient of zero, two give a positive one
MODES = {1: (0.7, 0.0), 2: (0.0, 0.4)}


def x_only_state(p):
    """U1 = U1(x) on every (K, J) plane, U2 = U3 = 0: on the orthogonal test
    grids the eta/zeta differences of a (K, J)-constant field vanish exactly,
    so the only strain rate is S11 = dU1/dx."""
    shape = spectral_shape(p)
    cu1 = np.zeros(shape, np.complex128)
    for m, (a, b) in MODES.items():
        cu1[:, :, m] = 0.5 * (a - 1j * b)
    z = np.zeros(shape, np.complex128)
    return (cu1, z.copy(), z.copy(), z.copy(), z.copy())


def dynamic_coefficient(p):
    """numpy evaluation of les_chan.F90:475-834 for the x-only field: the
    filter FILTER_VAR(2) (1/4, 1/2, 1/4, periodic), M = (alpha D)^2 F(|S|)
    F(S11) - F(D^2 |S| S11), L = F(U1^2) - F(U1)^2, C = max(0, -0.5
    sum(M L)/sum(M M)), NU_T = C D^2 |S|, with |S| = sqrt(2) |S11| and
    D = (DX J)^(1/3) per (K, J).  Returns C D^2 and |S|."""
    x = np.arange(p.nx) * p.lx / p.nx
    u, s11 = np.zeros(p.nx), np.zeros(p.nx)
    for m, (a, b) in MODES.items():
        kx = 2 * math.pi * m / p.lx
        u += a * np.cos(kx * x) + b * np.sin(kx * x)
        s11 += -a * kx * np.sin(kx * x) + b * kx * np.cos(kx * x)
    sm = np.sqrt(2.0 * s11 * s11)
    F = lambda v: 0.25 * np.roll(v, 1) + 0.5 * v + 0.25 * np.roll(v, -1)
    shape_m = F(sm) * F(s11) * ALPHA ** 2 - F(sm * s11)  # M / D^2
    L = F(u * u) - F(u) ** 2
    ratio = -0.5 * np.sum(shape_m * L) / np.sum(shape_m * shape_m)  # C * D^2
    return ratio, sm


def check_known_answer(p, jac, nu, cd, js, je, zs, ze, rtol):
    ratio, sm = dynamic_coefficient(p)
    assert ratio > 0
    dx = p.lx / p.nx
    for j in range(p.ny + 2):
        for k in range(p.nz + 2):
            inside = js <= j <= je and zs <= k <= ze
            if not inside:
                assert cd[j, k] == 0.0 and not nu[j, k].any(), (j, k)
                continue
            d2 = (dx * jac[j, k]) ** (2.0 / 3.0)
            assert cd[j, k] == pytest.approx(ratio / d2, rel=rtol), (j, k)
            assert np.allclose(nu[j, k, :p.nx], ratio * sm, rtol=rtol, atol=1e-16), (j, k)
            assert not nu[j, k, p.nx:].any()


def test_oracle_dynamic_coefficient_known_answer():
    p, xp, yp, _ = les_case("small")
    o = oracle_for(p, xp, yp, x_only_state(p))
    o.rk_substep(1)
    nu, cd = o.les_state()
    jac = ekref.metrics_from_grid(p, xp, yp)["int_jacob"]
    check_known_answer(p, jac, nu, cd, 1, p.ny, 1, p.nz, 1e-12)


def test_oracle_zero_coefficient_is_plain_path():
    """CREATE_NEW_FLOW with TIME_STEP 2..4 outside FIRST_TIME: the LES
    branches run with C_DYN = 0, which leaves the plain path's result."""
    p, xp, yp, st = les_case("sheared")
    p.create_new_flow = 1
    a = oracle_for(p, xp, yp, st)
    a.les_set_first_time(False)
    a.set_time(0.0, 1)
    q = type(p).from_buffer_copy(p)
    q.les = 0
    b = ekref.Oracle(q, ekref.metrics_from_grid(q, xp, yp))
    b.upload(*st)
    b.set_time(0.0, 1)
    a.step(2)
    b.step(2)
    for x, y in zip(a.download(), b.download()):
        assert np.array_equal(x, y)
    nu, cd = a.les_state()
    assert not nu.any() and not cd.any()


# --------------------------------------------------------------------------- GPU

def gpu_for(p, xp, yp, st):
    from ekman_bl_gb300.duct import DuctSolver
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    g.set_les_metrics(les_metrics_from_grid(p, xp, yp))
    g.upload(*st)
    return g


def compare(g, o, tol, what=""):
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
        e = rel_l2(x, y)
        assert e <= tol, f"{what} {name}: rel L2 {e:.3e} > {tol:.1e}"
    ng, cg = g.les_state()
    no, co = o.les_state()
    assert rel_l2(ng, no) <= tol, f"{what} NU_T {rel_l2(ng, no):.3e}"
    assert rel_l2(cg, co) <= tol, f"{what} C_DYN {rel_l2(cg, co):.3e}"


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_les_substeps_match_oracle(case):
    p, xp, yp, st = les_case(case)
    g, o = gpu_for(p, xp, yp, st), oracle_for(p, xp, yp, st)
    for rk in (1, 2, 3):
        g.rk_duct(rk)
        o.rk_substep(rk)
        compare(g, o, 1e-11, f"rk{rk}")
        for f in (EK_F_CF1, EK_F_CF2, EK_F_CF3, EK_F_CFTH, EK_F_CR1):
            assert rel_l2(g.get_field(f), o.get_field(f)) < 1e-11, (rk, f)
    nu, cd = g.les_state()
    assert cd.max() > 0 and nu.max() > 0


@pytest.mark.gpu
def test_les_steps_match_oracle():
    """Ten steps from TIME_STEP 0: FIRST_TIME in step 1, C_DYN kept in steps
    2..4 and 6..9, recomputed at RK_STEP 1 of steps 5 and 10."""
    p, xp, yp, st = les_case("sheared")
    g, o = gpu_for(p, xp, yp, st), oracle_for(p, xp, yp, st)
    for n in range(10):
        g.step(1)
        o.step(1)
        compare(g, o, 1e-10, f"step {n + 1}")


@pytest.mark.gpu
def test_les_create_new_flow_start():
    """CREATE_NEW_FLOW: step 1 is the plain path; steps 2..4 run the LES
    branches with C_DYN = 0 (FIRST_TIME is over and 2..4 are not multiples
    of 5)."""
    p, xp, yp, st = les_case("small")
    p.create_new_flow = 1
    g, o = gpu_for(p, xp, yp, st), oracle_for(p, xp, yp, st)
    for n in range(3):
        g.step(1)
        o.step(1)
        compare(g, o, 1e-10, f"step {n + 1}")
    nu, cd = g.les_state()
    assert not cd.any() and not nu.any()


@pytest.mark.gpu
def test_les_known_answer():
    p, xp, yp, _ = les_case("small")
    g = gpu_for(p, xp, yp, x_only_state(p))
    g.rk_duct(1)
    nu, cd = g.les_state()
    check_known_answer(p, metrics_from_grid(p, xp, yp)["int_jacob"], nu, cd, 1, p.ny, 1, p.nz, 1e-12)


@pytest.mark.gpu
def test_les_restart_recomputes(tmp_path):
    """READ_FLOW starts a run: FIRST_TIME again, so C_DYN is recomputed in
    the restarted step as the oracle does after ekref_les_set_first_time."""
    p, xp, yp, st = les_case("small")
    g, o = gpu_for(p, xp, yp, st), oracle_for(p, xp, yp, st)
    g.step(2)
    o.step(2)
    g.write_restart(str(tmp_path / "f"), str(tmp_path / "t"))
    g.read_restart(str(tmp_path / "f"), str(tmp_path / "t"))
    o.les_set_first_time(True)
    g.step(1)
    o.step(1)
    compare(g, o, 1e-10, "restarted")


@pytest.mark.gpu
def test_les_mixed_precision_tracks_oracle():
    """The mixed-precision path with LES (FP32 V-cycles inside the FP64
    refinement, FP32 nonlinear-term transforms, float-float in the others)
    against the FP64 oracle at the same 1e-10 residual rule: within 1e-5
    relative L2 after three steps."""
    from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL
    p, xp, yp, st = les_case("small")
    p.mg_stop, p.mg_tol, p.mg_maxcy = EK_MG_STOP_RESIDUAL, 1e-10, 200
    o = oracle_for(p, xp, yp, st)
    q = type(p).from_buffer_copy(p)
    q.mg_maxcy, q.mg_fast, q.fft_fp32, q.ff_arith = 60, 1, 1, 1
    g = gpu_for(q, xp, yp, st)
    g.step(3)
    o.step(3)
    a, b = g.download(), o.download()
    for name, x, y in zip(("CU1", "CU2", "CU3", "CTH"), (a[0], a[1], a[2], a[4]), (b[0], b[1], b[2], b[4])):
        assert rel_l2(x, y) < 1e-5, name
    ng, _ = g.les_state()
    no, _ = o.les_state()
    assert rel_l2(ng, no) < 1e-4


@pytest.mark.gpu
def test_les_with_sponge_and_variable_dt():
    """LES together with sponge_th (SPONGE_TYPE 2, its CU2X reset at
    TIME_STEP 2) and VARIABLE_DT (the CFL step after each RK_STEP 3), on the
    non-orthogonal grid, against the oracle over three steps."""
    p, xp, yp, st = les_case("sheared")
    p.sponge_type, p.ny_s_t = 2, p.ny // 2
    p.nz_s_r = p.nz - 3
    p.nz_s_l = p.nz + 1 - p.nz_s_r
    p.save_stats_int = 4
    # CFL 1: steps near 4e-4, above the 1.0E-4 at which REM_DIV_CURV stops
    p.variable_dt, p.update_dt, p.cfl, p.delta_t_set = 1, 1, 1.0, 1.0
    sg, so = ekref.sponge_profiles(p, xp, yp)
    g, o = gpu_for(p, xp, yp, st), oracle_for(p, xp, yp, st)
    g.set_sponge(sg, so)
    o.set_sponge(sg, so)
    for n in range(3):
        g.step(1)
        o.step(1)
        tg, ng, dg = g.get_time()
        to, no, do = o.get_time()
        assert ng == no and abs(dg - do) <= 1e-12 * do, n
        compare(g, o, 1e-10, f"step {n + 1}")
