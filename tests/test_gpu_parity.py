"""GPU parity: the CUDA path through the C ABI against the oracle on the same
seeded inputs.  Tolerances: relative L2 <= 1e-10 after many steps of the
FP64 path (the bar of the reference's plain method), tighter for single
operations; multigrid cycle counts must match exactly."""
import math

import numpy as np
import pytest

from ekcases import refgrid_case, rel_l2, sheared_case, small_case
from ekman_bl_gb300 import build as ekbuild
from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
from ekman_bl_gb300.params import (EK_MG_STOP_RESIDUAL, EK_F_CF1, EK_F_CF2, EK_F_CF3, EK_F_CFTH, EK_F_CR1, WORKLOADS,
                                   workload_setup)
from oracle import ekref

pytestmark = pytest.mark.gpu

CASES = {"small": small_case, "sheared": sheared_case, "refgrid": refgrid_case}


@pytest.fixture(scope="module", autouse=True)
def _build():
    ekbuild.build()


def pair(case, **over):
    p, xp, yp, st = CASES[case]() if isinstance(case, str) else case
    for k, v in over.items():
        setattr(p, k, v)
    m = metrics_from_grid(p, xp, yp)
    g = DuctSolver(p, m)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    g.upload(*st)
    o.upload(*st)
    return p, g, o


def compare_state(g, o, tol, fields=True):
    a, b = g.download(), o.download()
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), a, b):
        e = rel_l2(x, y)
        assert e <= tol, f"{name}: rel L2 {e:.3e} > {tol:.1e}"
    return a, b


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
@pytest.mark.parametrize("stop", [0, 1])
def test_poisson_batch_matches_oracle(case, stop):
    p, xp, yp, _ = CASES[case]()
    p.mg_stop = stop
    if stop == 1:
        p.mg_tol, p.mg_maxcy = 1e-10, 40
    m = metrics_from_grid(p, xp, yp)
    g = DuctSolver(p, m)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    rng = np.random.default_rng(11)
    kx2 = np.array([0.0, 0.3, 1.0, 7.0, 50.0])
    rhs = rng.standard_normal((len(kx2), p.ny + 2, p.nz + 2))
    pg, sg, cg = g.multigrid_mudpack(rhs, kx2)
    po, so, co = o.poisson(rhs, kx2)
    assert (sg["min_cycles"], sg["max_cycles"], sg["n_not_converged"]) == \
        (so["min_cycles"], so["max_cycles"], so["n_not_converged"])
    assert cg == co
    for q in range(len(kx2)):
        assert rel_l2(pg[q], po[q]) < 1e-12, q


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_rem_div_matches_oracle(case):
    p, g, o = pair(case)
    g.rem_div_curv()
    o.rem_div()
    compare_state(g, o, 1e-12)
    assert rel_l2(g.get_field(EK_F_CR1), o.get_field(EK_F_CR1)) < 1e-12
    assert g.divergence() == pytest.approx(o.divergence(), rel=1e-6, abs=1e-14)


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_three_substeps_match_oracle(case):
    p, g, o = pair(case)
    for rk in (1, 2, 3):
        g.rk_duct(rk)
        o.rk_substep(rk)
        compare_state(g, o, 1e-11)
        for f in (EK_F_CF1, EK_F_CF2, EK_F_CF3, EK_F_CFTH, EK_F_CR1):
            assert rel_l2(g.get_field(f), o.get_field(f)) < 1e-11, (rk, f)
        assert g.mg_stats()["max_cycles"] == o.mg_stats()["max_cycles"]


def test_hundred_steps_neutral_64():
    """The CPU-runnable neutral case (64 x 65 x 65, 100 RK3 steps,
    dt = 1e-3): FP64 path within 1e-10 relative L2 of the oracle."""
    w = WORKLOADS["ekman_neutral_64x65x65"]
    p, g, o = pair(workload_setup(w))
    g.rem_div_curv()
    o.rem_div()
    g.step(100)
    o.step(100)
    compare_state(g, o, 1e-10)
    assert g.divergence() < 1e-8


def test_quirk_phi_fp32():
    """Q1: phi rounded to REAL*4 before the projection (duct.F90:2664)."""
    p, g, o = pair("small", quirk_phi_fp32=1)
    g.step(2)
    o.step(2)
    compare_state(g, o, 1e-6)


def test_nan_state_reports_error():
    p, g, o = pair("small")
    cu = g.download()
    cu[0][3, 3, 1] = np.nan
    g.upload(*cu)
    with pytest.raises(Exception) as e:
        g.step(1)
    assert "NAN" in str(e.value)


@pytest.mark.parametrize("nx", [16, 64, 256, 1024])
def test_fft_entry_points_match_oracle(nx):
    """ekgpu_fft_x_to_fourier / _to_physical against the oracle's transform."""
    torch = pytest.importorskip("torch")
    from ekman_bl_gb300.duct import fft_x
    nkx = nx // 3
    nlines = 37
    rng = np.random.default_rng(nx)
    x = np.zeros((nlines, nx + 2))
    x[:, :nx] = rng.standard_normal((nlines, nx))
    xd = torch.from_numpy(x).cuda()
    cd = torch.zeros((nlines, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    fft_x(True, nx, nkx, nlines, xd.data_ptr(), cd.data_ptr())
    torch.cuda.synchronize()
    want = ekref.fft_r2c(x, nkx)
    assert rel_l2(cd.cpu().numpy(), want) < 1e-14
    yd = torch.zeros((nlines, nx + 2), dtype=torch.float64, device="cuda")
    fft_x(False, nx, nkx, nlines, cd.data_ptr(), yd.data_ptr())
    torch.cuda.synchronize()
    assert rel_l2(yd.cpu().numpy(), ekref.fft_c2r(want, nkx)) < 1e-14


def test_fft_entry_point_rejects_bad_size():
    from ekman_bl_gb300.duct import EkError, fft_x
    with pytest.raises(EkError) as e:
        fft_x(True, 48, 16, 1, 1, 1)
    assert "power of two" in str(e.value)


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_mixed_precision_poisson_reaches_tolerance(case):
    """mg_fast = 1: FP64 refinement around FP32 line-smoothed V-cycles.  The
    FP64 residual of the returned phi, recomputed with the oracle's operator,
    must be <= tol for every non-singular problem, and phi must agree with
    the oracle's FP64 solve at the same tolerance."""
    p, xp, yp, _ = CASES[case]()
    p.mg_stop, p.mg_tol, p.mg_maxcy, p.mg_fast = 1, 1e-10, 60, 1
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    po_ = CASES[case]()[0]
    po_.mg_stop, po_.mg_tol, po_.mg_maxcy = 1, 1e-12, 200
    o = ekref.Oracle(po_, ekref.metrics_from_grid(po_, xp, yp))
    rng = np.random.default_rng(12)
    # the case's own wavenumbers kx = 2 pi k / LX, k = 1, 2, 5, NX/3
    kx2 = np.array([(2 * math.pi * k / p.lx) ** 2 for k in (1, 2, 5, p.nx // 3)])
    rhs = rng.standard_normal((len(kx2), p.ny + 2, p.nz + 2))
    rhs[:, 0, :] = 0
    rhs[:, -1, :] = 0
    pg, sg, cg = g.multigrid_mudpack(rhs, kx2)
    assert cg == 0 and sg["n_not_converged"] == 0, sg
    assert sg["max_cycles"] <= 40, sg
    po, so, co = o.poisson(rhs, kx2)
    for q in range(len(kx2)):
        r = rhs[q] - o.mg_apply(kx2[q], pg[q])
        assert np.linalg.norm(r) / np.linalg.norm(rhs[q]) <= 1.05e-10, q
        assert rel_l2(pg[q], po[q]) < 1e-6, q


def test_mixed_precision_steps_track_oracle():
    """Three RK3 steps with the mixed-precision projection vs the oracle's
    FP64 projection at the same 1e-10 residual."""
    p, xp, yp, st = small_case()
    p.mg_stop, p.mg_tol, p.mg_maxcy = 1, 1e-10, 60
    m = metrics_from_grid(p, xp, yp)
    p.mg_fast = 1
    g = DuctSolver(p, m)
    po_ = small_case()[0]
    po_.mg_stop, po_.mg_tol, po_.mg_maxcy = 1, 1e-10, 200
    o = ekref.Oracle(po_, ekref.metrics_from_grid(po_, xp, yp))
    g.upload(*st)
    o.upload(*st)
    g.step(3)
    o.step(3)
    a, b = g.download(), o.download()
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), a, b):
        assert rel_l2(x, y) < 1e-7, name
    assert g.divergence() < 1e-7


@pytest.mark.parametrize("ff", [1, 2])
def test_mixed_path_hundred_steps_neutral_64(ff):
    """The mixed-precision path (FP32 V-cycles inside FP64 refinement at
    1e-10, FP32 arithmetic in the nonlinear-term transforms; ff = 1: the
    state's transforms and ADI in float-float, ff = 2: in FP32 on
    increments) against the FP64 oracle after 100 steps of the 64 x 65 x 65
    case: velocity and buoyancy within 1e-5 relative L2, divergence below
    1e-8."""
    w = WORKLOADS["ekman_neutral_64x65x65"]
    p, xp, yp, st = workload_setup(w, EK_MG_STOP_RESIDUAL)
    p.mg_tol, p.mg_maxcy = 1e-10, 200
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    q = workload_setup(w, EK_MG_STOP_RESIDUAL)[0]
    q.mg_tol, q.mg_maxcy, q.mg_fast, q.fft_fp32, q.ff_arith = 1e-10, 60, 1, 1, ff
    g = DuctSolver(q, metrics_from_grid(q, xp, yp))
    g.upload(*st)
    o.upload(*st)
    g.rem_div_curv()
    o.rem_div()
    g.step(100)
    o.step(100)
    a, b = g.download(), o.download()
    errs = {n: rel_l2(x, y) for n, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), a, b)}
    print(f"mixed path ff_arith={ff} after 100 steps of 64x65x65:", errs)
    for name in ("CU1", "CU2", "CU3", "CTH"):
        assert errs[name] < 1e-5, name
    assert g.divergence() < 1e-8


def test_float_float_transforms_hundred_steps():
    """ff_arith = 1 on the FP64 path: the transforms in float-float arithmetic
    stay within 1e-10 of the FP64 oracle after 100 steps (measured ~1e-12)."""
    w = WORKLOADS["ekman_neutral_64x65x65"]
    p, xp, yp, st = workload_setup(w)
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    q = workload_setup(w)[0]
    q.ff_arith = 1
    g = DuctSolver(q, metrics_from_grid(q, xp, yp))
    g.upload(*st)
    o.upload(*st)
    g.rem_div_curv()
    o.rem_div()
    g.step(100)
    o.step(100)
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
        assert rel_l2(x, y) < 1e-10, name


def test_mixed_precision_poisson_tall_grid():
    """Lines longer than 287 rows take the line solver's 16-problem layout
    (up to 64 segments): a 17 x 321 grid (NZ+2 x NY+2) to 1e-10, checked with
    the oracle's operator."""
    p, xp, yp, _ = small_case(nx=16, ny2=321, nz2=17)
    p.mg_stop, p.mg_tol, p.mg_maxcy, p.mg_fast = 1, 1e-10, 60, 1
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    kx2 = np.array([(2 * math.pi * k / p.lx) ** 2 for k in (1, 3)])
    rhs = np.random.default_rng(5).standard_normal((len(kx2), p.ny + 2, p.nz + 2))
    rhs[:, 0, :] = 0
    rhs[:, -1, :] = 0
    pg, sg, cg = g.multigrid_mudpack(rhs, kx2)
    assert cg == 0 and sg["n_not_converged"] == 0, sg
    for q in range(len(kx2)):
        r = rhs[q] - o.mg_apply(kx2[q], pg[q])
        assert np.linalg.norm(r) / np.linalg.norm(rhs[q]) <= 1.05e-10, q
