"""CPU tests of the oracle: known answers that pin its FFT convention,
Thomas solver and 9-point multigrid, and its restated metrics."""
import math

import numpy as np
import pytest

from ekcases import refgrid_case, sheared_case, small_case
from oracle import ekref


def test_fft_known_answers():
    nx, nkx = 32, 10
    x = np.arange(nx) * 2 * math.pi / nx
    line = np.zeros(nx + 2)
    line[:nx] = 1.5 + 2.0 * np.cos(3 * x) - 0.5 * np.sin(7 * x)
    c = ekref.fft_r2c(line[None, :], nkx)[0]
    want = np.zeros(nx // 2 + 1, complex)
    want[0] = 1.5
    want[3] = 1.0            # (1/NX) sum 2cos(3x) e^{-i3x} = 1
    want[7] = 0.25j          # -0.5 sin(7x) -> -0.5/(2i) = +0.25i
    assert np.allclose(c, want, atol=1e-14)
    back = ekref.fft_c2r(c[None, :], nkx)[0]
    assert np.allclose(back, line, atol=1e-13)
    assert back[nx] == 0.0 and back[nx + 1] == 0.0


def test_fft_truncation_and_derivative():
    nx, nkx = 64, 21
    rng = np.random.default_rng(0)
    x = np.arange(nx) * 2 * math.pi / nx
    line = np.zeros(nx + 2)
    line[:nx] = np.cos(5 * x) + np.cos(25 * x)    # mode 25 > NX/3 is dropped
    c = ekref.fft_r2c(line[None, :], nkx)[0]
    assert abs(c[25]) == 0.0 and abs(c[5] - 0.5) < 1e-14
    # i k X is the x-derivative (forward sign convention exp(-ikx))
    d = ekref.fft_c2r((1j * np.arange(nx // 2 + 1) * c)[None, :], nkx)[0]
    assert np.allclose(d[:nx], -5 * np.sin(5 * x), atol=1e-12)
    # round trip of band-limited random data; Im of mode 0 is ignored
    cc = np.zeros(nx // 2 + 1, complex)
    cc[1:nkx + 1] = rng.standard_normal(nkx) + 1j * rng.standard_normal(nkx)
    cc[0] = 0.3 + 0.7j
    r = ekref.fft_c2r(cc[None, :], nkx)[0]
    c2 = ekref.fft_r2c(r[None, :], nkx)[0]
    cc[0] = 0.3
    assert np.allclose(c2, cc, atol=1e-13)


def test_thomas_matches_dense():
    rng = np.random.default_rng(3)
    n, nsys = 20, 5
    a = rng.standard_normal((n + 1, nsys))
    c = rng.standard_normal((n + 1, nsys))
    b = 4.0 + np.abs(a) + np.abs(c)
    g = rng.standard_normal((n + 1, nsys))
    x = ekref.thomas(a, b, c, g)
    for s in range(nsys):
        A = np.diag(b[:, s]) + np.diag(a[1:, s], -1) + np.diag(c[:-1, s], 1)
        assert np.allclose(A @ x[:, s], g[:, s], atol=1e-12)


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_multigrid_manufactured_solution(case):
    """Apply dismd2cr's operator to a chosen phi, solve with the residual
    rule, get phi back (kx != 0: the operator is nonsingular)."""
    p, xp, yp, _ = {"small": small_case, "sheared": sheared_case, "refgrid": refgrid_case}[case]()
    p.mg_stop, p.mg_tol, p.mg_maxcy = 1, 1e-12, 200
    m = ekref.metrics_from_grid(p, xp, yp)
    o = ekref.Oracle(p, m)
    rng = np.random.default_rng(5)
    kx2 = np.array([(2 * math.pi / p.lx) ** 2 * k * k for k in (1, 2, 5)])
    phi = rng.standard_normal((len(kx2), p.ny + 2, p.nz + 2))
    rhs = np.stack([o.mg_apply(kx2[q], phi[q]) for q in range(len(kx2))])
    sol, st, code = o.poisson(rhs, kx2)
    assert code == 0, st
    for q in range(len(kx2)):
        assert np.linalg.norm(sol[q] - phi[q]) / np.linalg.norm(phi[q]) < 1e-8


def test_multigrid_reference_stopping_rule():
    """MUDPACK's rule: at most maxcy = 6 cycles, relative change <= REAL*4 1e-6."""
    p, xp, yp, _ = small_case()
    m = ekref.metrics_from_grid(p, xp, yp)
    o = ekref.Oracle(p, m)
    rng = np.random.default_rng(6)
    kx2 = np.array([0.0, 1.0, 4.0])
    rhs = rng.standard_normal((3, p.ny + 2, p.nz + 2))
    _, st, _ = o.poisson(rhs, kx2)
    assert st["max_cycles"] <= 6
    zero = np.zeros((1, p.ny + 2, p.nz + 2))
    phi, st0, code = o.poisson(zero, np.array([1.0]))
    assert code == 0 and st0["max_cycles"] == 1 and not phi.any()


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_left_null_vector_of_the_kx0_operator(case):
    """z with A^T z = 0 for the singular kx = 0 operator: z . (A phi) = 0
    for any phi, |z| = 1; A 1 = 0 holds for the same operator."""
    p, xp, yp, _ = {"small": small_case, "sheared": sheared_case, "refgrid": refgrid_case}[case]()
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    z = o.mg_left_null()
    assert abs(np.linalg.norm(z) - 1.0) < 1e-12
    rng = np.random.default_rng(8)
    for _ in range(3):
        a = o.mg_apply(0.0, rng.standard_normal(z.shape))
        assert abs((z * a).sum()) <= 1e-14 * np.linalg.norm(a)
    assert np.abs(o.mg_apply(0.0, np.ones(z.shape))).max() < 1e-10


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_wellposed_kx0_solve(case):
    """Under the residual rule the kx = 0 problem is solved as a well-posed
    one: b' = b - (z.b) z, ||b' - A phi|| <= tol ||b'||, zero-mean phi, the
    same cycle cap as every problem.  Adding a compatible part to b moves phi
    by the exact solution of that part."""
    p, xp, yp, _ = {"small": small_case, "sheared": sheared_case, "refgrid": refgrid_case}[case]()
    p.mg_stop, p.mg_tol, p.mg_maxcy = 1, 1e-10, 200
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    z = o.mg_left_null()
    rng = np.random.default_rng(9)
    b = rng.standard_normal((1, p.ny + 2, p.nz + 2))
    phi, st, code = o.poisson(b, np.array([0.0]))
    assert code == 0 and st["n_not_converged"] == 0, st
    bp = b[0] - (z * b[0]).sum() * z
    r = bp - o.mg_apply(0.0, phi[0])
    assert np.linalg.norm(r) <= 1.0001e-10 * np.linalg.norm(bp)
    assert abs(phi[0].mean()) < 1e-12 * np.abs(phi[0]).max()
    # a manufactured zero-mean solution comes back
    want = rng.standard_normal(z.shape)
    want -= want.mean()
    got, st2, code2 = o.poisson(o.mg_apply(0.0, want)[None], np.array([0.0]))
    assert code2 == 0
    assert np.linalg.norm(got[0] - want) / np.linalg.norm(want) < 1e-7


def test_oracle_steps_keep_divergence_small():
    p, xp, yp, st = small_case(32, 33, 33)
    m = ekref.metrics_from_grid(p, xp, yp)
    o = ekref.Oracle(p, m)
    o.upload(*st)
    o.rem_div()
    for _ in range(3):
        o.step(1)
        assert np.isfinite(o.divergence()) and o.divergence() < 1e-6
    cu = o.download()
    assert all(np.isfinite(a).all() for a in cu)


def test_reference_grid_fixture():
    p, xp, yp, _ = refgrid_case()
    m = ekref.metrics_from_grid(p, xp, yp)
    dz = xp[0, 1] - xp[0, 0]
    # orthogonal after the 1e-8 truncation of JACOBI_TRANS; J ~ dz*dy
    assert np.abs(m["gmat_12"][:, 1:-2, 1:-2]).max() == 0.0
    dy = np.diff(yp[:, 5])
    jac = m["int_jacob"][1:p.ny + 1, 5]
    assert np.allclose(jac, dz * 0.5 * (dy[:-1] + dy[1:]), rtol=0.2)
    logged = np.load("tests/golden/grid_yz_sub4.npz")["logged_divergence"]
    assert logged.size > 0 and logged.max() < 1e-9
