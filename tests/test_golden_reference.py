"""The oracle against golden vectors from the reference's own source.

tests/golden/make_golden.py runs pieces of the reference tree's Fortran
through an interpreter of the Fortran subset they are written in
(tests/golden/fortran_interp.py: there is no Fortran compiler here) and
stores inputs and outputs as fixtures.  These tests give the oracle the
same inputs and require the same outputs, which pins the oracle's
restatement to the reference itself.

- mudpack_<case>.npz: MULTIGRID_MUDPACK (src/mg_solver2d.F90:75-201, phi_bc
  and cofcr of src/duct.F90:3867-3934, MUDPACK src/mud2cr.f, src/mudcom.f)
  with the reference's settings (FMG + at most 6 W(2,1) cycles, REAL*4 1e-6
  relative change) on the three test grids for kx^2 in {0, 0.3, 1, 7, 50}:
  the oracle's solve must agree bit for bit.
- step_<case>.npz: REM_DIV_CURV and two to five time steps of RK_DUCT
  (src/duct.F90:237-2850) on a uniform, a sheared and the reference's own
  grid (the last with a read-in TH_BAR), with sponge_th on, with phi kept
  in REAL*8, under VARIABLE_DT (COURANT_CURV_MPI), and with the dynamic
  Smagorinsky model (les_chan, les_chan_th) on all three grids: the
  oracle's state, divergences, time step and C_DYN must agree to rounding
  level, JACOBI_TRANS's metrics bit for bit.
"""
import os
import sys

import numpy as np
import pytest

from ekcases import golden_step_cases
from ekman_bl_gb300.params import default_params
from oracle import ekref

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.fail(f"{name} missing: regenerate with tests/golden/make_golden.py")
    return np.load(path)


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_oracle_poisson_equals_reference_mudpack(case):
    g = _fixture(f"mudpack_{case}.npz")
    p = default_params(int(g["nx"]), int(g["ny"]), int(g["nz"]))
    m = {k[len("metric_"):]: np.ascontiguousarray(g[k]) for k in g.files if k.startswith("metric_")}
    o = ekref.Oracle(p, m)
    phi, st, code = o.poisson(g["rhs"], g["kx2"])
    o.close()
    for q, k in enumerate(g["kx2"]):
        ref = g["phi"][q]
        assert np.array_equal(phi[q], ref), (q, k, np.abs(phi[q] - ref).max(), np.abs(ref).max())


def _step_case(name, exact_inputs=True):
    """The fixture and the case's regenerated inputs.  The inputs come from
    numpy's transcendental functions, whose last bits differ between CPU
    architectures; a rounding-level comparison needs the very inputs the
    fixture was made from (checked by digest), a GPU-level one does not."""
    g = _fixture(f"step_{name}.npz")
    sys.path.insert(0, GOLDEN)
    from make_golden import case_digest
    p, xp, yp, st, tb, steps = golden_step_cases()[name]
    if exact_inputs:
        assert case_digest(st, tb) == str(g["inputs_sha256"]), \
            "regenerated inputs differ from the fixture's: another numpy or CPU architecture, or a changed case"
    assert (p.nx, p.ny, p.nz, steps) == (int(g["nx"]), int(g["ny"]), int(g["nz"]), int(g["steps"]))
    return g, p, xp, yp, st, tb, steps


def _oracle_steps(p, xp, yp, st, tb, steps, by_substep):
    m = ekref.metrics_from_grid(p, xp, yp)
    if tb is not None:
        m["th_bar"][:p.ny + 2, :p.nz + 2] = tb
    o = ekref.Oracle(p, m)
    try:
        if p.sponge_type:
            o.set_sponge(*ekref.sponge_profiles(p, xp, yp))
        if p.les:
            o.set_les_metrics(ekref.les_metrics_from_grid(p, xp, yp))
        o.upload(*st)
        o.set_time(p.time, p.time_step)
        o.rem_div()
        divs = [o.divergence()]
        if by_substep:
            # the driver loop spelled out (diablo.F90:109-158): TIME_STEP + 1,
            # RK_DUCT three times, TIME + DELTA_T (the one COURANT_CURV_MPI
            # may have set), FIRST_TIME = .FALSE.
            for _ in range(steps):
                t, ts, _ = o.get_time()
                o.set_time(t, ts + 1)
                for rk in (1, 2, 3):
                    o.rk_substep(rk)
                    divs.append(o.divergence())
                o.set_time(t + o.get_time()[2], ts + 1)
                if p.les:
                    o.les_set_first_time(False)
        else:
            o.step(steps)
        extra = {"time": o.get_time()[0], "delta_t": o.get_time()[2]}
        if p.les:
            extra["c_dyn"] = o.les_state()[1]
        return np.stack(o.download()), divs, extra
    finally:
        o.close()


STEP_CASES = ["small", "sheared", "refgrid", "sponge", "small_phi64", "cfl", "les_small", "les_sheared",
              "les_refgrid"]


@pytest.mark.parametrize("case", STEP_CASES)
def test_oracle_steps_equal_reference_rk_duct(case):
    """REM_DIV_CURV and two RK3 steps of the oracle against the reference's
    own RK_DUCT.  The interpreter evaluates each Fortran expression in
    source order while the oracle's C++ groups a few sums differently, so
    the bar is rounding level: 5e-14 relative L2 for velocity and scalar,
    1e-12 for the pressure, the divergence after every projection to 1e-10
    relative, TIME and DELTA_T (set by COURANT_CURV_MPI in the CFL run) to
    1e-13 and C_DYN of the LES runs to 1e-13 of its largest value.  ekref_step gives the same state as
    the substeps."""
    g, p, xp, yp, st, tb, steps = _step_case(case)
    got, divs, extra = _oracle_steps(p, xp, yp, st, tb, steps, True)
    assert np.array_equal(got, _oracle_steps(p, xp, yp, st, tb, steps, False)[0])
    for k, v in extra.items():
        # C_DYN is a ratio of sums that cancel: its bar is relative to its largest value
        atol = 1e-13 * np.abs(g[k]).max() if k == "c_dyn" else 0.0
        np.testing.assert_allclose(v, g[k], rtol=1e-13, atol=atol, err_msg=k)
    nkx = p.nx // 3
    ref = g["state"]
    for f, name in enumerate(("CU1", "CU2", "CU3", "CP", "CTH")):
        den = np.linalg.norm(ref[f])
        err = np.linalg.norm(got[f, ..., :nkx + 1] - ref[f]) / (den if den > 0 else 1.0)
        # CP sums the Poisson solutions, whose conditioning (~1e3 here) lifts
        # rounding-level differences in their right-hand sides
        assert err <= (1e-12 if name == "CP" else 5e-14), (name, err)
    high = g["state_high"] if "state_high" in g.files else np.zeros_like(got[..., nkx + 1:])
    assert np.array_equal(got[..., nkx + 1:], high)
    np.testing.assert_allclose(divs, g["divergence"], rtol=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("case", STEP_CASES)
def test_gpu_steps_against_reference_rk_duct(case):
    """The library's FP64 path (MUDPACK's own iteration) against the same
    fixtures.  With phi kept in REAL*8 the bar is the plain path's 1e-10;
    where phi is rounded to REAL*4 as the reference does, last-bit
    differences in phi can round the other way, so 1e-6 (the bar of the
    quirk_phi_fp32 tests)."""
    from ekman_bl_gb300 import build as ekbuild
    from ekman_bl_gb300.duct import DuctSolver, les_metrics_from_grid, metrics_from_grid, sponge_profiles
    ekbuild.build()
    g, p, xp, yp, st, tb, steps = _step_case(case, exact_inputs=False)
    m = metrics_from_grid(p, xp, yp)
    if tb is not None:
        m["th_bar"][:p.ny + 2, :p.nz + 2] = tb
    s = DuctSolver(p, m)
    try:
        if p.sponge_type:
            s.set_sponge(*sponge_profiles(p, xp, yp))
        if p.les:
            s.set_les_metrics(les_metrics_from_grid(p, xp, yp))
        s.upload(*st)
        s.set_time(p.time, p.time_step)
        s.rem_div_curv()
        s.step(steps)
        got = np.stack(s.download())
        div = s.divergence()
        t, _, dt = s.get_time()
    finally:
        s.close()
    tol = 1e-6 if p.quirk_phi_fp32 else 1e-10
    nkx = p.nx // 3
    for f, name in enumerate(("CU1", "CU2", "CU3", "CP", "CTH")):
        ref = g["state"][f]
        err = np.linalg.norm(got[f, ..., :nkx + 1] - ref) / np.linalg.norm(ref)
        assert err <= (100 * tol if name == "CP" else tol), (name, err)
    assert div == pytest.approx(float(g["divergence"][-1]), rel=1e-3 if p.quirk_phi_fp32 else 1e-7)
    assert dt == pytest.approx(float(g["delta_t"]), rel=1e-10) and t == pytest.approx(float(g["time"]), rel=1e-10)


@pytest.mark.parametrize("case", ["sheared", "refgrid", "les_sheared", "les_refgrid"])
def test_metrics_equal_reference_jacobi_trans(case):
    """JACOBI_TRANS (src/diablo.F90:1088-1570) as the reference computes it
    from the grid file, the LES branch's GMAT_*_y/_z on the LES runs: the
    oracle's metrics and the library's host routines are equal bit for
    bit."""
    from ekman_bl_gb300.duct import les_metrics_from_grid, metrics_from_grid
    g, p, xp, yp, st, tb, steps = _step_case(case)
    if p.les:
        pairs = (ekref.les_metrics_from_grid(p, xp, yp), les_metrics_from_grid(p, xp, yp))
    else:
        pairs = (ekref.metrics_from_grid(p, xp, yp), metrics_from_grid(p, xp, yp))
    keys = [k[len("metric_"):] for k in g.files if k.startswith("metric_")]
    assert len(keys) == (6 if p.les else 8)
    for m in pairs:
        for k in keys:
            ref = g[f"metric_{k}"]
            assert np.array_equal(m[k], ref), (k, np.abs(m[k] - ref).max())
