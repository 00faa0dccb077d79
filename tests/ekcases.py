"""Small seeded cases shared by the tests (sizes the oracle finishes in
seconds).  Fields are synthetic: a laminar Ekman spiral plus Gaussian noise,
as described in ekman_bl_gb300.params."""
from __future__ import annotations

import math
import os

import numpy as np

from ekman_bl_gb300.params import (EK_MG_STOP_RELCHANGE, EK_YMAX, EK_YMIN, EK_ZMAX, EK_ZMIN, Workload,
                                   default_params, ekman_state, make_grid, workload_setup)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def small_case(nx=16, ny2=17, nz2=17, ri=0.1, seed=0, mg_stop=EK_MG_STOP_RELCHANGE):
    w = Workload("small", nx, ny2, nz2, 400.0, 0.7, ri, 1e-3, 10, 1e-10, 0.01, 4 * math.pi, 0.4, seed)
    return workload_setup(w, mg_stop)


def sheared_case(nx=16, ny2=17, nz2=33, seed=1):
    """Non-orthogonal grid: streamwise points shifted with height, so GMAT_12
    and the diagonal MUDPACK couplings are nonzero."""
    p, xp, yp, st = small_case(nx, ny2, nz2, seed=seed)
    dz = xp[0, 1] - xp[0, 0]
    j = np.arange(p.ny + 2)[:, None]
    xp = xp + 0.3 * dz * np.sin(2 * math.pi * j / (p.ny + 1))
    return p, np.ascontiguousarray(xp), yp, st


def refgrid_case(nx=16, seed=2, stride=1):
    """The reference's own y-z grid (rundir_unst/GRID_YZ.dat, every 4th
    point; every 8th with stride 2) with the shipped input.dat physics:
    NU=1.3e-4, F_0=1e-4, WBULK0=0.05, LX=60, scalar bottom BC type 5 with
    C1=1.56e-3."""
    g = np.load(os.path.join(GOLDEN, "grid_yz_sub4.npz"))
    xp = np.ascontiguousarray(g["xpoint"][::stride, ::stride])
    yp = np.ascontiguousarray(g["ypoint"][::stride, ::stride])
    ny2, nz2 = xp.shape
    p = default_params(nx, ny2 - 2, nz2 - 2)
    p.nu, p.f0, p.wbulk0, p.lx, p.delta_t = 1.3e-4, 1.0e-4, 0.05, 60.0, 3.0
    p.pr, p.ri_tau, p.cont_strat = 1.0, 0.0, 0
    p.th_bc[EK_YMIN], p.th_bc[EK_YMAX], p.th_bc[EK_ZMIN], p.th_bc[EK_ZMAX] = 5, 1, 6, 6
    p.th_bc_c1[EK_YMIN] = 1.56e-3
    st = ekman_state(p, yp, 0.01, seed)
    return p, xp, yp, st


def sponge_case(sponge_type, dynamic=True, save_stats_int=4, nx=16):
    """small_case with sponge_th on (SPONGE_TYPE 1 parabolic, 2 exponential):
    a top sponge from NY_S_T = NY/2 and streamwise sponges on the last and
    first four K.  dynamic=False puts WBULK0 exactly in the top layer of the
    mean streamwise flow, so the dynamic mean-flow branch stays idle."""
    p, xp, yp, st = small_case(nx=nx)
    p.sponge_type = sponge_type
    p.ny_s_t = p.ny // 2
    p.nz_s_r = p.nz - 3           # streamwise sponge on the last 4 K and first ones
    p.nz_s_l = p.nz + 1 - p.nz_s_r
    p.save_stats_int = save_stats_int
    p.time_step = 0
    st = [a.copy() for a in st]
    if not dynamic:
        # upper layer of CU3X(0,K,J) exactly WBULK0: |mean - WBULK0| = 0
        st[2][p.ny_s_t:, :, 0] = p.wbulk0
    return p, xp, yp, st


def les_case(case="small", noise=0.3, seed=4, **grid):
    """A test grid with the dynamic Smagorinsky terms on from the first step
    (CREATE_NEW_FLOW = 0) and a noisier state; grid goes to the grid's case
    function (nx, stride)."""
    base = {"small": small_case, "sheared": sheared_case, "refgrid": refgrid_case}[case]
    p, xp, yp, _ = base(**grid)
    st = ekman_state(p, yp, noise, seed)
    if case != "refgrid":
        # a nonzero scalar and Kelvin-Helmholtz-like shear for a lively subgrid field
        st = list(st)
        rng = np.random.default_rng(seed + 1)
        sub = (p.ny, p.nz, p.nx // 3)
        st[4][1:p.ny + 1, 1:p.nz + 1, 1:p.nx // 3 + 1] += noise * (rng.standard_normal(sub) + 1j * rng.standard_normal(sub))
    p.les, p.les_model_type, p.les_model_type_th, p.create_new_flow = 1, 2, 1, 0
    return p, xp, yp, tuple(st)


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0)


def cfl_case(cfl, delta_t_set, nx=16):
    """small_case under VARIABLE_DT: COURANT_CURV_MPI after every step's
    RK_STEP = 3 ADI (UPDATE_DT = 1)."""
    p, xp, yp, st = small_case(nx=nx)
    p.variable_dt, p.update_dt, p.cfl, p.delta_t_set = 1, 1, cfl, delta_t_set
    return p, xp, yp, st


def th_bar_profile(p, xpoint, ypoint):
    """A read-in background scalar TH_BAR [J, K] for runs without
    CONT_STRAT (JACOBI_TRANS reads it from density_data_input.dat): linear
    in height with a 10 % modulation along z, so that its GMAT_12 terms are
    nonzero on a curvilinear grid."""
    zz = xpoint - xpoint.min()
    yy = ypoint.max() - ypoint
    return 1e-3 * yy * (1.0 + 0.1 * np.sin(2 * math.pi * zz / zz.max()))


def golden_step_cases():
    """The runs of the reference's RK_DUCT kept as fixtures (step_<name>.npz):
    name -> (p, xpoint, ypoint, state, th_bar or None, steps).  p has
    quirk_phi_fp32 = 1, the reference's own rounding of phi, except in
    small_phi64.  les_small's five steps cover C_DYN computed with
    FIRST_TIME, kept, and recomputed at TIME_STEP 5."""
    out = {}
    for name, case, steps in (("small", small_case, 2), ("sheared", lambda: sheared_case(nx=8), 2),
                              ("refgrid", lambda: refgrid_case(8, stride=2), 2),
                              ("sponge", lambda: sponge_case(2, True, save_stats_int=4, nx=8), 2),
                              ("small_phi64", lambda: small_case(nx=8), 2),
                              ("cfl", lambda: cfl_case(0.2, 1.0, nx=8), 2),
                              ("les_small", lambda: les_case("small"), 5),
                              ("les_sheared", lambda: les_case("sheared", nx=8), 2),
                              ("les_refgrid", lambda: les_case("refgrid", nx=8, stride=2), 2)):
        p, xp, yp, st = case()
        p.quirk_phi_fp32 = 0 if name.endswith("phi64") else 1
        tb = None if p.cont_strat else th_bar_profile(p, xp, yp)
        out[name] = (p, xp, yp, st, tb, steps)
    return out
