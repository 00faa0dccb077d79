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


def refgrid_case(nx=16, seed=2):
    """The reference's own y-z grid (rundir_unst/GRID_YZ.dat, every 4th
    point) with the shipped input.dat physics: NU=1.3e-4, F_0=1e-4,
    WBULK0=0.05, LX=60, scalar bottom BC type 5 with C1=1.56e-3."""
    g = np.load(os.path.join(GOLDEN, "grid_yz_sub4.npz"))
    xp, yp = g["xpoint"], g["ypoint"]
    ny2, nz2 = xp.shape
    p = default_params(nx, ny2 - 2, nz2 - 2)
    p.nu, p.f0, p.wbulk0, p.lx, p.delta_t = 1.3e-4, 1.0e-4, 0.05, 60.0, 3.0
    p.pr, p.ri_tau, p.cont_strat = 1.0, 0.0, 0
    p.th_bc[EK_YMIN], p.th_bc[EK_YMAX], p.th_bc[EK_ZMIN], p.th_bc[EK_ZMAX] = 5, 1, 6, 6
    p.th_bc_c1[EK_YMIN] = 1.56e-3
    st = ekman_state(p, yp, 0.01, seed)
    return p, xp, yp, st


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0)
