"""Runs pieces of the reference's own Fortran through fortran_interp (TEST
INFRASTRUCTURE).  Used by make_golden.py to produce golden vectors from the
reference tree; nothing here runs when the tests run.

The reference is compiled for a grid through its `grid_def` include file and
talks to MPI through `mpif.h`; both are generated here for one rank and the
requested sizes.  The MUDPACK grid shape (iixp, jjyq, iiex, jjey) is the
one the oracle and the library pick: p * 2^(k-1) + 1 with the smallest p >= 3.
"""
from __future__ import annotations

import os

import numpy as np

from fortran_interp import Runtime

MPIF_H = """
      integer MPI_STATUS_SIZE, MPI_DOUBLE_PRECISION, MPI_INTEGER, MPI_CHARACTER
      integer MPI_LOGICAL, MPI_DOUBLE_COMPLEX, MPI_COMM_WORLD, MPI_SUM, MPI_MIN, MPI_MAX
      integer MPI_REAL8, MPI_COMPLEX16, MPI_MAX_PROCESSOR_NAME
      parameter (MPI_STATUS_SIZE=5, MPI_DOUBLE_PRECISION=1, MPI_INTEGER=2, MPI_CHARACTER=3)
      parameter (MPI_LOGICAL=4, MPI_DOUBLE_COMPLEX=5, MPI_COMM_WORLD=0, MPI_SUM=1, MPI_MIN=2, MPI_MAX=3)
      parameter (MPI_REAL8=1, MPI_COMPLEX16=5, MPI_MAX_PROCESSOR_NAME=64)
"""


def mg_shape(n):
    """(p, k) with n = p * 2^(k-1) + 1, the smallest p >= 3 (else p = 2)."""
    m, best = n - 1, None
    for k in range(1, 31):
        if (1 << (k - 1)) > m:
            break
        if m % (1 << (k - 1)):
            continue
        p = m >> (k - 1)
        if p < 2:
            continue
        if best is None or (p >= 3 and (best[0] < 3 or p < best[0])):
            best = (p, k)
    return best


def grid_def(nx, ny, nz, n_th=1):
    """The reference's grid_def for one MPI rank (NP = 1)."""
    ixp, iex = mg_shape(nz + 2)
    jyq, jey = mg_shape(ny + 2)
    return f"""
	PARAMETER (NX = {nx})
	PARAMETER (NY = {ny})
	PARAMETER (NZ = {nz})
	PARAMETER (N_TH = {n_th})
	PARAMETER (NZ_S_R = NZ+2)
	PARAMETER (NZ_S_L = NZ + 1 - NZ_S_R)
	PARAMETER (NY_S_T = {max(1, (2 * ny) // 3)})
      PARAMETER (NKX=NX/3)
        INTEGER NYC, NZC, LEVELS, NM
        PARAMETER (NYC=3)
        PARAMETER (NZC=17)
        PARAMETER (NM=177045)
        PARAMETER (LEVELS=8)
	PARAMETER (NP= 1)
	PARAMETER (NZV=ceiling(real(NZ+2)/real(NP))*NP)
	PARAMETER (NXV=ceiling(real(NX+2)/real(NP))*NP)
	PARAMETER (NXP=NXV/NP-1)
	PARAMETER (NZP=NZV/NP-1)
	PARAMETER (NKXV=ceiling(real(NKX+1)/real(NP))*NP)
	PARAMETER (NKXP=NKXV/NP-1)
	PARAMETER (NX2V=ceiling(real(NXV/2)/real(NP))*NP)
	PARAMETER (NX2P=NX2V/NP-1)
	PARAMETER (iixp = {ixp} , jjyq = {jyq}, iiex = {iex}, jjey = {jey} )
	PARAMETER (nnx=iixp*2**(iiex-1)+1, nny=jjyq*2**(jjey-1)+1)
	PARAMETER (llwork=(7*(nnx+2)*(nny+2)+44*nnx*nny)/3 )
"""


SOURCES = ["modules.F90", "mg_solver2d.F90", "mud2cr.f", "mudcom.f", "duct.F90", "boundary.F90", "mpi_duct.F90",
           "ALLOCATION.F90", "diablo.F90"]


def runtime(ref_root, nx, ny, nz, n_th=1):
    """A Runtime holding the reference's hot-path sources built for a grid."""
    rt = Runtime()
    inc = {"grid_def": grid_def(nx, ny, nz, n_th), "mpif.h": MPIF_H}
    for f in SOURCES:
        rt.load(os.path.join(ref_root, "src", f), inc)
    return rt


def set_metrics(rt, m, nz, ny):
    """The metric module arrays (run_variable) from oracle-layout arrays:
    2-D [J, K], face [f, J, K] -> Fortran (0:NZ+2, 0:NY+2[, 2])."""
    for nm in ("gmat_11", "gmat_12", "gmat_22", "cjob_11", "cjob_12", "cjob_21", "cjob_22"):
        rt.allocate("run_variable", nm, [(0, nz + 2), (0, ny + 2), (1, 2)])
        rt.var("run_variable", nm).a[...] = np.transpose(m[nm], (2, 1, 0))
    rt.allocate("run_variable", "int_jacob", [(0, nz + 2), (0, ny + 2)])
    rt.var("run_variable", "int_jacob").a[...] = m["int_jacob"].T


def multigrid_mudpack(rt, kx2, rhs_mg):
    """MULTIGRID_MUDPACK (mg_solver2d.F90:75-201) for one real problem:
    kx2_c = kx2, RHS_TMP = -rhs_mg (phi_bc hands -RHS_TMP to mud2cr, so
    rhs_mg is the right-hand side mud2cr solves with), MUDPACK_BC 0 0 2 2.
    rhs_mg is [J, K]; returns phi [J, K] on (0:NZ+1, 0:NY+1)."""
    rt.module("mg_vari").values["mudpack_bc"].a[...] = [0, 0, 2, 2]
    rt.set_var("fft_var", "kx2_c", float(kx2))
    rt.var("pr_rem", "rhs_tmp").a[...] = -np.asarray(rhs_mg).T
    ptmp = rt.var("pr_rem", "p_tmp")
    ptmp.a[...] = 0.0
    rt.call("multigrid_mudpack", ptmp)
    return ptmp.a.T.copy()
