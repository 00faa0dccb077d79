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


def grid_def(nx, ny, nz, n_th=1, sponge=None):
    """The reference's grid_def for one MPI rank (NP = 1); sponge = (NY_S_T,
    NZ_S_R, NZ_S_L), the first points of the sponge layers."""
    ixp, iex = mg_shape(nz + 2)
    jyq, jey = mg_shape(ny + 2)
    ny_s_t, nz_s_r, nz_s_l = sponge if sponge else (max(1, (2 * ny) // 3), nz + 2, -1)
    return f"""
	PARAMETER (NX = {nx})
	PARAMETER (NY = {ny})
	PARAMETER (NZ = {nz})
	PARAMETER (N_TH = {n_th})
	PARAMETER (NZ_S_R = {nz_s_r})
	PARAMETER (NZ_S_L = {nz_s_l})
	PARAMETER (NY_S_T = {ny_s_t})
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
           "ALLOCATION.F90", "diablo.F90", "les_chan.F90", "les_chan_th.F90"]


def runtime(ref_root, nx, ny, nz, n_th=1, sponge=None, phi64=False):
    """A Runtime holding the reference's hot-path sources built for a grid.
    phi64: REM_DIV_CURV's CMPLX(P_TMP2, P_TMP) (duct.F90:2664, 2700) keeps
    phi in REAL*8 instead of rounding it to default REAL."""
    rt = Runtime()
    if phi64:
        rt.cmplx_default = "c16"
    inc = {"grid_def": grid_def(nx, ny, nz, n_th, sponge), "mpif.h": MPIF_H}
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


# ---------------------------------------------------------------------------
# time stepping: INITIALIZE's READ_FLOW path, then the driver's DO RK_STEP
def _fft_stubs(rt, nx, nz, ny):
    """FFT_X_TO_FOURIER_OP / FFT_X_TO_PHYSICAL_OP, whose source (fft.F90) is
    missing from the reference tree: the oracle's line transforms, forward
    (1/NX) sum u e^{-2 pi i k n/NX} for k <= NKX = NX/3 and zero above,
    inverse the Hermitian sum over k <= NKX.  VARP(0:NX+1, 0:NZP, 0:NY+1)
    and CVARP(0:NX/2, 0:NZP, 0:NY+1) share storage (EQUIVALENCE), so each
    reads its input before it writes its output."""
    from oracle import ekref
    nk, ny2, nkx = nz + 2, ny + 2, nx // 3

    def lines(jmin, jmax, kmin, kmax):
        j0, j1, k0, k1 = (int(x.flat[0]) for x in (jmin, jmax, kmin, kmax))
        return [(j, k) for j in range(j0, j1 + 1) for k in range(k0, k1 + 1)]

    def as_real(a):
        f = a.flat.view(np.float64) if a.flat.dtype == np.complex128 else a.flat
        return f[:(nx + 2) * nk * ny2].reshape((nx + 2, nk, ny2), order="F")

    def as_cplx(a):
        f = a.flat.view(np.complex128) if a.flat.dtype == np.float64 else a.flat
        return f[:(nx // 2 + 1) * nk * ny2].reshape((nx // 2 + 1, nk, ny2), order="F")

    def forward(varp, cvarp, jmin, jmax, kmin, kmax):
        sel = lines(jmin, jmax, kmin, kmax)
        x = np.stack([as_real(varp)[:, k, j] for j, k in sel])
        c = ekref.fft_r2c(x, nkx)
        out = as_cplx(cvarp)
        for (j, k), row in zip(sel, c):
            out[:, k, j] = row

    def inverse(cvarp, varp, jmin, jmax, kmin, kmax):
        sel = lines(jmin, jmax, kmin, kmax)
        c = np.stack([as_cplx(cvarp)[:, k, j] for j, k in sel])
        y = ekref.fft_c2r(c, nkx)
        out = as_real(varp)
        for (j, k), row in zip(sel, y):
            out[:, k, j] = row

    rt.provide("fft_x_to_fourier_op", forward)
    rt.provide("fft_x_to_physical_op", inverse)


def _mpi_stubs(rt):
    """MPI with one rank: the collectives copy their send buffers."""
    def copy(sbuf, scount, stype, rbuf, *rest):
        n = int(scount.flat[0])
        rbuf.flat[:n] = sbuf.flat[:n]
        rest[-1].flat[0] = 0

    def bcast(buf, count, dtype, root, comm, ierr):
        ierr.flat[0] = 0

    for name in ("mpi_alltoall", "mpi_gather", "mpi_allgather"):
        rt.provide(name, copy)
    rt.provide("mpi_bcast", bcast)
    rt.provide("mpi_barrier", lambda comm, ierr: None)


def duct_setup(rt, p, xpoint, ypoint, state, th_bar=None):
    """The module state INITIALIZE (diablo.F90:193-668) leaves on its
    READ_FLOW path, with input.dat's values taken from the run parameters p
    and the flow from state (CU1X, CU2X, CU3X, CPX, CTHX as [J, K, I]):
    allocate_var, INITIALIZE's derived sizes, JACOBI_TRANS on the grid
    points (GRID_YZ.dat written from xpoint / ypoint; without CONT_STRAT it
    reads TH_BAR [J, K], zero if None, from density_data_input.dat),
    INIT_FFT's wavenumbers, the RKW3 constants, INIT_DUCT, the spectral
    arrays, the state.  INIT_FLAG is left .FALSE.: the first projection's
    discarded extra solve leaves no state behind.  The two SAVE_STATS_CURVI
    calls that end INITIALIZE are not made: they take the flow through
    physical space and back, which changes it in the last bit."""
    nx, ny, nz = p.nx, p.ny, p.nz
    _fft_stubs(rt, nx, nz, ny)
    _mpi_stubs(rt)
    R = "run_variable"
    sv = rt.set_var
    sv("grid", "lx", p.lx)
    sv("time_step_var", "delta_t", p.delta_t)
    sv("time_step_var", "delta_t_set", p.delta_t_set)
    for k, v in (("nu", p.nu), ("f_0", p.f0), ("wbulk0", p.wbulk0), ("px0", p.px0), ("f_type", p.f_type),
                 ("omega0", p.omega0), ("amp_omega0", p.amp_omega0), ("time", p.time), ("time_step", p.time_step),
                 ("cont_strat", bool(p.cont_strat)), ("mudpack_use", True), ("les", bool(p.les)),
                 ("les_model_type", p.les_model_type), ("les_model_type_th", p.les_model_type_th),
                 ("wall_model_type", 0), ("sponge_type", p.sponge_type), ("variable_dt", bool(p.variable_dt)),
                 ("update_dt", p.update_dt), ("cfl", p.cfl), ("ic_type", p.ic_type),
                 ("create_new_flow", bool(p.create_new_flow)), ("int_treat", False), ("wave_abs", False),
                 ("save_stats_int", p.save_stats_int), ("first_time", True)):
        sv(R, k, v)
    rt.var(R, "pr").a[0] = p.pr
    rt.var(R, "ri_tau").a[0] = p.ri_tau
    walls = ("ymin", "ymax", "zmin", "zmax")
    for f, bc, c1 in (("u", p.u_bc, p.u_bc_c1), ("v", p.v_bc, p.v_bc_c1), ("w", p.w_bc, p.w_bc_c1)):
        for i, wall in enumerate(walls):
            sv(R, f"{f}_bc_{wall}", bc[i])
            sv(R, f"{f}_bc_{wall}_c1", c1[i])
    for i, wall in enumerate(walls):
        rt.var(R, f"th_bc_{wall}").a[0] = p.th_bc[i]
        rt.var(R, f"th_bc_{wall}_c1").a[0] = p.th_bc_c1[i]
    rt.module("mg_vari").values["mudpack_bc"].a[...] = [0, 0, 2, 2]
    sv("mg_vari", "init_flag", False)
    sv("mpi_var", "rank", 0)
    sv("mpi_var", "nproces", 1)
    rt.call("allocate_var")
    if p.les:
        rt.call("allocation_les_var")
    # the sizes INITIALIZE derives after reading input.dat (diablo.F90:398-408);
    # grid_def's NXP = NXV/NP - 1 = NX + 1 with NP = 1
    sv("domain", "nxm", nx - 1)
    sv("domain", "nym", ny - 1)
    sv("domain", "nzm", nz - 1)
    sv("domain", "nxp_l", nx - 1)
    sv("domain", "nx2p_l", nx // 3)
    gx, dx = rt.var("grid", "gx").a, rt.var("grid", "dx").a
    for i in range(nx + 2):
        gx[i] = (i * p.lx) / nx
        dx[i] = p.lx / nx
    # JACOBI_TRANS reads the grid points (J outer, K inner) from GRID_YZ.dat
    rt.files["GRID_YZ.dat"] = "".join(f"{float(xpoint[j, k])!r} {float(ypoint[j, k])!r}\n"
                                      for j in range(ny + 2) for k in range(nz + 2))
    tb = np.zeros((ny + 2, nz + 2)) if th_bar is None else th_bar
    rt.files["density_data_input.dat"] = "".join(f"{float(tb[j, k])!r}\n"
                                                 for j in range(ny + 2) for k in range(nz + 2))
    rt.call("jacobi_trans")
    # INIT_FFT (fft.F90, missing): KXP(I) = I (2 pi) / LX, KX2P = KXP^2, CIKXP = i KXP
    kxp = np.array([i * (2.0 * np.pi) / p.lx for i in range(nx // 2 + 1)])
    rt.var("fft_var", "kxp").a[...] = kxp
    rt.var("fft_var", "kx2p").a[...] = kxp * kxp
    rt.var("fft_var", "cikxp").a[...] = 1j * kxp
    h = rt.var(R, "h_bar").a
    h[0], h[1], h[2] = p.delta_t * (8.0 / 15.0), p.delta_t * (2.0 / 15.0), p.delta_t * (5.0 / 15.0)
    b = rt.var(R, "beta_bar").a
    b[0], b[1], b[2] = 1.0, 25.0 / 8.0, 9.0 / 4.0
    z = rt.var(R, "zeta_bar").a
    z[0], z[1], z[2] = 0.0, -17.0 / 8.0, -5.0 / 4.0
    rt.call("init_duct")
    for name in ("u", "v", "w", "p", "th", "r1", "r2", "r3", "rth", "f1", "f2", "f3", "fth"):
        rt.call(f"allocation_{name}", False)
    set_state(rt, state)


def set_state(rt, state):
    R = "run_variable"
    for name, a in zip(("cu1x", "cu2x", "cu3x", "cpx"), state[:4]):
        rt.var(R, name).a[...] = np.transpose(a, (2, 1, 0))
    rt.var(R, "cthx").a[..., 0] = np.transpose(state[4], (2, 1, 0))
    for name in ("cf1x", "cf2x", "cf3x", "cfthx"):
        rt.var(R, name).a[...] = 0.0


def get_state(rt):
    R = "run_variable"
    out = [np.ascontiguousarray(np.transpose(rt.var(R, n).a, (2, 1, 0))) for n in ("cu1x", "cu2x", "cu3x", "cpx")]
    out.append(np.ascontiguousarray(np.transpose(rt.var(R, "cthx").a[..., 0], (2, 1, 0))))
    return out


def record_divergence(rt):
    """Collect the divergence REM_DIV_CURV prints after each projection: the
    one-value MPI_COMBINE_STATS(DIV, 1, 1) of the step (duct.F90:2801-2813)."""
    rt.divergence = []
    combine = rt.proc("mpi_combine_stats")

    def wrapped(stat, zs, ys):
        combine(stat, zs, ys)
        if int(zs.flat[0]) * int(ys.flat[0]) == 1:
            rt.divergence.append(float(stat.flat[0]))
    rt.provide("mpi_combine_stats", wrapped)


def rem_div_curv(rt):
    rt.call("rem_div_curv")


def rk_step(rt):
    """One time step of the driver loop (diablo.F90:109-168): TIME_STEP + 1,
    DO RK_STEP = 1, 3: CALL RK_DUCT, TIME + DELTA_T, FIRST_TIME = .FALSE.
    RI_TAU stays RI_FINAL without INT_TREAT.  The runs made here stop short
    of SAVE_STATS_INT: SAVE_STATS_CURVI (flow_statistics.F90:2) takes the
    flow through physical space and back, which changes it in the last bit,
    and writes files."""
    R = "run_variable"
    rt.var(R, "time_step")[0] += 1
    for rk in (1, 2, 3):
        rt.set_var(R, "rk_step", rk)
        rt.call("rk_duct")
    rt.var(R, "time")[0] += rt.var("time_step_var", "delta_t")[0]
    rt.set_var(R, "first_time", False)
