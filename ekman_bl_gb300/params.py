"""Run parameters, geometry and synthetic initial fields of the duct substep.

`EkParams`, `EkMetrics` and `EkMgStats` mirror the structs of include/ekgpu.h
field for field.  The parameter names follow the reference's input.dat and
grid_def (src/diablo.F90:242-337, rundir_unst/grid_def).  The named
workloads below stand in for a dataset: the reference ships no benchmark
data, so fields are synthetic and seeded.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

EK_YMIN, EK_YMAX, EK_ZMIN, EK_ZMAX = 0, 1, 2, 3
EK_MG_STOP_RELCHANGE, EK_MG_STOP_RESIDUAL = 0, 1
(EK_F_CU1, EK_F_CU2, EK_F_CU3, EK_F_CP, EK_F_CTH, EK_F_CF1, EK_F_CF2, EK_F_CF3,
 EK_F_CFTH, EK_F_CR1) = range(10)

STATUS = {0: "EK_OK", 1: "EK_ERR_ARG", 2: "EK_ERR_CUDA", 3: "EK_ERR_NOT_CONVERGED",
          4: "EK_ERR_NAN", 5: "EK_ERR_TIMEOUT", 6: "EK_ERR_STATE",
          7: "EK_ERR_IO", 8: "EK_ERR_DT"}

# REAL*4 literal 10.0**(-6) of mg_solver2d.F90:188, widened to REAL*8.
MUDPACK_TOLMAX = float(np.float32(10.0) ** np.float32(-6))


class EkParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("lx", C.c_double), ("nu", C.c_double), ("delta_t", C.c_double),
        ("f0", C.c_double), ("wbulk0", C.c_double),
        ("f_type", C.c_int),
        ("px0", C.c_double), ("omega0", C.c_double), ("amp_omega0", C.c_double), ("time", C.c_double),
        ("n_th", C.c_int), ("pr", C.c_double), ("ri_tau", C.c_double),
        ("cont_strat", C.c_int), ("ic_type", C.c_int),
        ("u_bc", C.c_int * 4), ("v_bc", C.c_int * 4), ("w_bc", C.c_int * 4), ("th_bc", C.c_int * 4),
        ("u_bc_c1", C.c_double * 4), ("v_bc_c1", C.c_double * 4),
        ("w_bc_c1", C.c_double * 4), ("th_bc_c1", C.c_double * 4),
        ("mudpack_bc", C.c_int * 4),
        ("mg_ixp", C.c_int), ("mg_jyq", C.c_int), ("mg_iex", C.c_int), ("mg_jey", C.c_int),
        ("mg_maxcy", C.c_int), ("mg_kcycle", C.c_int), ("mg_iprer", C.c_int), ("mg_ipost", C.c_int),
        ("mg_intpol", C.c_int), ("mg_stop", C.c_int), ("mg_tol", C.c_double),
        ("quirk_phi_fp32", C.c_int), ("mg_fast", C.c_int), ("sponge_type", C.c_int), ("les", C.c_int),
        ("ny_s_t", C.c_int), ("nz_s_r", C.c_int), ("nz_s_l", C.c_int), ("save_stats_int", C.c_int),
        ("time_step", C.c_int), ("variable_dt", C.c_int), ("update_dt", C.c_int),
        ("cfl", C.c_double), ("delta_t_set", C.c_double), ("fft_fp32", C.c_int),
        ("ff_arith", C.c_int), ("les_model_type", C.c_int), ("les_model_type_th", C.c_int),
        ("create_new_flow", C.c_int),
    ]


class EkMetrics(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in (
        "int_jacob", "gmat_11", "gmat_12", "gmat_22", "cjob_11", "cjob_12", "cjob_21", "cjob_22", "th_bar")]


class EkMgStats(C.Structure):
    _fields_ = [("nprob", C.c_int), ("min_cycles", C.c_int), ("max_cycles", C.c_int),
                ("n_not_converged", C.c_int), ("max_relchange", C.c_double), ("max_residual", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# ek_stats: the scalars, then the (0:NZ+1, 0:NY+1) planes, in header order
STATS_SCALARS = ("ubulk", "vbulk", "thbulk", "urms_b", "vrms_b", "wrms_b", "u3_probe", "u1_probe")
STATS_PLANES = ("urms", "vrms", "wrms", "uv", "uw", "wv", "pu", "pv", "tke", "dudy", "dwdy", "dudz", "dwdz",
                "omega_x", "thrms", "thv", "thw", "dthdy", "dthdz", "rig",
                "mean_u1", "mean_u2", "mean_u3", "mean_p", "mean_th")


class EkStats(C.Structure):
    _fields_ = [(n, C.c_double) for n in STATS_SCALARS] + [(n, C.POINTER(C.c_double)) for n in STATS_PLANES]


def stats_struct(p: "EkParams"):
    """An EkStats whose planes point into fresh (NY+2, NZ+2) arrays (the
    Fortran (0:NZ+1, 0:NY+1) layout); returns (struct, arrays)."""
    arrs = {n: np.zeros((p.ny + 2, p.nz + 2)) for n in STATS_PLANES}
    st = EkStats()
    for n, a in arrs.items():
        setattr(st, n, as_ptr(a))
    return st, arrs


def stats_dict(st: EkStats, arrs: dict) -> dict:
    out = {n: getattr(st, n) for n in STATS_SCALARS}
    out.update(arrs)
    return out


def default_params(nx: int, ny: int, nz: int) -> EkParams:
    """The shipped rundir_unst/input.dat choices for the Ekman layer
    (input.dat:21-62): no-slip bottom (type 0), stress-free top (type 1),
    periodic streamwise (type 6), MUDPACK BC 0 0 2 2, W(2,1) cycles with cubic
    prolongation, at most 6 cycles to a relative change of 1e-6."""
    p = EkParams()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.lx = 4.0 * math.pi
    p.nu = 1.0e-3
    p.delta_t = 1.0e-3
    p.f0 = 1.0
    p.wbulk0 = 1.0
    p.f_type = 1
    p.px0 = 0.0
    p.n_th = 1
    p.pr = 1.0
    p.ri_tau = 0.0
    p.cont_strat = 1
    p.ic_type = 7
    for arr in (p.u_bc, p.v_bc, p.w_bc, p.th_bc):
        arr[EK_YMIN], arr[EK_YMAX], arr[EK_ZMIN], arr[EK_ZMAX] = 0, 1, 6, 6
    for arr in (p.u_bc_c1, p.v_bc_c1, p.w_bc_c1, p.th_bc_c1):
        for i in range(4):
            arr[i] = 0.0
    p.mudpack_bc[0], p.mudpack_bc[1], p.mudpack_bc[2], p.mudpack_bc[3] = 0, 0, 2, 2
    p.mg_maxcy, p.mg_kcycle, p.mg_iprer, p.mg_ipost, p.mg_intpol = 6, 2, 2, 1, 3
    p.mg_stop = EK_MG_STOP_RELCHANGE
    p.mg_tol = MUDPACK_TOLMAX
    p.quirk_phi_fp32 = 0
    # sponge extents as grid_def writes them (streamwise sponge off:
    # NZ_S_R = NZ+2, NZ_S_L = NZ+1-NZ_S_R), SAVE_STATS_INT of input.dat
    p.sponge_type = 0
    p.ny_s_t = (2 * ny) // 3
    p.nz_s_r = nz + 2
    p.nz_s_l = nz + 1 - p.nz_s_r
    p.save_stats_int = 100
    p.time_step = 0
    # fixed time step (VARIABLE_DT off); CFL, UPDATE_DT of the shipped input.dat
    p.variable_dt = 0
    p.update_dt = 1
    p.cfl = 0.8
    p.delta_t_set = p.delta_t
    # LES off; the shipped model choice (input.dat:11) when it is switched on
    p.les, p.les_model_type, p.les_model_type_th, p.create_new_flow = 0, 2, 1, 1
    return p


@dataclass
class Workload:
    """A named synthetic Ekman-layer case (sizes as NX, NY+2, NZ+2)."""
    name: str
    nx: int
    ny2: int
    nz2: int
    re: float
    pr: float
    ri: float
    delta_t: float
    steps: int
    mg_tol: float
    noise: float
    lx_d: float          # spanwise period, in Ekman depths
    cell_d: float        # y-z cell size (uniform z, mean y), in Ekman depths
    seed: int = 0
    les: int = 0         # dynamic-Smagorinsky LES; the synthetic field stands in for a
                         # restart file (CREATE_NEW_FLOW = .FALSE.)

    def params(self, mg_stop: int = EK_MG_STOP_RELCHANGE) -> EkParams:
        p = default_params(self.nx, self.ny2 - 2, self.nz2 - 2)
        # Re = G*delta/nu on the Ekman depth delta = sqrt(2 nu / f), G = f = 1
        p.f0, p.wbulk0 = 1.0, 1.0
        p.nu = 2.0 / (self.re * self.re)
        p.pr, p.ri_tau = self.pr, self.ri
        p.delta_t = self.delta_t
        p.lx = self.lx_d * self.ekman_depth
        p.mg_stop = mg_stop
        p.mg_tol = MUDPACK_TOLMAX if mg_stop == EK_MG_STOP_RELCHANGE else self.mg_tol
        if mg_stop == EK_MG_STOP_RESIDUAL:
            # a cap well above the ~55 W-cycles MUDPACK's point smoother needs
            # at 1e-8 on these grids (the mixed solver needs <= 7)
            p.mg_maxcy = 100
        if self.les:
            p.les, p.create_new_flow = 1, 0
        return p

    @property
    def ekman_depth(self) -> float:
        return math.sqrt(2.0 * (2.0 / (self.re * self.re)))


# The reference's named cases (CPU-runnable neutral case, the stratified
# plain-path case, the large stratified case, the LES case), with the
# vertical size rounded up to MUDPACK's p*2^k+1.
WORKLOADS = {
    "ekman_neutral_64x65x65": Workload("ekman_neutral_64x65x65", 64, 65, 65, 400.0, 1.0, 0.0, 1.0e-3, 100,
                                       1e-10, 0.01, 4.0 * math.pi, 0.4),
    # cells of 0.35 / 0.3 Ekman depths keep the streamwise advective CFL near
    # 0.6 at the named time steps (0.25 depths went unstable within 25 steps)
    "ekman_strat_256x257x193": Workload("ekman_strat_256x257x193", 256, 257, 193, 800.0, 0.7, 0.1, 5.0e-4, 200,
                                        1e-10, 0.01, 64.0, 0.35),
    "ekman_strat_512x385x257": Workload("ekman_strat_512x385x257", 512, 385, 257, 1000.0, 0.7, 0.1, 3.0e-4, 200,
                                        1e-8, 0.01, 128.0, 0.3),
    # the LES case: Re = 2000, Ri = 0.15; twice the spanwise and about 1.3 and
    # 1.5 times the vertical and streamwise points of the large stratified
    # case at the same cell sizes in Ekman depths, and half its time step (the
    # depth halves with Re, so the advective CFL stays at ~0.6)
    "ekman_les_1024x513x385": Workload("ekman_les_1024x513x385", 1024, 513, 385, 2000.0, 0.7, 0.15, 1.5e-4, 500,
                                       1e-8, 0.01, 256.0, 0.3, les=1),
}


def mudpack_form(n: int, pmax: int = 8) -> bool:
    """True when n = p*2^(k-1) + 1 with 2 <= p <= pmax: MUDPACK's grid
    form (mud2cr.f:134-135) with a coarsest grid of at most pmax + 1 points,
    so that the multigrid has a full hierarchy."""
    m = n - 1
    while m > pmax and m % 2 == 0:
        m //= 2
    return 2 <= m <= pmax


def mudpack_size(n: int, pmax: int = 8) -> int:
    """The smallest n' >= n of MUDPACK form with p <= pmax (384 -> 385,
    200 -> 225, 100 -> 113).  The reference's mud2cr only runs sides of
    that form; a run on any other side is set up on the next one."""
    m = max(n, 3)
    while not mudpack_form(m, pmax):
        m += 1
    return m


ENSEMBLE_MEMBERS = 8


def ensemble_workloads(members: int = ENSEMBLE_MEMBERS, seed: int = 0, lo: int = 64, hi: int = 256):
    """An ensemble of independent stratified Ekman-layer runs on uneven grids:
    per member, NX from {64, 128, 256} (the transforms take powers of two)
    and NY+2, NZ+2 drawn uniformly from [lo, hi] with numpy default_rng(seed),
    then rounded up to MUDPACK form (mudpack_size).  Re = 400, Pr = 0.7,
    Ri = 0.1, dt = 1e-3, cells of 0.4 Ekman depths and a spanwise period of
    4 pi * NX/64 depths (the 64x65x65 case's cell sizes).  Returns
    [(drawn (NY+2, NZ+2), Workload)]."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(members):
        nx = int(rng.choice([64, 128, 256]))
        ny2, nz2 = (int(v) for v in rng.integers(lo, hi + 1, size=2))
        ny2r, nz2r = mudpack_size(ny2), mudpack_size(nz2)
        w = Workload(f"ensemble{m}_{nx}x{ny2r}x{nz2r}", nx, ny2r, nz2r, 400.0, 0.7, 0.1, 1.0e-3, 100,
                     1e-8, 0.01, 4.0 * math.pi * nx / 64, 0.4, seed=seed + m)
        out.append(((ny2, nz2), w))
    return out


def make_grid(p: EkParams, ly: float, lz: float, stretch: float = 1.8):
    """GRID_YZ.dat-style points xpoint/ypoint(0:NZ+1, 0:NY+1) (column-major,
    K fastest): uniform streamwise z (period NZ*dz) and a tanh-stretched
    vertical y clustered at the bottom wall."""
    nz2, ny2 = p.nz + 2, p.ny + 2
    dz = lz / p.nz
    z = np.arange(nz2) * dz
    j = np.arange(ny2)
    y = ly * (1.0 + np.tanh(stretch * (j / (ny2 - 1) - 1.0)) / math.tanh(stretch))
    xpoint = np.ascontiguousarray(np.broadcast_to(z[None, :], (ny2, nz2)))
    ypoint = np.ascontiguousarray(np.broadcast_to(y[:, None], (ny2, nz2)))
    return xpoint, ypoint  # arrays indexed [J, K] == Fortran (K, J)


def spectral_shape(p: EkParams):
    """numpy shape [J, K, I] of a complex Fourier-space field (Fortran (I,K,J))."""
    return (p.ny + 2, p.nz + 2, p.nx // 2 + 1)


def ekman_state(p: EkParams, ypoint: np.ndarray, noise: float, seed: int):
    """Laminar Ekman spiral in kx = 0 plus seeded Gaussian noise on
    kx = 1..NX/3 of every velocity component and of the scalar, interior
    points only.  u3 = G(1 - e^-eta cos eta), u1 = G e^-eta sin eta,
    eta = y/delta (steady balance of the Coriolis and viscous terms of
    duct.F90:461-473 with the geostrophic wind WBULK0 = G)."""
    shape = spectral_shape(p)
    g = p.wbulk0
    delta = math.sqrt(2.0 * p.nu / p.f0)
    eta = ypoint / delta  # [J, K]
    cu = [np.zeros(shape, np.complex128) for _ in range(3)]
    cu[0][:, :, 0] = g * np.exp(-eta) * np.sin(eta)
    cu[2][:, :, 0] = g * (1.0 - np.exp(-eta) * np.cos(eta))
    cth = np.zeros(shape, np.complex128)
    rng = np.random.default_rng(seed)
    nkx = p.nx // 3
    interior = (slice(1, p.ny + 1), slice(1, p.nz + 1), slice(1, nkx + 1))
    sub = (p.ny, p.nz, nkx)
    for f in (*cu, cth):
        f[interior] += noise * g * (rng.standard_normal(sub) + 1j * rng.standard_normal(sub)) / math.sqrt(2.0)
    cp = np.zeros(shape, np.complex128)
    return cu[0], cu[1], cu[2], cp, cth


def workload_setup(w: Workload, mg_stop: int = EK_MG_STOP_RELCHANGE):
    """Parameters, grid and initial state of a named workload."""
    p = w.params(mg_stop)
    h = w.cell_d * w.ekman_depth
    xpoint, ypoint = make_grid(p, ly=(p.ny + 1) * h, lz=p.nz * h)
    state = ekman_state(p, ypoint, w.noise, w.seed)
    return p, xpoint, ypoint, state


def as_ptr(a: np.ndarray):
    assert a.dtype in (np.float64, np.complex128) and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))
