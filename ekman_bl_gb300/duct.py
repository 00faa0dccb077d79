"""Host-side mirror of the reference's duct-substep interface, over the C ABI.

The reference (ekman_bl) exposes its hot path as Fortran subroutines that
act on module globals: RK_DUCT (src/duct.F90:237-2469), REM_DIV_CURV
(src/duct.F90:2472-2818) and MULTIGRID_MUDPACK (src/mg_solver2d.F90:75-201).
`DuctSolver` keeps the same operations and names, with the module state held
on the GPU by libekgpu.so.  Every call goes through the C ABI of
include/ekgpu.h; there is no CPU fallback -- if the library or a GPU is
missing, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
import warnings

import numpy as np

from .params import STATUS, EkMetrics, EkMgStats, EkParams, EkStats, as_ptr, spectral_shape, stats_dict, stats_struct

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libekgpu.so")
_D = C.POINTER(C.c_double)
_lib = None

EXPORTS = [
    "ekgpu_default_params", "ekgpu_create", "ekgpu_destroy", "ekgpu_last_error", "ekgpu_set_stream",
    "ekgpu_set_metrics", "ekgpu_metrics_from_grid", "ekgpu_upload_state", "ekgpu_download_state",
    "ekgpu_get_field", "ekgpu_put_field", "ekgpu_rk_substep", "ekgpu_step", "ekgpu_ensemble_step", "ekgpu_rem_div",
    "ekgpu_poisson_batch", "ekgpu_poisson_batch_device", "ekgpu_last_divergence", "ekgpu_last_mg_stats",
    "ekgpu_mg_counters", "ekgpu_set_step_graph",
    "ekgpu_launch_count", "ekgpu_set_timing", "ekgpu_get_timing", "ekgpu_timing_class_name",
    "ekgpu_fft_x_to_fourier", "ekgpu_fft_x_to_physical", "ekgpu_fft_x_to_fourier_noalloc", "ekgpu_fft_table_count",
    "ekgpu_sponge_profiles", "ekgpu_set_sponge", "ekgpu_set_time", "ekgpu_get_time",
    "ekgpu_save_flow", "ekgpu_read_flow", "ekgpu_save_stats",
    "ekgpu_unet_create", "ekgpu_unet_destroy", "ekgpu_unet_last_error", "ekgpu_unet_num_params",
    "ekgpu_unet_set_params", "ekgpu_unet_get_params", "ekgpu_unet_forward", "ekgpu_unet_set_tcgen05",
    "ekgpu_unet_train_step",
    "ekgpu_unet_gradient", "ekgpu_guess_geometry", "ekgpu_set_poisson_guess", "ekgpu_set_pair_sink",
    "ekgpu_pair_count", "ekgpu_last_guess_stats", "ekgpu_mg_autotune", "ekgpu_mg_set_layout", "ekgpu_mg_levels", "ekgpu_mg_tail_levels",
    "ekgpu_les_metrics_from_grid", "ekgpu_set_les_metrics", "ekgpu_les_set_first_time", "ekgpu_les_get",
]

LES_METRICS = ("gmat_11_y", "gmat_12_y", "gmat_22_y", "gmat_11_z", "gmat_12_z", "gmat_22_z")


class EkError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def lib_path() -> str:
    return _LIB_PATH


def load_library():
    """Load libekgpu.so (built by ekman_bl_gb300.build); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise RuntimeError(f"{_LIB_PATH} is missing: run `python -m ekman_bl_gb300.build` (needs nvcc)")
    L = C.CDLL(_LIB_PATH)
    P = C.POINTER(EkParams)
    V = C.c_void_p
    L.ekgpu_default_params.argtypes = [P]
    L.ekgpu_create.argtypes = [P, C.POINTER(V)]
    L.ekgpu_destroy.argtypes = [V]
    L.ekgpu_destroy.restype = None
    L.ekgpu_last_error.argtypes = [V]
    L.ekgpu_last_error.restype = C.c_char_p
    L.ekgpu_set_stream.argtypes = [V, V]
    L.ekgpu_set_metrics.argtypes = [V, C.POINTER(EkMetrics)]
    L.ekgpu_metrics_from_grid.argtypes = [P, _D, _D] + [_D] * 9
    L.ekgpu_sponge_profiles.argtypes = [P, _D, _D, _D, _D]
    L.ekgpu_set_sponge.argtypes = [V, _D, _D]
    L.ekgpu_set_time.argtypes = [V, C.c_double, C.c_int]
    L.ekgpu_get_time.argtypes = [V, _D, C.POINTER(C.c_int), _D]
    L.ekgpu_upload_state.argtypes = [V] + [_D] * 5
    L.ekgpu_download_state.argtypes = [V] + [_D] * 5
    L.ekgpu_save_flow.argtypes = [V, C.c_char_p, C.c_char_p]
    L.ekgpu_read_flow.argtypes = [V, C.c_char_p, C.c_char_p]
    L.ekgpu_save_stats.argtypes = [V, C.POINTER(EkStats)]
    F = C.POINTER(C.c_float)
    L.ekgpu_unet_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(V)]
    L.ekgpu_unet_destroy.argtypes = [V]
    L.ekgpu_unet_destroy.restype = None
    L.ekgpu_unet_last_error.argtypes = [V]
    L.ekgpu_unet_last_error.restype = C.c_char_p
    L.ekgpu_unet_num_params.argtypes = [V]
    L.ekgpu_unet_num_params.restype = C.c_long
    L.ekgpu_unet_set_params.argtypes = [V, F]
    L.ekgpu_unet_get_params.argtypes = [V, F]
    L.ekgpu_unet_forward.argtypes = [V, V, C.c_int, V, V]
    L.ekgpu_unet_set_tcgen05.argtypes = [V, C.c_int]
    L.ekgpu_unet_train_step.argtypes = [V, V, V, C.c_int, C.c_int, C.c_int, C.c_double, _D, V]
    L.ekgpu_unet_gradient.argtypes = [V, V, V, C.c_int, C.c_int, C.c_int, _D, V, F, V]
    L.ekgpu_guess_geometry.argtypes = [V, C.c_int] + [C.POINTER(C.c_int)] * 4
    L.ekgpu_set_poisson_guess.argtypes = [V, V, C.c_int]
    L.ekgpu_set_pair_sink.argtypes = [V, V, V, C.c_int, C.c_int]
    L.ekgpu_pair_count.argtypes = [V, C.POINTER(C.c_int)]
    L.ekgpu_last_guess_stats.argtypes = [V, _D, _D]
    L.ekgpu_mg_autotune.argtypes = [V, C.c_int, C.c_char_p, C.c_int]
    L.ekgpu_mg_set_layout.argtypes = [V, C.c_int, C.c_int, C.c_int, C.c_int]
    L.ekgpu_mg_levels.argtypes = [V, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]
    L.ekgpu_mg_tail_levels.argtypes = [V, C.POINTER(C.c_int)]
    L.ekgpu_les_metrics_from_grid.argtypes = [P, _D, _D] + [_D] * 6
    L.ekgpu_set_les_metrics.argtypes = [V] + [_D] * 6
    L.ekgpu_les_set_first_time.argtypes = [V, C.c_int]
    L.ekgpu_les_get.argtypes = [V, _D, _D]
    L.ekgpu_get_field.argtypes = [V, C.c_int, _D]
    L.ekgpu_put_field.argtypes = [V, C.c_int, _D]
    L.ekgpu_rk_substep.argtypes = [V, C.c_int]
    L.ekgpu_step.argtypes = [V, C.c_int]
    L.ekgpu_ensemble_step.argtypes = [C.POINTER(V), C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.ekgpu_rem_div.argtypes = [V]
    L.ekgpu_poisson_batch.argtypes = [V, _D, _D, _D, C.c_int, C.POINTER(EkMgStats)]
    L.ekgpu_poisson_batch_device.argtypes = [V, V, V, V, C.c_int, C.POINTER(EkMgStats)]
    L.ekgpu_last_divergence.argtypes = [V, _D]
    L.ekgpu_last_mg_stats.argtypes = [V, C.POINTER(EkMgStats)]
    L.ekgpu_mg_counters.argtypes = [V, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.ekgpu_set_step_graph.argtypes = [V, C.c_int]
    L.ekgpu_launch_count.argtypes = [V]
    L.ekgpu_launch_count.restype = C.c_longlong
    L.ekgpu_set_timing.argtypes = [V, C.c_int]
    L.ekgpu_get_timing.argtypes = [V, _D, C.POINTER(C.c_longlong), _D, C.c_int]
    L.ekgpu_timing_class_name.argtypes = [C.c_int]
    L.ekgpu_timing_class_name.restype = C.c_char_p
    L.ekgpu_fft_table_count.argtypes = []
    for n in ("ekgpu_fft_x_to_fourier", "ekgpu_fft_x_to_physical", "ekgpu_fft_x_to_fourier_noalloc"):
        getattr(L, n).argtypes = [C.c_int, C.c_int, C.c_long, V, V, V]
    _lib = L
    return L


def restart_file_names(kind: str, rank: int = 0, n_th: int = 1, backup_index: int = 0):
    """The restart file names of SAVE_FLOW, BACKUP_FLOW and READ_FLOW
    (diablo.F90:781-809, 861-882, 938-950): kind "saved" or "res"
    (last_saved/), or "backup" (backup/, suffix _mmmm = backup_index mod
    10000).  Rank digits RRR = (rank+1) mod 1000, scalar digits NN = N mod
    100.  Returns (flow name, [scalar names])."""
    r = f"{(rank + 1) % 1000:03d}"
    if kind in ("saved", "res"):
        d, ext = "last_saved", "." + kind
    elif kind == "backup":
        d, ext = "backup", f".saved_{backup_index % 10000:04d}"
    else:
        raise ValueError(f"restart kind {kind!r}: one of saved, res, backup")
    flow = f"{d}/diablo_{r}{ext}"
    ths = [f"{d}/diablo_th{n % 100:02d}_{r}{ext}" for n in range(1, n_th + 1)]
    return flow, ths


def metrics_from_grid(p: EkParams, xpoint: np.ndarray, ypoint: np.ndarray) -> dict:
    """JACOBI_TRANS (src/diablo.F90:1088-1570) through ekgpu_metrics_from_grid.
    Arrays in C order: 2-D [J, K] = Fortran (0:NZ+2, 0:NY+2); face [f, J, K]."""
    L = load_library()
    n2 = (p.ny + 3, p.nz + 3)
    out = {"int_jacob": np.zeros(n2), "th_bar": np.zeros(n2)}
    for k in ("gmat_11", "gmat_12", "gmat_22", "cjob_11", "cjob_12", "cjob_21", "cjob_22"):
        out[k] = np.zeros((2,) + n2)
    xp = np.ascontiguousarray(xpoint, np.float64)
    yp = np.ascontiguousarray(ypoint, np.float64)
    st = L.ekgpu_metrics_from_grid(C.byref(p), as_ptr(xp), as_ptr(yp), *[as_ptr(out[k]) for k in (
        "int_jacob", "gmat_11", "gmat_12", "gmat_22", "cjob_11", "cjob_12", "cjob_21", "cjob_22", "th_bar")])
    if st:
        raise EkError(st, "ekgpu_metrics_from_grid")
    return out


def les_metrics_from_grid(p: EkParams, xpoint: np.ndarray, ypoint: np.ndarray) -> dict:
    """GMAT_*_y / GMAT_*_z of JACOBI_TRANS's LES branch (src/diablo.F90:1379-1467)
    through ekgpu_les_metrics_from_grid; face layout [f, J, K] like GMAT_11."""
    L = load_library()
    out = {k: np.zeros((2, p.ny + 3, p.nz + 3)) for k in LES_METRICS}
    xp = np.ascontiguousarray(xpoint, np.float64)
    yp = np.ascontiguousarray(ypoint, np.float64)
    st = L.ekgpu_les_metrics_from_grid(C.byref(p), as_ptr(xp), as_ptr(yp), *[as_ptr(out[k]) for k in LES_METRICS])
    if st:
        raise EkError(st, "ekgpu_les_metrics_from_grid")
    return out


def sponge_profiles(p: EkParams, xpoint: np.ndarray, ypoint: np.ndarray):
    """SPONGE_SIGMA(0:NY+1) and SPONGE_SIGMA_OUT(0:NZ+1) of
    src/diablo.F90:1489-1556 through ekgpu_sponge_profiles."""
    L = load_library()
    sig, sig_out = np.zeros(p.ny + 2), np.zeros(p.nz + 2)
    xp = np.ascontiguousarray(xpoint, np.float64)
    yp = np.ascontiguousarray(ypoint, np.float64)
    st = L.ekgpu_sponge_profiles(C.byref(p), as_ptr(xp), as_ptr(yp), as_ptr(sig), as_ptr(sig_out))
    if st:
        raise EkError(st, "ekgpu_sponge_profiles")
    return sig, sig_out


class DuctSolver:
    """GPU-resident RK3 duct substep (one context = one set of module arrays)."""

    def __init__(self, p: EkParams, metrics: dict):
        self.p = p
        self._L = load_library()
        h = C.c_void_p()
        st = self._L.ekgpu_create(C.byref(p), C.byref(h))
        self._h = h
        if st:
            msg = self._L.ekgpu_last_error(h).decode() if h.value else ""
            self.close()
            raise EkError(st, msg)
        self._metrics = {k: np.ascontiguousarray(v, np.float64) for k, v in metrics.items()}
        m = EkMetrics()
        for k in ("int_jacob", "gmat_11", "gmat_12", "gmat_22", "cjob_11", "cjob_12", "cjob_21", "cjob_22", "th_bar"):
            setattr(m, k, as_ptr(self._metrics[k]))
        self._check(self._L.ekgpu_set_metrics(h, C.byref(m)))

    # -- plumbing -----------------------------------------------------------
    def _check(self, st, allow=()):
        if st and st not in allow:
            raise EkError(st, self._L.ekgpu_last_error(self._h).decode())
        return st

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.ekgpu_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None):
        self._check(self._L.ekgpu_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def set_sponge(self, sponge_sigma, sponge_sigma_out):
        """SPONGE_SIGMA(0:NY+1), SPONGE_SIGMA_OUT(0:NZ+1) read by sponge_th."""
        self._sponge = [np.ascontiguousarray(a, np.float64) for a in (sponge_sigma, sponge_sigma_out)]
        self._check(self._L.ekgpu_set_sponge(self._h, *[as_ptr(a) for a in self._sponge]))

    def set_time(self, time: float, time_step: int):
        self._check(self._L.ekgpu_set_time(self._h, float(time), int(time_step)))

    # -- LES (les_chan / les_chan_th) ----------------------------------------
    def set_les_metrics(self, m: dict):
        """Upload GMAT_*_y / GMAT_*_z (les_metrics_from_grid)."""
        self._les_metrics = [np.ascontiguousarray(m[k], np.float64) for k in LES_METRICS]
        self._check(self._L.ekgpu_set_les_metrics(self._h, *[as_ptr(a) for a in self._les_metrics]))

    def les_set_first_time(self, flag: bool):
        """FIRST_TIME: recompute C_DYN in every substep until cleared."""
        self._check(self._L.ekgpu_les_set_first_time(self._h, int(bool(flag))))

    def les_state(self):
        """(NU_T in the physical layout [J, K, I], C_DYN [J, K])."""
        p = self.p
        nu = np.zeros((p.ny + 2, p.nz + 2, p.nx + 2))
        cd = np.zeros((p.ny + 2, p.nz + 2))
        self._check(self._L.ekgpu_les_get(self._h, as_ptr(nu), as_ptr(cd)))
        return nu, cd

    def get_time(self):
        """(TIME, TIME_STEP, DELTA_T)."""
        t, n, dt = C.c_double(), C.c_int(), C.c_double()
        self._check(self._L.ekgpu_get_time(self._h, C.byref(t), C.byref(n), C.byref(dt)))
        return t.value, n.value, dt.value

    # -- state ----------------------------------------------------------------
    def upload(self, cu1, cu2, cu3, cp, cth):
        arrs = [np.ascontiguousarray(a, np.complex128) for a in (cu1, cu2, cu3, cp, cth)]
        self._check(self._L.ekgpu_upload_state(self._h, *[as_ptr(a) for a in arrs]))

    def download(self, out=None):
        """CU1X, CU2X, CU3X, CPX, CTHX; into the five arrays of `out` when
        given (C-contiguous complex128 of the spectral shape, e.g. pinned)."""
        shape = spectral_shape(self.p)
        arrs = list(out) if out is not None else [np.zeros(shape, np.complex128) for _ in range(5)]
        for a in arrs:
            if a.shape != shape or a.dtype != np.complex128 or not a.flags.c_contiguous:
                raise ValueError("download: out arrays must be C-contiguous complex128 of the spectral shape")
        self._check(self._L.ekgpu_download_state(self._h, *[as_ptr(a) for a in arrs]))
        return arrs

    # -- restart files ----------------------------------------------------------
    def write_restart(self, flow_path: str, th_path: str | None = None):
        """The file writes of SAVE_FLOW / BACKUP_FLOW (diablo.F90:813-833,
        886-907): records [NX NY NZ TIME TIME_STEP] and [CU1X CU2X CU3X CPX]
        to flow_path, the header and [CTHX] to th_path."""
        self._check(self._L.ekgpu_save_flow(self._h, os.fsencode(flow_path),
                                            None if th_path is None else os.fsencode(th_path)))

    def read_restart(self, flow_path: str, th_path: str | None = None):
        """The file reads of READ_FLOW (diablo.F90:953-987); sets TIME and
        TIME_STEP from the headers.  A wrong-dimension file raises EkError
        (EK_ERR_IO) with the state unchanged."""
        self._check(self._L.ekgpu_read_flow(self._h, os.fsencode(flow_path),
                                            None if th_path is None else os.fsencode(th_path)))

    def save_flow(self, final: bool = False, root: str = ".", rank: int = 0):
        """SAVE_FLOW(FINAL) (diablo.F90:753-837): creates last_saved/ when
        missing and writes diablo_RRR.saved (.res when final) plus one scalar
        file per N_TH.  Returns the paths written."""
        d = os.path.join(root, "last_saved")
        os.makedirs(d, exist_ok=True)
        kind = "res" if final else "saved"
        flow, ths = restart_file_names(kind, rank, self.p.n_th)
        flow, ths = os.path.join(root, flow), [os.path.join(root, t) for t in ths]
        self.write_restart(flow, ths[0] if ths else None)
        return [flow] + ths

    def backup_flow(self, backup_flow_int: int, root: str = ".", rank: int = 0):
        """BACKUP_FLOW (diablo.F90:841-915): backup/diablo_RRR.saved_mmmm with
        m = TIME_STEP / BACKUP_FLOW_INT.  Returns the paths written."""
        os.makedirs(os.path.join(root, "backup"), exist_ok=True)
        _, step, _ = self.get_time()
        flow, ths = restart_file_names("backup", rank, self.p.n_th, step // backup_flow_int)
        flow, ths = os.path.join(root, flow), [os.path.join(root, t) for t in ths]
        self.write_restart(flow, ths[0] if ths else None)
        return [flow] + ths

    def read_flow(self, root: str = ".", rank: int = 0, read_th: bool = True):
        """READ_FLOW (diablo.F90:918-1072): last_saved/diablo_RRR.saved and,
        when read_th (the scalar is not CREATE_NEW_TH), its scalar file."""
        flow, ths = restart_file_names("saved", rank, self.p.n_th)
        th = os.path.join(root, ths[0]) if (read_th and ths) else None
        self.read_restart(os.path.join(root, flow), th)

    # -- statistics -------------------------------------------------------------
    def save_stats(self, root: str | None = None, save_stats_int: int | None = None,
                   xpoint=None, ypoint=None) -> dict:
        """SAVE_STATS_CURVI (flow_statistics.F90:2-1023): the plane statistics
        as a dict of scalars and (NY+2, NZ+2) planes.  The state goes through
        physical space and back and CF1X..CF3X are zeroed, as in the
        reference.  With root, also appends plane_data/time_bulk.txt and
        writes plot_binary's data_tec_KKKKK.pln (needs xpoint, ypoint)."""
        st, arrs = stats_struct(self.p)
        self._check(self._L.ekgpu_save_stats(self._h, C.byref(st)))
        out = stats_dict(st, arrs)
        if root is not None:
            from .stats_io import write_stats_files
            time, step, dt = self.get_time()
            every = save_stats_int if save_stats_int is not None else self.p.save_stats_int
            th_bar = self._metrics.get("th_bar")
            if th_bar is None:
                th_bar = np.zeros((self.p.ny + 3, self.p.nz + 3))
            out["files"] = write_stats_files(root, time, dt, step, every, xpoint, ypoint, th_bar, out)
        return out

    # -- line-solver layouts (tile-shape autotuner) -------------------------------
    def mg_autotune(self, reps: int = 3) -> list:
        """Time every valid layout of the mixed solver's line solves per level
        and direction and keep the fastest; returns the timings."""
        import json
        buf = C.create_string_buffer(1 << 16)
        self._check(self._L.ekgpu_mg_autotune(self._h, reps, buf, len(buf)))
        return json.loads(buf.value.decode())

    def mg_set_layout(self, level: int, direction: int, lanes: int, seg: int = 8):
        """Problems per block (8/16/32) and segment rows (4/8) of the line
        solves at one level and direction (0 y-lines, 1 x-lines); 0 = default."""
        self._check(self._L.ekgpu_mg_set_layout(self._h, level, direction, lanes, seg))

    def mg_tail_levels(self) -> int:
        """ltop: the mixed solver's coarse levels 1..ltop run as one launch per
        cycle (no line-solve layouts to tune there); 0 = none."""
        n = C.c_int()
        self._check(self._L.ekgpu_mg_tail_levels(self._h, C.byref(n)))
        return n.value

    def mg_levels(self):
        """[(nx, ny)] of the multigrid levels, coarsest first."""
        n = C.c_int()
        nx, ny = (C.c_int * 32)(), (C.c_int * 32)()
        self._check(self._L.ekgpu_mg_levels(self._h, C.byref(n), nx, ny, 32))
        return [(nx[i], ny[i]) for i in range(n.value)]

    # -- learned initial guess of the Poisson problems ----------------------------
    def guess_geometry(self, factor: int):
        """(h, w, hv, wv): the network image size and its valid part."""
        v = [C.c_int() for _ in range(4)]
        self._check(self._L.ekgpu_guess_geometry(self._h, factor, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def set_poisson_guess(self, net, factor: int = 4):
        """Start the kx^2 != 0 problems of each mixed solve from net's
        prediction (None: from zero)."""
        self._guess_net = net
        self._check(self._L.ekgpu_set_poisson_guess(self._h, None if net is None else net.handle, factor))

    def set_pair_sink(self, x_ptr: int | None, t_ptr: int | None, capacity: int = 0, factor: int = 4):
        """Collect (input [h][w][2], target [h][w]) FP32 pairs into device
        buffers after each projection solve; None stops."""
        self._check(self._L.ekgpu_set_pair_sink(self._h, C.c_void_p(x_ptr or 0), C.c_void_p(t_ptr or 0),
                                                capacity, factor))

    def pair_count(self) -> int:
        n = C.c_int()
        self._check(self._L.ekgpu_pair_count(self._h, C.byref(n)))
        return n.value

    def last_guess_stats(self):
        """(mean |b - A g|/|b| after the scaled guess, mean corrections) of
        the last mixed solve, over the kx^2 != 0 problems."""
        r, m = C.c_double(), C.c_double()
        self._check(self._L.ekgpu_last_guess_stats(self._h, C.byref(r), C.byref(m)))
        return r.value, m.value

    def get_field(self, f: int):
        a = np.zeros(spectral_shape(self.p), np.complex128)
        self._check(self._L.ekgpu_get_field(self._h, f, as_ptr(a)))
        return a

    def put_field(self, f: int, a):
        a = np.ascontiguousarray(a, np.complex128)
        self._check(self._L.ekgpu_put_field(self._h, f, as_ptr(a)))

    # -- the reference operations ---------------------------------------------
    # EK_ERR_NOT_CONVERGED (a projection problem stopped at mg_maxcy above
    # the residual rule's tolerance) leaves a complete, valid state: these
    # calls return the code and warn instead of raising.
    def _solve_status(self, st):
        self._check(st, allow=(3,))
        if st == 3:
            warnings.warn(f"EK_ERR_NOT_CONVERGED: {self._L.ekgpu_last_error(self._h).decode()}", RuntimeWarning,
                          stacklevel=3)
        return st

    def rk_duct(self, rk_step: int):
        """RK_DUCT: one RK3 substep (duct.F90:237-2469)."""
        return self._solve_status(self._L.ekgpu_rk_substep(self._h, rk_step))

    def step(self, nsteps: int = 1):
        """nsteps times DO RK_STEP=1,3; CALL RK_DUCT (diablo.F90:152-154)."""
        return self._solve_status(self._L.ekgpu_step(self._h, nsteps))

    def rem_div_curv(self):
        """REM_DIV_CURV: projection of the current state (duct.F90:2472-2818)."""
        return self._solve_status(self._L.ekgpu_rem_div(self._h))

    def set_step_graph(self, on: bool):
        """Let step() run each RK3 step as one captured CUDA graph (default
        on; applies to the mixed solver with a fixed time step)."""
        self._check(self._L.ekgpu_set_step_graph(self._h, 1 if on else 0))

    def mg_counters(self):
        """(real Poisson problems solved, of them stopped at the cycle cap)
        since the context was created."""
        a, b = C.c_longlong(), C.c_longlong()
        self._check(self._L.ekgpu_mg_counters(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def multigrid_mudpack(self, rhs: np.ndarray, kx2: np.ndarray):
        """Batched MULTIGRID_MUDPACK: rhs[nprob, NY+2, NZ+2] (MUDPACK grid,
        K fastest), one kx^2 per problem; returns (phi, stats, status)."""
        rhs = np.ascontiguousarray(rhs, np.float64)
        kx2 = np.ascontiguousarray(kx2, np.float64)
        phi = np.zeros_like(rhs)
        st = EkMgStats()
        code = self._L.ekgpu_poisson_batch(self._h, as_ptr(rhs), as_ptr(phi), as_ptr(kx2), len(kx2), C.byref(st))
        self._check(code, allow=(3,))
        return phi, st.as_dict(), code

    def multigrid_mudpack_device(self, rhs_ptr: int, phi_ptr: int, kx2_ptr: int, nprob: int):
        st = EkMgStats()
        code = self._L.ekgpu_poisson_batch_device(self._h, C.c_void_p(rhs_ptr), C.c_void_p(phi_ptr),
                                                   C.c_void_p(kx2_ptr), nprob, C.byref(st))
        self._check(code, allow=(3,))
        return st.as_dict(), code

    def divergence(self) -> float:
        d = C.c_double()
        self._check(self._L.ekgpu_last_divergence(self._h, C.byref(d)))
        return d.value

    def mg_stats(self) -> dict:
        s = EkMgStats()
        self._check(self._L.ekgpu_last_mg_stats(self._h, C.byref(s)))
        return s.as_dict()

    def launch_count(self) -> int:
        return int(self._L.ekgpu_launch_count(self._h))

    def set_timing(self, on: bool):
        self._check(self._L.ekgpu_set_timing(self._h, 1 if on else 0))

    def timing(self) -> dict:
        """Per-kernel-class totals {name: (ms, launches, algorithmic bytes)}
        since set_timing."""
        n = 32
        ms = (C.c_double * n)()
        cnt = (C.c_longlong * n)()
        by = (C.c_double * n)()
        k = self._L.ekgpu_get_timing(self._h, ms, cnt, by, n)
        if k < 0:
            self._check(k)
        return {self._L.ekgpu_timing_class_name(i).decode(): (ms[i], int(cnt[i]), by[i]) for i in range(k)}


def ensemble_step(members, nsteps: int = 1, raise_on_error: bool = True) -> list:
    """Advance an ensemble of independent runs (DuctSolvers of any sizes)
    by nsteps RK3 steps each, concurrently on one GPU (ekgpu_ensemble_step:
    each member on its own stream and host thread).  Returns the members'
    status codes; with raise_on_error, raises the first failing member's
    EkError after every member has finished."""
    members = list(members)
    L = load_library()
    n = len(members)
    handles = (C.c_void_p * max(n, 1))(*[m._h.value for m in members])
    status = (C.c_int * max(n, 1))()
    r = L.ekgpu_ensemble_step(handles, n, nsteps, status)
    codes = [int(status[i]) for i in range(n)]
    if r and raise_on_error:
        for m, c in zip(members, codes):
            if c and c != 3:  # NOT_CONVERGED leaves the member's state valid
                m._check(c)
        if any(c not in (0, 3) for c in codes) or not codes:
            raise EkError(r, "ekgpu_ensemble_step: bad arguments")
    return codes


def fft_x(forward: bool, nx: int, nkx: int, nlines: int, in_ptr: int, out_ptr: int, stream_ptr: int | None = None):
    """The context-free x-transforms (ekgpu_fft_x_to_fourier / _to_physical)
    on device buffers given as raw pointers."""
    L = load_library()
    fn = L.ekgpu_fft_x_to_fourier if forward else L.ekgpu_fft_x_to_physical
    st = fn(nx, nkx, nlines, C.c_void_p(in_ptr), C.c_void_p(out_ptr), C.c_void_p(stream_ptr or 0))
    if st:
        raise EkError(st, L.ekgpu_last_error(None).decode())


class UNet:
    """The learned-guess network (ekgpu_unet_*): device images are given by
    address (e.g. torch CUDA tensors' data_ptr()), FP32 NHWC."""

    def __init__(self, cin: int, channels: int, max_batch: int, h: int, w: int):
        self._L = load_library()
        hdl = C.c_void_p()
        st = self._L.ekgpu_unet_create(cin, channels, max_batch, h, w, C.byref(hdl))
        if st:
            raise EkError(st, "ekgpu_unet_create")
        self._h = hdl
        self.cin, self.channels, self.max_batch, self.h, self.w = cin, channels, max_batch, h, w

    @property
    def handle(self):
        return self._h

    def _check(self, st):
        if st:
            raise EkError(st, self._L.ekgpu_unet_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.ekgpu_unet_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nparams(self) -> int:
        return int(self._L.ekgpu_unet_num_params(self._h))

    def set_params(self, params: np.ndarray):
        a = np.ascontiguousarray(params, np.float32)
        assert a.size == self.nparams()
        self._check(self._L.ekgpu_unet_set_params(self._h, a.ctypes.data_as(C.POINTER(C.c_float))))

    def get_params(self) -> np.ndarray:
        a = np.zeros(self.nparams(), np.float32)
        self._check(self._L.ekgpu_unet_get_params(self._h, a.ctypes.data_as(C.POINTER(C.c_float))))
        return a

    def forward(self, x_ptr: int, n: int, y_ptr: int, stream: int | None = None):
        self._check(self._L.ekgpu_unet_forward(self._h, C.c_void_p(x_ptr), n, C.c_void_p(y_ptr),
                                               C.c_void_p(stream or 0)))

    def set_tcgen05(self, on: bool):
        """Forward convolutions on the tcgen05 tensor-core kernel where their
        channel counts allow it (the default), or all on the mma.sync one."""
        self._check(self._L.ekgpu_unet_set_tcgen05(self._h, int(bool(on))))

    def train_step(self, x_ptr: int, t_ptr: int, n: int, hv: int, wv: int, lr: float,
                   stream: int | None = None) -> float:
        loss = C.c_double()
        self._check(self._L.ekgpu_unet_train_step(self._h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), n, hv, wv, lr,
                                                  C.byref(loss), C.c_void_p(stream or 0)))
        return loss.value

    def gradient(self, x_ptr: int, t_ptr: int, n: int, hv: int, wv: int, y_ptr: int | None = None,
                 stream: int | None = None):
        """(loss, flat parameter gradient) without an update."""
        loss = C.c_double()
        g = np.zeros(self.nparams(), np.float32)
        self._check(self._L.ekgpu_unet_gradient(self._h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), n, hv, wv,
                                                C.byref(loss), C.c_void_p(y_ptr or 0),
                                                g.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(stream or 0)))
        return loss.value, g
