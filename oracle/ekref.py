"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/libekref.so (built by oracle/Makefile from the C++
restatement of the reference's RK_DUCT / REM_DIV_CURV / MUDPACK path).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module; it is the checker, never the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from ekman_bl_gb300.params import (EkMetrics, EkMgStats, EkParams, EkStats, as_ptr, spectral_shape, stats_dict,
                                   stats_struct)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libekref.so")
_lib = None
_D = C.POINTER(C.c_double)


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        P = C.POINTER(EkParams)
        L.ekref_create.argtypes = [P, C.POINTER(C.c_void_p)]
        L.ekref_destroy.argtypes = [C.c_void_p]
        L.ekref_last_error.argtypes = [C.c_void_p]
        L.ekref_last_error.restype = C.c_char_p
        L.ekref_set_threads.argtypes = [C.c_int]
        L.ekref_metrics_from_grid.argtypes = [P, _D, _D] + [_D] * 9
        L.ekref_set_metrics.argtypes = [C.c_void_p, C.POINTER(EkMetrics)]
        L.ekref_sponge_profiles.argtypes = [P, _D, _D, _D, _D]
        L.ekref_set_sponge.argtypes = [C.c_void_p, _D, _D]
        L.ekref_set_time.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.ekref_get_time.argtypes = [C.c_void_p, _D, C.POINTER(C.c_int), _D]
        L.ekref_upload_state.argtypes = [C.c_void_p] + [_D] * 5
        L.ekref_download_state.argtypes = [C.c_void_p] + [_D] * 5
        L.ekref_get_field.argtypes = [C.c_void_p, C.c_int, _D]
        L.ekref_put_field.argtypes = [C.c_void_p, C.c_int, _D]
        L.ekref_rk_substep.argtypes = [C.c_void_p, C.c_int]
        L.ekref_step.argtypes = [C.c_void_p, C.c_int]
        L.ekref_rem_div.argtypes = [C.c_void_p]
        L.ekref_poisson_batch.argtypes = [C.c_void_p, _D, _D, _D, C.c_int, C.POINTER(EkMgStats)]
        L.ekref_last_divergence.argtypes = [C.c_void_p, _D]
        L.ekref_last_mg_stats.argtypes = [C.c_void_p, C.POINTER(EkMgStats)]
        L.ekref_fft_r2c.argtypes = [C.c_int, C.c_int, C.c_long, _D, _D]
        L.ekref_fft_c2r.argtypes = [C.c_int, C.c_int, C.c_long, _D, _D]
        L.ekref_thomas_real.argtypes = [C.c_int, C.c_int, _D, _D, _D, _D]
        L.ekref_mg_apply.argtypes = [C.c_void_p, C.c_double, _D, _D]
        L.ekref_mg_left_null.argtypes = [C.c_void_p, _D]
        L.ekref_save_stats.argtypes = [C.c_void_p, C.POINTER(EkStats)]
        L.ekref_les_metrics_from_grid.argtypes = [P, _D, _D] + [_D] * 6
        L.ekref_set_les_metrics.argtypes = [C.c_void_p] + [_D] * 6
        L.ekref_les_set_first_time.argtypes = [C.c_void_p, C.c_int]
        L.ekref_les_get.argtypes = [C.c_void_p, _D, _D]
        _lib = L
    return _lib


def metrics_from_grid(p: EkParams, xpoint: np.ndarray, ypoint: np.ndarray) -> dict:
    """JACOBI_TRANS restated (diablo.F90:1088-1570); arrays shaped like the
    Fortran ones in C order: 2-D [J, K] = (0:NZ+2, 0:NY+2), face [f, J, K]."""
    n2 = (p.ny + 3, p.nz + 3)
    out = {"int_jacob": np.zeros(n2), "th_bar": np.zeros(n2)}
    for k in ("gmat_11", "gmat_12", "gmat_22", "cjob_11", "cjob_12", "cjob_21", "cjob_22"):
        out[k] = np.zeros((2,) + n2)
    xp = np.ascontiguousarray(xpoint, np.float64)
    yp = np.ascontiguousarray(ypoint, np.float64)
    st = lib().ekref_metrics_from_grid(C.byref(p), as_ptr(xp), as_ptr(yp), as_ptr(out["int_jacob"]),
                                       as_ptr(out["gmat_11"]), as_ptr(out["gmat_12"]), as_ptr(out["gmat_22"]),
                                       as_ptr(out["cjob_11"]), as_ptr(out["cjob_12"]), as_ptr(out["cjob_21"]),
                                       as_ptr(out["cjob_22"]), as_ptr(out["th_bar"]))
    if st:
        raise RuntimeError(f"ekref_metrics_from_grid failed: {st}")
    return out


LES_METRICS = ("gmat_11_y", "gmat_12_y", "gmat_22_y", "gmat_11_z", "gmat_12_z", "gmat_22_z")


def les_metrics_from_grid(p: EkParams, xpoint: np.ndarray, ypoint: np.ndarray) -> dict:
    """GMAT_*_y / GMAT_*_z of JACOBI_TRANS (diablo.F90:1379-1467), face layout [f, J, K]."""
    n3 = (2, p.ny + 3, p.nz + 3)
    out = {k: np.zeros(n3) for k in LES_METRICS}
    xp = np.ascontiguousarray(xpoint, np.float64)
    yp = np.ascontiguousarray(ypoint, np.float64)
    st = lib().ekref_les_metrics_from_grid(C.byref(p), as_ptr(xp), as_ptr(yp), *[as_ptr(out[k]) for k in LES_METRICS])
    if st:
        raise RuntimeError(f"ekref_les_metrics_from_grid failed: {st}")
    return out


def sponge_profiles(p: EkParams, xpoint: np.ndarray, ypoint: np.ndarray):
    """The oracle's SPONGE_SIGMA / SPONGE_SIGMA_OUT (diablo.F90:1489-1556)."""
    sig, sig_out = np.zeros(p.ny + 2), np.zeros(p.nz + 2)
    xp = np.ascontiguousarray(xpoint, np.float64)
    yp = np.ascontiguousarray(ypoint, np.float64)
    st = lib().ekref_sponge_profiles(C.byref(p), as_ptr(xp), as_ptr(yp), as_ptr(sig), as_ptr(sig_out))
    if st:
        raise RuntimeError(f"ekref_sponge_profiles failed: {st}")
    return sig, sig_out


def metrics_struct(m: dict) -> EkMetrics:
    s = EkMetrics()
    for k in ("int_jacob", "gmat_11", "gmat_12", "gmat_22", "cjob_11", "cjob_12", "cjob_21", "cjob_22", "th_bar"):
        setattr(s, k, as_ptr(m[k]))
    return s


class Oracle:
    """The oracle context, shaped like the product's DuctSolver."""

    def __init__(self, p: EkParams, metrics: dict, threads: int = 0):
        self.p = p
        L = lib()
        if threads:
            L.ekref_set_threads(threads)
        h = C.c_void_p()
        st = L.ekref_create(C.byref(p), C.byref(h))
        self._h = h
        if st:
            msg = L.ekref_last_error(h).decode() if h else ""
            raise ValueError(f"ekref_create: {st} {msg}")
        self._metrics = metrics
        self._check(L.ekref_set_metrics(h, C.byref(metrics_struct(metrics))))

    def _check(self, st):
        if st:
            raise RuntimeError(f"oracle status {st}: {lib().ekref_last_error(self._h).decode()}")
        return st

    def close(self):
        if self._h:
            lib().ekref_destroy(self._h)
            self._h = None

    __del__ = close

    def upload(self, cu1, cu2, cu3, cp, cth):
        arrs = [np.ascontiguousarray(a, np.complex128) for a in (cu1, cu2, cu3, cp, cth)]
        self._check(lib().ekref_upload_state(self._h, *[as_ptr(a) for a in arrs]))

    def download(self):
        shape = spectral_shape(self.p)
        arrs = [np.zeros(shape, np.complex128) for _ in range(5)]
        self._check(lib().ekref_download_state(self._h, *[as_ptr(a) for a in arrs]))
        return arrs

    def get_field(self, f):
        a = np.zeros(spectral_shape(self.p), np.complex128)
        self._check(lib().ekref_get_field(self._h, f, as_ptr(a)))
        return a

    def put_field(self, f, a):
        a = np.ascontiguousarray(a, np.complex128)
        self._check(lib().ekref_put_field(self._h, f, as_ptr(a)))

    def rk_substep(self, rk):
        return self._check(lib().ekref_rk_substep(self._h, rk))

    def step(self, n=1):
        return self._check(lib().ekref_step(self._h, n))

    def set_sponge(self, sponge_sigma, sponge_sigma_out):
        self._sponge = [np.ascontiguousarray(a, np.float64) for a in (sponge_sigma, sponge_sigma_out)]
        self._check(lib().ekref_set_sponge(self._h, *[as_ptr(a) for a in self._sponge]))

    def set_time(self, time: float, time_step: int):
        self._check(lib().ekref_set_time(self._h, float(time), int(time_step)))

    def get_time(self):
        t, n, dt = C.c_double(), C.c_int(), C.c_double()
        lib().ekref_get_time(self._h, C.byref(t), C.byref(n), C.byref(dt))
        return t.value, n.value, dt.value

    def rem_div(self):
        return self._check(lib().ekref_rem_div(self._h))

    def poisson(self, rhs: np.ndarray, kx2: np.ndarray):
        rhs = np.ascontiguousarray(rhs, np.float64)
        phi = np.zeros_like(rhs)
        kx2 = np.ascontiguousarray(kx2, np.float64)
        st = EkMgStats()
        code = lib().ekref_poisson_batch(self._h, as_ptr(rhs), as_ptr(phi), as_ptr(kx2), len(kx2), C.byref(st))
        if code not in (0, 3):
            self._check(code)
        return phi, st.as_dict(), code

    def mg_apply(self, kx2: float, phi: np.ndarray):
        phi = np.ascontiguousarray(phi, np.float64)
        out = np.zeros_like(phi)
        self._check(lib().ekref_mg_apply(self._h, kx2, as_ptr(phi), as_ptr(out)))
        return out

    def mg_left_null(self):
        """Left null vector z of the finest kx = 0 operator, [NY+2, NZ+2]."""
        z = np.zeros((self.p.ny + 2, self.p.nz + 2))
        self._check(lib().ekref_mg_left_null(self._h, as_ptr(z)))
        return z

    def divergence(self):
        d = C.c_double()
        lib().ekref_last_divergence(self._h, C.byref(d))
        return d.value

    def mg_stats(self):
        s = EkMgStats()
        lib().ekref_last_mg_stats(self._h, C.byref(s))
        return s.as_dict()

    def set_les_metrics(self, m: dict):
        self._les = [np.ascontiguousarray(m[k], np.float64) for k in LES_METRICS]
        self._check(lib().ekref_set_les_metrics(self._h, *[as_ptr(a) for a in self._les]))

    def les_set_first_time(self, flag: bool):
        self._check(lib().ekref_les_set_first_time(self._h, int(bool(flag))))

    def les_state(self):
        """(NU_T in the physical layout [J, K, I], C_DYN [J, K])."""
        p = self.p
        nu = np.zeros((p.ny + 2, p.nz + 2, p.nx + 2))
        cd = np.zeros((p.ny + 2, p.nz + 2))
        self._check(lib().ekref_les_get(self._h, as_ptr(nu), as_ptr(cd)))
        return nu, cd

    def save_stats(self) -> dict:
        """SAVE_STATS_CURVI restated: the statistics and the state round trip."""
        st, arrs = stats_struct(self.p)
        self._check(lib().ekref_save_stats(self._h, C.byref(st)))
        return stats_dict(st, arrs)


def fft_r2c(x: np.ndarray, nkx: int) -> np.ndarray:
    """x: (..., NX+2) real lines -> (..., NX/2+1) complex."""
    nx = x.shape[-1] - 2
    xx = np.ascontiguousarray(x, np.float64)
    out = np.zeros(x.shape[:-1] + (nx // 2 + 1,), np.complex128)
    lib().ekref_fft_r2c(nx, nkx, int(np.prod(x.shape[:-1])), as_ptr(xx), as_ptr(out))
    return out


def fft_c2r(c: np.ndarray, nkx: int) -> np.ndarray:
    nx = (c.shape[-1] - 1) * 2
    cc = np.ascontiguousarray(c, np.complex128)
    out = np.zeros(c.shape[:-1] + (nx + 2,), np.float64)
    lib().ekref_fft_c2r(nx, nkx, int(np.prod(c.shape[:-1])), as_ptr(cc), as_ptr(out))
    return out


def thomas(a, b, c, g):
    """THOMAS_REAL on arrays shaped [n+1, nsys] (Fortran (0:nsys-1, 0:n))."""
    a, b, c, g = (np.ascontiguousarray(x, np.float64).copy() for x in (a, b, c, g))
    n = a.shape[0] - 1
    nsys = a.shape[1]
    lib().ekref_thomas_real(nsys, n, as_ptr(a), as_ptr(b), as_ptr(c), as_ptr(g))
    return g
