"""CPU checks of the C ABI: the library loads without a GPU, exports every
entry point include/ekgpu.h declares, validates parameters before touching
the device, and its host-side metrics equal the oracle's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from ekcases import refgrid_case, sheared_case, small_case
from ekman_bl_gb300 import build as ekbuild
from ekman_bl_gb300.duct import EXPORTS, load_library, metrics_from_grid
from ekman_bl_gb300.params import EkParams, default_params
from oracle import ekref

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ekgpu.h")


@pytest.fixture(scope="module")
def lib():
    ekbuild.build()
    return load_library()


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ekgpu_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol(lib):
    names = declared()
    assert set(names) == set(EXPORTS)
    for n in names:
        assert hasattr(lib, n), n


@pytest.mark.parametrize("field,value,msg", [
    ("nx", 48, "power of two"), ("ic_type", 5, "IC_TYPE"), ("sponge_type", 3, "SPONGE"),
    ("save_stats_int", 0, "SAVE_STATS_INT"),
    ("les_model_type", 1, "LES_MODEL_TYPE"), ("les_model_type_th", 2, "LES_MODEL_TYPE_TH"),
    ("f_type", 0, "F_TYPE"), ("mg_ixp", 3, "Mudpack")])
def test_create_rejects_unsupported(lib, field, value, msg):
    p = default_params(16, 15, 15)
    setattr(p, field, value)
    if field.startswith("les_"):
        p.les = 1
    if field == "save_stats_int":
        p.sponge_type = 2
    if field == "mg_ixp":  # grid_def shape that does not match NZ+2 = 17
        p.mg_iex, p.mg_jyq, p.mg_jey = 3, 4, 3
    h = C.c_void_p()
    st = lib.ekgpu_create(C.byref(p), C.byref(h))
    assert st == 1
    assert msg in lib.ekgpu_last_error(h).decode()
    lib.ekgpu_destroy(h)


def test_create_rejects_unsupported_bc(lib):
    p = default_params(16, 15, 15)
    p.w_bc[2] = 0   # U3 Dirichlet at z-min needs the U3_BAR profile
    h = C.c_void_p()
    assert lib.ekgpu_create(C.byref(p), C.byref(h)) == 1
    lib.ekgpu_destroy(h)


def test_default_params(lib):
    p = EkParams()
    assert lib.ekgpu_default_params(C.byref(p)) == 0
    assert (p.mg_maxcy, p.mg_kcycle, p.mg_iprer, p.mg_ipost, p.mg_intpol) == (6, 2, 2, 1, 3)
    assert list(p.mudpack_bc) == [0, 0, 2, 2]
    assert p.mg_tol == float(np.float32(1e-6))


@pytest.mark.parametrize("case", [small_case, sheared_case, refgrid_case])
def test_host_metrics_equal_oracle(lib, case):
    p, xp, yp, _ = case()
    a = metrics_from_grid(p, xp, yp)
    b = ekref.metrics_from_grid(p, xp, yp)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
