"""Ensembles of differently sized runs on one GPU (ekgpu_ensemble_step).

The reference runs each ensemble member as its own job of the same code
(RK_DUCT, src/duct.F90:237-2469, driven by diablo.F90:152-154); the GPU path
steps every member on its own stream from its own host thread.

CPU: the MUDPACK size helpers (mud2cr.f:134-135 grid form), the seeded
uneven-grid ensemble, and the C ABI's argument checks.
GPU: members of different NX, NY and NZ stepped together against the
oracle (FP64 path, relative L2 <= 1e-10 after two steps); the mixed path's
members stepped together equal the same members stepped one at a time; a
failing member leaves the others stepping and reports its own status.
"""
import ctypes as C

import pytest

from ekcases import rel_l2, small_case
from ekman_bl_gb300 import build as ekbuild
from ekman_bl_gb300.duct import DuctSolver, ensemble_step, load_library, metrics_from_grid
from ekman_bl_gb300.params import (ENSEMBLE_MEMBERS, EK_MG_STOP_RESIDUAL, ensemble_workloads, mudpack_form,
                                   mudpack_size)
from oracle import ekref


def test_mudpack_size_is_the_next_admissible_side():
    for n in range(3, 700):
        m = mudpack_size(n)
        assert m >= n and mudpack_form(m)
        assert not any(mudpack_form(k) for k in range(n, m))
    assert [mudpack_size(n) for n in (384, 512, 64, 257, 193, 200)] == [385, 513, 65, 257, 193, 225]
    # p*2^(k-1)+1 with 2 <= p <= 8: a multigrid hierarchy down to <= 9 points
    assert mudpack_form(385) and mudpack_form(257) and mudpack_form(97)
    assert not mudpack_form(384) and not mudpack_form(209)


def test_ensemble_workloads_are_seeded_uneven_and_admissible():
    a = ensemble_workloads(seed=0)
    b = ensemble_workloads(seed=0)
    assert len(a) == ENSEMBLE_MEMBERS
    assert [w.name for _, w in a] == [w.name for _, w in b]
    assert [w.name for _, w in a] != [w.name for _, w in ensemble_workloads(seed=1)]
    drawn = [s for (d, _) in a for s in d]
    assert all(64 <= s <= 256 for s in drawn)
    # the draw mixes sides of MUDPACK form and sides that need rounding up
    assert any(mudpack_form(s) for s in drawn) and not all(mudpack_form(s) for s in drawn)
    for (ny2, nz2), w in a:
        assert w.nx in (64, 128, 256)
        assert w.ny2 == mudpack_size(ny2) and w.nz2 == mudpack_size(nz2)
    assert len({(w.nx, w.ny2, w.nz2) for _, w in a}) > 1


def test_ensemble_step_rejects_bad_arguments():
    L = load_library()
    st = (C.c_int * 2)()
    assert L.ekgpu_ensemble_step(None, 1, 1, st) == 1
    h = (C.c_void_p * 2)(0x1000, 0x2000)
    assert L.ekgpu_ensemble_step(h, 0, 1, st) == 1
    assert L.ekgpu_ensemble_step(h, 2, -1, st) == 1
    assert L.ekgpu_ensemble_step((C.c_void_p * 2)(0x1000, None), 2, 1, st) == 1
    assert L.ekgpu_ensemble_step((C.c_void_p * 2)(0x1000, 0x1000), 2, 1, st) == 1


# members of different NX, NY+2 and NZ+2 (small enough for the oracle)
SIZES = [(16, 17, 17), (32, 33, 25), (8, 21, 33), (16, 25, 41)]


def _member(i, nx, ny2, nz2, **over):
    p, xp, yp, st = small_case(nx, ny2, nz2, seed=10 + i)
    for k, v in over.items():
        setattr(p, k, v)
    return p, xp, yp, st


@pytest.fixture(scope="module")
def _built():
    ekbuild.build()


@pytest.mark.gpu
def test_ensemble_members_match_oracle(_built):
    gs, os_ = [], []
    for i, sz in enumerate(SIZES):
        p, xp, yp, st = _member(i, *sz)
        g = DuctSolver(p, metrics_from_grid(p, xp, yp))
        g.upload(*st)
        o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
        o.upload(*st)
        gs.append(g)
        os_.append(o)
    assert ensemble_step(gs, 2) == [0] * len(gs)
    for i, (g, o) in enumerate(zip(gs, os_)):
        o.step(2)
        for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
            assert rel_l2(x, y) <= 1e-10, (SIZES[i], name)
        assert g.divergence() == pytest.approx(o.divergence(), rel=1e-6, abs=1e-14)
        g.close()


@pytest.mark.gpu
def test_mixed_ensemble_equals_members_alone(_built):
    mixed = dict(mg_stop=EK_MG_STOP_RESIDUAL, mg_tol=1e-10, mg_maxcy=60, mg_fast=1, fft_fp32=1, ff_arith=1)
    together, alone = [], []
    for i, sz in enumerate(SIZES):
        p, xp, yp, st = _member(i, *sz, **mixed)
        for group in (together, alone):
            g = DuctSolver(p, metrics_from_grid(p, xp, yp))
            g.upload(*st)
            group.append(g)
    assert ensemble_step(together, 3) == [0] * len(SIZES)
    for g in alone:
        g.step(3)
    for i, (a, b) in enumerate(zip(together, alone)):
        for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), a.download(), b.download()):
            assert rel_l2(x, y) <= 1e-13, (SIZES[i], name)
        a.close()
        b.close()


@pytest.mark.gpu
def test_failing_member_leaves_the_others_stepping(_built):
    gs, ref = [], []
    for i, sz in enumerate(SIZES[:3]):
        # member 1 asks for LES but never gets its LES metrics
        p, xp, yp, st = _member(i, *sz, **({"les": 1} if i == 1 else {}))
        g = DuctSolver(p, metrics_from_grid(p, xp, yp))
        g.upload(*st)
        gs.append(g)
        if i != 1:
            r = DuctSolver(p, metrics_from_grid(p, xp, yp))
            r.upload(*st)
            r.step(1)
            ref.append(r)
    codes = ensemble_step(gs, 1, raise_on_error=False)
    assert codes == [0, 6, 0]  # EK_ERR_STATE for the member without LES metrics
    assert "LES metrics" in gs[1]._L.ekgpu_last_error(gs[1]._h).decode()
    for g, r in zip((gs[0], gs[2]), ref):
        for x, y in zip(g.download(), r.download()):
            assert rel_l2(x, y) <= 1e-13
    with pytest.raises(Exception, match="LES metrics"):
        ensemble_step(gs, 1)
    for g in gs + ref:
        g.close()
