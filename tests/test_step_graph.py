"""Whole RK3 steps run as CUDA graphs (ekgpu_step with the mixed solver).

A step replayed from its captured graph must equal the same step run
launch by launch, bit for bit: the graph holds the same kernels in the same
order, and the correction cycles that the eager path stops from the host
stop inside the graph at the same check.  Covered: the plain mixed step,
sponge_th with its CU2X reset (a key of its own), the LES schedule of
C_DYN (FIRST_TIME and every fifth step), a re-capture after the autotuner
changes the line-solve layouts, and the status a graph-run step reports for
a capped solve and for a NaN divergence.
"""
import numpy as np
import pytest

from ekcases import les_case, small_case, sponge_case
from ekman_bl_gb300 import build as ekbuild
from ekman_bl_gb300.duct import DuctSolver, les_metrics_from_grid, metrics_from_grid, sponge_profiles
from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _build():
    ekbuild.build()


def _mixed(p, ff=1):
    p.mg_stop, p.mg_tol, p.mg_maxcy, p.mg_fast, p.fft_fp32, p.ff_arith = EK_MG_STOP_RESIDUAL, 1e-10, 60, 1, 1, ff
    return p


def _pair(case, ff=1):
    p, xp, yp, st = case
    _mixed(p, ff)
    out = []
    for on in (True, False):
        g = DuctSolver(p, metrics_from_grid(p, xp, yp))
        g.set_step_graph(on)
        if p.les:
            g.set_les_metrics(les_metrics_from_grid(p, xp, yp))
        if p.sponge_type:
            g.set_sponge(*sponge_profiles(p, xp, yp))
        g.upload(*st)
        out.append(g)
    return out


def _same(a, b):
    for x, y, n in zip(a.download(), b.download(), ("CU1", "CU2", "CU3", "CP", "CTH")):
        assert np.array_equal(x, y), n
    assert a.divergence() == b.divergence()
    sa, sb = a.mg_stats(), b.mg_stats()
    for k in ("nprob", "min_cycles", "max_cycles", "n_not_converged", "max_residual"):
        assert sa[k] == sb[k], (k, sa, sb)


@pytest.mark.parametrize("variant", ["plain", "sponge", "les", "plain_inc", "sponge_inc"])
def test_graph_steps_equal_eager_steps(variant):
    """(_inc: the state path in FP32 increment form, ff_arith = 2.)"""
    ff = 2 if variant.endswith("_inc") else 1
    variant = variant.replace("_inc", "")
    if variant == "plain":
        case = small_case()
    elif variant == "sponge":
        # SAVE_STATS_INT = 4: the CU2X reset fires at TIME_STEP 2, 4, 6
        p, xp, yp, st = sponge_case(2, True, save_stats_int=4)
        case = (p, xp, yp, st)
    else:
        case = les_case("small")
    g, e = _pair(case, ff)
    try:
        for _ in range(7):  # the LES C_DYN recomputation falls on TIME_STEP 5
            assert g.step(1) == 0 and e.step(1) == 0
            _same(g, e)
        # steps 2..7 replayed graphs; the eager solver issued every launch
        assert g.get_time() == e.get_time()
        assert 0 < g.launch_count() <= e.launch_count() * 1.05
    finally:
        g.close()
        e.close()


def test_graph_recaptured_after_autotune():
    g, e = _pair(small_case())
    try:
        g.step(2)
        e.step(2)
        for s in (g, e):
            s.mg_autotune(reps=1)
        for lev in range(2, len(g.mg_levels()) + 1):
            for d in (0, 1):
                g.mg_set_layout(lev, d, 8, 8)
                e.mg_set_layout(lev, d, 8, 8)
        g.step(3)
        e.step(3)
        _same(g, e)
    finally:
        g.close()
        e.close()


def test_graph_step_reports_not_converged():
    p, xp, yp, st = small_case()
    _mixed(p)
    p.mg_maxcy = 1
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        with pytest.warns(RuntimeWarning, match="NOT_CONVERGED"):
            assert g.step(1) == 3   # eager
        n0 = g.mg_counters()[1]
        with pytest.warns(RuntimeWarning, match="NOT_CONVERGED"):
            assert g.step(2) == 3   # from the graph
        assert g.mg_counters()[1] > n0 and g.mg_stats()["max_cycles"] == 1
    finally:
        g.close()


def test_graph_step_reports_nan():
    p, xp, yp, st = small_case()
    _mixed(p)
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    try:
        g.upload(*st)
        g.step(2)  # eager, then a captured graph
        cu = g.download()
        cu[0][3, 3, 1] = np.nan
        g.upload(*cu)
        with pytest.raises(Exception) as e:
            g.step(1)
        assert "NAN" in str(e.value)
    finally:
        g.close()


def test_ensemble_graph_equals_members_stepped_alone():
    """Members of different sizes stepped as one graph launch per ensemble
    step equal the same members stepped one at a time without graphs."""
    from ekman_bl_gb300.duct import ensemble_step
    from test_ensemble import SIZES, _member
    together, alone = [], []
    for i, (nx, ny2, nz2) in enumerate(SIZES[:3]):
        p, xp, yp, st = _member(i, nx, ny2, nz2)
        _mixed(p)
        for group, on in ((together, True), (alone, False)):
            s = DuctSolver(p, metrics_from_grid(p, xp, yp))
            s.set_step_graph(on)
            s.upload(*st)
            group.append(s)
    try:
        # the first call steps the members on their own threads (an eager
        # step each, then their own graphs); the second one launches one
        # graph per ensemble step
        assert ensemble_step(together, 2) == [0, 0, 0]
        n0 = sum(s.launch_count() for s in together)
        assert ensemble_step(together, 3) == [0, 0, 0]
        assert sum(s.launch_count() for s in together) > n0
        for s in alone:
            assert s.step(5) == 0
        for a, b in zip(together, alone):
            _same(a, b)
            assert a.get_time() == b.get_time()
    finally:
        for s in together + alone:
            s.close()


@pytest.mark.parametrize("variant", ["plain", "sponge"])
def test_concurrent_branches_equal_one_chain(variant):
    """The increment form's concurrent branches (each field's chain on its own
    stream, a captured step's divergence check on a side stream) against the
    same steps as one chain of launches (the per-kernel timer forces that),
    bit for bit: the branches share no array, so no ordering between them
    can change a result.  The sponge case crosses sponge_th's CU2X reset."""
    if variant == "plain":
        case = small_case()
    else:
        p, xp, yp, st = sponge_case(2, True, save_stats_int=4)
        case = (p, xp, yp, st)
    g, e = _pair(case, 2)
    try:
        e.set_step_graph(False)
        e.set_timing(True)
        for _ in range(5):
            assert g.step(1) == 0 and e.step(1) == 0
            _same(g, e)
    finally:
        g.close()
        e.close()
