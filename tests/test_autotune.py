"""Tile-shape autotuner of the mixed solver's line solves.

Each problem's arithmetic does not depend on the problems per block (8, 16
or 32): a line's segments and separators are all the problem's own lane.  So
with 8-row segments every layout gives the default solve bit for bit.  With
4-row segments the elimination order changes: the solve then meets the same
tolerance in the same number of cycles and agrees to that tolerance.
"""
import math

import numpy as np
import pytest

from ekcases import small_case
from ekman_bl_gb300.params import EK_MG_STOP_RESIDUAL

pytestmark = pytest.mark.gpu


def mixed_solver():
    from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
    p, xp, yp, st = small_case(nx=32, ny2=129, nz2=65, mg_stop=EK_MG_STOP_RESIDUAL)
    p.mg_tol, p.mg_maxcy, p.mg_fast = 1e-10, 60, 1
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    g.upload(*st)
    return p, g


def batch(p, seed=3):
    kx2 = np.array([(2 * math.pi * k / p.lx) ** 2 for k in (1, 2, 3, 5, 8, 10)])
    rhs = np.random.default_rng(seed).standard_normal((len(kx2), p.ny + 2, p.nz + 2))
    rhs[:, 0, :] = 0
    rhs[:, -1, :] = 0
    return rhs, kx2


def test_layouts_give_identical_solves():
    p, g = mixed_solver()
    rhs, kx2 = batch(p)
    phi0, st0, c0 = g.multigrid_mudpack(rhs, kx2)
    assert c0 == 0
    ngrid = len(g.mg_levels())
    for lanes in (8, 16, 32):
        for lev in range(2, ngrid + 1):
            for d in (0, 1):
                g.mg_set_layout(lev, d, lanes, 8)
        phi, st, c = g.multigrid_mudpack(rhs, kx2)
        assert c == 0 and st["max_cycles"] == st0["max_cycles"] and st["min_cycles"] == st0["min_cycles"]
        assert np.array_equal(phi, phi0), lanes


def test_short_segments_meet_the_tolerance():
    p, g = mixed_solver()
    rhs, kx2 = batch(p, seed=5)
    phi0, st0, _ = g.multigrid_mudpack(rhs, kx2)
    ngrid = len(g.mg_levels())
    for lanes in (8, 16):
        for lev in range(2, ngrid + 1):
            for d in (0, 1):
                g.mg_set_layout(lev, d, lanes, 4)
        phi, st, c = g.multigrid_mudpack(rhs, kx2)
        assert c == 0 and st["n_not_converged"] == 0 and st["max_residual"] <= p.mg_tol
        assert abs(st["max_cycles"] - st0["max_cycles"]) <= 1
        assert np.linalg.norm(phi - phi0) <= 1e-8 * np.linalg.norm(phi0)


def test_autotune_picks_valid_layouts_and_changes_nothing():
    p, g = mixed_solver()
    rhs, kx2 = batch(p, seed=4)
    phi0, st0, _ = g.multigrid_mudpack(rhs, kx2)
    a0 = g.download()
    rep = g.mg_autotune(reps=2)
    levels = g.mg_levels()
    # the coarse levels 1..ltop run as one launch per cycle, with no layouts
    ltop = g.mg_tail_levels()
    assert 1 <= ltop < len(levels)
    first = max(2, ltop + 1)
    assert len(rep) == 2 * (len(levels) - first + 1)
    assert sorted({row["level"] for row in rep}) == list(range(first, len(levels) + 1))
    for row in rep:
        assert row["lanes"] in (8, 16, 32) and row["seg"] in (4, 8)
        assert f'{row["lanes"]}x{row["seg"]}' in row["us"]
        assert all(v > 0 for v in row["us"].values())
        nx, ny = levels[row["level"] - 1]
        assert row["n"] == (nx if row["dir"] == "x" else ny)
    # the state is untouched, and a solve after tuning is the same solve
    for x, y in zip(g.download(), a0):
        assert np.array_equal(x, y)
    phi, st, c = g.multigrid_mudpack(rhs, kx2)
    assert c == 0 and st["max_residual"] <= p.mg_tol
    assert np.linalg.norm(phi - phi0) <= 1e-8 * np.linalg.norm(phi0)


def test_autotune_needs_the_mixed_solver():
    from ekman_bl_gb300.duct import DuctSolver, EkError, metrics_from_grid
    p, xp, yp, st = small_case()
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    with pytest.raises(EkError):
        g.mg_autotune()
