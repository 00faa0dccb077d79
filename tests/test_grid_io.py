"""GRID_YZ.dat and density_data_input.dat (src/diablo.F90:1118-1158), read on
the host; the metrics built from a file read back equal those of the arrays
written."""
import os

import numpy as np
import pytest

from ekcases import GOLDEN, small_case
from ekman_bl_gb300.duct import metrics_from_grid
from ekman_bl_gb300.grid_io import read_density, read_grid_yz, write_grid_yz


def test_round_trip(tmp_path):
    p, xp, yp, _ = small_case()
    path = str(tmp_path / "GRID_YZ.dat")
    write_grid_yz(path, xp, yp)
    x2, y2 = read_grid_yz(path, p.ny, p.nz)
    assert np.array_equal(x2, xp) and np.array_equal(y2, yp)
    m1, m2 = metrics_from_grid(p, xp, yp), metrics_from_grid(p, x2, y2)
    for k in m1:
        assert np.array_equal(m1[k], m2[k]), k


def test_reference_grid_sample(tmp_path):
    """The committed every-4th-point sample of the reference grid written
    out and read back."""
    g = np.load(os.path.join(GOLDEN, "grid_yz_sub4.npz"))
    xp, yp = g["xpoint"], g["ypoint"]
    path = str(tmp_path / "GRID_YZ.dat")
    write_grid_yz(path, xp, yp)
    x2, y2 = read_grid_yz(path, xp.shape[0] - 2, xp.shape[1] - 2)
    assert np.array_equal(x2, xp) and np.array_equal(y2, yp)


def test_list_directed_forms(tmp_path):
    """Free-form lines as Fortran list-directed output writes them: E and D
    exponents, comma separators, blank lines, trailing values ignored."""
    path = tmp_path / "g.dat"
    lines = ["  0.000000000000000E+000  0.000000000000000E+000", "", "   1.12500000000000       2.5D-01",
             "3.0, 4.0, 99.0", "-1.0d0 5e-1"]
    path.write_text("\n".join(lines) + "\n")
    x, y = read_grid_yz(str(path), 0, 0)
    assert x.tolist() == [[0.0, 1.125], [3.0, -1.0]] and y.tolist() == [[0.0, 0.25], [4.0, 0.5]]
    with pytest.raises(ValueError, match="expected"):
        read_grid_yz(str(path), 1, 0)


def test_density(tmp_path):
    path = tmp_path / "density_data_input.dat"
    vals = np.arange(12.0).reshape(3, 4)        # NY = 1, NZ = 2
    path.write_text("\n".join(f"{v:.17g}" for v in vals.ravel()) + "\n")
    tb = read_density(str(path), 1, 2)
    assert tb.shape == (4, 5)
    assert np.array_equal(tb[:3, :4], vals) and not tb[3].any() and not tb[:, 4].any()
