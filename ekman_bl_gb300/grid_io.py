"""The grid and background-density files JACOBI_TRANS reads
(src/diablo.F90:1118-1158), on the host.

  GRID_YZ.dat               one line per point, J outer, K inner:
                            READ(21,*) xpoint(K,J), ypoint(K,J), J, K = 0..NY+1, 0..NZ+1
  density_data_input.dat    READ(31,*) TH_BAR(K,J) in the same order, read
                            only when CONT_STRAT is false (otherwise
                            TH_BAR = -ypoint(K,J) + ypoint(0,NY+1))

Arrays are numpy (NY+2, NZ+2), the Fortran (0:NZ+1, 0:NY+1) layout.  The
metrics themselves come from ekgpu_metrics_from_grid.
"""
from __future__ import annotations

import numpy as np


def _values(path: str, per_line: int, count: int) -> np.ndarray:
    """The first per_line list-directed values of each of count lines
    (Fortran D exponents accepted); fewer lines is an error, as a Fortran
    READ past the end of the file is."""
    out = np.empty((count, per_line))
    n = 0
    with open(path) as f:
        for line in f:
            if n == count:
                break
            tok = line.replace(",", " ").split()
            if not tok:
                continue
            if len(tok) < per_line:
                raise ValueError(f"{path}: line {n + 1} has {len(tok)} values, {per_line} expected")
            out[n] = [float(t.replace("D", "E").replace("d", "e")) for t in tok[:per_line]]
            n += 1
    if n < count:
        raise ValueError(f"{path}: {n} points, {count} expected (NY+2)*(NZ+2)")
    return out


def read_grid_yz(path: str, ny: int, nz: int):
    """xpoint, ypoint from a GRID_YZ.dat file."""
    v = _values(path, 2, (ny + 2) * (nz + 2))
    return (np.ascontiguousarray(v[:, 0].reshape(ny + 2, nz + 2)),
            np.ascontiguousarray(v[:, 1].reshape(ny + 2, nz + 2)))


def write_grid_yz(path: str, xpoint: np.ndarray, ypoint: np.ndarray):
    """A GRID_YZ.dat for read_grid_yz and for the reference's own reader:
    two values per line, J outer, K inner, full REAL*8 precision."""
    with open(path, "w") as f:
        for x, y in zip(np.asarray(xpoint).ravel(), np.asarray(ypoint).ravel()):
            f.write(f"{x:25.16E} {y:25.16E}\n")


def read_density(path: str, ny: int, nz: int) -> np.ndarray:
    """TH_BAR(0:NZ+1, 0:NY+1) from density_data_input.dat, as the
    (NY+3, NZ+3) metric-layout array ekgpu_set_metrics takes (the extra
    row and column, TH_BAR(NZ+2,:) and TH_BAR(:,NY+2), zero)."""
    v = _values(path, 1, (ny + 2) * (nz + 2))[:, 0].reshape(ny + 2, nz + 2)
    tb = np.zeros((ny + 3, nz + 3))
    tb[:ny + 2, :nz + 2] = v
    return tb
