"""The oracle against golden vectors from the reference's own source.

tests/golden/make_golden.py runs pieces of the reference tree's Fortran
through an interpreter of the Fortran subset they are written in
(tests/golden/fortran_interp.py: there is no Fortran compiler here) and
stores inputs and outputs as fixtures.  These tests give the oracle the
same inputs and require the same outputs, which pins the oracle's
restatement to the reference itself.

- mudpack_<case>.npz: MULTIGRID_MUDPACK (src/mg_solver2d.F90:75-201, phi_bc
  and cofcr of src/duct.F90:3867-3934, MUDPACK src/mud2cr.f, src/mudcom.f)
  with the reference's settings (FMG + at most 6 W(2,1) cycles, REAL*4 1e-6
  relative change) on the three test grids for kx^2 in {0, 0.3, 1, 7, 50}:
  the oracle's solve must agree bit for bit.
"""
import os

import numpy as np
import pytest

from ekman_bl_gb300.params import default_params
from oracle import ekref

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.fail(f"{name} missing: regenerate with tests/golden/make_golden.py")
    return np.load(path)


@pytest.mark.parametrize("case", ["small", "sheared", "refgrid"])
def test_oracle_poisson_equals_reference_mudpack(case):
    g = _fixture(f"mudpack_{case}.npz")
    p = default_params(int(g["nx"]), int(g["ny"]), int(g["nz"]))
    m = {k[len("metric_"):]: np.ascontiguousarray(g[k]) for k in g.files if k.startswith("metric_")}
    o = ekref.Oracle(p, m)
    phi, st, code = o.poisson(g["rhs"], g["kx2"])
    o.close()
    for q, k in enumerate(g["kx2"]):
        ref = g["phi"][q]
        assert np.array_equal(phi[q], ref), (q, k, np.abs(phi[q] - ref).max(), np.abs(ref).max())
