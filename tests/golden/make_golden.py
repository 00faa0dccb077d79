"""Regenerate the fixtures in this directory from the reference tree.

grid_yz_sub4.npz: the reference's own curvilinear y-z grid
(rundir_unst/GRID_YZ.dat, 321 x 129 points read J-outer / K-inner as in
JACOBI_TRANS, src/diablo.F90:1124-1128) subsampled every 4th point in both
directions to 81 x 33 (both still MUDPACK sizes p*2^k+1), and the divergence
values the reference printed after each projection (rundir_unst/log), kept as
a magnitude check.

mudpack_<case>.npz: MULTIGRID_MUDPACK (src/mg_solver2d.F90:75-201, with
phi_bc and cofcr of src/duct.F90:3867-3934 and MUDPACK's src/mud2cr.f and
src/mudcom.f) run on the three test grids of tests/ekcases.py for several
kx^2 and seeded right-hand sides -- the reference's own source executed by
fortran_interp.py, so the oracle's restatement of the Poisson solver is
checked against the reference itself.  Each file holds the metric arrays
the solve used, the right-hand sides, kx^2 and the reference's phi.

Run where the reference tree is available, with its root as the argument:
    python tests/golden/make_golden.py <path of the ekman_bl tree>
"""
import os
import re
import sys

import numpy as np


def main(ref_root: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    pts = np.loadtxt(os.path.join(ref_root, "rundir_unst", "GRID_YZ.dat"))
    nk, nj = 321, 129
    z = pts[:, 0].reshape(nj, nk)
    y = pts[:, 1].reshape(nj, nk)
    zs = np.ascontiguousarray(z[::4, ::4])
    ys = np.ascontiguousarray(y[::4, ::4])
    divs = []
    with open(os.path.join(ref_root, "rundir_unst", "log")) as f:
        for line in f:
            m = re.search(r"Divergence after the projection step:\s*([-+0-9.Ee]+)", line)
            if m:
                divs.append(float(m.group(1)))
    np.savez_compressed(os.path.join(here, "grid_yz_sub4.npz"), xpoint=zs, ypoint=ys,
                        logged_divergence=np.array(divs))
    print("wrote grid_yz_sub4.npz", zs.shape, len(divs), "divergence values")


MUDPACK_KX2 = (0.0, 0.3, 1.0, 7.0, 50.0)


def mudpack_goldens(ref_root: str) -> None:
    """Reference MULTIGRID_MUDPACK solves on the test grids."""
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.join(here, ".."))
    sys.path.insert(0, os.path.join(here, "..", ".."))
    import reference_run as rr
    from ekcases import refgrid_case, sheared_case, small_case
    from oracle import ekref
    for name, case in (("small", small_case), ("sheared", sheared_case), ("refgrid", refgrid_case)):
        p, xp, yp, _ = case()
        m = ekref.metrics_from_grid(p, xp, yp)
        rt = rr.runtime(ref_root, p.nx, p.ny, p.nz)
        rr.set_metrics(rt, m, p.nz, p.ny)
        rng = np.random.default_rng(40 + len(name))
        rhs = rng.standard_normal((len(MUDPACK_KX2), p.ny + 2, p.nz + 2))
        phi = np.stack([rr.multigrid_mudpack(rt, k, rhs[q]) for q, k in enumerate(MUDPACK_KX2)])
        out = {f"metric_{k}": v for k, v in m.items()}
        np.savez_compressed(os.path.join(here, f"mudpack_{name}.npz"), nx=p.nx, ny=p.ny, nz=p.nz,
                            kx2=np.array(MUDPACK_KX2), rhs=rhs, phi=phi, **out)
        print(f"wrote mudpack_{name}.npz", rhs.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the ekman_bl tree>")
    main(sys.argv[1])
    mudpack_goldens(sys.argv[1])
