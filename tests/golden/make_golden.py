"""Regenerate the fixtures in this directory from the reference tree.

grid_yz_sub4.npz: the reference's own curvilinear y-z grid
(rundir_unst/GRID_YZ.dat, 321 x 129 points read J-outer / K-inner as in
JACOBI_TRANS, src/diablo.F90:1124-1128) subsampled every 4th point in both
directions to 81 x 33 (both still MUDPACK sizes p*2^k+1), and the divergence
values the reference printed after each projection (rundir_unst/log), kept as
a magnitude check.

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


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the ekman_bl tree>")
    main(sys.argv[1])
