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

step_<case>.npz: the reference's time stepping -- REM_DIV_CURV
(src/duct.F90:2472-2850), then per step DO RK_STEP = 1,3: CALL RK_DUCT
(src/duct.F90:237-2460, with src/boundary.F90, src/mpi_duct.F90,
src/ALLOCATION.F90, and JACOBI_TRANS and INIT_DUCT for the set-up) -- on
the cases of tests/ekcases.golden_step_cases: the state after the steps
(modes 0..NKX; the ones above are zero), the divergence printed after
every projection, TIME and DELTA_T, C_DYN of the LES runs, JACOBI_TRANS's
metrics on the two curvilinear grids (the LES ones on the LES runs of
those grids), and a SHA-256 of the inputs, so the test knows that it
regenerated the same ones.  fft.F90 is missing from the reference tree:
the x-transforms are the oracle's (1/NX forward, unnormalised inverse,
modes above NKX zero), and MPI with one rank copies.

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


def case_digest(st, th_bar):
    """SHA-256 of a case's inputs: the state's bytes, then TH_BAR's."""
    import hashlib
    h = hashlib.sha256()
    for a in st:
        h.update(np.ascontiguousarray(a, np.complex128).tobytes())
    if th_bar is not None:
        h.update(np.ascontiguousarray(th_bar, np.float64).tobytes())
    return h.hexdigest()


def step_goldens(ref_root: str, only=None) -> None:
    """Reference time steps: REM_DIV_CURV, then per step DO RK_STEP = 1,3:
    RK_DUCT, on the cases of tests/ekcases.golden_step_cases (those named
    in only, if given)."""
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.join(here, ".."))
    sys.path.insert(0, os.path.join(here, "..", ".."))
    import reference_run as rr
    from ekcases import golden_step_cases
    for name, (p, xp, yp, st, tb, steps) in golden_step_cases().items():
        if only and name not in only:
            continue
        sponge = (p.ny_s_t, p.nz_s_r, p.nz_s_l) if p.sponge_type else None
        rt = rr.runtime(ref_root, p.nx, p.ny, p.nz, sponge=sponge, phi64=not p.quirk_phi_fp32)
        rr.duct_setup(rt, p, xp, yp, st, tb)
        # JACOBI_TRANS's metrics on the curvilinear grids, in the oracle's layout
        metrics = {}
        names = []
        if name in ("sheared", "refgrid"):
            names = [("run_variable", nm) for nm in ("int_jacob", "gmat_11", "gmat_12", "gmat_22", "cjob_11",
                                                     "cjob_12", "cjob_21", "cjob_22")]
        if name in ("les_sheared", "les_refgrid"):
            names = [("les_chan_var", f"gmat_{a}_{d}") for a in ("11", "12", "22") for d in ("y", "z")]
        for mod, nm in names:
            a = rt.var(mod, nm).a
            metrics[f"metric_{nm}"] = a.T if a.ndim == 2 else np.transpose(a, (2, 1, 0))
        rr.record_divergence(rt)
        rr.rem_div_curv(rt)
        for _ in range(steps):
            rr.rk_step(rt)
        state = np.stack(rr.get_state(rt))
        extra = {"time": rt.var("run_variable", "time")[0], "delta_t": rt.var("time_step_var", "delta_t")[0]}
        if p.les:
            extra["c_dyn"] = rt.var("les_chan_var", "c_dyn").a.T.copy()
        nkx = p.nx // 3
        # the modes above NKX are kept only where they are not all zero
        high = {"state_high": state[..., nkx + 1:]} if np.any(state[..., nkx + 1:]) else {}
        np.savez_compressed(os.path.join(here, f"step_{name}.npz"), nx=p.nx, ny=p.ny, nz=p.nz, steps=steps,
                            quirk_phi_fp32=p.quirk_phi_fp32, inputs_sha256=case_digest(st, tb),
                            state=state[..., :nkx + 1], divergence=np.array(rt.divergence), **high, **metrics,
                            **extra)
        print(f"wrote step_{name}.npz", state.shape, len(rt.divergence), "divergences")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the ekman_bl tree>")
    main(sys.argv[1])
    mudpack_goldens(sys.argv[1])
    step_goldens(sys.argv[1])
