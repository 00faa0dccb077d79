"""SAVE_STATS_CURVI (src/flow_statistics.F90:2-1023) and its file output.

CPU: the oracle's statistics against the Fortran formulas written out here
in numpy (loops over the same index ranges, fluctuations from the oracle's
own inverse transform); the oracle's state round trip; the .pln record and
the time_bulk.txt line.  GPU: the library against the oracle on the same
state (the mode-0 gradient planes bit for bit, the x-sums within 1e-12), the
state it leaves behind, and a run that keeps stepping after the call.
"""
import math
import struct

import numpy as np
import pytest

from ekcases import rel_l2, sheared_case, small_case
from ekman_bl_gb300.params import EK_F_CF1, EK_F_CF3, EK_F_CFTH, STATS_PLANES
from ekman_bl_gb300.stats_io import PLN_ORDER, plane_binary_payload, stats_file_name, time_bulk_line, write_record
from oracle import ekref


def cases():
    out = []
    p, xp, yp, st = small_case()
    out.append(("strat", p, xp, yp, st))
    p, xp, yp, st = sheared_case()
    p.cont_strat = 0                       # the TH_BAR gradient term of dthdy
    out.append(("sheared", p, xp, yp, st))
    p, xp, yp, st = small_case(seed=4)
    p.amp_omega0, p.omega0 = 0.3, 0.0146   # TKE scaled by (AMP_OMEGA0/OMEGA0)**(-2)
    out.append(("oscill", p, xp, yp, st))
    return out


CASES = cases()


def formula_stats(p, m, st):
    """flow_statistics.F90:80-555 and 846-920 written out with NP = 1."""
    NX, NY, NZ = p.nx, p.ny, p.nz
    cu1, cu2, cu3, cp, cth = st
    R1, R2, R3, T, Pm = (a[:, :, 0].real for a in (cu1, cu2, cu3, cth, cp))   # [j, k]
    phys = [ekref.fft_c2r(a, p.nx // 3) for a in (cu1, cu2, cu3, cp, cth)]    # [j, k, i]
    U1, U2, U3, PX, TH = (a[:, :, :NX] for a in phys)
    jac = m["int_jacob"]
    c11, c12, c21, c22 = (m[k] for k in ("cjob_11", "cjob_12", "cjob_21", "cjob_22"))
    tb = m["th_bar"]
    out = {}
    out["urms"] = np.sqrt(((U1 - R1[..., None]) ** 2).sum(-1) / NX)
    out["vrms"] = np.sqrt(((U2 - R2[..., None]) ** 2).sum(-1) / NX)
    out["wrms"] = np.sqrt(((U3 - R3[..., None]) ** 2).sum(-1) / NX)
    pmean = np.zeros_like(Pm)
    pmean[1:NY + 1, 1:NZ + 1] = Pm[1:NY + 1, 1:NZ + 1]
    u1, u2, u3 = U1 - R1[..., None], U2 - R2[..., None], U3 - R3[..., None]
    pp = PX - pmean[..., None]
    for name, a, b in (("uv", u1, u2), ("uw", u1, u3), ("wv", u3, u2), ("pu", u3, pp), ("pv", u2, pp)):
        v = (a * b).sum(-1) / NX
        v[:, 0] = 0.0
        v[:, NZ + 1] = 0.0
        out[name] = v
    e = R1 ** 2 + R2 ** 2 + R3 ** 2
    out["tke"] = e * (p.amp_omega0 / p.omega0) ** -2.0 if p.amp_omega0 != 0 else e
    cav = lambda A, k, j: 0.125 * (A[0, j, k] + A[0, j + 1, k] + A[1, j, k] + A[1, j, k + 1])
    z = lambda: np.zeros((NY + 2, NZ + 2))
    dudy, dwdy, dudz, dwdz, omx, dthdy, dthdz, rig = (z() for _ in range(8))
    wb = p.w_bc
    js = 1 if wb[0] in (0, 1, 6, 7, 3) else 2
    je = NY if wb[1] in (0, 1, 6, 7, 3) else NY - 1
    zs = 1 if p.u_bc[2] in (1, 6) else 2
    ze = NZ if p.u_bc[3] in (1, 6) else NZ - 1
    for k in range(1, NZ + 1):
        for j in range(1, NY + 1):
            a11, a12, a21, a22, J = cav(c11, k, j), cav(c12, k, j), cav(c21, k, j), cav(c22, k, j), jac[j, k]
            gy = lambda F: (a12 * (F[j, k + 1] - F[j, k - 1]) + a22 * (F[j + 1, k] - F[j - 1, k])) / J
            gz = lambda F: (a21 * (F[j + 1, k] - F[j - 1, k]) + a11 * (F[j, k + 1] - F[j, k - 1])) / J
            if zs <= k <= ze and js <= j <= je:
                dudy[j, k], dwdy[j, k] = gy(R1), gy(R3)
            dudz[j, k], dwdz[j, k] = gz(R1), gz(R3)
            omx[j, k] = gy(R3) - gz(R2)
            dthdy[j, k] = gy(T) + (0.0 if p.cont_strat else gy(tb))
            dthdz[j, k] = gz(T)
    for a in (dudy, dwdy, dudz, dwdz, omx):
        a[0, 1:NZ + 1] = a[1, 1:NZ + 1]
        a[NY + 1, 1:NZ + 1] = a[NY, 1:NZ + 1]
    dudz[1:NY + 1, 1] = dudz[1:NY + 1, 2]
    dwdz[1:NY + 1, 1] = dwdz[1:NY + 1, 2]
    for a in (dthdy, dthdz):
        a[1:NY + 1, 0] = a[1:NY + 1, 1]
        a[1:NY + 1, NZ + 1] = a[1:NY + 1, NZ]
        a[0, :] = 2.0 * a[1, :] - a[2, :]
        a[NY + 1, :] = 2.0 * a[NY, :] - a[NY - 1, :]
    for k in range(1, NZ + 1):
        for j in range(1, NY + 1):
            b = dthdy[j, k] - 1.0 if p.cont_strat else dthdy[j, k]
            den = dwdy[j, k] ** 2 + dudy[j, k] ** 2
            rig[j, k] = -p.ri_tau * b * 1e18 if dwdy[j, k] == 0.0 else -p.ri_tau * b / den
    out.update(dudy=dudy, dwdy=dwdy, dudz=dudz, dwdz=dwdz, omega_x=omx, dthdy=dthdy, dthdz=dthdz, rig=rig)
    th = TH - T[..., None]
    out["thrms"] = np.sqrt((th ** 2).sum(-1) / NX)
    out["thv"] = (th * u2).sum(-1) / NX
    out["thw"] = (th * u3).sum(-1) / NX
    corner = lambda F: 0.25 * (F[1:, 1:] + F[1:, :-1] + F[:-1, :-1] + F[:-1, 1:])
    n = float(NY * NZ)
    out["ubulk"] = corner(R3)[:NY, :NZ].sum() / n
    out["vbulk"] = corner(R1)[:NY, :NZ].sum() / n
    out["thbulk"] = corner(T)[:NY, :NZ].sum() / n
    area = jac[1:NY + 1, 1:NZ + 1].sum()
    for s, q in (("urms_b", "urms"), ("vrms_b", "vrms"), ("wrms_b", "wrms")):
        out[s] = (corner(out[q])[:NY, :NZ] * jac[1:NY + 1, 1:NZ + 1]).sum() / area
    out["u3_probe"] = phys[2][NY, 2, NX + 1]
    out["u1_probe"] = phys[0][NY, 2, NX + 1]
    return out


def oracle_for(p, xp, yp, st):
    o = ekref.Oracle(p, ekref.metrics_from_grid(p, xp, yp))
    o.upload(*st)
    return o


@pytest.mark.parametrize("name,p,xp,yp,st", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_formulas(name, p, xp, yp, st):
    m = ekref.metrics_from_grid(p, xp, yp)
    o = oracle_for(p, xp, yp, st)
    got = o.save_stats()
    want = formula_stats(p, m, st)
    for k, v in want.items():
        if np.ndim(v) == 0:
            assert got[k] == pytest.approx(v, rel=1e-12, abs=1e-300), k
        else:
            np.testing.assert_allclose(got[k], v, rtol=1e-11, atol=1e-14 * (np.abs(v).max() + 1e-300), err_msg=k)
    assert got["u3_probe"] == 0.0 and got["u1_probe"] == 0.0   # padding point NX+1
    assert np.abs(got["dwdy"]).max() > 0 and np.abs(got["uv"]).max() > 0 and np.abs(got["thv"]).max() > 0


def test_oracle_round_trip_state():
    name, p, xp, yp, st = CASES[0]
    o = oracle_for(p, xp, yp, st)
    o.put_field(EK_F_CF1, np.ones_like(st[0]))
    o.put_field(EK_F_CFTH, np.ones_like(st[0]))
    got = o.save_stats()
    after = o.download()
    nkx = p.nx // 3
    for a, b in zip(after, st):
        want = ekref.fft_r2c(ekref.fft_c2r(b, nkx), nkx)
        np.testing.assert_allclose(a, want, rtol=0, atol=1e-15 * np.abs(want).max())
        assert not a[:, :, nkx + 1:].any()
    assert not o.get_field(EK_F_CF1).any() and o.get_field(EK_F_CFTH).all()
    assert np.array_equal(got["mean_u1"], after[0][:, :, 0].real)


def test_pln_record(tmp_path):
    rng = np.random.default_rng(0)
    ny2, nz2 = 7, 5
    st = {n: rng.standard_normal((ny2, nz2)) for n in STATS_PLANES}
    xp, yp = rng.standard_normal((ny2, nz2)), rng.standard_normal((ny2, nz2))
    tb = rng.standard_normal((ny2 + 1, nz2 + 1))
    path = tmp_path / "x.pln"
    with open(path, "wb") as f:
        write_record(f, plane_binary_payload(xp, yp, tb, st))
    raw = path.read_bytes()
    n = 25 * ny2 * nz2 * 8
    assert struct.unpack_from("<i", raw, 0)[0] == n and struct.unpack_from("<i", raw, 4 + n)[0] == n
    planes = np.frombuffer(raw[4:4 + n], np.float64).reshape(25, ny2, nz2)
    assert PLN_ORDER[0] == "xpoint" and np.array_equal(planes[0], xp) and np.array_equal(planes[1], yp)
    assert np.array_equal(planes[5], st["mean_th"] + tb[:ny2, :nz2])     # TH_WH
    assert np.array_equal(planes[9], st["urms"]) and np.array_equal(planes[24], st["mean_p"])
    assert np.array_equal(planes[16], st["rig"]) and np.array_equal(planes[19], st["tke"])
    assert stats_file_name(1200, 100) == "plane_data/data_tec_00012.pln"
    assert stats_file_name(100 * 123456, 100) == "plane_data/data_tec_23456.pln"


def test_time_bulk_line():
    st = {"ubulk": 0.0123456789, "vbulk": -1.5, "u3_probe": 0.0, "u1_probe": 12345.6789}
    line = time_bulk_line(2.5, 3e-4, st)
    assert line == "      2.5000000      0.0003000      0.0123457     -1.5000000      0.0000000  12345.6789000\n"
    assert len(line) == 6 * 15 + 1


# --------------------------------------------------------------------------- GPU

EXACT = ("tke", "dudy", "dwdy", "dudz", "dwdz", "omega_x", "dthdy", "dthdz", "rig")


@pytest.mark.gpu
@pytest.mark.parametrize("name,p,xp,yp,st", CASES, ids=[c[0] for c in CASES])
def test_gpu_stats_match_oracle(name, p, xp, yp, st):
    from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    g.upload(*st)
    g.put_field(EK_F_CFTH, np.ones_like(st[0]))
    o = oracle_for(p, xp, yp, st)
    a, b = g.save_stats(), o.save_stats()
    for k in EXACT:
        assert np.array_equal(a[k], b[k]), k                     # mode-0 formulas: bit for bit
    # the mean planes after the round trip: roundoff of the transforms, on
    # the scale of the state (a mode-0 plane that is zero comes back as ~1e-18)
    scale = max(np.abs(f).max() for f in st)
    for k in STATS_PLANES:
        if k not in EXACT:
            atol = 1e-14 * scale if k.startswith("mean_") else 1e-13 * (np.abs(b[k]).max() + 1e-300)
            np.testing.assert_allclose(a[k], b[k], rtol=1e-12, atol=atol, err_msg=k)
    for k in ("ubulk", "vbulk", "thbulk", "urms_b", "vrms_b", "wrms_b", "u3_probe", "u1_probe"):
        assert a[k] == pytest.approx(b[k], rel=1e-12, abs=1e-15), k
    for x, y in zip(g.download(), o.download()):
        assert rel_l2(x, y) < 1e-14
    assert not g.get_field(EK_F_CF1).any() and not g.get_field(EK_F_CF3).any()
    assert g.get_field(EK_F_CFTH).all()


@pytest.mark.gpu
def test_gpu_stats_mid_run(tmp_path):
    """Steps, statistics with the file output, more steps: the state and the
    files follow the oracle."""
    from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
    name, p, xp, yp, st = CASES[0]
    p.save_stats_int = 2
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    g.upload(*st)
    o = oracle_for(p, xp, yp, st)
    g.step(2)
    o.step(2)
    a = g.save_stats(root=str(tmp_path), xpoint=xp, ypoint=yp)
    b = o.save_stats()
    scale = max(np.abs(f).max() for f in st)
    for k in STATS_PLANES:
        atol = 1e-11 * scale if k.startswith("mean_") else 1e-11 * (np.abs(b[k]).max() + 1e-300)
        np.testing.assert_allclose(a[k], b[k], rtol=1e-9, atol=atol, err_msg=k)
    g.step(2)
    o.step(2)
    for nm, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), o.download()):
        assert rel_l2(x, y) < 1e-10, nm
    pln = tmp_path / "plane_data" / "data_tec_00001.pln"
    raw = pln.read_bytes()
    n2 = (p.ny + 2) * (p.nz + 2)
    assert struct.unpack_from("<i", raw, 0)[0] == 25 * 8 * n2
    planes = np.frombuffer(raw[4:4 + 25 * 8 * n2], np.float64).reshape(25, p.ny + 2, p.nz + 2)
    assert np.array_equal(planes[PLN_ORDER.index("urms")], a["urms"])
    line = (tmp_path / "plane_data" / "time_bulk.txt").read_text().splitlines()
    assert len(line) == 1 and float(line[0][30:45]) == pytest.approx(a["ubulk"], abs=1e-7)
