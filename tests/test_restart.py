"""Restart files: SAVE_FLOW, BACKUP_FLOW, READ_FLOW (src/diablo.F90:753-1072).

CPU: the file names against the Fortran CHAR arithmetic written out here;
the oracle's record layout against an independent parse of the bytes
(marker values, header offsets, subrecord signs); the oracle's dimension
check.  GPU: the library's files byte for byte equal to the oracle's (with
and without subrecord splits), the library reading oracle-written files,
error cases leaving the state unchanged, and a run restarted from a file
equal to the uninterrupted run.
"""
import os
import struct

import numpy as np
import pytest

from ekcases import rel_l2, small_case
from ekman_bl_gb300.duct import EkError, restart_file_names
from ekman_bl_gb300.params import EK_F_CF1, EK_F_CF2
from oracle import restart


def fortran_name(prefix, i, ext, n=None):
    """FNAME / FNAME_TH as diablo.F90:781-809 builds them, digit by digit."""
    d = lambda v: chr(v + 48)
    s = prefix
    if n is not None:
        s += d(n % 100 // 10) + d(n % 10) + "_"
    return s + d(i % 1000 // 100) + d(i % 100 // 10) + d(i % 10) + ext


@pytest.mark.parametrize("rank", [0, 7, 41, 998, 1000])
def test_file_names(rank):
    i = rank + 1
    for kind in ("saved", "res"):
        flow, ths = restart_file_names(kind, rank, n_th=1)
        assert flow == fortran_name("last_saved/diablo_", i, "." + kind)
        assert ths == [fortran_name("last_saved/diablo_th", i, "." + kind, 1)]
    for m in (0, 3, 57, 12345):
        mm = "".join(chr(v + 48) for v in (m % 10000 // 1000, m % 1000 // 100, m % 100 // 10, m % 10))
        flow, ths = restart_file_names("backup", rank, n_th=1, backup_index=m)
        assert flow == fortran_name("backup/diablo_", i, ".saved_" + mm)
        assert ths == [fortran_name("backup/diablo_th", i, ".saved_" + mm, 1)]
    assert restart_file_names("saved", rank, n_th=0)[1] == []


def parse_records(raw):
    """Independent parse: list of (leading marker, payload, trailing marker)."""
    out, pos = [], 0
    while pos < len(raw):
        (lead,) = struct.unpack_from("<i", raw, pos)
        k = abs(lead)
        payload = raw[pos + 4:pos + 4 + k]
        (tail,) = struct.unpack_from("<i", raw, pos + 4 + k)
        out.append((lead, payload, tail))
        pos += 8 + k
    assert pos == len(raw)
    return out


def small_state(seed=0):
    p, xp, yp, st = small_case(seed=seed)
    return p, st


def test_oracle_record_layout(tmp_path):
    p, st = small_state()
    path = tmp_path / "f"
    restart.write_flow(path, (p.nx, p.ny, p.nz), 1.25, 17, st[:4])
    recs = parse_records(path.read_bytes())
    assert len(recs) == 2
    lead, head, tail = recs[0]
    assert lead == tail == 24
    assert struct.unpack("<3i", head[:12]) == (p.nx, p.ny, p.nz)
    assert struct.unpack("<d", head[12:20])[0] == 1.25
    assert struct.unpack("<i", head[20:24])[0] == 17
    lead, data, tail = recs[1]
    assert lead == tail == 4 * st[0].size * 16
    # (I, K, J) order: I fastest, complex*16 as (re, im)
    j, k, i = 3, 5, 2
    nk, ni = p.nz + 2, p.nx // 2 + 1
    off = ((j * nk + k) * ni + i) * 16
    assert struct.unpack_from("<2d", data, off) == (st[0][j, k, i].real, st[0][j, k, i].imag)
    off2 = st[0].size * 16 * 3 + off  # CPX is the fourth array of the record
    assert struct.unpack_from("<2d", data, off2) == (st[3][j, k, i].real, st[3][j, k, i].imag)


def test_oracle_subrecords(tmp_path):
    p, st = small_state()
    path = tmp_path / "f"
    smax = 1000
    restart.write_flow(path, (p.nx, p.ny, p.nz), 0.5, 3, st[:4], smax=smax)
    recs = parse_records(path.read_bytes())
    total = 4 * st[0].size * 16
    nsub = -(-total // smax)
    assert len(recs) == 1 + nsub
    assert recs[0][0] == recs[0][2] == 24
    data = recs[1:]
    for n, (lead, payload, tail) in enumerate(data):
        last, first = n == nsub - 1, n == 0
        assert abs(lead) == abs(tail) == len(payload)
        assert (lead < 0) == (not last)
        assert (tail < 0) == (not first)
    assert b"".join(r[1] for r in data) == b"".join(a.tobytes() for a in st[:4])
    time, step, back = restart.read_flow(path, (p.nx, p.ny, p.nz), 4)
    assert (time, step) == (0.5, 3)
    for a, b in zip(back, st[:4]):
        assert np.array_equal(a, b)


def test_oracle_dimension_check(tmp_path):
    p, st = small_state()
    path = tmp_path / "f"
    restart.write_flow(path, (p.nx, p.ny + 1, p.nz), 0.0, 0, st[:4])
    with pytest.raises(ValueError, match="wrong dimensions"):
        restart.read_flow(path, (p.nx, p.ny, p.nz), 4)


# --------------------------------------------------------------------------- GPU

def solver(seed=0):
    from ekman_bl_gb300.duct import DuctSolver, metrics_from_grid
    p, xp, yp, st = small_case(seed=seed)
    g = DuctSolver(p, metrics_from_grid(p, xp, yp))
    g.upload(*st)
    return p, g, st


@pytest.mark.gpu
@pytest.mark.parametrize("smax", [None, 1000, 4096])
def test_save_matches_oracle_bytes(tmp_path, monkeypatch, smax):
    if smax is not None:
        monkeypatch.setenv("EKGPU_FORTRAN_SUBRECORD", str(smax))
    p, g, _ = solver()
    g.step(2)
    g.set_time(0.375, 42)
    g.write_restart(str(tmp_path / "gpu.saved"), str(tmp_path / "gpu_th.saved"))
    st = g.download()
    dims = (p.nx, p.ny, p.nz)
    kw = {} if smax is None else {"smax": smax}
    restart.write_flow(tmp_path / "ora.saved", dims, 0.375, 42, st[:4], **kw)
    restart.write_flow(tmp_path / "ora_th.saved", dims, 0.375, 42, st[4:], **kw)
    assert (tmp_path / "gpu.saved").read_bytes() == (tmp_path / "ora.saved").read_bytes()
    assert (tmp_path / "gpu_th.saved").read_bytes() == (tmp_path / "ora_th.saved").read_bytes()


@pytest.mark.gpu
def test_read_oracle_file(tmp_path):
    p, g, _ = solver()
    _, _, st = solver(seed=5)
    dims = (p.nx, p.ny, p.nz)
    restart.write_flow(tmp_path / "f", dims, 2.5, 11, st[:4], smax=777)
    restart.write_flow(tmp_path / "t", dims, 2.75, 12, st[4:], smax=5000)
    g.step(1)
    g.read_restart(str(tmp_path / "f"), str(tmp_path / "t"))
    for name, a, b in zip(("CU1", "CU2", "CU3", "CP", "CTH"), g.download(), st):
        assert np.array_equal(a, b), name
    t, n, _ = g.get_time()
    assert (t, n) == (2.75, 12)           # the scalar file's header is read last
    assert not g.get_field(EK_F_CF1).any() and not g.get_field(EK_F_CF2).any()
    # without the scalar file CTHX is left alone (NUM_READ_TH = 0)
    _, _, st2 = solver(seed=6)
    restart.write_flow(tmp_path / "f2", dims, 4.0, 20, st2[:4])
    g.read_restart(str(tmp_path / "f2"))
    got = g.download()
    assert np.array_equal(got[0], st2[0]) and np.array_equal(got[4], st[4])
    assert g.get_time()[:2] == (4.0, 20)


@pytest.mark.gpu
def test_read_errors_leave_state(tmp_path):
    p, g, _ = solver()
    g.step(1)
    before = g.download()
    t0 = g.get_time()
    dims = (p.nx, p.ny, p.nz)
    _, _, st = solver(seed=3)
    bad = {
        "dims": ((p.nx * 2, p.ny, p.nz), None),
        "truncated": (dims, -100),
        "markers": (dims, "flip"),
    }
    for name, (d, cut) in bad.items():
        path = tmp_path / name
        restart.write_flow(path, d, 9.0, 99, st[:4])
        raw = bytearray(path.read_bytes())
        if cut == "flip":
            raw[-1] ^= 0x01               # trailing marker of the data record
        elif cut is not None:
            raw = raw[:cut]
        path.write_bytes(bytes(raw))
        with pytest.raises(EkError) as e:
            g.read_restart(str(path))
        assert e.value.code == 7, name    # EK_ERR_IO
        if name == "dims":
            assert "wrong dimensions" in str(e.value)
        for a, b in zip(g.download(), before):
            assert np.array_equal(a, b), name
        assert g.get_time() == t0
    with pytest.raises(EkError):
        g.read_restart(str(tmp_path / "missing"))
    # a good flow file with a bad scalar file: nothing is read
    restart.write_flow(tmp_path / "good", dims, 9.0, 99, st[:4])
    restart.write_flow(tmp_path / "badth", (p.nx, p.ny, p.nz + 2), 9.0, 99, st[4:])
    with pytest.raises(EkError):
        g.read_restart(str(tmp_path / "good"), str(tmp_path / "badth"))
    for a, b in zip(g.download(), before):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_restarted_run_continues(tmp_path):
    """SAVE_FLOW after 2 steps, READ_FLOW into a fresh context, 2 more steps:
    the same state as 4 uninterrupted steps."""
    p, a, _ = solver()
    a.step(2)
    t2 = a.get_time()[:2]
    paths = a.save_flow(root=str(tmp_path))
    assert [os.path.relpath(x, tmp_path) for x in paths] == list(
        [restart_file_names("saved", 0, 1)[0]] + restart_file_names("saved", 0, 1)[1])
    backup = a.backup_flow(1, root=str(tmp_path))
    assert backup[0].endswith("backup/diablo_001.saved_0002")
    a.step(2)
    p2, b, _ = solver(seed=9)
    b.read_flow(root=str(tmp_path))
    assert b.get_time()[:2] == t2 and t2[1] == 2
    b.step(2)
    for name, x, y in zip(("CU1", "CU2", "CU3", "CP", "CTH"), b.download(), a.download()):
        assert rel_l2(x, y) < 1e-13, name
    assert b.get_time()[:2] == a.get_time()[:2]
