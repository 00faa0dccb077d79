"""Oracle: restart files of SAVE_FLOW / BACKUP_FLOW / READ_FLOW
(src/diablo.F90:753-1072), restated in numpy.  Test infrastructure only: the
tests compare the library's writer and reader with these functions.

The reference writes with FORM="UNFORMATTED", sequential access
(diablo.F90:813-833): one record per WRITE statement, framed by 4-byte
record-length markers in host byte order.  Records longer than 2**31 - 9
bytes are split into subrecords, the leading marker negative when another
subrecord follows and the trailing marker negative when one precedes it
(the record layout documented for the Intel and GNU Fortran runtimes; the
reference builds with ifort, Makefile:8).  No restart file ships with the
reference, so the format is pinned by that documented layout, not by a
golden file.

  flow file    [NX NY NZ TIME TIME_STEP]  int32 x3, real*8, int32 (24 bytes)
               [CU1X CU2X CU3X CPX]       each (0:NX/2, 0:NZ+1, 0:NY+1) complex*16
  scalar file  [NX NY NZ TIME TIME_STEP] [CTHX(:,:,:,N)]

Arrays here are numpy (NY+2, NZ+2, NX/2+1) complex128, C order, which is
the Fortran (I, K, J) order.
"""
from __future__ import annotations

import struct

import numpy as np

SUBRECORD_MAX = 2147483639
HEADER = struct.Struct("<3idi")


def _write_record(f, payload: bytes, smax: int = SUBRECORD_MAX):
    n = len(payload)
    pos, first = 0, True
    while True:
        k = min(n - pos, smax)
        more = pos + k < n
        f.write(struct.pack("<i", -k if more else k))
        f.write(payload[pos:pos + k])
        f.write(struct.pack("<i", k if first else -k))
        pos += k
        first = False
        if not more:
            break


def _read_record(f) -> bytes:
    parts, first = [], True
    while True:
        (lead,) = struct.unpack("<i", f.read(4))
        k = abs(lead)
        parts.append(f.read(k))
        (tail,) = struct.unpack("<i", f.read(4))
        if abs(tail) != k or (tail < 0) == first or len(parts[-1]) != k:
            raise ValueError("corrupt record markers")
        first = False
        if lead >= 0:
            return b"".join(parts)


def write_flow(path, dims, time, time_step, fields, smax: int = SUBRECORD_MAX):
    """WRITE(10) NX, NY, NZ, TIME, TIME_STEP; WRITE(10) CU1X, CU2X, CU3X, CPX
    (diablo.F90:813-820); for a scalar file pass fields=[CTHX] (827-828)."""
    nx, ny, nz = dims
    with open(path, "wb") as f:
        _write_record(f, HEADER.pack(nx, ny, nz, float(time), int(time_step)), smax)
        _write_record(f, b"".join(np.ascontiguousarray(a, np.complex128).tobytes() for a in fields), smax)


def read_flow(path, dims, nfields):
    """READ (10) NX_T, NY_T, NZ_T, TIME, TIME_STEP; the dimension check
    (diablo.F90:953-963, raising where the reference STOPs); then nfields
    arrays of the spectral shape from the next record (966-969)."""
    nx, ny, nz = dims
    with open(path, "rb") as f:
        head = _read_record(f)
        nxt, nyt, nzt, time, step = HEADER.unpack(head[:HEADER.size])
        if (nxt, nyt, nzt) != (nx, ny, nz):
            raise ValueError("Error: old flowfield wrong dimensions.")
        data = _read_record(f)
    shape = (ny + 2, nz + 2, nx // 2 + 1)
    n = int(np.prod(shape))
    if len(data) < nfields * n * 16:
        raise ValueError("data record too short")
    arr = np.frombuffer(data, np.complex128, count=nfields * n).reshape((nfields,) + shape)
    return time, step, [a.copy() for a in arr]
