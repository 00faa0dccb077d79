"""File output of SAVE_STATS_CURVI's plane statistics
(src/flow_statistics.F90:389-407, 941-977, 2636-2686), written on the host
from the planes ekgpu_save_stats returns.

  plane_data/time_bulk.txt        one line per call: TIME, DELTA_T, UBULK,
                                  VBULK, U3X(NXP,2,NY), U1X(NXP,2,NY) in
                                  FORMAT(6f15.7), appended
  plane_data/data_tec_KKKKK.pln   plot_binary: one Fortran unformatted record
                                  of 25 (0:NZ+1, 0:NY+1) REAL*8 planes,
                                  K = TIME_STEP / SAVE_STATS_INT mod 100000

The Tecplot file (plot_tecplot, linked against tecio) and the plane dumps
are not written.
"""
from __future__ import annotations

import os
import struct

import numpy as np

SUBRECORD_MAX = 2147483639  # Intel / GNU Fortran: largest subrecord payload


def write_record(f, payload: bytes, smax: int = SUBRECORD_MAX):
    """One Fortran unformatted sequential record: 4-byte length markers in
    host (little-endian) order; a record over smax bytes is split, the
    leading marker negative when a subrecord follows, the trailing marker
    negative when one precedes."""
    n, pos, first = len(payload), 0, True
    while True:
        k = min(n - pos, smax)
        more = pos + k < n
        f.write(struct.pack("<i", -k if more else k))
        f.write(payload[pos:pos + k])
        f.write(struct.pack("<i", k if first else -k))
        pos, first = pos + k, False
        if not more:
            return


def stats_file_name(time_step: int, save_stats_int: int) -> str:
    """'plane_data/data_tec_' // five digits of TIME_STEP/SAVE_STATS_INT // '.pln'
    (flow_statistics.F90:967-973)."""
    k = time_step // save_stats_int
    return f"plane_data/data_tec_{k % 100000:05d}.pln"


def time_bulk_line(time: float, delta_t: float, st: dict) -> str:
    """WRITE(66,565) ... with 565 FORMAT(6f15.7)."""
    vals = (time, delta_t, st["ubulk"], st["vbulk"], st["u3_probe"], st["u1_probe"])
    return "".join(f"{v:15.7f}" for v in vals) + "\n"


PLN_ORDER = ("xpoint", "ypoint", "mean_u3", "mean_u2", "mean_u1", "th_wh", "mean_th", "wrms", "vrms", "urms",
             "wv", "uv", "pv", "thrms", "thv", "thw", "rig", "dthdy", "dthdz", "tke", "omega_x", "dwdy", "dwdz",
             "dudy", "mean_p")


def plane_binary_payload(xpoint: np.ndarray, ypoint: np.ndarray, th_bar: np.ndarray, st: dict) -> bytes:
    """The record plot_binary writes (flow_statistics.F90:2670-2675):
    xpoint, ypoint, the mode-0 planes, TH_WH = DBLE(CTHX(0,:,:)) + TH_BAR
    and the statistics, each (0:NZ+1, 0:NY+1) with K fastest."""
    ny2, nz2 = st["urms"].shape
    planes = dict(st)
    planes["xpoint"] = np.asarray(xpoint, np.float64).reshape(ny2, nz2)
    planes["ypoint"] = np.asarray(ypoint, np.float64).reshape(ny2, nz2)
    tb = np.asarray(th_bar, np.float64).reshape(ny2 + 1, nz2 + 1)[:ny2, :nz2]  # TH_BAR(0:NZ+2,0:NY+2)
    planes["th_wh"] = st["mean_th"] + tb
    return b"".join(np.ascontiguousarray(planes[n], np.float64).tobytes() for n in PLN_ORDER)


def write_stats_files(root: str, time: float, delta_t: float, time_step: int, save_stats_int: int,
                      xpoint, ypoint, th_bar, st: dict) -> list:
    """The rank-0 file output of one SAVE_STATS_CURVI call; creates
    plane_data/ when missing.  Returns the paths written."""
    d = os.path.join(root, "plane_data")
    os.makedirs(d, exist_ok=True)
    tb = os.path.join(d, "time_bulk.txt")
    with open(tb, "a") as f:
        f.write(time_bulk_line(time, delta_t, st))
    pln = os.path.join(root, stats_file_name(time_step, save_stats_int))
    with open(pln, "wb") as f:
        write_record(f, plane_binary_payload(xpoint, ypoint, th_bar, st))
    return [tb, pln]
