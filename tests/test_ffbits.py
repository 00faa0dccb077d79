"""The integer-pipe double <-> float conversions (ekman_bl_gb300/csrc/
ek_ffbits.h) against the compiler's conversions, bit for bit, on random
doubles over 140 binades (the header compiles as plain C++)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ffbits_bit_exact(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "ffbits_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "ekman_bl_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "ffbits_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
