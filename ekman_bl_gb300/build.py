"""Build libekgpu.so (the C-ABI library with the sm_103a kernels) in-tree.

Each translation unit is compiled separately and in parallel with nvcc for
sm_103a only; the shared library lands in ekman_bl_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libekgpu.so")
SOURCES = ["ek_api.cu", "ek_fft.cu", "ek_rk.cu", "ek_mg.cu", "ek_mgfast.cu", "ek_host.cpp", "ek_io.cpp", "ek_stats.cu", "ek_unet.cu", "ek_guess.cu", "ek_les.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libekgpu.so")
    return path


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
    if src.endswith(".cu"):
        cmd += ARCH
    else:
        cmd += ["-x", "c++", "-Xcompiler", "-fopenmp"]
    subprocess.run(cmd, check=True)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "ekgpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc(), "-shared", "-o", tmp, *objs, *ARCH, "-lcudart", "-lgomp"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
