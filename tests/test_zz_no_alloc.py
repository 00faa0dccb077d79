"""The allocation-free forward x-transform, checked against the regular one.

ekgpu_fft_x_to_fourier_noalloc serves callers that may not allocate device
memory (their application owns the GPU's memory through its own pool, or
they run a time-critical loop that cannot afford cudaMalloc/cudaFree).  It
keeps its twiddle scratch in a fixed device array instead.  This test calls
both entry points through the C ABI on the same inputs, twice in a row with
different sizes (so the second call must overwrite what the first left in
the shared array), and requires the same results within the tolerance the
other transform tests use.  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

from ekman_bl_gb300 import build as ekbuild
from ekman_bl_gb300.duct import load_library

pytestmark = pytest.mark.gpu


def _transform(fn, nx, nkx, x, torch):
    nlines = x.shape[0]
    xd = torch.from_numpy(x).cuda()
    out = torch.zeros((nlines, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    st = fn(nx, nkx, nlines, C.c_void_p(xd.data_ptr()), C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    return st, out.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    ekbuild.build()
    L = load_library()
    L.ekgpu_fft_x_to_fourier_noalloc.argtypes = [C.c_int, C.c_int, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(2024)
    for nx, nlines in ((1024, 29), (64, 300)):
        nkx = nx // 3
        x = np.zeros((nlines, nx + 2))
        x[:, :nx] = rng.standard_normal((nlines, nx))
        st_a, a = _transform(L.ekgpu_fft_x_to_fourier_noalloc, nx, nkx, x, torch)
        st_b, b = _transform(L.ekgpu_fft_x_to_fourier, nx, nkx, x, torch)
        assert st_a == 0 and st_b == 0
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-14
        assert not a[:, nkx + 1:].any()


def test_noalloc_allocates_no_table():
    """A size no other call of this process used: the regular entry point
    would allocate a twiddle table for it, the allocation-free one must not."""
    torch = pytest.importorskip("torch")
    ekbuild.build()
    L = load_library()
    L.ekgpu_fft_x_to_fourier_noalloc.argtypes = [C.c_int, C.c_int, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p]
    nx = 512
    x = np.zeros((7, nx + 2))
    x[:, :nx] = np.random.default_rng(5).standard_normal((7, nx))
    before = L.ekgpu_fft_table_count()
    st, _ = _transform(L.ekgpu_fft_x_to_fourier_noalloc, nx, nx // 3, x, torch)
    assert st == 0
    assert L.ekgpu_fft_table_count() == before


def test_noalloc_rejects_sizes_beyond_its_scratch():
    ekbuild.build()
    L = load_library()
    L.ekgpu_fft_x_to_fourier_noalloc.argtypes = [C.c_int, C.c_int, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p]
    st = L.ekgpu_fft_x_to_fourier_noalloc(2048, 600, 1, None, None, None)
    assert st == 1
    assert b"1024" in L.ekgpu_last_error(None)
