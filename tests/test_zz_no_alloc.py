"""The allocation-free dense solve, m25_dense_solve_noalloc.

It serves callers whose device memory belongs to another allocator (a
framework's caching allocator, a fixed arena) and that cannot let this
library call cudaMalloc / cudaFree while they run: they hand in device
buffers for Z, B, X and the pivots, and the library's only scratch is one
static device array. Checked through the C ABI against m25_dense_solve on
the same systems, on calls in a row (the array keeps the previous call's
contents, which each call must clear). The third order, 4000, is above what
the fp64 cluster panel holds (about 2900 trailing rows), so its first panels
run the cooperative panel kernel, whose grid-barrier words and candidate
pivot rows live in the static array. The buffers below are allocated by this
test, which plays the caller.

This file is collected last on purpose, so that a run that stops at the
first failure has run every other test before it.
"""

import ctypes as C

import numpy as np
import pytest

from mom25d_gb300 import engine as E

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, the fp64 tolerance of the other dense-solve tests


def system(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A += 2 * np.sqrt(n) * np.eye(n) * (0.3 + 0.2j)
    A[:3, :3] = 0  # pivoting is required
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    return A, B


def test_noalloc_solve_matches_dense_solve(gpu):
    import torch

    lib = E.load()
    ctx = E.Context(0)
    info = np.zeros(2, np.int32)
    for call, n in enumerate((700, 1301, 4000)):
        A, B = system(n, 100 + call)
        # the existing entry point, host buffers
        Xref = np.zeros_like(B)
        Zref = A.copy()  # overwritten by its LU factors; held here until the call returns
        E.check(lib.m25_dense_solve(ctx.h, n, 2, E.M25_FP64, Zref.ctypes.data, B.ctypes.data, Xref.ctypes.data,
                                    E.M25_ON_HOST, 0.0, 0, E.ptr(info, C.c_int32)))
        # the allocation-free entry point on caller-owned device buffers
        dZ = torch.from_numpy(A.copy()).cuda()
        dB = torch.from_numpy(B.copy()).cuda()
        dX = torch.zeros_like(dB)
        dpiv = torch.zeros(n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        E.check(lib.m25_dense_solve_noalloc(n, 2, dZ.data_ptr(), dB.data_ptr(), dX.data_ptr(), dpiv.data_ptr(), None,
                                            E.ptr(info, C.c_int32)))
        X = dX.cpu().numpy()
        assert info[1] == 0
        assert np.abs(X - Xref).max() <= TOL * np.abs(Xref).max(), call
        assert np.abs(A @ X - B).max() <= 1e-10 * np.abs(B).max()
        piv = dpiv.cpu().numpy()
        assert piv.min() >= 0 and piv.max() < n and np.all(piv >= np.arange(n))
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    import torch

    lib = E.load()
    buf = torch.zeros(16, dtype=torch.complex128, device="cuda")
    piv = torch.zeros(16, dtype=torch.int32, device="cuda")
    info = np.zeros(2, np.int32)
    n = 24576 + 1  # M25_NOALLOC_MAX_N + 1: refused before any buffer is touched
    rc = lib.m25_dense_solve_noalloc(n, 1, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), piv.data_ptr(), None,
                                     E.ptr(info, C.c_int32))
    assert rc == E.M25_ERR_VALUE
    assert b"exceeds the maximum" in lib.m25_last_error()
