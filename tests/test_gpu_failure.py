"""Failure paths on the GPU, made without any fault: a bounded wait of the
triangular solve that runs out (a context-level poll limit too short for the
solve), and a sweep that stops part-way and resumes from its checkpoint
(Engine/tests/test_robustness.py:28-61 in mom25d)."""

import ctypes as C

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import engine as E
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _system(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A += 2 * np.sqrt(n) * np.eye(n)
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    return A, B


def _solve(ctx, A, B, precision):
    n = A.shape[0]
    Z = np.ascontiguousarray(A.copy())
    X = np.zeros_like(B)
    info = np.zeros(2, np.int32)
    E.check(ctx.lib.m25_dense_solve(ctx.h, n, B.shape[1], precision, Z.ctypes.data, B.ctypes.data, X.ctypes.data,
                                    E.M25_ON_HOST, 1e-14, 60, E.ptr(info, C.c_int32)))
    return X


@pytest.mark.parametrize("precision", [E.M25_FP64, E.M25_MIXED])
def test_triangular_solve_wait_runs_out_and_context_recovers(gpu, precision):
    """With one poll per ready-flag wait the wavefront solve of a 3000 x 3000
    system (47 dependent blocks) cannot finish: every block gives up, the
    call raises RuntimeError naming the wait, and the same context then
    solves the same system correctly with the default limit."""
    A, B = _system(3000, 11)
    Xr = np.linalg.solve(A, B)
    ctx = E.Context(0)
    try:
        E.check(ctx.lib.m25_ctx_set_wait_limit(ctx.h, 1))
        with pytest.raises(RuntimeError, match="wait of the triangular solve ran out"):
            _solve(ctx, A, B, precision)
        E.check(ctx.lib.m25_ctx_set_wait_limit(ctx.h, 0))
        X = _solve(ctx, A, B, precision)
        assert np.abs(X - Xr).max() <= 1e-11 * np.abs(Xr).max()
        # and once more: nothing of the failed call is left behind
        X = _solve(ctx, A, B, precision)
        assert np.abs(X - Xr).max() <= 1e-11 * np.abs(Xr).max()
    finally:
        ctx.close()


def test_wait_limit_rejects_a_negative_value(gpu):
    ctx = E.Context(0)
    try:
        assert ctx.lib.m25_ctx_set_wait_limit(ctx.h, -1) == E.M25_ERR_VALUE
    finally:
        ctx.close()


def test_checkpoint_resume(gpu, tmp_path):
    """A sweep killed after two of three frequencies resumes from its
    checkpoint: only the missing frequency is computed again and S is the
    uninterrupted sweep's; a sweep over other frequencies starts afresh."""
    lay, st, m, _ = workloads.build(G, "line")
    f = np.array([3.0, 5.0, 7.0]) * 1e9
    sol = Solver(m, st, verbose=False)
    try:
        ck = str(tmp_path / "ck.npz")
        full = sol.sweep(f, checkpoint=ck)
        d = dict(np.load(ck))
        assert d["done"].all()
        # a run killed after the first two frequencies
        d["done"][2] = False
        d["S"][2] = 0
        np.savez(ck, **d)
        calls = []
        point = sol.point
        sol.point = lambda fr, *a, **k: calls.append(fr) or point(fr, *a, **k)
        again = sol.sweep(f, checkpoint=ck)
        assert calls == [f[2]]
        np.testing.assert_array_equal(again.S, full.S)
        # a sweep the checkpoint does not describe computes every point
        calls.clear()
        sol.sweep(f[:2], checkpoint=ck)
        assert len(calls) == 2
    finally:
        sol.close()


def test_checkpoint_of_a_killed_sweep(gpu, tmp_path):
    """A point that fails part-way through a sweep leaves the checkpoint of
    the points before it; the restarted sweep computes only the rest."""
    lay, st, m, _ = workloads.build(G, "line")
    f = np.array([2.0, 4.0, 6.0, 8.0]) * 1e9
    sol = Solver(m, st, verbose=False)
    try:
        ref = sol.sweep(f)
        ck = str(tmp_path / "ck.npz")
        point = sol.point
        seen = []

        def dies_at_third(fr, *a, **k):
            seen.append(fr)
            if len(seen) == 3:
                raise RuntimeError("killed")
            return point(fr, *a, **k)

        sol.point = dies_at_third
        with pytest.raises(RuntimeError, match="killed"):
            sol.sweep(f, checkpoint=ck)
        assert list(np.load(ck)["done"]) == [True, True, False, False]
        calls = []
        sol.point = lambda fr, *a, **k: calls.append(fr) or point(fr, *a, **k)
        again = sol.sweep(f, checkpoint=ck)
        assert calls == [f[2], f[3]]
        np.testing.assert_array_equal(again.S, ref.S)
    finally:
        sol.close()
