"""The learned Green's remainder: the engine's MLP kernels against the
oracle (oracle/mlp.py), training, and the surrogate tables with their judge
against the Sommerfeld tabulation."""

import time

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import engine as E
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Greens, Solver
from mom25d_gb300.surrogate import MLP, GreensSurrogate
from oracle import mlp as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("layers,n_out", [(1, 3), (3, 6), (2, 54)])
def test_mlp_loss_and_gradient_match_oracle(gpu, layers, n_out):
    ctx = E.Context(0)
    net = MLP(ctx, 2, n_out, layers=layers, seed=3)
    rng = np.random.default_rng(layers)
    p = (rng.standard_normal(net.count) * 0.2).astype(np.float32)
    net.set_params(p)
    np.testing.assert_array_equal(net.params(), p)
    X = rng.uniform(-1, 1, (300, 2)).astype(np.float32)
    Y = rng.standard_normal((300, n_out)).astype(np.float32)
    loss, g = net.loss_grad(X, Y)
    lo, go = O.loss_grad(p.astype(float), X.astype(float), Y.astype(float), layers)
    assert abs(loss - lo) <= 1e-5 * lo
    # fp32 kernels against the float64 oracle
    assert np.abs(g - go).max() <= 2e-5 * np.abs(go).max(), np.abs(g - go).max() / np.abs(go).max()
    f = net(X)
    fo = O.forward(p.astype(float), X.astype(float), layers, n_out)[0]
    assert np.abs(f - fo).max() <= 1e-5 * np.abs(fo).max()
    net.close()
    ctx.close()


def test_mlp_training_fits_a_smooth_function(gpu):
    ctx = E.Context(0)
    net = MLP(ctx, 2, 2, layers=3, seed=0)
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (8192, 2))
    Y = np.stack([np.sin(2 * X[:, 0]) * np.cos(X[:, 1]), X[:, 0] * X[:, 1]], 1)
    loss0, _ = net.loss_grad(X, Y)
    loss = net.train(X, Y, steps=3000, batch=2048, lr=3e-3, lr_min=1e-5, seed=1)
    assert loss < 1e-4 * loss0, (loss0, loss)
    # deterministic: the same seed gives the same network
    net2 = MLP(ctx, 2, 2, layers=3, seed=0)
    loss2 = net2.train(X, Y, steps=3000, batch=2048, lr=3e-3, lr_min=1e-5, seed=1)
    assert loss2 == loss
    net.close()
    net2.close()
    ctx.close()


@pytest.fixture(scope="module")
def lpf_surrogate(gpu):
    lay, st, m, freqs = workloads.build(G, "lpf")
    sol = Solver(m, st, verbose=False, precision="mixed")
    t0 = time.perf_counter()
    sur = GreensSurrogate(sol, 0.5e9, 8e9)
    print(f"surrogate: {sur.nsamples} samples in {sur.sample_seconds:.2f} s, trained in {sur.train_seconds:.2f} s, "
          f"loss {sur.train_loss:.3e} (total {time.perf_counter() - t0:.2f} s)")
    yield sol, sur, freqs
    sur.close()
    sol.close()


def plan(rho, near, stride):
    """The radii a learned table integrates (the engine's rule, restated):
    every radius below `near`, then every stride-th radius and the last (the
    knots), and the middle radius of each gap between knots (validation).
    Returns (integrated, knots, validation, rest) index arrays."""
    n = rho.size
    n0 = int(np.searchsorted(rho, near, side="left"))
    knots = list(range(n0)) + list(range(n0, n, stride))
    if knots[-1] != n - 1:
        knots.append(n - 1)
    knots = np.array(knots)
    val = np.array([(a + b) // 2 for a, b in zip(knots[:-1], knots[1:]) if b - a >= 2], int)
    ie = np.union1d(knots, val)
    return ie, knots, val, np.setdiff1d(np.arange(n), ie)


def test_surrogate_tables_and_judge(lpf_surrogate):
    """Learned tables on the LPF stack: the integrated radii carry the
    Sommerfeld integral bit for bit; the other radii hold the network plus a
    not-a-knot spline of its residual through the integrated radii (checked
    against scipy); the judge's error is the error of the knots-only spline
    at the validation radii; a rejected table is the plain one bit for bit."""
    from scipy.interpolate import CubicSpline

    sol, sur, freqs = lpf_surrogate
    sol.surrogate = sur
    tol0, sur.tol = sur.tol, 4e-5  # a looser judge, so that some tables take the learned path
    out = []
    for f in (0.6e9, 2.3e9, 4.1e9, 7.9e9):
        g = Greens(sol, f)
        res, (used, err, nint) = g.remainder()
        g_ref = Greens(sol, f, surrogate=False)
        ref, (_, _, nref) = g_ref.remainder()
        rho = g.rho
        ie, kn, va, rest = plan(rho, sur.near * sur.a, sur.stride)
        smax = np.abs(ref[ie]).max()
        net = sur.predict(rho, f)
        cs = CubicSpline(rho[kn], ref[kn] - net[kn], bc_type="not-a-knot", axis=0)
        judged = np.abs(net[va] + cs(rho[va]) - ref[va]).max() / smax
        true_err = np.abs(res - ref).max() / np.abs(ref).max()
        out.append((f, used, err, judged, true_err, nint, nref))
        assert nref == rho.size
        # the judge, restated (the network's fp32 outputs at the device's features
        # and at numpy's may differ in the last bit: ~6e-8 of the largest remainder)
        assert abs(err - judged) <= 0.05 * judged + 1e-7, (err, judged)
        assert used == (err <= sur.tol)
        if used:
            assert nint == ie.size
            np.testing.assert_array_equal(res[ie], ref[ie])
            cs2 = CubicSpline(rho[ie], ref[ie] - net[ie], bc_type="not-a-knot", axis=0)
            fill = net[rest] + cs2(rho[rest])
            assert np.abs(res[rest] - fill).max() <= 2e-7 * smax
            assert true_err <= sur.tol
        else:
            assert nint == rho.size
            np.testing.assert_array_equal(res, ref)
        g.close()
        g_ref.close()
    print("(f, used, judged error, judged error restated, error vs Sommerfeld, radii integrated, radii):", out)
    assert any(o[1] for o in out)
    sur.tol = tol0
    sol.surrogate = None


def test_surrogate_sweep_within_mixed_bar(lpf_surrogate):
    """S of the mixed path with the learned remainder (default judge
    tolerance) within 1e-5 of the mixed path without it."""
    sol, sur, freqs = lpf_surrogate
    f = np.asarray(freqs, float)[::25]
    r0 = sol.sweep(f)
    sol.surrogate = sur
    r1 = sol.sweep(f)
    sol.surrogate = None
    d = np.abs(r1.S - r0.S).max()
    print("max |dS| with the learned remainder:", d)
    assert d <= 1e-5


def _greens_ms(sol, f, surrogate):
    """Device time of one frequency's Green's tables (CUDA events around the
    table kernels, the engine's stage timer), the table's remainder info
    (used, judged error, radii integrated) and its radii."""
    import ctypes as C

    ms = (C.c_double * 11)()
    E.check(sol.ctx.lib.m25_ctx_timing(sol.ctx.h, 1, None, None))
    g = Greens(sol, f, surrogate=surrogate)
    res, info = g.remainder()
    sol.ctx.synchronize()
    E.check(sol.ctx.lib.m25_ctx_timing(sol.ctx.h, 0, ms, None))
    rho = g.rho
    g.close()
    return ms[0], info, rho, res


def test_learned_remainder_pays_on_the_via_transition(gpu):
    """The two-layer via transition (4 level pairs x 3 kernels per radius):
    a network trained on ~1e6 of the engine's own Sommerfeld remainders over
    1-20 GHz. At the default judge tolerance it is accepted at most
    frequencies; each accepted table integrates fewer radii and takes less
    device time than the plain tabulation; the network's correction through
    the knots is judged more accurate than a spline of the integral alone
    through the same knots (what the network adds); and the sweep's S stays
    within 1e-5 of the plain tabulation's."""
    from scipy.interpolate import CubicSpline

    lay, st, m, freqs = workloads.build(G, "via")
    sol = Solver(m, st, verbose=False, precision="mixed")
    try:
        sur = GreensSurrogate(sol, 1e9, 20e9, nfreq=1024, nrad=1024, steps=20000)
        print(f"{sur.nsamples} samples in {sur.sample_seconds:.2f} s, trained in {sur.train_seconds:.2f} s, "
              f"loss {sur.train_loss:.3e}")
        assert sur.nsamples >= 1_000_000
        sol.surrogate = sur
        fs = np.linspace(1.5e9, 19.5e9, 10)
        for f in fs[:2]:  # warm-up of both paths
            _greens_ms(sol, f, True)
            _greens_ms(sol, f, False)
        rows = []
        for f in fs:
            t_sur, (used, err, nint), rho, _ = _greens_ms(sol, f, True)
            t_ref, _, _, ref = _greens_ms(sol, f, False)
            ie, kn, va, rest = plan(rho, sur.near * sur.a, sur.stride)
            cs = CubicSpline(rho[kn], ref[kn], bc_type="not-a-knot", axis=0)
            plain_err = np.abs(cs(rho[va]) - ref[va]).max() / np.abs(ref[ie]).max()
            rows.append((f / 1e9, used, err, plain_err, nint, rho.size, t_sur, t_ref))
        print("(f GHz, learned table used, judged error, knots-only spline error, radii integrated, radii, "
              "ms with, ms without):")
        for r in rows:
            print("  %.1f %d %.2e %.2e %d %d %.3f %.3f" % r)
        accepted = [r for r in rows if r[1]]
        assert len(accepted) >= len(rows) // 2, rows
        assert all(r[4] < r[5] for r in accepted)  # fewer Sommerfeld radii
        assert sum(r[6] for r in accepted) < sum(r[7] for r in accepted), rows  # less device time
        assert np.median([r[2] / r[3] for r in rows]) < 1.0  # the network beats the spline alone
        f = freqs[::4]
        r1 = sol.sweep(f)
        sol.surrogate = None
        r0 = sol.sweep(f)
        d = np.abs(r1.S - r0.S).max()
        print("max |dS| with the learned remainder:", d)
        assert d <= 1e-5
        sur.close()
    finally:
        sol.close()
