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


def test_surrogate_tables_and_judge(lpf_surrogate):
    """In-band tables from the learned remainder: the judge's verdict
    matches the actual error against the full Sommerfeld remainder, and a
    rejected network leaves the Sommerfeld table untouched."""
    sol, sur, freqs = lpf_surrogate
    sol.surrogate = sur
    tol0, sur.tol = sur.tol, 4e-5  # a looser judge, so that some tables take the learned path
    out = []
    t_sur = t_ref = 0.0
    for f in (0.6e9, 2.3e9, 4.1e9, 7.9e9):
        t0 = time.perf_counter()
        g = Greens(sol, f)
        res, (used, err) = g.remainder()
        t1 = time.perf_counter()
        g_ref = Greens(sol, f, surrogate=False)
        ref, _ = g_ref.remainder()
        t_sur += t1 - t0
        t_ref += time.perf_counter() - t1
        true_err = np.abs(res - ref).max() / np.abs(ref).max()
        raw = np.abs(sur.predict(g.rho, f) - ref).max() / np.abs(ref).max()
        out.append((f, used, err, true_err, raw))
        if used:
            assert true_err <= 1.5 * sur.tol, (f, err, true_err)
        else:
            assert true_err == 0.0
        # the judge's estimate (at radii it did not fit) tracks the actual error
        if used:
            assert 0.5 * true_err <= err <= 2 * true_err, (f, err, true_err)
        g.close()
        g_ref.close()
    print("(f, used, judged error, error vs Sommerfeld, network alone):", out)
    print(f"Sommerfeld radii per table: {2 * sur.ncheck - 1} with the network, {g_ref.rho.size} without; "
          f"table time with / without: {t_sur / 4 * 1e3:.2f} / {t_ref / 4 * 1e3:.2f} ms")
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
