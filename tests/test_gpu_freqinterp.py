"""GPU tests of the frequency interpolation (m25_interp_*, FreqInterp):
the store / interpolation kernels against oracle/freqinterp.py, and
interpolated sweeps against mom25d's own FreqInterp sweeps
(tests/golden/*_interp.npz)."""

import ctypes as C

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import engine as E
from mom25d_gb300 import workloads
from mom25d_gb300.freqinterp import FreqInterp
from mom25d_gb300.solver import Solver
from oracle import freqinterp as OI

from conftest import golden

pytestmark = pytest.mark.gpu

CASES = {"tee": {}, "shunt_via": dict(step=1.5e9)}


@pytest.mark.parametrize("single", [0, 1])
def test_interp_kernels_match_oracle(gpu, single):
    """Anchor transform and Lagrange interpolation on random matrices with via
    unknowns (rows and columns >= nb), complex128 and complex64 anchors."""
    rng = np.random.default_rng(7)
    n, nb = 301, 280
    pos = rng.uniform(-0.02, 0.02, (n, 3))
    fa = np.array([1e9, 2e9, 3e9, 4e9])
    ke = lambda f: 1.7 * 2 * np.pi * f / 299792458.0  # noqa: E731
    Zs = [rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) for _ in fa]
    ctx = E.Context(0)
    h = C.c_void_p()
    E.check(ctx.lib.m25_interp_create(ctx.h, n, nb, E.ptr(pos), 4, single, C.byref(h)))
    ip = E.Handle(ctx, h, ctx.lib.m25_interp_destroy)
    for s, (f, Z) in enumerate(zip(fa, Zs)):
        Zc = np.ascontiguousarray(Z)
        E.check(ctx.lib.m25_interp_store(ip.h, s, Zc.ctypes.data, n, E.M25_ON_HOST, f, ke(f)))
    f = 2.4e9
    L = OI.weights(fa, f, [0, 1, 2, 3])
    slots = np.array([0, 1, 2, 3], np.int32)
    out = np.empty((n, n), complex)
    E.check(ctx.lib.m25_interp_eval(ip.h, 4, E.ptr(slots, C.c_int32), E.ptr(L), f, ke(f), out.ctypes.data, n,
                                    E.M25_ON_HOST))
    dt = np.complex64 if single else np.complex128
    Ws = [OI.store(Z, pos, nb, fi, ke(fi), dt) for fi, Z in zip(fa, Zs)]
    ref = OI.evaluate(Ws, L, pos, nb, f, ke(f))
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < (1e-6 if single else 1e-13), err
    ip.close()
    ctx.close()


@pytest.mark.parametrize("name", list(CASES))
def test_interpolated_sweep_matches_reference(gpu, name):
    """Solver.sweep with a FreqInterp: anchors, interpolated Z at the
    off-anchor frequency and S of mom25d's interpolated sweep (fp64 path)."""
    g = golden(name + "_interp")
    lay, st, m, _ = workloads.build(G, name)
    sol = Solver(m, st, verbose=False)
    ip = FreqInterp(**CASES[name]).setup(sol, g["freqs"])
    np.testing.assert_array_equal(ip.anchors, g["anchors"])
    Zi = ip.impedance(float(g["f_mid"]))
    rows = g["Z_rows_idx"]
    assert np.abs(Zi[rows] - g["Zi_rows"]).max() <= 1e-10 * np.abs(g["Zi_rows"]).max()
    ip.close()
    r = sol.sweep(g["freqs"], interp=FreqInterp(**CASES[name]))
    assert r.info["interp_fills"] == len(g["anchors"])
    assert np.abs(r.S - g["S"]).max() < 1e-6
    sol.close()


def test_interpolated_sweep_auto_and_mixed(gpu):
    """interp="auto" picks the interpolation on the tee (37 frequencies, 6
    anchors) as mom25d does; the mixed precision within 1e-5 of mom25d."""
    g = golden("tee_interp")
    lay, st, m, _ = workloads.build(G, "tee")
    sol = Solver(m, st, verbose=False, precision="mixed")
    r = sol.sweep(g["freqs"], interp="auto")
    assert r.info["interp_anchors"] == len(g["anchors"])
    assert np.abs(r.S - g["S"]).max() < 1e-5
    sol.close()


def test_resident_anchors_on_concurrent_workers(gpu):
    """Resident anchors (all filled first) read by four workers give the S of
    the windowed single-worker sweep (the same anchors, the same kernels)."""
    g = golden("tee_interp")
    lay, st, m, _ = workloads.build(G, "tee")
    sol = Solver(m, st, verbose=False)
    r1 = sol.sweep(g["freqs"], interp=FreqInterp(resident=False))
    assert r1.info["workers"] == 1
    r4 = sol.sweep(g["freqs"], interp=FreqInterp(resident=True), workers=4)
    assert r4.info["workers"] == 4 and r4.info["interp_fills"] == len(g["anchors"])
    assert np.abs(r4.S - r1.S).max() < 1e-12
    sol.close()


def test_complex64_anchors(gpu):
    """complex64 anchors (the reference's choice when complex128 would not
    fit) stay within its stated ~5e-5 of the complex128 interpolation at low
    frequency (bound 5e-4 over the tee's band)."""
    g = golden("tee_interp")
    lay, st, m, _ = workloads.build(G, "tee")
    sol = Solver(m, st, verbose=False)
    r = sol.sweep(g["freqs"], interp=FreqInterp(dtype=np.complex64))
    assert np.abs(r.S - g["S"]).max() < 5e-4
    sol.close()
