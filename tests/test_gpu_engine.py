"""GPU parity tests: the CUDA engine against the CPU oracle and against
fixtures made by running mom25d (tests/golden). Tolerances are written in
each test; fp64 stages must agree to rounding, the mixed path to 1e-5 in S.
"""

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Solver, dense_solve
from oracle import sweep as O

from conftest import fp64_tol, gamma_floor, golden

pytestmark = pytest.mark.gpu


def build(name, **kw):
    lay, st, m, freqs = workloads.build(G, name, **kw)
    return lay, st, m, freqs


@pytest.fixture(scope="module")
def line(gpu):
    lay, st, m, freqs = build("line")
    sol = Solver(m, st, verbose=False)
    yield sol, O.Sweep(m, st)
    sol.close()


@pytest.fixture(scope="module")
def shunt(gpu):
    lay, st, m, freqs = build("shunt_via")
    sol = Solver(m, st, verbose=False)
    yield sol, O.Sweep(m, st)
    sol.close()


# ---------------------------------------------------------------- Green's tables
@pytest.mark.parametrize("f", [0.5e9, 7e9, 20e9])
def test_slab_tables_match_oracle(line, f):
    sol, ref = line
    g = sol.greens(f)
    S, c, coef = g.tables()
    k = ref.kernels(f)
    np.testing.assert_array_equal(g.rho, k.rho_tab)
    for m, tab in enumerate((k.SA, k.SV, k.SW)):
        err = np.abs(S[m, 0, 0] - tab).max() / np.abs(tab).max()
        assert err < 1e-12, (m, err)
    # cubic coefficients against scipy's not-a-knot spline (the cubic term
    # carries the cancellation of the slope system: 1e-8), and the spline
    # values between the nodes (1e-12)
    c_ref = k.pair().spl.c  # (4, n-1, 2)
    for m in range(2):
        err = np.abs(coef[0, :, :, m] - c_ref[:, :, m].T).max() / np.abs(c_ref[:, :, m]).max()
        assert err < 1e-8, (m, err)
        mid = 0.5 * (g.rho[1:] + g.rho[:-1])
        dx = (mid - g.rho[:-1])[:, None] ** np.arange(3, -1, -1)[None]
        val = np.sum(coef[0, :, :, m] * dx, 1)
        ref_val = k.pair().spl(mid)[:, m]
        assert np.abs(val - ref_val).max() < 1e-12 * np.abs(ref_val).max()
    np.testing.assert_allclose(c[1, 0, 0], k.cv, rtol=1e-15)
    g.close()


@pytest.mark.parametrize("name", ["via", "stripline"])
def test_layered_tables_match_oracle(gpu, name):
    """Two levels with air above (via transition), and one level under a PEC
    cover (stripline)."""
    lay, st, m, _ = build(name)
    sol = Solver(m, st, verbose=False)
    ref = O.Sweep(m, st)
    f = 10e9
    g = sol.greens(f)
    S, c, coef = g.tables()
    k = ref.kernels(f)
    np.testing.assert_array_equal(g.rho, k.rho_tab)
    L = len(m.layer_names)
    for i in range(L):
        for j in range(L):
            p = k.pair(i, j)
            np.testing.assert_allclose(c[:, i, j], [p.cA, p.cV, p.cW], rtol=1e-12, atol=1e-14)
            for mm, tab in enumerate((p.spl(g.rho)[:, 0], p.spl(g.rho)[:, 1], p.splw(g.rho))):
                err = np.abs(S[mm, i, j] - tab).max() / np.abs(tab).max()
                assert err < 1e-11, (i, j, mm, err)
    g.close()
    sol.close()


# ------------------------------------------------------------------------ fill
@pytest.mark.parametrize("f", [2e9, 7e9])
def test_fill_fp64_matches_oracle(line, f):
    sol, ref = line
    Z = sol.impedance(f)
    Zo = ref.impedance(f)
    assert np.abs(Z - Zo).max() <= 1e-12 * np.abs(Zo).max()
    assert np.abs(Z - Z.T).max() <= 1e-15 * np.abs(Z).max()  # symmetrised in the gather


def test_fill_with_via_matches_oracle(shunt):
    sol, ref = shunt
    f = 3e9
    Z = sol.impedance(f)
    Zo = ref.impedance(f)
    scale = np.abs(Zo).max()
    nb = sol.mesh.n_basis
    assert np.abs(Z[:nb, :nb] - Zo[:nb, :nb]).max() <= 1e-12 * scale
    # via rows and the via-via block
    assert np.abs(Z[nb:] - Zo[nb:]).max() <= 1e-11 * np.abs(Zo[nb:]).max()


@pytest.mark.parametrize("name", ["tee", "via", "bandpass_0", "lpf"])
def test_fill_fp64_matches_reference_rows(gpu, name):
    g = golden(name)
    base = "bandpass" if name.startswith("bandpass") else name
    kw = {"k": 0} if name.startswith("bandpass") else {}
    lay, st, m, _ = build(base, **kw)
    sol = Solver(m, st, verbose=False)
    Z = sol.impedance(float(g["f0"]))
    rows = g["Z_rows_idx"]
    assert np.abs(Z[rows] - g["Z_rows"]).max() <= 1e-11 * np.abs(g["Z_rows"]).max()
    assert np.abs(np.diag(Z) - g["Z_diag"]).max() <= 1e-11 * np.abs(g["Z_diag"]).max()
    sol.close()


def test_fill_mixed_close_to_fp64(line):
    sol, _ = line
    f = 7e9
    Z64 = sol.impedance(f, precision="fp64")
    Z32 = sol.impedance(f, precision="mixed_fill32")
    assert Z32.dtype == np.complex64
    assert np.abs(Z32 - Z64).max() <= 3e-6 * np.abs(Z64).max()


def test_fill_mixed_close_to_fp64_fill(line):
    """precision 'mixed' keeps the near pairs' singular parts and sums in fp64
    and evaluates their smooth parts and all mid / far pairs in fp32: a
    complex128 Z within 1e-6 of the fp64 fill (relative to max |Z|)."""
    sol, _ = line
    for f in (2e9, 7e9):
        Z64 = sol.impedance(f, precision="fp64")
        Zm = sol.impedance(f, precision="mixed")
        assert Zm.dtype == np.complex128
        err = np.abs(Zm - Z64).max() / np.abs(Z64).max()
        assert 0 < err < 1e-6, err


# ----------------------------------------------------------------------- solve
@pytest.mark.parametrize("n", [1, 2, 63, 65, 130, 700])
def test_dense_solve_fp64_vs_lapack(gpu, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A += n * np.eye(n) * (0.3 + 0.1j)
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    X = dense_solve(A, B)
    Xr = np.linalg.solve(A, B)
    assert np.abs(X - Xr).max() <= 1e-12 * np.abs(Xr).max()


def test_dense_solve_needs_pivoting(gpu):
    # zero leading diagonal: partial pivoting is required
    rng = np.random.default_rng(3)
    n = 200
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A[0, 0] = 0
    A[:5, :5] = 0
    B = rng.standard_normal((n, 1)) + 0j
    X = dense_solve(A, B)
    assert np.abs(A @ X - B).max() <= 1e-10 * np.abs(B).max()


@pytest.mark.parametrize("n", [64, 300, 1000])
def test_dense_solve_mixed_refines_to_fp64(gpu, n):
    rng = np.random.default_rng(n + 1)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A += 3 * np.sqrt(n) * np.eye(n)
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    X = dense_solve(A, B, precision="mixed", tol=1e-15)
    Xr = np.linalg.solve(A, B)
    assert np.abs(X - Xr).max() <= 1e-12 * np.abs(Xr).max()


def test_dense_solve_mixed_ill_conditioned(gpu):
    """cond ~1e7 (cond u32 ~ 1, where classical refinement with a complex64 LU
    stalls): GMRES refinement reaches the fp64 solution's accuracy."""
    rng = np.random.default_rng(7)
    n = 400
    U, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    Vm, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    s = np.logspace(0, -7, n)
    A = (U * s) @ Vm.conj().T
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    X = dense_solve(A, B, precision="mixed")
    Xr = np.linalg.solve(A, B)
    assert np.abs(X - Xr).max() <= 1e-5 * np.abs(Xr).max()
    r = A @ X - B
    assert np.linalg.norm(r) <= 1e-13 * (np.abs(A).sum(1).max() * np.linalg.norm(X) + np.linalg.norm(B))


def test_singular_matrix_raises(gpu):
    A = np.zeros((10, 10), complex)
    with pytest.raises(RuntimeError):
        dense_solve(A, np.ones((10, 1)))


# --------------------------------------------------------------------- sweeps
def test_line_sweep_fp64_matches_reference(line):
    sol, ref = line
    g = golden("line")
    r = sol.sweep(g["freqs"])
    # three times the floor of mom25d's own Nelder-Mead wave fit (conftest.fit_floor)
    assert np.abs(r.S - g["S"]).max() < fp64_tol("line")
    assert np.abs(r.gamma - g["gamma"]).max() < 1e-6 * np.abs(g["gamma"]).max()
    assert np.abs(r.z0 - g["z0"]).max() < 1e-6 * np.abs(g["z0"]).max()
    assert np.abs(r.renormalize(50) - g["S50"]).max() < fp64_tol("line")


def test_deembed_stages_match_oracle(line):
    sol, ref = line
    f = 7e9
    S, z0, gam, zl, res, x, _ = sol.point(f, keep_currents=True)
    q, phi, I, V = sol.last_deembed()
    k = ref.kernels(f)
    Zo = ref.impedance(f, k)
    xo = O.dense_solve(Zo, ref.excitations())
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    qo = O.charges(sol.mesh, x, 2 * np.pi * f)
    assert np.abs(q - qo).max() <= 1e-12 * np.abs(qo).max()
    pts = np.concatenate([pm.vpts for pm in ref.pm])
    phio = O.line_voltage(sol.mesh, k, q, pts, "top")
    assert np.abs(phi - phio).max() <= 1e-11 * np.abs(phio).max()
    Io = np.concatenate([pm.currents(x) for pm in ref.pm])
    assert np.abs(I - Io).max() <= 1e-13 * np.abs(Io).max()
    So = ref.deembed(f, k, x, q)[0]
    assert np.abs(S - So).max() < fp64_tol("line")


def test_shunt_via_sweep_matches_reference(shunt):
    sol, _ = shunt
    g = golden("shunt_via")
    r = sol.sweep(g["freqs"])
    assert np.abs(r.S - g["S"]).max() < fp64_tol("shunt_via")


def test_tee_sweep_matches_reference(gpu):
    g = golden("tee")
    lay, st, m, _ = build("tee")
    idx = [0, 12, 24, 36]
    # fp64 and mixed (fp64 singular parts of the fill, complex64 LU + fp64
    # GMRES refinement) are held to the reference's fit floor; the all-fp32 fill loses the
    # low-frequency scalar-potential cancellation (~1e-4 at 1 GHz)
    for prec, tol in (("fp64", fp64_tol("tee")), ("mixed", 1e-6), ("mixed_fill32", 3e-4)):
        sol = Solver(m, st, verbose=False, precision=prec)
        r = sol.sweep(g["freqs"][idx])
        assert np.abs(r.S - g["S"][idx]).max() < tol, prec
        sol.close()


def test_lpf_headline_workload_matches_reference(gpu):
    """N = 5943 at the fixture's frequencies (11 of the 101, 0.5 to 8 GHz):
    fp64 within three fit floors, mixed within 1e-5 (on 4 workers, as the
    bench runs it)."""
    g = golden("lpf")
    lay, st, m, _ = build("lpf")
    for prec, tol, workers in (("fp64", fp64_tol("lpf"), 1), ("mixed", 1e-5, 4)):
        sol = Solver(m, st, verbose=False, precision=prec)
        r = sol.sweep(g["freqs"], workers=workers)
        dS = np.abs(r.S - g["S"]).max(axis=(1, 2))
        print(prec, "max |dS| per frequency", dS)
        assert dS.max() < tol, (prec, dS)
        sol.close()


@pytest.mark.parametrize("name", ["shunt_via", "via"])
def test_mixed_sweep_with_vias_matches_reference(gpu, name):
    """The mixed precision with via unknowns (the fill writes a complex128 Z,
    split for the complex64 LU and the refinement) within 1e-5 of mom25d."""
    g = golden(name)
    lay, st, m, _ = build(name)
    sol = Solver(m, st, verbose=False, precision="mixed")
    r = sol.sweep(g["freqs"])
    assert np.abs(r.S - g["S"]).max() < 1e-5
    sol.close()


@pytest.mark.parametrize("name", ["line", "via"])
def test_mixed_point_falls_back_to_fp64(gpu, name):
    """A refinement target the complex64 LU cannot reach (1e-30 in 8 steps)
    sends each point through the fp64 fill and LU: the same S as the fp64
    sweep, refine_steps -1 and every frequency listed as a fallback."""
    g = golden(name)
    lay, st, m, _ = build(name)
    ref = Solver(m, st, verbose=False, precision="fp64")
    r64 = ref.sweep(g["freqs"])
    ref.close()
    sol = Solver(m, st, verbose=False, precision="mixed", refine_tol=1e-30, max_refine=8)
    r = sol.sweep(g["freqs"])
    sol.close()
    assert r.info["refine_steps"] == [-1] * len(g["freqs"])
    assert r.info["fp64_fallback"] == [float(f) for f in g["freqs"]]
    assert np.abs(r.S - r64.S).max() < 1e-12


def test_via_transition_sweep_matches_reference(gpu):
    g = golden("via")
    lay, st, m, _ = build("via")
    sol = Solver(m, st, verbose=False)
    r = sol.sweep(g["freqs"])
    assert np.abs(r.S - g["S"]).max() < fp64_tol("via")
    sol.close()


def test_bad_mesh_is_rejected(gpu):
    lay, st, m, _ = build("line")
    m.tri_basis = m.tri_basis.copy()
    m.tri_basis[0, 0] = 10 ** 6
    sol = Solver(m, st, verbose=False)
    with pytest.raises(ValueError):
        sol.geometry()
    sol.close()


# ------------------------------------------------ LU factors, tensor cores
def _lu_reconstruct(F, piv):
    n = F.shape[0]
    L = np.tril(F, -1) + np.eye(n)
    U = np.triu(F)
    perm = np.arange(n)
    for i, p in enumerate(piv):
        perm[[i, p]] = perm[[p, i]]
    return L @ U, perm


@pytest.mark.parametrize("n", [300, 1000, 1280, 1302, 1344])
def test_lu_complex64_tensor_cores_reconstruct(gpu, n):
    """complex64 LU with tcgen05 3xTF32 trailing updates: P L U = A to fp32
    accuracy. The tensor cores' fp32 accumulation rounds differently from
    SIMT fused multiply-adds, so the bound against the SIMT factorisation is
    a factor of 16; a wrong tile or operand split gives O(1) errors. (The
    pivot sequences may part where two candidates tie to rounding, so the
    factors themselves are not compared.) The orders end the blocks of 128
    columns in each way: a second panel of 44, 40 or 22 columns, a full block
    with no trailing matrix (1280) and a single last panel (1344)."""
    import ctypes as C

    from mom25d_gb300 import engine as E

    ctx = E.Context(0)
    rng = np.random.default_rng(n)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    errs = {}
    for flags in (0, E.M25_LU_NO_TENSOR_CORES):
        F = A.copy()
        piv = np.zeros(n, np.int32)
        info = np.zeros(1, np.int32)
        E.check(ctx.lib.m25_lu_factor(ctx.h, n, E.M25_MIXED, F.ctypes.data, n, E.ptr(piv, C.c_int32), E.M25_ON_HOST,
                                      flags, E.ptr(info, C.c_int32)))
        LU, perm = _lu_reconstruct(F.astype(np.complex128), piv)
        err = np.abs(LU - A[perm]).max() / np.abs(A).max()
        assert info[0] == 0
        assert err < 5e-5 * np.sqrt(n / 300), (flags, err)
        errs[flags] = err
    print("P L U - A, tensor cores / SIMT:", errs)
    assert errs[0] <= 16 * errs[E.M25_LU_NO_TENSOR_CORES], errs
    ctx.close()


@pytest.mark.parametrize("n", [40, 64, 65, 127, 128, 129, 193, 257, 511])
def test_lu_complex64_tensor_cores_small_and_odd_orders(gpu, n):
    """The blocked tensor-core LU on small and odd orders, rows padded to an
    even length (16-byte rows, as the mixed solve stores its LU): a single
    panel, a block without a second panel's full width, blocks that end
    exactly, and odd trailing sizes of the rank-64 and rank-128 updates."""
    import ctypes as C

    from mom25d_gb300 import engine as E

    ctx = E.Context(0)
    rng = np.random.default_rng(1000 + n)
    lda = n + (n & 1)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    F = np.zeros((n, lda), np.complex64)
    F[:, :n] = A
    piv = np.zeros(n, np.int32)
    info = np.zeros(1, np.int32)
    E.check(ctx.lib.m25_lu_factor(ctx.h, n, E.M25_MIXED, F.ctypes.data, lda, E.ptr(piv, C.c_int32), E.M25_ON_HOST,
                                  0, E.ptr(info, C.c_int32)))
    LU, perm = _lu_reconstruct(F[:, :n].astype(np.complex128), piv)
    err = np.abs(LU - A[perm]).max() / np.abs(A).max()
    assert info[0] == 0
    assert err < 5e-5, err
    ctx.close()


@pytest.mark.parametrize("tile_n", [128, 192])
@pytest.mark.parametrize("n", [257, 1302])
def test_lu_complex64_tensor_cores_each_tile_shape(gpu, n, tile_n):
    """Every update of the factorisation in tiles of 128 or of 192 real
    columns (the context's tile-shape knob, which otherwise picks 128 only for
    the narrow updates): P L U = A to fp32 accuracy either way."""
    import ctypes as C

    from mom25d_gb300 import engine as E

    ctx = E.Context(0)
    E.check(ctx.lib.m25_ctx_set_tuning(ctx.h, 0, 0, 0, tile_n))
    with pytest.raises(ValueError):
        E.check(ctx.lib.m25_ctx_set_tuning(ctx.h, 0, 0, 0, 96))
    rng = np.random.default_rng(2000 + n)
    lda = n + (n & 1)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    F = np.zeros((n, lda), np.complex64)
    F[:, :n] = A
    piv = np.zeros(n, np.int32)
    info = np.zeros(1, np.int32)
    E.check(ctx.lib.m25_lu_factor(ctx.h, n, E.M25_MIXED, F.ctypes.data, lda, E.ptr(piv, C.c_int32), E.M25_ON_HOST,
                                  0, E.ptr(info, C.c_int32)))
    LU, perm = _lu_reconstruct(F[:, :n].astype(np.complex128), piv)
    err = np.abs(LU - A[perm]).max() / np.abs(A).max()
    assert info[0] == 0
    assert err < 5e-5 * np.sqrt(max(n, 300) / 300), err
    ctx.close()


# ------------------------------------------------------- concurrent points
def test_sweep_workers_match_one_worker(gpu):
    """Points in flight on separate engine contexts give the results of the
    one-at-a-time sweep (every stage is deterministic)."""
    lay, st, m, freqs = build("line")
    f = np.linspace(2e9, 14e9, 5)
    s1 = Solver(m, st, verbose=False, precision="mixed")
    r1 = s1.sweep(f)
    s1.close()
    s2 = Solver(m, st, verbose=False, precision="mixed")
    r2 = s2.sweep(f, workers=3)
    s2.close()
    assert r2.info["workers"] == 3
    for a, b in ((r1.S, r2.S), (r1.gamma, r2.gamma), (r1.z0, r2.z0), (r1.fit_residual, r2.fit_residual)):
        np.testing.assert_allclose(a, b, rtol=1e-15, atol=0)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_lossless_line_sweep_matches_reference(gpu, prec):
    """Lossless substrate: the device fit searches beta alone (gamma = j beta)
    by Brent's bounded method as mom25d does (solver.py:654-662); gamma
    purely imaginary and equal to mom25d's, S within three fit floors
    (fp64) or 1e-5 (mixed), no bound warning on this line, and the fit's
    iteration counts reported per group."""
    import ctypes as C
    import warnings

    from mom25d_gb300 import engine as E

    g = golden("line_lossless")
    lay, st, m, _ = build("line_lossless")
    sol = Solver(m, st, verbose=False, precision=prec)
    try:
        with warnings.catch_warnings():
            warnings.simplefilter("error", RuntimeWarning)
            r = sol.sweep(g["freqs"])
        assert np.all(r.gamma.real == 0)
        dS = np.abs(r.S - g["S"]).max(axis=(1, 2))
        dg = (np.abs(r.gamma - g["gamma"]) / np.abs(g["gamma"])).max(axis=1)
        print(prec, "max |dS|", dS, "gamma", dg)
        # where the line is electrically short (2 GHz) the fit's objective is
        # flat in beta and the search stops anywhere within the floor
        if prec == "fp64":
            assert dg.max() < 3 * gamma_floor("line_lossless")
        tol = fp64_tol("line_lossless") if prec == "fp64" else 1e-5
        assert dS.max() < tol
        it = np.zeros(len(sol.groups), np.int32)
        E.check(sol.ctx.lib.m25_deembed_fit_info(sol.port_data().h, E.ptr(it, C.c_int32)))
        assert np.all(it > 1) and np.all(it < 500), it
    finally:
        sol.close()
