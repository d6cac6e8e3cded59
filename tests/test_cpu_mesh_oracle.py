"""CPU tests: the grid mesher and the oracle against fixtures generated by
running mom25d itself (tests/golden/make_golden.py)."""

import hashlib

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from oracle import kernels as K
from oracle import sweep as O

from conftest import golden


def mesh_digest(m):
    h = hashlib.sha256()
    for a in (m.nodes, m.tris, m.tri_basis, m.tri_sign, m.edge_len, m.tri_layer):
        h.update(np.ascontiguousarray(a).tobytes())
    for s in m.via_segments:
        h.update(repr((s["via"], s["top"], s["bottom"])).encode())
        for k in ("top_tris", "bottom_tris"):
            if s[k] is not None:
                h.update(np.asarray(s[k], np.int64).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", ["line", "line_lossless", "shunt_via", "tee", "via", "lpf", "bandpass_0",
                                  "bandpass_3", "bandpass_7", "bandpass_11", "bandpass_14", "gcpw", "stripline"])
def test_mesh_identical_to_reference(name):
    import os

    from conftest import GOLDEN

    if not os.path.exists(os.path.join(GOLDEN, name + ".npz")):
        pytest.skip(f"no fixture {name}")
    g = golden(name)
    base = "bandpass" if name.startswith("bandpass") else name
    kw = {"k": int(name.split("_")[1])} if name.startswith("bandpass") else {}
    lay, st, m, _ = workloads.build(G, base, **kw)
    stack = st if hasattr(st, "layers") else st.to_stackup()
    m.assign_levels(sorted(m.layer_names, key=stack.level_z))
    assert m.n_unknowns == int(g["N"]) and len(m.tris) == int(g["Nt"])
    assert mesh_digest(m) == str(g["mesh_sha"])


def test_potential_integrals_known_answers():
    g = golden("kernels")
    for d in (0.0, 0.254e-3):
        I0, I1 = K.potential_integrals(g["V"], g["r"], d)
        np.testing.assert_allclose(I0, g[f"I0_{d:g}"], rtol=1e-13, atol=1e-20)
        np.testing.assert_allclose(I1, g[f"I1_{d:g}"], rtol=1e-13, atol=1e-20)


def test_potential_integrals_vs_brute_force():
    """Closed form against a fine midpoint rule (the reference's own check, 2e-3)."""
    V = np.array([[[0, 0], [1.0, 0.2], [0.3, 0.9]]])
    r = np.array([[0.4, 0.3], [2.0, -0.5], [0.5, 0.1]])
    I0, I1 = K.potential_integrals(V, r)
    n = 600
    u, v = np.meshgrid((np.arange(n) + 0.5) / n, (np.arange(n) + 0.5) / n)
    msk = u + v < 1
    e1, e2 = V[0, 1] - V[0, 0], V[0, 2] - V[0, 0]
    P = V[0, 0] + u[msk, None] * e1 + v[msk, None] * e2
    w = 0.5 * abs(e1[0] * e2[1] - e1[1] * e2[0]) / msk.sum()
    for k in range(len(r)):
        d = P - r[k]
        R = np.hypot(d[:, 0], d[:, 1])
        assert I0[0, k] == pytest.approx((w / R).sum(), rel=4e-3)


def test_slab_kernels_match_reference():
    g = golden("kernels")
    s = K.SlabKernels(5e9, 3.55, 0.508e-3, 0.0027, rho_max=0.03, zs_ground=0.02 + 0.02j)
    np.testing.assert_array_equal(s.rho_tab, g["slab_rho_tab"])
    for a, b in ((s.SA, g["slab_SA"]), (s.SV, g["slab_SV"]), (s.SW, g["slab_SW"])):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    R = g["slab_R"]
    p = s.pair()
    for a, b in ((p.gA(R), g["slab_gA"]), (p.gV(R), g["slab_gV"]), (p.gW(R), g["slab_gW"])):
        assert np.max(np.abs(a - b) * 4 * np.pi * R) < 1e-12


def test_air_slab_equals_images():
    """eps_r = 1 over ground: source plus negative image (the reference's test, 1e-6)."""
    h = 0.5e-3
    for f in (1e9, 10e9):
        s = K.SlabKernels(f, 1.0, h, rho_max=0.06)
        k = s.k0
        R = np.array([1e-5, 1e-4, 5e-4, 2e-3, 1e-2, 0.03, 0.06])
        R2 = np.sqrt(R ** 2 + 4 * h ** 2)
        exact = (np.exp(-1j * k * R) / R - np.exp(-1j * k * R2) / R2) / (4 * np.pi)
        p = s.pair()
        assert np.max(np.abs(p.gA(R) - exact) * 4 * np.pi * R) < 1e-6
        assert np.max(np.abs(p.gV(R) - exact) * 4 * np.pi * R) < 1e-6


def test_layered_one_layer_equals_slab():
    f = 3e9
    s = K.SlabKernels(f, 3.55, 0.508e-3, 0.002, rho_max=0.04)
    lk = K.LayeredKernels(f, [(0.508e-3, 3.55, 0.002)], [1], [0.508e-3], rho_max=0.04)
    R = np.array([1e-5, 1e-4, 5e-4, 2e-3, 1e-2, 0.03])
    for a, b in ((lk.pair(0, 0).gA(R), s.pair().gA(R)), (lk.pair(0, 0).gV(R), s.pair().gV(R)),
                 (lk.pair(0, 0).gW(R), s.pair().gW(R))):
        assert np.max(np.abs(a - b) * 4 * np.pi * R) < 1e-12


def test_via_inductance_known_answer():
    g = golden("kernels")
    vias = [G.Via((0, 0), 0.3e-3), G.Via((1e-3, 0.2e-3), 0.2e-3)]
    spans = np.array([[0.0, 0.508e-3], [0.0, 0.508e-3]])
    L = O.via_block_L(vias, spans, (0.0, 0.508e-3))
    np.testing.assert_allclose(L, g["via_L"], rtol=1e-13)


@pytest.mark.parametrize("name", ["tee", "bandpass_0", "via"])
def test_oracle_fill_matches_reference_rows(name):
    """The oracle's fill against mom25d's Z rows and diagonal on the larger
    cases: a tee, a band-pass variant and the two-level via transition (its
    via row, whose entries are small against the RWG self terms, on its own
    scale: the levels must be ordered by height as Solver does)."""
    g = golden(name)
    base = name.split("_")[0]
    lay, st, m, _ = workloads.build(G, base, **({"k": 0} if base == "bandpass" else {}))
    sw = O.Sweep(m, st)
    Z = sw.impedance(float(g["f0"]))
    rows = g["Z_rows_idx"]
    assert np.abs(Z[rows] - g["Z_rows"]).max() <= 1e-13 * np.abs(g["Z_rows"]).max()
    assert np.abs(np.diag(Z) - g["Z_diag"]).max() <= 1e-13 * np.abs(g["Z_diag"]).max()
    for k, r in enumerate(rows):
        if r >= m.n_basis:  # via unknowns
            assert np.abs(Z[r] - g["Z_rows"][k]).max() <= 1e-13 * np.abs(g["Z_rows"][k]).max()


@pytest.mark.parametrize("name", ["line", "shunt_via"])
def test_oracle_fill_and_sweep_match_reference(name):
    g = golden(name)
    lay, st, m, _ = workloads.build(G, name)
    sw = O.Sweep(m, st)
    f0 = float(g["f0"])
    Z = sw.impedance(f0)
    if "Z" in g.files:
        assert np.abs(Z - g["Z"]).max() <= 1e-13 * np.abs(g["Z"]).max()
    else:
        rows = g["Z_rows_idx"]
        assert np.abs(Z[rows] - g["Z_rows"]).max() <= 1e-13 * np.abs(g["Z_rows"]).max()
        assert np.abs(np.diag(Z) - g["Z_diag"]).max() <= 1e-13 * np.abs(g["Z_diag"]).max()
    x = O.dense_solve(Z.copy(), sw.excitations())
    # the currents agree to ~cond(Z) x 1e-16 (cond ~1e7 with the shunt via)
    assert np.abs(x - g["x"]).max() <= 1e-8 * np.abs(g["x"]).max()
    S, z0, gam, zl, res = sw.sweep(g["freqs"])
    # the reference's own Nelder-Mead wave fit moves gamma by ~4e-8 under 1e-15
    # perturbations of its inputs: S agrees to that floor, not to 1e-9
    assert np.abs(S - g["S"]).max() < 1e-6
    assert np.abs(gam - g["gamma"]).max() < 1e-6 * np.abs(g["gamma"]).max()


def test_oracle_lossless_sweep_matches_reference():
    """A lossless substrate takes mom25d's bounded search over beta
    (gamma = j beta, Engine/mom25d/solver.py:654-662): the oracle's sweep
    gives mom25d's gamma (purely imaginary) and S (lossless line)."""
    from conftest import fp64_tol, gamma_floor

    g = golden("line_lossless")
    lay, st, m, _ = workloads.build(G, "line_lossless")
    assert mesh_digest(m) == str(g["mesh_sha"])
    sw = O.Sweep(m, st)
    S, z0, gam, zl, res = sw.sweep(g["freqs"])
    assert np.all(gam.real == 0) and np.all(g["gamma"].real == 0)
    # where the line is short (2 GHz) the objective is flat in beta: even
    # mom25d's own beta moves within the floor with its BLAS thread count
    assert (np.abs(gam - g["gamma"]) / np.abs(g["gamma"])).max() < 3 * gamma_floor("line_lossless")
    assert np.abs(S - g["S"]).max() < fp64_tol("line_lossless")


def test_stripline_tables_equal_reference():
    """The oracle's layered kernels under a PEC cover (a shorted top layer,
    V = 0 on the cover; mom25d/layered.py:257-275) against mom25d's own
    tables of the stripline stack (tests/golden/stripline.npz): the leading
    coefficients and the smooth parts' spline values at the radii."""
    import os

    from conftest import GOLDEN

    if not os.path.exists(os.path.join(GOLDEN, "stripline.npz")):
        pytest.skip("no stripline fixture")
    g = golden("stripline")
    lay, st, m, _ = workloads.build(G, "stripline")
    zl = [st.level_z(n) for n in m.layer_names]
    lk = K.LayeredKernels(float(g["f0"]), [(d.t, d.eps_r, d.tand) for d in st.layers],
                          [st.metals[n] for n in m.layer_names], zl, rho_max=float(g["rho_max"]), top="pec")
    np.testing.assert_array_equal(lk.rho_tab, g["rho_tab"])
    p = lk.pairs[0, 0]
    np.testing.assert_allclose([p.cA, p.cV, p.cW], g["pair00_c"], rtol=1e-12, atol=1e-15)
    # mom25d's spline coefficients evaluated at the knots: the tabulated smooth parts
    c = g["pair00_spl_c"]  # (4, n - 1, 2) PPoly coefficients of [S_A, S_V]
    ref_SA, ref_SV = c[3, :, 0], c[3, :, 1]
    mine = p.spl(g["rho_tab"][:-1])
    for k, ref in ((0, ref_SA), (1, ref_SV)):
        assert np.abs(mine[:, k] - ref).max() <= 1e-10 * np.abs(ref).max(), k
