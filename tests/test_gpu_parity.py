"""Parity of every stage of the sweep point against fixtures made by running
mom25d itself (tests/golden, make_golden.py), on every workload that has one.

Bars:
- every stage before the wave fit (currents x, charges q, line voltages phi,
  cut currents I and cut voltages V), fp64 path: 1e-9 relative to the
  largest entry, or three times that stage's conditioning floor where that is
  larger. The floors (tests/golden/x_floor.npz, made by running mom25d) are
  how far mom25d's own stage moves when its Z is perturbed by 1e-13 relative,
  the level at which the two fills agree: x by 5e-10 to 3e-7 (the part of x
  that moves carries almost no charge), q, phi, I and V by far less, except
  on the ill-conditioned N = 25284 grounded CPW at 1 GHz;
- S of the fp64 path: three times the floor of mom25d's own wave fit
  (conftest.fit_floor: 8e-9 to 6e-8 by workload), or three times the spread
  of mom25d's S under the same Z perturbation where that is larger;
- S of the mixed path: 1e-5.
"""

import os

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Solver

from conftest import GOLDEN, fp64_tol, golden

pytestmark = pytest.mark.gpu

STAGE_TOL = 1e-9


def stage_floor(name, stage):
    """How far mom25d's own value of a stage moves under a 1e-13 relative
    perturbation of its Z (0 when not measured)."""
    path = os.path.join(GOLDEN, "x_floor.npz")
    if not os.path.exists(path):
        return 0.0
    d = np.load(path)
    key = f"{name}_{stage}" if f"{name}_{stage}" in d.files else (name if stage == "x" and name in d.files else None)
    return float(d[key]) if key else 0.0


def stage_tol(name, stage):
    """The bar of one pre-fit stage (see the module docstring)."""
    return max(STAGE_TOL, 3.0 * stage_floor(name, stage))


def s_tol(name):
    """The fp64 bar of S: the wave-fit floor, or the Z-perturbation spread."""
    return max(fp64_tol(name), 3.0 * stage_floor(name, "S"))


def _have(name):
    return os.path.exists(os.path.join(GOLDEN, name + ".npz"))


def _build(name):
    if name.startswith("bandpass_"):
        return workloads.build(G, "bandpass", k=int(name.split("_")[1]))
    return workloads.build(G, name)


VARIANTS = [f"bandpass_{k}" for k in (0, 3, 7, 11, 14)]
STAGE_CASES = ["line", "shunt_via", "tee", "via", "lpf", "stripline"] + VARIANTS


@pytest.mark.parametrize("name", STAGE_CASES)
def test_prefit_stages_match_reference(gpu, name):
    """x, q, phi, I, V of the fp64 point at the fixture's first frequency."""
    if not _have(name):
        pytest.skip(f"no fixture {name}")
    g = golden(name)
    if "phi" not in g.files:
        pytest.skip(f"fixture {name} predates the stage arrays")
    lay, st, m, _ = _build(name)
    sol = Solver(m, st, verbose=False, precision="fp64")
    try:
        out = sol.point(float(g["f0"]), keep_currents=True)
        x = out[5]
        q, phi, I, V = sol.last_deembed()
        errs = {}
        for key, got in (("x", x), ("q", q), ("phi", phi), ("I", I), ("V", V)):
            ref = g[key]
            assert got.shape == ref.shape, (key, got.shape, ref.shape)
            errs[key] = np.abs(got - ref).max() / np.abs(ref).max()
        bars = {k: stage_tol(name, k) for k in errs}
        print(name, {k: f"{v:.1e} (bar {bars[k]:.1e})" for k, v in errs.items()})
        assert all(errs[k] <= bars[k] for k in errs), (errs, bars)
    finally:
        sol.close()


@pytest.mark.parametrize("name", VARIANTS)
def test_bandpass_variant_sweeps_match_reference(gpu, name):
    """Coupled-line band-pass variants of N 1524 to 4972: fp64 within three
    fit floors, mixed within 1e-5, at the fixture's frequencies."""
    if not _have(name):
        pytest.skip(f"no fixture {name}")
    g = golden(name)
    lay, st, m, _ = _build(name)
    assert m.n_unknowns == g["N"]
    for prec, tol in (("fp64", s_tol(name)), ("mixed", 1e-5)):
        sol = Solver(m, st, verbose=False, precision=prec)
        try:
            r = sol.sweep(g["freqs"], workers=2)
            dS = np.abs(r.S - g["S"]).max()
            print(name, prec, f"max |dS| {dS:.2e}")
            assert dS < tol, (prec, dS)
        finally:
            sol.close()


def test_gcpw_large_workload_matches_reference(gpu):
    """The via-fenced grounded CPW, N = 25284 with 84 vias (the largest
    workload). Mixed precision: at 10.35 GHz the complex64 LU + refinement
    within 1e-5; at 1 GHz the refinement stalls (cond(Z) u32 > 1) and the
    point falls back to the fp64 fill and LU, which must then meet the fp64
    bar."""
    if not _have("gcpw"):
        pytest.skip("no fixture gcpw")
    g = golden("gcpw")
    lay, st, m, _ = _build("gcpw")
    assert m.n_unknowns == g["N"]
    sol = Solver(m, st, verbose=False, precision="mixed")
    try:
        r = sol.sweep(g["freqs"])
        dS = np.abs(r.S - g["S"]).max(axis=(1, 2))
        print("gcpw max |dS| per frequency", dS, r.info)
        fb = set(r.info["fp64_fallback"])
        for i, f in enumerate(g["freqs"]):
            assert dS[i] < (s_tol("gcpw") if float(f) in fb else 1e-5), (f, dS[i])
    finally:
        sol.close()


def test_gcpw_prefit_stages_match_reference(gpu):
    """x, q, phi, I, V of the fp64 point at 1 GHz on the N = 25284 mesh."""
    if not _have("gcpw"):
        pytest.skip("no fixture gcpw")
    g = golden("gcpw")
    lay, st, m, _ = _build("gcpw")
    sol = Solver(m, st, verbose=False, precision="fp64")
    try:
        x = sol.point(float(g["f0"]), keep_currents=True)[5]
        q, phi, I, V = sol.last_deembed()
        errs = {k: np.abs(got - g[k]).max() / np.abs(g[k]).max()
                for k, got in (("x", x), ("q", q), ("phi", phi), ("I", I), ("V", V))}
        bars = {k: stage_tol("gcpw", k) for k in errs}
        print("gcpw", {k: f"{v:.1e} (bar {bars[k]:.1e})" for k, v in errs.items()})
        assert all(errs[k] <= bars[k] for k in errs), (errs, bars)
        Z = sol.impedance(float(g["f0"]))
        rows = g["Z_rows_idx"]
        assert np.abs(Z[rows] - g["Z_rows"]).max() <= 1e-11 * np.abs(g["Z_rows"]).max()
        assert np.abs(np.diag(Z) - g["Z_diag"]).max() <= 1e-11 * np.abs(g["Z_diag"]).max()
    finally:
        sol.close()


def test_stripline_under_a_pec_cover(gpu):
    """The centred stripline under a PEC cover (mom25d's Engine/tests/
    test_multilayer.py:59-76): S of the fp64 path within three fit floors of
    mom25d's and the mixed path within 1e-5 (tests/golden/stripline.npz), and
    mom25d's physics checks: eps_eff = eps_r within 3e-3, the line impedance
    within 1.5 % of the zero-thickness formula eta0 / (4 sqrt(eps_r)) K(k) /
    K(k'), k = sech(pi W / 2 b), and |S11| < 5e-3."""
    from scipy.special import ellipk

    if not _have("stripline"):
        pytest.skip("no fixture stripline")
    g = golden("stripline")
    lay, st, m, _ = _build("stripline")
    er, hh, W = 3.66, 0.254e-3, 0.4e-3
    b = 2 * hh
    k = 1 / np.cosh(np.pi * W / (2 * b))
    z0 = 376.730313668 / (4 * np.sqrt(er)) * ellipk(k ** 2) / ellipk(1 - k ** 2)
    for prec, tol in (("fp64", s_tol("stripline")), ("mixed", 1e-5)):
        sol = Solver(m, st, verbose=False, precision=prec)
        try:
            r = sol.sweep(g["freqs"])
            dS = np.abs(r.S - g["S"]).max()
            print("stripline", prec, f"|dS| {dS:.1e}", r.eeff[:, 0], r.z0_line[:, 0].real, z0)
            assert dS < tol, (prec, dS)
            np.testing.assert_allclose(r.eeff[:, 0], er, rtol=3e-3)
            np.testing.assert_allclose(r.z0_line[:, 0].real, z0, rtol=0.015)
            assert np.all(np.abs(r.S[:, 0, 0]) < 5e-3)
        finally:
            sol.close()
