"""CPU tests of the frequency interpolation (FreqInterp): the host logic of
mom25d_gb300/freqinterp.py (anchors, phase ratio, step, basis centres,
window, weights) and the oracle's transform with the oracle's own fill,
both against fixtures made by mom25d's FreqInterp
(tests/golden/make_golden.py --interp)."""

from types import SimpleNamespace

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.freqinterp import FreqInterp
from oracle import freqinterp as OI
from oracle import sweep as O

from conftest import golden

CASES = {"tee": {}, "shunt_via": dict(step=1.5e9)}


def host_solver(name):
    """What FreqInterp.setup reads of a Solver, without a device."""
    lay, sub, m, _ = workloads.build(G, name)
    st = sub if hasattr(sub, "layers") else sub.to_stackup()  # as Solver.__init__
    order = sorted(list(m.layer_names), key=st.level_z)
    if getattr(m, "level_order", None) != order:
        m.assign_levels(order)
    zl = np.array([st.level_z(n) for n in m.layer_names])
    return SimpleNamespace(mesh=m, stack=st, zl=zl, ports=m.layout.ports), m, st


@pytest.mark.parametrize("name", list(CASES))
def test_anchor_grid_matches_reference(name):
    g = golden(name + "_interp")
    sol, m, _ = host_solver(name)
    assert m.n_unknowns == int(g["N"])
    ip = FreqInterp(**CASES[name]).setup(sol, g["freqs"])
    np.testing.assert_allclose(ip.pos, g["pos"], rtol=0, atol=1e-15)
    assert ip.nb == int(g["nb"])
    assert ip.k_ratio == pytest.approx(float(g["k_ratio"]), rel=1e-15)
    assert ip.step == pytest.approx(float(g["step"]), rel=1e-15)
    np.testing.assert_array_equal(ip.anchors, g["anchors"])
    for f, win, L in zip(g["freqs"], g["windows"], g["weights"]):
        assert ip._window(f) == list(win)
        np.testing.assert_array_equal(ip.weights(f, ip._window(f)), L)
        assert OI.window(ip.anchors, ip.order, f) == list(win)


def test_oracle_interpolated_z_matches_reference():
    """The oracle's fill at the anchors of the window, transformed and
    interpolated by oracle/freqinterp.py: the reference's interpolated Z
    rows (shunt via: RWG and via unknowns)."""
    g = golden("shunt_via_interp")
    lay, st, m, _ = workloads.build(G, "shunt_via")
    sw = O.Sweep(m, st)
    anchors, fm = g["anchors"], float(g["f_mid"])
    idx = OI.window(anchors, int(g["order"]), fm)
    kr = float(g["k_ratio"])
    ke = lambda f: kr * 2 * np.pi * f / 299792458.0  # noqa: E731
    Ws = [OI.store(sw.impedance(float(anchors[i])), g["pos"], int(g["nb"]), float(anchors[i]),
                   ke(float(anchors[i]))) for i in idx]
    Z = OI.evaluate(Ws, OI.weights(anchors, fm, idx), g["pos"], int(g["nb"]), fm, ke(fm))
    rows = g["Z_rows_idx"]
    ref = g["Zi_rows"]
    assert np.abs(Z[rows] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_oracle_interpolated_sweep_matches_reference():
    """The oracle's fill at every anchor, the transform, the Lagrange
    combination at each frequency, solve and de-embedding: mom25d's
    interpolated S on the shunt via (25 frequencies, 5 anchors)."""
    g = golden("shunt_via_interp")
    lay, st, m, _ = workloads.build(G, "shunt_via")
    sw = O.Sweep(m, st)
    anchors, order, nb = g["anchors"], int(g["order"]), int(g["nb"])
    kr = float(g["k_ratio"])
    ke = lambda f: kr * 2 * np.pi * f / 299792458.0  # noqa: E731
    W = [OI.store(sw.impedance(float(fa)), g["pos"], nb, float(fa), ke(float(fa))) for fa in anchors]
    S = []
    for f in g["freqs"]:
        idx = OI.window(anchors, order, f)
        Z = OI.evaluate([W[i] for i in idx], OI.weights(anchors, f, idx), g["pos"], nb, f, ke(f))
        kern = sw.kernels(f)
        x = O.dense_solve(Z, sw.excitations())
        q = O.charges(m, x, kern.omega)
        S.append(sw.deembed(f, kern, x, q)[0])
    assert np.abs(np.array(S) - g["S"]).max() < 1e-6


def test_order_limit():
    with pytest.raises(ValueError):
        FreqInterp(order=8)
    assert FreqInterp(order=7).order == 7
