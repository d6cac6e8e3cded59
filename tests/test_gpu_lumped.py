"""GPU tests of sweeps with a lumped component (Layout.add_lumped): S of the
loaded line, with the value overridden per sweep and with an open gap, and
the loaded currents, against mom25d (tests/golden/lumped_line.npz)."""

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Solver

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-6), ("mixed", 1e-5)])
def test_lumped_sweeps_match_reference(gpu, precision, tol):
    g = golden("lumped_line")
    lay, st, m, _ = workloads.build(G, "lumped_line")
    sol = Solver(m, st, verbose=False, precision=precision)
    r = sol.sweep(g["freqs"], keep_currents=True)
    assert np.abs(r.S - g["S"]).max() < tol
    assert np.abs(r.currents[0] - g["x"]).max() < 100 * tol * np.abs(g["x"]).max()
    np.testing.assert_allclose(sol.lumped_currents(r.currents[0]), g["I_gap"], rtol=100 * tol)
    r2 = sol.sweep(g["freqs"], values={"Z1": "C 1p"}, workers=2)
    assert np.abs(r2.S - g["C1p_S"]).max() < tol
    r3 = sol.sweep(g["freqs"], values={"Z1": None})
    assert np.abs(r3.S - g["open_S"]).max() < tol
    sol.close()


def test_component_sweep_matches_reference(gpu):
    import os

    from conftest import GOLDEN

    g = golden("component_line")
    lay, st, m, _ = workloads.build(G, "component_line", block=os.path.join(GOLDEN, "block.s2p"))
    sol = Solver(m, st, verbose=False)
    r = sol.sweep(g["freqs"])
    assert np.abs(r.S - g["S"]).max() < 1e-6
    sol.close()
