"""GPU test of the sweep outputs behind SweepResult.matched_currents,
wave_currents and Network.currents: the engine's wave amplitudes and
currents against mom25d's line sweep (tests/golden/line_network.npz)."""

import os

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Solver

from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu


def test_waves_currents_and_connect_match_reference(gpu):
    g = golden("line_network")
    lay, st, m, _ = workloads.build(G, "line")
    sol = Solver(m, st, verbose=False)
    r = sol.sweep(g["freqs"], keep_currents=True)
    sol.close()
    # the wave amplitudes are the fit's coefficients: as S, to the fit's floor
    assert np.abs(r.waves - g["waves"]).max() < 1e-6 * np.abs(g["waves"]).max()
    for got, ref in ((r.matched_currents(0, 0), g["matched0"]), (r.wave_currents(0, [1.0, 0.5j]), g["wave0"])):
        assert np.abs(got - ref).max() < 1e-6 * np.abs(ref).max()
    net = r.connect(os.path.join(GOLDEN, "block.s2p"), [(1, 1)])
    assert np.abs(net.S - g["net_S"]).max() < 1e-6
    c = net.currents(0, 0)
    assert np.abs(c - g["net_currents0"]).max() < 1e-6 * np.abs(g["net_currents0"]).max()
