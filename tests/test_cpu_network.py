"""CPU tests of the network post-processing (mom25d_gb300/network.py,
SweepResult.connect / matched_currents / wave_currents) against the same
operations run by mom25d on its line sweep (tests/golden/line_network.npz,
block.s2p; tests/golden/make_golden.py --network)."""

import os

import numpy as np

from mom25d_gb300 import network as N
from mom25d_gb300.solver import SweepResult

from conftest import GOLDEN, golden


def reference_result(currents=None):
    g = golden("line_network")
    return SweepResult(g["freqs"], g["S"], g["z0"], g["gamma"], g["z0_line"], g["fit_residual"],
                       [str(n) for n in g["port_names"]], currents, g["waves"]), g


def test_touchstone_block_reads_as_written():
    blk = N.Touchstone(os.path.join(GOLDEN, "block.s2p"))
    assert blk.n == 2 and blk.z0 == 50.0
    assert blk.f[0] == 1e9
    s = blk.s(blk.f[0])
    # MA with a GHz axis, version-1 order S11 S21 S12 S22
    assert abs(s[0, 0] - 0.084 * np.exp(-1j * np.deg2rad(30.0))) < 1e-12
    assert abs(s[1, 0] - 0.69 * np.exp(-1j * np.deg2rad(90.0))) < 1e-12
    assert abs(s[1, 1] - 0.0924 * np.exp(-1j * np.deg2rad(45.0))) < 1e-12


def test_connect_matches_reference():
    r, g = reference_result()
    net = r.connect(os.path.join(GOLDEN, "block.s2p"), [(1, 1)])
    assert net.names == [str(n) for n in g["net_names"]]
    np.testing.assert_allclose(net.S, g["net_S"], rtol=0, atol=1e-13)


def test_renormalize_round_trip_and_reference():
    r, g = reference_result()
    S50 = r.renormalize(50.0)
    np.testing.assert_allclose(N.renormalize(r.S, r.z0, 50.0), S50, rtol=0, atol=1e-13)
    np.testing.assert_allclose(N.renormalize(S50, 50.0, r.z0), r.S, rtol=0, atol=1e-12)


def test_innerconnect_of_a_thru_is_identity():
    """Joining a matched thru between two ports of a network leaves the
    network with those ports shorted through: a 2-port thru joined to port 2
    of a 2-port gives back the 2-port."""
    rng = np.random.default_rng(3)
    SA = 0.3 * (rng.standard_normal((4, 2, 2)) + 1j * rng.standard_normal((4, 2, 2)))
    thru = np.zeros((4, 2, 2), complex)
    thru[:, 0, 1] = thru[:, 1, 0] = 1.0
    S, idx = N.connect(SA, thru, [(1, 0)])
    assert idx == [0, 3]
    np.testing.assert_allclose(S, SA, atol=1e-14)


def test_wave_currents_of_matched_drive_are_matched_currents():
    """With x the reference's currents (those of the same mom25d sweep),
    matched_currents and wave_currents reproduce mom25d's."""
    gn0 = golden("line_network")
    r, gn = reference_result(currents=[gn0["x0"]] + [None] * (len(gn0["freqs"]) - 1))
    np.testing.assert_allclose(r.matched_currents(0, 0), gn["matched0"], rtol=0, atol=1e-12 * np.abs(gn["matched0"]).max())
    np.testing.assert_allclose(r.wave_currents(0, [1.0, 0.5j]), gn["wave0"], rtol=0, atol=1e-12 * np.abs(gn["wave0"]).max())


def test_touchstone_formats_units_and_port_order(tmp_path):
    """DB and RI formats, MHz and Hz axes, comments, a 3-port file (rows in
    row order; only 2-ports use the column order S11 S21 S12 S22), the
    interpolation between points and the range check."""
    p = tmp_path / "a.s2p"
    p.write_text("! comment\n# MHZ S DB R 75\n100 -6 90 -20 0 -30 0 -1 -90 ! tail\n"
                 "300 -6 90 -20 0 -30 0 -1 -90\n")
    t = N.Touchstone(str(p))
    assert t.z0 == 75.0 and t.n == 2
    np.testing.assert_allclose(t.f, [1e8, 3e8])
    s = t.s(2e8)
    assert abs(s[0, 0] - 10 ** (-6 / 20) * 1j) < 1e-12
    assert abs(s[1, 0] - 10 ** (-20 / 20)) < 1e-12  # second pair of a 2-port line is S21
    assert abs(s[0, 1] - 10 ** (-30 / 20)) < 1e-12
    q = tmp_path / "b.s3p"
    vals = " ".join(f"{k} {-k}" for k in range(1, 10))
    q.write_text(f"# HZ S RI\n1e9 {vals}\n2e9 {vals}\n")
    t3 = N.Touchstone(str(q))
    s3 = t3.s(1.5e9)
    assert s3[0, 1] == 2 - 2j and s3[1, 0] == 4 - 4j and s3[2, 2] == 9 - 9j
    import pytest

    with pytest.raises(ValueError):
        t3.s(3e9)
