"""Internal S-parameter ports on the GPU against mom25d's own sweeps
(tests/golden/gap_port_line.npz, via_port_line.npz): the feeds' wave fits
over every port's excitation on the device, the internal ports' rows, the
reference impedances and S assembled on the host."""

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Solver

from conftest import fp64_tol, golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["gap_port_line", "via_port_line"])
def test_internal_port_sweep_matches_reference(gpu, name, prec):
    g = golden(name)
    lay, st, m, _ = workloads.build(G, name)
    sol = Solver(m, st, verbose=False, precision=prec)
    try:
        r = sol.sweep(g["freqs"], keep_currents=True)
        assert r.port_names == [str(s) for s in g["port_names"]]
        tol = fp64_tol() if prec == "fp64" else 1e-5
        dS = np.abs(r.S - g["S"]).max()
        print(name, prec, f"max |dS| {dS:.2e}")
        assert dS < tol
        assert np.abs(r.z0 - g["z0"]).max() < tol * 100 * np.abs(g["z0"]).max()
        np.testing.assert_array_equal(r.z0[:, 2], 50.0)
        P = len(lay.ports)
        assert np.abs(r.gamma[:, :P] - g["gamma"][:, :P]).max() < 1e-6 * np.abs(g["gamma"][:, :P]).max()
        assert r.waves.shape == g["waves"].shape
        if prec == "fp64":
            x, xr = r.currents[0], g["x0"]
            assert np.abs(x - xr).max() <= 1e-7 * np.abs(xr).max()
    finally:
        sol.close()


def test_internal_ports_only_take_the_host_path(gpu):
    """The device's whole-point call refuses ports whose solutions carry
    internal-port columns (they are de-embedded with host currents)."""
    lay, st, m, _ = workloads.build(G, "gap_port_line")
    sol = Solver(m, st, verbose=False)
    try:
        sol.port_data()
        with pytest.raises(ValueError, match="internal-port"):
            import ctypes as C

            from mom25d_gb300 import engine as E

            P = len(sol.ports)
            S = np.zeros((P, P), complex)
            z0, gam, zl, res = np.zeros(P), np.zeros(P, complex), np.zeros(P, complex), np.zeros(P)
            info = np.zeros(2, np.int32)
            g = sol.greens(4e9)
            F = lambda a: E.ptr(a.view(np.float64))  # noqa: E731
            E.check(sol.ctx.lib.m25_sweep_point(sol.ctx.h, sol.geometry().h, g.h, sol.port_data().h, 0.0, 0.0, 0.0,
                                                0.0, E.M25_FP64, E.ptr(E.f64(sol.beta0(4e9))), 1e-12, 60, None, F(S),
                                                E.ptr(z0), F(gam), F(zl), E.ptr(res), E.ptr(info, C.c_int32)))
    finally:
        sol.close()
