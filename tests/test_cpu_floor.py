"""The reference's own reproducibility floor in S (tests/golden/fit_floor.npz,
made by running mom25d: make_golden.py --floor). It bounds how closely any
re-implementation, the oracle included, can match mom25d's S, and sets the
fp64 bars of the parity tests (three times the floor of each workload)."""

import numpy as np
import pytest

from conftest import fit_floor, fp64_tol, golden


def test_floor_fixture_covers_the_parity_workloads():
    d = golden("fit_floor")
    assert set(d["cases"]) == {"line", "tee", "via", "bandpass_0", "lpf", "line_lossless"}
    for c in d["cases"]:
        for mode in ("fit", "x"):
            dS = d[f"{c}_dS_{mode}"]
            assert dS.shape == (len(d[f"{c}_eps"]), len(d[f"{c}_freqs"]))
            assert np.all(np.isfinite(dS))


@pytest.mark.parametrize("case", ["line", "tee", "via", "bandpass_0", "lpf", "line_lossless"])
def test_floor_does_not_shrink_with_the_perturbation(case):
    """The floor is a property of the fit, not of the perturbation: inputs
    moved by 1e-15 already move S by within a factor of 30 of what 1e-10
    does (a linear response would scale by 1e5), and the worst case of each
    workload lies between 1e-9 and 1e-7 -- a hundred times above the 1e-9
    bar the fp64 path is asked for, and a tenth of the 1e-6 held before."""
    d = golden("fit_floor")
    for mode in ("fit", "x"):
        per_eps = d[f"{case}_dS_{mode}"].max(axis=1)
        assert per_eps[0] > per_eps[-1] / 30, (mode, per_eps)
    f = fit_floor(case)
    assert 1e-9 < f < 1e-7, f
    # gamma moves by the same kind of amount (relative)
    assert d[f"{case}_dgamma_fit"].max() < 1e-6


def test_fp64_bar_is_three_floors():
    cases = ("line", "tee", "via", "bandpass_0", "lpf", "line_lossless")
    for case in cases:
        assert fp64_tol(case) == 3 * fit_floor(case)
    # a workload without its own measurement takes the largest floor
    assert fit_floor("gcpw") == max(fit_floor(c) for c in cases)
