"""Batched sweeps of geometry variants of uneven N (mom25d_gb300/batch.py)
against mom25d's own sweeps of each variant (tests/golden/bandpass_*.npz)."""

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.autotune import Tuning
from mom25d_gb300.batch import VariantBatch
from mom25d_gb300.solver import Solver

from conftest import golden

pytestmark = pytest.mark.gpu

KS = (0, 3, 7, 11, 14)  # N 1524, 2164, 3064, 3982, 4972


def _solvers(precision):
    out = []
    for k in KS:
        lay, st, mesh, _ = workloads.build(G, "bandpass", k=k)
        out.append(Solver(mesh, st, verbose=False, precision=precision))
    return out


@pytest.mark.parametrize("tuning", [None, "fixed"])
def test_variant_batch_matches_reference(gpu, tuning):
    """Five band-pass variants, each at its fixture's frequencies, through one
    batch on four worker contexts shared by all variants: every S within 1e-5
    of mom25d's (mixed precision), with the measured tuning table or with
    one fixed set of knobs."""
    sols = _solvers("mixed")
    try:
        tun = Tuning.fixed(panel_cluster_min=8, wave_ctas=16, tc_chunk=2) if tuning == "fixed" else None
        with VariantBatch(sols, tuning=tun) as batch:
            res = batch.sweep([golden(f"bandpass_{k}")["freqs"] for k in KS], workers=4)
            again = batch.sweep([golden(f"bandpass_{k}")["freqs"] for k in KS], workers=4)  # contexts reused
        assert len(res) == len(KS)
        for k, r in zip(KS, res):
            g = golden(f"bandpass_{k}")
            dS = np.abs(r.S - g["S"]).max()
            print(f"bandpass_{k} N={g['N']} max |dS| {dS:.2e}", r.info["batch"])
            assert dS < 1e-5, (k, dS)
            assert r.info["workers"] == 4
        assert res[0].info["batch"]["points"] == sum(len(golden(f"bandpass_{k}")["freqs"]) for k in KS)
        for a, b in zip(res, again):
            np.testing.assert_array_equal(a.S, b.S)
    finally:
        for s in sols:
            s.close()


def test_variant_batch_equals_separate_sweeps(gpu):
    """The batch gives each variant the S of its own sweep (same precision,
    default knobs) to the wave fit's floor, and leaves the solvers usable."""
    sols = _solvers("fp64")[:2]
    try:
        f = np.array([2e9, 6e9, 10e9])
        with VariantBatch(sols, tuning=Tuning.fixed()) as batch:
            res = batch.sweep(f, workers=3)
        for s, r in zip(sols, res):
            r1 = s.sweep(f)
            assert np.abs(r.S - r1.S).max() < 1e-7
    finally:
        for s in sols:
            s.close()
