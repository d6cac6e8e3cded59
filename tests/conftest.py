import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built engine")


def golden(name):
    import numpy as np

    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def gpu():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test without a CUDA device")
    from mom25d_gb300 import engine

    engine.load()
    return True


def fit_floor(name=None):
    """mom25d's own reproducibility floor in S for a workload: the largest
    |S - S0| its sweep showed when the inputs of its wave fit, or its RWG
    currents, were multiplied by 1 + eps (n1 + j n2) with eps from 1e-15 to
    1e-10 (tests/golden/fit_floor.npz, made by make_golden.py --floor). The
    Nelder-Mead wave fit stops anywhere inside a flat valley of its
    objective, so even eps = 1e-15 moves S by about this much: no
    re-implementation can be held closer to mom25d's S than the floor.
    Workloads without a measurement of their own take the largest one."""
    d = golden("fit_floor")
    floors = {str(c): max(float(d[f"{c}_dS_fit"].max()), float(d[f"{c}_dS_x"].max())) for c in d["cases"]}
    if name is not None and name in floors:
        return floors[name]
    return max(floors.values())


def fp64_tol(name=None):
    """The bar of the fp64 path's S against mom25d's: three times the fit floor."""
    return 3.0 * fit_floor(name)


def gamma_floor(name=None):
    """The same floor for the fitted propagation constant, relative to |gamma|."""
    d = golden("fit_floor")
    floors = {str(c): max(float(d[f"{c}_dgamma_fit"].max()), float(d[f"{c}_dgamma_x"].max())) for c in d["cases"]}
    if name is not None and name in floors:
        return floors[name]
    return max(floors.values())
