"""GB300-native (sm_103a) engine for mom25d's per-frequency sweep path:
Green's tables, RWG impedance fill, dense complex LU + solve and port
de-embedding, behind mom25d's Layout / Stackup / Solver / sweep() API."""

from .constants import C0, EPS0, ETA0, MU0, GHz, MHz, mm, um
from .layout import CoplanarGround, Layout, Mesh, Port, Via
from .stack import Dielectric, Stackup, Substrate


def __getattr__(name):
    # the CUDA-backed parts load the engine library on first use
    if name in ("Solver", "SweepResult", "PortModel", "dense_solve", "assemble"):
        from . import solver

        return getattr(solver, name)
    raise AttributeError(name)
