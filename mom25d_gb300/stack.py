"""Dielectric stack descriptions: Substrate (one grounded slab) and Stackup
(layers bottom to top with named metal levels), as mom25d/solver.py:42-76
and mom25d/layered.py:52-180 define them: air above the top layer
(top="air") or a PEC cover on it (top="pec", e.g. a stripline). Inner PEC
planes (sections) are not part of this engine."""

from dataclasses import dataclass

import numpy as np

from .constants import MU0

GND = "gnd"


def surface_impedance(freq, sigma, t):
    """One-sided skin-effect impedance of a conductor slab of thickness t,
    k_c coth(k_c t) / sigma with k_c = sqrt(j w mu0 sigma); -> 1/(sigma t) at DC."""
    if not sigma:
        return 0.0
    w = 2 * np.pi * freq
    kc = np.sqrt(1j * w * MU0 * sigma)
    return kc / sigma / np.tanh(kc * t)


@dataclass
class Dielectric:
    t: float
    eps_r: float
    tand: float = 0.0


@dataclass
class Stackup:
    layers: list
    metals: dict = None
    top: str = "air"
    sigma: float = None
    t: float = 35e-6
    ground_loss: bool = True
    planes: dict = None

    def __post_init__(self):
        if not self.layers:
            raise ValueError("stackup needs at least one dielectric layer")
        self.layers = [d if isinstance(d, Dielectric) else Dielectric(*d) for d in self.layers]
        n = len(self.layers)
        if self.metals is None:
            self.metals = {"top": n}
        if self.top not in ("air", "pec"):
            raise ValueError("top must be 'air' or 'pec'")
        for name, k in self.metals.items():
            if name == GND:
                raise ValueError("'gnd' is reserved for the ground plane")
            if not 1 <= k <= n:
                raise ValueError(f"metal level {name}: interface {k} not in 1..{n}")
            if k == n and self.top == "pec":
                raise ValueError(f"metal level {name} would lie on the PEC cover")
        self.planes = dict(self.planes or {})
        if self.planes:
            raise ValueError("inner PEC planes are not part of this engine")
        self.bounds = [0, n]
        self.z = np.concatenate([[0.0], np.cumsum([d.t for d in self.layers])])

    @classmethod
    def microstrip(cls, eps_r, h, tand=0.0, sigma=None, t=35e-6, ground_loss=True):
        return cls([Dielectric(h, eps_r, tand)], {"top": 1}, "air", sigma, t, ground_loss)

    @property
    def lossless(self):
        return not self.sigma and not any(d.tand for d in self.layers)

    def level_z(self, name):
        if name == GND:
            return 0.0
        return float(self.z[self.metals[name]])

    def section(self, name):
        return 0

    def level_h(self, name):
        return self.level_z(name)

    def eps_below(self, name):
        k = self.metals[name]
        t = np.array([d.t for d in self.layers[:k]])
        e = np.array([d.eps_r for d in self.layers[:k]])
        return float(t @ e / t.sum())

    def covered(self, name):
        return self.metals[name] < len(self.layers) or self.top == "pec"

    def surface_impedance(self, freq, t=None):
        return surface_impedance(freq, self.sigma, self.t if t is None else t)


@dataclass
class Substrate:
    """Grounded dielectric slab with conductors on top."""

    eps_r: float
    h: float
    tand: float = 0.0
    sigma: float = None
    t: float = 35e-6
    ground_loss: bool = True

    @property
    def lossless(self):
        return not self.tand and not self.sigma

    def surface_impedance(self, freq):
        return surface_impedance(freq, self.sigma, self.t)

    def to_stackup(self):
        return Stackup.microstrip(self.eps_r, self.h, self.tand, self.sigma, self.t, self.ground_loss)
