"""Lumped components across delta gaps (Layout.add_lumped): their one-port
values (Engine/mom25d/lumped.py:17-90).

A load Z across a gap adds Z l l^T to the MoM matrix (l: the gap edges'
signed lengths, Mesh.lumped_vectors); the solver applies every load at once
with the Woodbury identity after one solve for the port and gap excitations
(Solver._load_lumped), so values can change per sweep without a new fill
(Solver.sweep(..., values=...)).

Values: R, L, C, combined with series / parallel, a number (ohm), a callable
f -> Z, or a string such as 'R 50', 'C 1p', 'R 10 + L 0.5n', 'C 1p || R 1k'.
"""

import numpy as np

_SCALE = (("G", 1e9), ("M", 1e6), ("k", 1e3), ("", 1.0), ("m", 1e-3), ("u", 1e-6), ("n", 1e-9), ("p", 1e-12),
          ("f", 1e-15))
_SUFFIX = {"f": 1e-15, "p": 1e-12, "n": 1e-9, "u": 1e-6, "m": 1e-3, "k": 1e3, "M": 1e6, "G": 1e9}


class Value:
    """A one-port impedance Z(f) [ohm] with a readable description."""

    def __init__(self, fz, desc):
        self.fz, self.desc = fz, desc

    def z(self, f):
        return complex(self.fz(f))

    def __repr__(self):
        return self.desc


def _label(x, unit):
    for prefix, k in _SCALE:
        if abs(x) >= k:
            return f"{x / k:g} {prefix}{unit}"
    return f"{x:g} {unit}"


def R(r):
    r = float(r)
    return Value(lambda f: complex(r), _label(r, "ohm"))


def L(l):
    l = float(l)
    return Value(lambda f: 2j * np.pi * f * l, _label(l, "H"))


def C(c):
    c = float(c)
    return Value(lambda f: 1 / (2j * np.pi * f * c), _label(c, "F"))


def series(*vals):
    vs = [as_value(v) for v in vals]
    return Value(lambda f: sum(v.z(f) for v in vs), "(" + " + ".join(map(repr, vs)) + ")")


def parallel(*vals):
    vs = [as_value(v) for v in vals]
    return Value(lambda f: 1 / sum(1 / v.z(f) for v in vs), "(" + " || ".join(map(repr, vs)) + ")")


def as_value(v):
    """A Value from a Value, a number (ohm) or a callable f -> Z."""
    if isinstance(v, Value):
        return v
    if callable(v):
        return Value(v, getattr(v, "__name__", "Z(f)"))
    if np.isreal(v):
        return R(float(np.real(v)))
    z = complex(v)
    return Value(lambda f: z, f"{z} ohm")


def _number(text):
    t = text.strip()
    if t and t[-1] in _SUFFIX:
        return float(t[:-1]) * _SUFFIX[t[-1]]
    return float(t)


def _element(text):
    kind, val = text.split()
    makers = {"R": R, "L": L, "C": C}
    if kind.upper() not in makers:
        raise ValueError(f"lumped value {text!r}: R, L or C expected")
    return makers[kind.upper()](_number(val))


def parse(text):
    """'R 50', 'C 1p', 'L 2.2n', 'R 10 + L 0.5n', 'C 1p || R 1k' -> Value
    (lumped.py:71-90; series-mounted .s2p parts are not part of this engine)."""
    t = text.strip()
    if t.lower().endswith(".s2p"):
        raise ValueError("series parts from .s2p files are not part of this engine")
    if "||" in t:
        return parallel(*[parse(p) for p in t.split("||")])
    if "+" in t:
        return series(*[_element(p) for p in t.split("+")])
    return _element(t)
