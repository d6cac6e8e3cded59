"""S-parameter networks after a sweep: Touchstone blocks, joining ports,
renormalisation (Engine/mom25d/network.py:1-103, lumped.Touchstone
lumped.py:93-148).

Host-side arithmetic on (F, n, n) matrices: none of it is on the GPU path.
Two ports k, l of one network are joined by the sub-network interconnection
formula (Compton; scikit-rf's innerconnect):

  S'_ij = S_ij + [S_il S_kj (1 - S_lk) + S_il S_lj S_kk
                  + S_ik S_lj (1 - S_kl) + S_ik S_kj S_ll] / D,
  D = (1 - S_kl)(1 - S_lk) - S_kk S_ll,

and two networks are joined by placing them side by side and joining the
connected port pairs one after another.
"""

import numpy as np

_UNITS = {"HZ": 1.0, "KHZ": 1e3, "MHZ": 1e6, "GHZ": 1e9}


class Touchstone:
    """N-port block from a Touchstone v1 file (.sNp; MA, DB or RI; any
    frequency unit; one real reference impedance). s(f) interpolates the real
    and imaginary parts linearly in frequency; z(f) is the impedance matrix."""

    def __init__(self, path):
        self.path = str(path)
        digits = "".join(ch for ch in self.path.rsplit(".", 1)[-1] if ch.isdigit())
        if not digits:
            raise ValueError(f"{self.path}: no port count in the extension (.sNp)")
        n = int(digits)
        fmt, unit, z0 = "MA", 1e9, 50.0
        nums = []
        with open(self.path) as fh:
            for line in fh:
                line = line.split("!", 1)[0].strip()
                if not line:
                    continue
                if line.startswith("#"):
                    tok = line[1:].upper().split()
                    for i, t in enumerate(tok):
                        if t in _UNITS:
                            unit = _UNITS[t]
                        elif t in ("MA", "DB", "RI"):
                            fmt = t
                        elif t == "R" and i + 1 < len(tok):
                            z0 = float(tok[i + 1])
                    continue
                nums.extend(float(x) for x in line.split())
        per = 1 + 2 * n * n
        if not nums or len(nums) % per:
            raise ValueError(f"{self.path}: {len(nums)} numbers are not rows of {per}")
        v = np.asarray(nums).reshape(-1, per)
        self.f = v[:, 0] * unit
        a, b = v[:, 1::2], v[:, 2::2]
        if fmt == "RI":
            s = a + 1j * b
        else:
            mag = a if fmt == "MA" else 10.0 ** (a / 20.0)
            s = mag * np.exp(1j * np.deg2rad(b))
        s = s.reshape(-1, n, n)
        if n == 2:  # version-1 two-ports list S11 S21 S12 S22 (column by column)
            s = np.swapaxes(s, 1, 2)
        self.s_data, self.n, self.z0 = s, n, z0
        self.desc = f"Touchstone {self.path.rsplit('/', 1)[-1]} ({n}-port)"

    def s(self, f):
        """S at f (n x n)."""
        lo, hi = self.f[0], self.f[-1]
        if not lo * (1 - 1e-9) <= f <= hi * (1 + 1e-9):
            raise ValueError(f"{self.path}: {f / 1e9:g} GHz outside {lo / 1e9:g}-{hi / 1e9:g} GHz")
        flat = self.s_data.reshape(len(self.f), -1)
        re = np.array([np.interp(f, self.f, flat[:, c].real) for c in range(flat.shape[1])])
        im = np.array([np.interp(f, self.f, flat[:, c].imag) for c in range(flat.shape[1])])
        return (re + 1j * im).reshape(self.n, self.n)

    def z(self, f):
        s = self.s(f)
        eye = np.eye(self.n)
        return self.z0 * (eye + s) @ np.linalg.inv(eye - s)

    def __repr__(self):
        return self.desc


def innerconnect(S, k, l):
    """Join ports k and l of S (F, n, n) -> (F, n-2, n-2)."""
    S = np.asarray(S)
    keep = [i for i in range(S.shape[-1]) if i not in (k, l)]
    Skk, Sll, Skl, Slk = S[:, k, k], S[:, l, l], S[:, k, l], S[:, l, k]
    D = (1 - Skl) * (1 - Slk) - Skk * Sll
    col_k, col_l = S[:, keep, k][:, :, None], S[:, keep, l][:, :, None]  # S_ik, S_il
    row_k, row_l = S[:, k, keep][:, None, :], S[:, l, keep][:, None, :]  # S_kj, S_lj
    e = lambda v: v[:, None, None]  # noqa: E731
    num = (col_l * row_k * e(1 - Slk) + col_l * row_l * e(Skk) + col_k * row_l * e(1 - Skl)
           + col_k * row_k * e(Sll))
    return S[:, keep][:, :, keep] + num / e(D)


def connect(SA, SB, pairs):
    """Join port a of SA to port b of SB for every (a, b) in pairs (0-based).
    Returns (S, idx): the remaining ports, SA's then SB's, and for each the
    port number in the side-by-side numbering (SB's ports offset by SA's
    count)."""
    SA, SB = np.asarray(SA), np.asarray(SB)
    na, nb = SA.shape[-1], SB.shape[-1]
    S = np.zeros((SA.shape[0], na + nb, na + nb), complex)
    S[:, :na, :na] = SA
    S[:, na:, na:] = SB
    idx = list(range(na + nb))
    for a, b in pairs:
        k, l = idx.index(a), idx.index(na + b)
        S = innerconnect(S, k, l)
        idx = [p for p in idx if p not in (a, na + b)]
    return S, idx


def renormalize(S, z_old, z_new):
    """S (F, n, n) from per-port real reference impedances z_old to z_new
    (each (F, n) or broadcastable), through the impedance matrix."""
    S = np.asarray(S)
    nf, n = S.shape[0], S.shape[-1]
    zo = np.broadcast_to(np.asarray(z_old, float), (nf, n))
    zn = np.broadcast_to(np.asarray(z_new, float), (nf, n))
    eye = np.eye(n)
    out = np.empty_like(S)
    for f in range(nf):
        ro, rn = np.sqrt(zo[f]), np.sqrt(zn[f])
        Z = ro[:, None] * np.linalg.solve(eye - S[f], eye + S[f]) * ro[None, :]
        Zn = Z / (rn[:, None] * rn[None, :])
        out[f] = np.linalg.solve(Zn + eye, Zn - eye)
    return out


class Network:
    """S-parameters on named ports with one real reference impedance (the
    result of SweepResult.connect)."""

    def __init__(self, freqs, S, names, z0=50.0):
        self.freqs, self.S, self.names, self.z0 = np.asarray(freqs), np.asarray(S), list(names), z0
        self._source = None

    def db(self, i, j):
        return 20 * np.log10(np.abs(self.S[:, i, j]))

    def currents(self, fi, port):
        """Layout coefficients at frequency index fi for a unit incident wave
        on `port` (name or index) of this network, its other ports matched:
        the connected blocks set what returns into the layout ports they are
        attached to (needs a sweep with keep_currents=True)."""
        if self._source is None:
            raise ValueError("currents: this network does not come from SweepResult.connect")
        res, model, pairs, idx, z0 = self._source
        q = self.names.index(port) if isinstance(port, str) else int(port)
        SL = res.renormalize(z0)[fi]
        SB = model.s(self.freqs[fi])
        nl, nb = SL.shape[0], SB.shape[0]
        drive = np.zeros(nl + nb, complex)
        drive[idx[q]] = 1.0
        # incident waves a = [a_layout, a_block]: across a joined pair (i, k)
        # each side's incident wave is the other side's reflected one
        M = np.eye(nl + nb, dtype=complex)
        for i, k in pairs:
            M[i, nl:] -= SB[k]
            M[nl + k, :nl] -= SL[i]
            drive[i] = drive[nl + k] = 0.0
        a = np.linalg.solve(M, drive)
        return res.wave_currents(fi, a[:nl], z0)

    def write_touchstone(self, path):
        n = len(self.names)
        with open(path, "w") as fh:
            fh.write("! mom25d_gb300 network, ports: " + ", ".join(self.names) + "\n")
            fh.write(f"# HZ S RI R {self.z0:g}\n")
            for f, s in zip(self.freqs, self.S):
                m = s.T if n == 2 else s  # version-1 two-port order S11 S21 S12 S22
                fh.write(f"{f:.9e} " + " ".join(f"{v.real:.9e} {v.imag:.9e}" for v in m.ravel()) + "\n")
