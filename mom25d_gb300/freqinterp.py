"""Frequency interpolation of the impedance matrix between anchor fills: the
GPU form of mom25d's FreqInterp (Engine/mom25d/freqinterp.py:27-197).

Z is filled exactly at evenly spaced anchor frequencies. With the propagation
phase between basis functions taken out and the 1/(j w) of the scalar
potential undone, W = j w Z exp(+j k_e R_mn) is smooth in frequency; between
anchors it is Lagrange-interpolated from the order + 1 nearest anchors and
Z = W~ exp(-j k_e R) / (j w). The anchors live on the device (m25_interp,
complex128 unless that would take more than about half the free device
memory, then complex64); the interpolation, the solve and the de-embedding of
a point run there (m25_interp_point). The window, the weights and the choice
of anchors are the reference's. Where every anchor of the band fits in the
device memory (a few GB at N ~ 6k) they are all filled first and kept
("resident"): the points then depend on nothing but the anchors and run on
the sweep's concurrent workers like exact-fill points. Otherwise the order + 1
anchors of the window are kept, as in mom25d, and an ascending sweep fills
every anchor once.
"""

import ctypes as C

import numpy as np

from . import engine as E
from .constants import C0


class FreqInterp:
    """Z interpolated between exact fills, for Solver.sweep(..., interp=FreqInterp(...)).

    The arguments are mom25d's (Engine/mom25d/freqinterp.py:27-88) plus one:
    step      anchor spacing [Hz]; the anchors cover the swept band at even
              spacing. None derives it from the layout: 0.35 c / (k_ratio D)
              with D the largest distance between two basis centres.
    order     Lagrange order; order + 1 anchors enter each point (1..7 here).
    k_ratio   the phase taken out before interpolating is exp(-j k_ratio k0 R);
              None estimates k_ratio as the square root of a quasi-static
              effective permittivity of the stack.
    check     also fill exactly the first swept frequency that sits at least
              a quarter step away from every anchor, and print how far the
              interpolated Z is from it.
    block     kept for signature compatibility (the host implementation in
              mom25d walks the rows in blocks; the device kernels do not).
    dtype     anchor storage: np.complex128, np.complex64, or None for
              complex128 when it fits in device memory, else complex64.
    resident  (not in mom25d) None keeps all anchors of the band on the
              device when they need under 40 % of its free memory; True or
              False forces the choice.
    """

    def __init__(self, step=None, order=3, k_ratio=None, check=False, block=1024, dtype=None, resident=None):
        if not 1 <= int(order) <= 7:
            raise ValueError("FreqInterp: order 1..7 (the device interpolation combines up to 8 anchors)")
        self.step, self.order, self.k_ratio, self.check, self.block = step, order, k_ratio, check, block
        self.dtype = dtype
        self.resident = resident
        self._resident = False  # this setup's choice
        self.solver = None
        self._ip = None

    # ----------------------------------------------------------- setup
    def setup(self, solver, freqs):
        """Anchors for the band of freqs, basis centres, k_ratio and step
        (freqinterp.py:54-88); the device slots are made on first use."""
        self.close()
        self.solver = solver
        f = np.asarray(freqs, float)
        lo, hi = f.min(), f.max()
        self._slot_of = {}
        self.n_fills = 0
        self.fill_time = 0.0
        self.pos = basis_centres(solver)
        self.nb = solver.mesh.n_basis
        if self.k_ratio is None:
            self.k_ratio = float(np.sqrt(eps_eff(solver)))
        if self.step is None:
            ext = np.ptp(self.pos, axis=0)
            self.step = 0.35 * C0 / (max(self.k_ratio, 1.0) * float(np.linalg.norm(ext)))
        n = max(self.order + 1, int(np.ceil((hi - lo) / self.step - 1e-9)) + 1)
        self.anchors = np.linspace(lo, hi, n) if hi > lo else lo + self.step * (np.arange(n) - n // 2)
        self._checked = not self.check
        return self

    def _device(self):
        if self._ip is None:
            sol = self.solver
            N = len(self.pos)
            free, total = C.c_uint64(), C.c_uint64()
            E.check(sol.ctx.lib.m25_ctx_mem_info(sol.ctx.h, C.byref(free), C.byref(total)))
            if self.dtype is None:
                need = (self.order + 1) * N * N * 16 + 3 * N * N * 16  # anchors + Z + LU work
                self.dtype = np.complex128 if need < 0.5 * free.value else np.complex64
            single = int(np.dtype(self.dtype) == np.complex64)
            fits = len(self.anchors) * N * N * np.dtype(self.dtype).itemsize < 0.4 * free.value
            self._resident = fits if self.resident is None else bool(self.resident)
            nslots = len(self.anchors) if self._resident else self.order + 1
            h = C.c_void_p()
            pos = np.ascontiguousarray(self.pos, np.float64)
            E.check(sol.ctx.lib.m25_interp_create(sol.ctx.h, N, self.nb, E.ptr(pos), nslots, single, C.byref(h)))
            self._ip = E.Handle(sol.ctx, h, sol.ctx.lib.m25_interp_destroy)
            self._free = list(range(nslots))
        return self._ip

    def fill_all(self, freqs=None):
        """Resident anchors: fill every anchor now (and run the check at the
        first frequency of freqs between anchors), so that points can then
        be taken in any order and by several workers."""
        self._device()
        if not self._resident:
            raise RuntimeError("the anchors of this band do not fit in the device memory together")
        self._slots(list(range(len(self.anchors))))
        if not self._checked and freqs is not None:
            for f in freqs:
                if np.min(np.abs(self.anchors - f)) > 0.25 * self.step:
                    self.impedance(f)
                    break
            self._checked = True

    def _window(self, f):
        """Indices of the order+1 anchors used at f: centred on the anchor
        interval holding f (freqinterp.py:124-132)."""
        n, k = len(self.anchors), self.order + 1
        j = int(np.clip(np.searchsorted(self.anchors, f, side="right") - 1, 0, n - 2))
        i0 = min(max(j - (k - 1) // 2, 0), n - k)
        return list(range(i0, i0 + k))

    def weights(self, f, idx):
        """Lagrange weights of the anchors idx at f (freqinterp.py:134-141)."""
        fa = self.anchors[idx]
        L = np.ones(len(idx))
        for a in range(len(idx)):
            for b in range(len(idx)):
                if a != b:
                    L[a] *= (f - fa[b]) / (fa[a] - fa[b])
        return L

    def ke(self, f):
        return self.k_ratio * 2 * np.pi * f / C0

    def _slots(self, idx):
        """Device slots of the anchors idx: anchors outside the window are
        evicted, missing ones filled (freqinterp.py:107-122, 147-151)."""
        import time

        ip = self._device()
        if not self._resident:
            for i in list(self._slot_of):
                if i not in idx:
                    self._free.append(self._slot_of.pop(i))
        sol = self.solver
        for i in idx:
            if i in self._slot_of:
                continue
            slot = self._free.pop()
            fa = float(self.anchors[i])
            t = time.time()
            g = sol.greens(fa)
            zs = complex(sol.surface_impedance(fa))
            prec = E.M25_MIXED if sol.precision == "mixed" else E.M25_FP64
            E.check(sol.ctx.lib.m25_interp_anchor(sol.ctx.h, sol.geometry().h, g.h, ip.h, slot, zs.real, zs.imag,
                                                  zs.real, zs.imag, prec, self.ke(fa)))
            E.check(sol.ctx.lib.m25_ctx_synchronize(sol.ctx.h))
            g.close()
            self.fill_time += time.time() - t
            self.n_fills += 1
            self._slot_of[i] = slot
        return [self._slot_of[i] for i in idx]

    # ---------------------------------------------------------- public
    def impedance(self, f):
        """Interpolated Z at f as a host complex128 array
        (freqinterp.py:145-168)."""
        idx = self._window(f)
        slots = np.array(self._slots(idx), np.int32)
        L = self.weights(f, idx)
        N = len(self.pos)
        Z = np.empty((N, N), complex)
        E.check(self.solver.ctx.lib.m25_interp_eval(self._ip.h, len(idx), E.ptr(slots, C.c_int32), E.ptr(L), float(f),
                                                    self.ke(f), Z.ctypes.data, N, E.M25_ON_HOST))
        if not self._checked and np.min(np.abs(self.anchors - f)) > 0.25 * self.step:
            self._checked = True
            self.report_error(f, Z)
        return Z

    def point(self, f, keep_currents=False, solver=None):
        """One sweep point with the interpolated Z: the outputs of
        Solver.point (S, z0, gamma, z0_line, residual, currents, info).
        solver: a concurrent worker of the sweep (its own engine context) that
        reads resident anchors; default the solver of setup."""
        sol = solver or self.solver
        if sol.Lm is not None:  # lumped loads: the interpolated Z through the host solve and Woodbury
            if sol is not self.solver:
                raise RuntimeError("lumped loads with an interpolated Z run on the sweep's own solver")
            g = sol.greens(f)
            out = sol._lumped_point(f, g, self.impedance(f), keep_currents)
            g.close()
            return out
        idx = self._window(f)
        if sol is not self.solver:
            if not self._resident or any(i not in self._slot_of for i in idx):
                raise RuntimeError("another worker's point needs resident, filled anchors (fill_all)")
            slots = np.array([self._slot_of[i] for i in idx], np.int32)
        else:
            if not self._checked and np.min(np.abs(self.anchors - f)) > 0.25 * self.step:
                self.impedance(f)  # prints the check
            slots = np.array(self._slots(idx), np.int32)
        L = self.weights(f, idx)
        g = sol.greens(f)
        P = len(sol.ports)
        n = sol.mesh.n_unknowns
        S = np.zeros((P, P), complex)
        z0 = np.zeros(P)
        gam = np.zeros(P, complex)
        zl = np.zeros(P, complex)
        res = np.zeros(P)
        x = np.zeros((n, P), complex) if keep_currents else None
        info = np.zeros(2, np.int32)
        b0 = E.f64(sol.beta0(f))
        F = lambda a: E.ptr(a.view(np.float64)) if a is not None else None  # noqa: E731
        prec = E.M25_MIXED if sol.precision == "mixed" else E.M25_FP64
        E.check(sol.ctx.lib.m25_interp_point(
            sol.ctx.h, sol.geometry().h, g.h, sol.port_data().h, self._ip.h, len(idx), E.ptr(slots, C.c_int32),
            E.ptr(L), self.ke(f), prec, E.ptr(b0), sol.refine_tol, sol.max_refine, F(x), F(S), E.ptr(z0), F(gam),
            F(zl), E.ptr(res), E.ptr(info, C.c_int32)))
        g.close()
        return sol._fixed_z0(S, z0) + (gam, zl, res, x, dict(refine_steps=int(info[0]),
                                                               fp64_fallback=bool(info[0] < 0),
                                                               waves=sol.last_waves()))

    def report_error(self, f, Zi=None):
        """Fill Z exactly at f and compare: the relative Frobenius error of
        the interpolated Z in each block (RWG-RWG, RWG-via and via-via,
        taken apart because the via entries are orders of magnitude larger);
        prints them and returns the worst (Engine/mom25d/freqinterp.py:151-170)."""
        Zi = self.impedance(f) if Zi is None else Zi
        Ze = self.solver.impedance(f, precision="fp64")
        nb = self.nb
        blocks = {"RWG": (slice(0, nb), slice(0, nb)), "RWG-via": (slice(0, nb), slice(nb, None)),
                  "via-via": (slice(nb, None), slice(nb, None))}
        errs = {}
        for k, (a, b) in blocks.items():
            ne = np.linalg.norm(Ze[a, b])
            if ne > 0:
                errs[k] = np.linalg.norm(Zi[a, b] - Ze[a, b]) / ne
        err = max(errs.values())
        spacing = np.diff(self.anchors).mean() / 1e9
        parts = "; ".join(f"{k}: {v:.1e}" for k, v in errs.items())
        print(f"  interpolated Z vs exact fill at {f / 1e9:.4f} GHz -- {parts} "
              f"[order {self.order}, anchor spacing {spacing:.3g} GHz]")
        self.last_error = err
        return err

    def close(self):
        if self._ip is not None:
            self._ip.close()
            self._ip = None


def basis_centres(solver):
    """(N, 3) centres of the unknowns: RWG edge midpoints on their level, via
    segments at mid-span between their end levels (freqinterp.py:60-71)."""
    m = solver.mesh
    zl = solver.zl[m.edge_layer]
    pos = np.c_[m.edge_mid, zl]
    segs = getattr(m, "via_segments", None) or []
    if segs:
        st = solver.stack
        via_z = {n: st.level_z(n) for n in list(m.layer_names) + list(getattr(m, "planes", []))}
        via_z["gnd"] = 0.0
        zc = [0.5 * (via_z[g["bottom"]] + via_z[g["top"]]) for g in segs]
        xy = [m.vias[g["via"]].xy for g in segs]
        pos = np.r_[pos, np.c_[xy, zc]]
    return pos


def eps_eff(solver):
    """Quasi-static eps_eff of the stack under the first port's level, for the
    phase extraction only (freqinterp.py:199-209)."""
    st = solver.stack
    layer = solver.ports[0].layer if solver.ports else solver.mesh.layer_names[0]
    e = st.eps_below(layer)
    return e if st.covered(layer) else 0.5 * (e + 1)
