"""ORACLE (test infrastructure only; never imported by the product path).

CPU restatement of mom25d's spectral-domain Green's functions and the
closed-form 1/R triangle integrals, used to check the CUDA engine:

  slab kernels         mom25d/greens.py:82-212   (GroundedSlabGreens)
  layered kernels      mom25d/layered.py:238-405 (LayeredGreens: TL recursion,
                       leading terms, tabulation)
  potential integrals  mom25d/integrals.py:24-67 (Wilton et al. 1984)

Third-party arithmetic it relies on, as mom25d does: scipy.special j0 / jv
(real / complex J0), scipy.interpolate.CubicSpline (not-a-knot).
"""

import numpy as np
from scipy.interpolate import CubicSpline
from scipy.special import j0, jv

C0 = 299792458.0
MU0 = 4e-7 * np.pi
EPS0 = 1.0 / (MU0 * C0 ** 2)

# Dunavant degree-5 7-point and the 3-point rule (barycentric; weights sum to 1),
# mom25d/integrals.py:5-16
_A1, _B1 = 0.059715871789770, 0.470142064105115
_A2, _B2 = 0.797426985353087, 0.101286507323456
TRI7_BARY = np.array([[1 / 3, 1 / 3, 1 / 3], [_A1, _B1, _B1], [_B1, _A1, _B1], [_B1, _B1, _A1],
                      [_A2, _B2, _B2], [_B2, _A2, _B2], [_B2, _B2, _A2]])
TRI7_W = np.array([0.225] + [0.132394152788506] * 3 + [0.125939180544827] * 3)
TRI3_BARY = np.array([[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3]])
TRI3_W = np.full(3, 1 / 3)


def quad_points(verts, bary):
    return np.einsum("kv,nvd->nkd", bary, verts)


def potential_integrals(verts, r, d=0.0):
    """I0 = Int_T 1/R dS', I1 = Int_T (r' - r)/R dS' (in-plane part) for
    triangles verts (N,3,2) and observers r (K,2) at height d above the
    plane (mom25d/integrals.py:24-67): sum over the three edges of the
    edge-line terms (log and, off-plane, arctan)."""
    d = abs(float(d))
    I0 = np.zeros((verts.shape[0], r.shape[0]))
    I1 = np.zeros((verts.shape[0], r.shape[0], 2))
    for i in range(3):
        a = verts[:, (i + 1) % 3][:, None, :]
        b = verts[:, (i + 2) % 3][:, None, :]
        e = b - a
        le = np.sqrt((e * e).sum(-1, keepdims=True))
        t_hat = e / le
        n_hat = np.stack([t_hat[..., 1], -t_hat[..., 0]], -1)
        da, db = a - r[None], b - r[None]
        sa, sb = (da * t_hat).sum(-1), (db * t_hat).sum(-1)
        p = (da * n_hat).sum(-1)
        Ra = np.sqrt(da[..., 0] ** 2 + da[..., 1] ** 2 + d * d)
        Rb = np.sqrt(db[..., 0] ** 2 + db[..., 1] ** 2 + d * d)
        q2 = p * p + d * d
        with np.errstate(divide="ignore", invalid="ignore"):
            fb = np.where(sb >= 0, Rb + sb, q2 / (Rb - sb))
            fa = np.where(sa >= 0, Ra + sa, q2 / (Ra - sa))
            lg = np.log(fb / fa)
        lg = np.where(np.sqrt(q2) <= 1e-12 * le[..., 0], 0.0, lg)
        I0 += p * lg
        if d:
            I0 -= d * (np.arctan2(p * sb, q2 + d * Rb) - np.arctan2(p * sa, q2 + d * Ra))
        I1 += 0.5 * n_hat * (q2 * lg + sb * Rb - sa * Ra)[..., None]
    return I0, I1


def gauss_panels(a, b, n_panels, order):
    x, w = np.polynomial.legendre.leggauss(order)
    edges = np.linspace(a, b, n_panels + 1)
    half = 0.5 * np.diff(edges)
    mid = 0.5 * (edges[1:] + edges[:-1])
    return (mid[:, None] + half[:, None] * x).ravel(), (half[:, None] * w).ravel()


def sqrt_re_pos(z):
    s = np.sqrt(z)
    return np.where(s.real < 0, -s, s)


def rho_grid(rho_max, lam, tmin):
    """Tabulation radii: step min(lambda/80, max(t/25, rho/25)) from 0 past rho_max
    (mom25d/greens.py:180-183, layered.py:384-387)."""
    r = [0.0]
    while r[-1] < rho_max:
        r.append(r[-1] + min(lam / 80, max(tmin / 25, r[-1] / 25)))
    return np.array(r)


def lifted_path(k0, kref, tmin, rho_max, order=12):
    """Sommerfeld path: a sine-lifted arc over [0, T] then the real axis to
    kmax (mom25d/greens.py:138-155, layered.py:343-358)."""
    T = 1.3 * kref + k0
    a = min(0.5 * k0, 1.0 / rho_max)
    n1 = int(np.clip(np.ceil(2 * T / a), 100, 3000))
    t, w = gauss_panels(0.0, T, n1, order)
    kc = t + 1j * a * np.sin(np.pi * t / T)
    wc = w * (1 + 1j * a * np.pi / T * np.cos(np.pi * t / T))
    kmax = max(40 * kref, 20.0 / tmin, T * 1.5)
    dk = min(np.pi / rho_max, 0.5 / tmin, kref)
    n2 = int(np.ceil((kmax - T) / dk))
    kr, wr = gauss_panels(T, kmax, n2, 8)
    return kc, wc, kr, wr


def hankel_sum(rho, coef, k, real_axis):
    """(nrho, ncoef): sum_k J0(k rho) coef[k, :]."""
    out = np.empty((rho.size, coef.shape[1]), complex)
    step = max(1, int(4e6 // k.size))
    for s in range(0, rho.size, step):
        arg = np.outer(rho[s:s + step], k)
        J = j0(arg.real) if real_axis else jv(0, arg)
        out[s:s + step] = J @ coef
    return out


class Pair:
    """Kernels between two levels: g = c / (4 pi R) + S(rho), R = sqrt(rho^2 + dz^2)."""

    def __init__(self, dz, cA, cV, cW, rho, SA, SV, SW):
        self.dz, self.cA, self.cV, self.cW = dz, cA, cV, cW
        self.rho = rho
        self.spl = CubicSpline(rho, np.stack([SA, SV], -1))
        self.splw = CubicSpline(rho, SW)

    def smooth(self, rho):
        S = self.spl(rho)
        return S[..., 0], S[..., 1]

    def smooth_w(self, rho):
        return self.splw(rho)

    def R(self, rho):
        return np.sqrt(np.asarray(rho) ** 2 + self.dz ** 2)

    def gA(self, rho):
        return self.cA / (4 * np.pi * self.R(rho)) + self.smooth(rho)[0]

    def gV(self, rho):
        return self.cV / (4 * np.pi * self.R(rho)) + self.smooth(rho)[1]

    def gW(self, rho):
        return self.cW / (4 * np.pi * self.R(rho)) + self.smooth_w(rho)


class SlabKernels:
    """One grounded slab, conductors on top (mom25d/greens.py:82-212)."""

    def __init__(self, freq, eps_r, h, tand=0.0, rho_max=0.1, zs_ground=0.0):
        self.freq, self.h = freq, h
        self.omega = 2 * np.pi * freq
        self.k0 = k0 = self.omega / C0
        self.epsc = e = eps_r * (1 - 1j * tand)
        self.k1 = k1 = k0 * np.sqrt(e)
        self.ka = np.sqrt(0.5 * (k0 ** 2 + k1 ** 2))
        self.cv = 2.0 / (e + 1.0)
        self.kv = np.sqrt((e * k0 ** 2 + k1 ** 2) / (e + 1.0))
        self.levels = ["top"]
        kc, wc, kr, wr = lifted_path(k0, abs(k1), h, rho_max)
        rho = rho_grid(rho_max, 2 * np.pi / abs(k1), h)
        res = 0.0
        for k, w, real in ((kc, wc, False), (kr, wr.astype(complex), True)):
            coef = np.stack([w * k * g / (2 * np.pi) for g in self.remainder(k.astype(complex))], 1)
            res = res + hankel_sum(rho, coef, k.real if real else k, real)
        with np.errstate(divide="ignore", invalid="ignore"):
            fa = np.where(rho > 0, np.expm1(-1j * self.ka * rho) / (4 * np.pi * rho), -1j * self.ka / (4 * np.pi))
            fv = np.where(rho > 0, np.expm1(-1j * self.kv * rho) / (4 * np.pi * rho), -1j * self.kv / (4 * np.pi))
        loss = 0.0
        if zs_ground:
            d = 2 * h
            loss = zs_ground / (1j * self.omega * MU0) * d / (2 * np.pi * (rho ** 2 + d ** 2) ** 1.5)
        self.rho_tab = rho
        self.SA = fa + res[:, 0] + loss
        self.SV = self.cv * fv + res[:, 1]
        self.SW = self.cv * fv + res[:, 2]
        self._pair = Pair(0.0, 1.0, self.cv, self.cv, rho, self.SA, self.SV, self.SW)

    def spectral(self, kr):
        k0, k1, h, e = self.k0, self.k1, self.h, self.epsc
        u0 = np.sqrt(kr ** 2 - k0 ** 2)
        u1 = sqrt_re_pos(kr ** 2 - k1 ** 2)
        x = u1 * h
        ex = np.exp(-2 * x)
        small = np.abs(x) < 1e-4
        with np.errstate(divide="ignore", invalid="ignore"):
            coth = np.where(small, 1 / h + u1 ** 2 * h / 3, u1 * (1 + ex) / (1 - ex))
            tanh = np.where(small, u1 ** 2 * h, u1 * (1 - ex) / (1 + ex))
            t_over_u = np.where(small, h, tanh / u1 ** 2)
        dte = u0 + coth
        dtm = e * u0 + tanh
        return 1.0 / dte, (u0 + tanh) / (dte * dtm), u0 * t_over_u / dtm

    def remainder(self, kr):
        gA, gV, gW = self.spectral(kr)
        ua = np.sqrt(kr ** 2 - self.ka ** 2)
        uv = np.sqrt(kr ** 2 - self.kv ** 2)
        return gA - 0.5 / ua, gV - 0.5 * self.cv / uv, gW - 0.5 * self.cv / uv

    def pair(self, i=0, j=0):
        return self._pair


class LayeredKernels:
    """Open multilayer stack, transmission-line form of Michalski & Zheng
    (mom25d/layered.py:217-405): TE/TM line voltages per level, leading
    c e^{-jkR}/(4 pi R) terms, remainder tabulated per level pair."""

    def __init__(self, freq, layers, il, zl, rho_max=0.1, zs_ground=0.0, top="air"):
        """layers [(t, eps_r, tand)] bottom to top; il: interface index of each
        mesh level (1..N); zl: its height; top: "air" or "pec" (a cover on
        the top layer, mom25d/layered.py:257-275)."""
        self.pec_top = top == "pec"
        self.freq = freq
        self.omega = 2 * np.pi * freq
        self.k0 = k0 = self.omega / C0
        self.t = np.array([d[0] for d in layers], float)
        self.epsc = np.array([d[1] * (1 - 1j * d[2]) for d in layers])
        self.kk = k0 * np.sqrt(self.epsc)
        self.il = np.asarray(il, int)
        self.zl = np.asarray(zl, float)
        self.h = float(self.t.sum())
        L = len(self.il)
        self.dz = np.abs(self.zl[:, None] - self.zl[None, :])
        self._leading()
        kref = np.abs(self.kk).max()
        tmin = self.t.min()
        kc, wc, kr, wr = lifted_path(k0, kref, tmin, rho_max)
        rho = rho_grid(rho_max, 2 * np.pi / kref, tmin)
        res = 0.0
        for k, w, real in ((kc, wc, False), (kr, wr.astype(complex), True)):
            rem = np.stack(self.remainder(k.astype(complex)))  # (3, L, L, K)
            coef = (w * k / (2 * np.pi))[None] * rem.reshape(-1, k.size)
            res = res + hankel_sum(rho, coef.T, k.real if real else k, real)
        res = res.T.reshape(3, L, L, rho.size)
        self.rho_tab = rho
        self.pairs = {}
        for i in range(L):
            for j in range(L):
                R = np.sqrt(rho ** 2 + self.dz[i, j] ** 2)
                S = []
                for m in range(3):
                    k = self.kx[min(m, 1), i, j]
                    with np.errstate(divide="ignore", invalid="ignore"):
                        f = np.where(R > 0, np.expm1(-1j * k * R) / (4 * np.pi * R), -1j * k / (4 * np.pi))
                    S.append(self.c[m, i, j] * f + res[m, i, j])
                if zs_ground:
                    d = self.zl[i] + self.zl[j]
                    S[0] = S[0] + zs_ground / (1j * self.omega * MU0) * d / (2 * np.pi * (rho ** 2 + d ** 2) ** 1.5)
                self.pairs[i, j] = Pair(self.dz[i, j], *self.c[:, i, j], rho, *S)

    def line_voltages(self, kr):
        """TE and TM interface voltages (L, N+1, K) for unit currents at each level."""
        N, K, L = len(self.t), kr.size, len(self.il)
        u = np.stack([sqrt_re_pos(kr ** 2 - k ** 2) for k in self.kk])
        u0 = np.sqrt(kr ** 2 - self.k0 ** 2)
        x = u * self.t[:, None]
        ex = np.exp(-2 * x)
        T = (1 - ex) / (1 + ex)
        Sh = 2 * np.exp(-x) / (1 + ex)
        out = []
        for y, yair in ((u, u0), (self.epsc[:, None] / u, 1.0 / u0)):
            ydn = np.empty((N + 1, K), complex)
            ydn[1] = y[0] / T[0]
            for k in range(2, N + 1):
                yl, yk, tk = ydn[k - 1], y[k - 1], T[k - 1]
                ydn[k] = yk * (yl + yk * tk) / (yk + yl * tk)
            yup = np.empty((N + 1, K), complex)
            if not self.pec_top:
                yup[N] = yair
            for k in range(N - 1, 0, -1):
                yk, tk = y[k], T[k]
                if k == N - 1 and self.pec_top:  # layer N shorted by the cover
                    yup[k] = yk / tk
                else:
                    yl = yup[k + 1]
                    yup[k] = yk * (yl + yk * tk) / (yk + yl * tk)
            V = np.zeros((L, N + 1, K), complex)
            for l, s in enumerate(self.il):
                V[l, s] = 1.0 / (ydn[s] + yup[s])
                for k in range(s, 1, -1):
                    V[l, k - 1] = V[l, k] * Sh[k - 1] / (1 + ydn[k - 1] / y[k - 1] * T[k - 1])
                for k in range(s, N):
                    if k + 1 == N and self.pec_top:
                        break  # V_N = 0 on the cover
                    V[l, k + 1] = V[l, k] * Sh[k] / (1 + yup[k + 1] / y[k] * T[k])
            out.append(V)
        return out[0], out[1], u

    def spectral(self, kr):
        Vh, Ve, u = self.line_voltages(kr)
        il = self.il
        gA = Vh[:, il].transpose(1, 0, 2)
        gV = ((Ve[:, il] + self.k0 ** 2 * Vh[:, il]) / kr ** 2).transpose(1, 0, 2)
        cum = np.cumsum(np.diff(Ve, axis=1) / u[None] ** 2, axis=1)
        gW = cum[:, il - 1].transpose(1, 0, 2)
        return gA, gV, gW

    def _leading(self):
        L = len(self.il)
        N = len(self.t)
        self.c = np.zeros((3, L, L), complex)
        self.kx = np.zeros((2, L, L), complex)
        kbig = 15.0 / self.t.min()
        big = None
        for i in range(L):
            for j in range(L):
                if i == j:
                    n = self.il[i]
                    eb, kb = self.epsc[n - 1], self.kk[n - 1]
                    ea, ka = (1.0, self.k0) if n == N else (self.epsc[n], self.kk[n])
                    cv = 2.0 / (ea + eb)
                    self.c[:, i, j] = (1.0, cv, cv)
                    self.kx[0, i, j] = np.sqrt(0.5 * (ka ** 2 + kb ** 2))
                    self.kx[1, i, j] = np.sqrt((eb * ka ** 2 + ea * kb ** 2) / (ea + eb))
                    continue
                if big is None:
                    big = [g[..., 0] for g in self.spectral(np.array([kbig], complex))]
                ux = np.sqrt(kbig ** 2 - self.k0 ** 2 + 0j)
                f = 2 * ux * np.exp(ux * self.dz[i, j])
                cA, cV, cW = (f * g[i, j] for g in big)
                if self.zl[j] < self.zl[i]:
                    cW = 0.0
                self.c[:, i, j] = (cA, cV, cW)
                self.kx[:, i, j] = self.k0
        self.c = np.where(np.abs(self.c.imag) < 1e-9 * np.abs(self.c), self.c.real, self.c)

    def remainder(self, kr):
        out = []
        for m, g in enumerate(self.spectral(kr)):
            kx = self.kx[min(m, 1)]
            ux = np.sqrt(kr[None, None] ** 2 - kx[..., None] ** 2)
            out.append(g - self.c[m][..., None] * np.exp(-ux * self.dz[..., None]) / (2 * ux))
        return out

    def pair(self, i, j):
        return self.pairs[i, j]
