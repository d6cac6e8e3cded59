"""Solver / sweep API of mom25d (Engine/mom25d/solver.py:673-1335) on the
GB300 engine.

The Python layer keeps mom25d's objects and their meaning (Solver, sweep,
SweepResult, PortModel data, port groups, checkpoint keys) and prepares the
small frequency-independent host arrays: test blocks, port cuts and voltage
points, the Sommerfeld path and tabulation radii of each frequency. Every
per-frequency computation of the sweep path runs on the GPU through the C
ABI: Green's tables, impedance fill, LU + solve, de-embedding. There is no
CPU fallback; without the CUDA library or a device the constructor raises.
"""

import ctypes as C
import os
import threading
import time
import zlib
from dataclasses import dataclass

import numpy as np

from . import analytic
from . import engine as E
from .constants import C0, EPS0, MU0

# ------------------------------------------------------------- host prep
_A1, _B1 = 0.059715871789770, 0.470142064105115
_A2, _B2 = 0.797426985353087, 0.101286507323456
TRI7_BARY = np.array([[1 / 3, 1 / 3, 1 / 3], [_A1, _B1, _B1], [_B1, _A1, _B1], [_B1, _B1, _A1],
                      [_A2, _B2, _B2], [_B2, _A2, _B2], [_B2, _B2, _A2]])
TRI7_W = np.array([0.225] + [0.132394152788506] * 3 + [0.125939180544827] * 3)


def morton_order(xy):
    """Z-order of points on a 16-bit lattice over their bounding square
    (ties keep input order); mom25d groups its test triangles the same way
    (Engine/mom25d/solver.py:294-304), which fixes the near/mid/far blocks."""
    span = max(float(np.ptp(xy, 0).max()), 1e-30)
    q = ((xy - xy.min(0)) / span * 65535).astype(np.uint64)

    def interleave(v):
        for shift, mask in ((8, 0x00FF00FF), (4, 0x0F0F0F0F), (2, 0x33333333), (1, 0x55555555)):
            v = (v | (v << np.uint64(shift))) & np.uint64(mask)
        return v

    return np.argsort(interleave(q[:, 0]) | (interleave(q[:, 1]) << np.uint64(1)), kind="stable")


def test_blocks(mesh, block=32):
    """(nblocks, 32) triangle slots: per level, Morton order, blocks of 32."""
    out = []
    tl = mesh.tri_layer
    for lt in range(len(mesh.layer_names)):
        on = np.nonzero(tl == lt)[0]
        if not on.size:
            continue
        order = on[morton_order(mesh.centroid[on])]
        for p0 in range(0, order.size, block):
            row = -np.ones(block, np.int32)
            pb = order[p0:p0 + block]
            row[:pb.size] = pb
            out.append(row)
    return np.stack(out)


def gauss_panels(a, b, n_panels, order):
    x, w = np.polynomial.legendre.leggauss(order)
    edges = np.linspace(a, b, n_panels + 1)
    half = 0.5 * np.diff(edges)
    mid = 0.5 * (edges[1:] + edges[:-1])
    return (mid[:, None] + half[:, None] * x).ravel(), (half[:, None] * w).ravel()


def sommerfeld_path(k0, kref, tmin, rho_max, order=12):
    """Lifted arc k = t + j a sin(pi t / T) over [0, T] (Gauss-Legendre panels)
    and the real axis [T, kmax]: T = 1.3 kref + k0, a = min(k0/2, 1/rho_max)
    (Engine/mom25d/greens.py:261-278, layered.py:343-358)."""
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


def tabulation_radii(rho_max, lam, tmin):
    """rho grid: steps min(lambda/80, max(t_min/25, rho/25)) up to rho_max
    (Engine/mom25d/greens.py:298-306)."""
    r = [0.0]
    while r[-1] < rho_max:
        r.append(r[-1] + min(lam / 80, max(tmin / 25, r[-1] / 25)))
    return np.array(r)


class Greens:
    """Green's tables of one frequency on the device (GroundedSlabGreens /
    LayeredGreens): rho grid, S_A/S_V/S_W tables, cubic coefficients."""

    def __init__(self, solver, freq, rho=None, surrogate=True):
        """rho: tabulation radii (default: mom25d's grid for this frequency);
        surrogate: use the solver's learned remainder when it covers freq."""
        st, mesh = solver.stack, solver.mesh
        self.freq = float(freq)
        self.omega = 2 * np.pi * freq
        self.k0 = k0 = self.omega / C0
        layers = st.layers
        eps = np.array([d.eps_r * (1 - 1j * d.tand) for d in layers])
        kk = k0 * np.sqrt(eps)
        t = np.array([d.t for d in layers], float)
        single = solver.single
        kref = abs(kk[0]) if single else np.abs(kk).max()
        tmin = t[0] if single else t.min()
        kc, wc, kr, wr = sommerfeld_path(k0, kref, tmin, solver.rho_max)
        self.rho = tabulation_radii(solver.rho_max, 2 * np.pi / kref, tmin) if rho is None else np.asarray(rho, float)
        zg = st.surface_impedance(freq) if st.ground_loss else 0.0
        zg = complex(zg)
        self.levels = list(mesh.layer_names)
        L = len(self.levels)
        arrs = dict(lt=E.f64(t), le=E.f64([d.eps_r for d in layers]), ld=E.f64([d.tand for d in layers]),
                    il=E.i32([st.metals[n] for n in self.levels]), lz=E.f64(solver.zl),
                    kc=E.f64(np.stack([kc.real, kc.imag], 1)), wc=E.f64(np.stack([wc.real, wc.imag], 1)),
                    kr=E.f64(kr), wr=E.f64(wr), rho=E.f64(self.rho))
        d = E.GreensDesc(self.freq, len(layers), E.ptr(arrs["lt"]), E.ptr(arrs["le"]), E.ptr(arrs["ld"]), L,
                         E.ptr(arrs["il"], C.c_int32), E.ptr(arrs["lz"]), int(single), zg.real, zg.imag,
                         float(st.z[-1]), kc.size, kr.size, E.ptr(arrs["kc"]), E.ptr(arrs["wc"]), E.ptr(arrs["kr"]),
                         E.ptr(arrs["wr"]), self.rho.size, E.ptr(arrs["rho"]), 15.0 / t.min())
        d.top_pec = int(getattr(st, "top", "air") == "pec")
        sur = getattr(solver, "surrogate", None) if surrogate else None
        self.surrogate_used = None
        if sur is not None and sur.covers(self.freq):
            arrs["sur_scale"] = E.f64(sur.scale)
            sur.fill_desc(d, E.ptr(arrs["sur_scale"]))
        h = C.c_void_p()
        E.check(solver.ctx.lib.m25_greens_create(solver.ctx.h, C.byref(d), C.byref(h)))
        self._h = E.Handle(solver.ctx, h, solver.ctx.lib.m25_greens_destroy)
        self.nlev = L
        self.h = h

    def remainder(self):
        """(res (nrho, 3 L^2) complex128, info): the Sommerfeld remainder of the
        tables (columns [A, V, W] x level pairs (i, j)), info = (learned
        remainder used, its judged relative error, number of radii the
        Sommerfeld integral ran at)."""
        res = np.zeros((self.rho.size, 3 * self.nlev ** 2), complex)
        info = np.zeros(3)
        E.check(self._h.ctx.lib.m25_greens_remainder(self.h, E.ptr(res.view(np.float64)), E.ptr(info)))
        return res, (bool(info[0]), float(info[1]), int(info[2]))

    def tables(self):
        """(S (3,L,L,nrho), c (3,L,L), coef (L*L, nrho-1, 4, 3)) complex128 host copies."""
        L, n = self.nlev, self.rho.size
        S = np.zeros((3, L, L, n), complex)
        c = np.zeros((3, L, L), complex)
        coef = np.zeros((L * L, n - 1, 4, 3), complex)
        E.check(self._h.ctx.lib.m25_greens_tables(self.h, E.ptr(S.view(np.float64)), E.ptr(c.view(np.float64)),
                                                  E.ptr(coef.view(np.float64))))
        return S, c, coef

    def close(self):
        self._h.close()


class PortModel:
    """The per-feed data of the de-embedding (Engine/mom25d/solver.py:570-610).

    - s: the grid cuts of the feed inside its fitting window, which keeps
      `margin` (default max(1.5 width, 4 h), h the height of the feed's level
      over ground) clear of the reference plane and of the delta gap; the
      wave fit needs at least four.
    - cuts: per window cut, the RWG edges on it and their signs
      (Mesh.cut_edges): the current toward the circuit is
      sum(sign * edge_len * x).
    - excitation: a 1 V delta gap at the gap cut, i.e. the signed edge
      lengths of the edges on that cut.
    - vpts: where the line voltage is sampled, 8 points per window cut: at
      -0.3, -0.1, 0.1 and 0.3 widths across the strip, on both sides of the
      cut at half the distance to the nearer neighbouring grid cut (the two
      sides average out the ripple of the alternating cell diagonals).
    """

    FRACTIONS = np.array([-0.3, -0.1, 0.1, 0.3])  # across the strip, in widths

    def __init__(self, mesh, port, h):
        self.port = port
        keep = port.margin if port.margin is not None else max(1.5 * port.width, 4 * h)
        grid_cuts = mesh.cut_positions(port)
        s = grid_cuts[(grid_cuts >= keep - 1e-12) & (grid_cuts <= port.s_gap - keep + 1e-12)]
        if s.size < 4:
            raise ValueError(f"port {port.name}: the wave fit needs 4 grid cuts between {keep * 1e3:.3g} mm "
                             f"and {(port.s_gap - keep) * 1e3:.3g} mm along the feed and found {s.size}; "
                             "lengthen the feed or refine the mesh")
        self.s = s
        self.cuts = [mesh.cut_edges(port, si) for si in s]
        gap_edges, gap_sign = mesh.cut_edges(port, port.s_gap)
        if gap_edges.size == 0:
            raise ValueError(f"port {port.name}: no mesh edge lies on the delta-gap cut")
        self.excitation = np.zeros(mesh.n_unknowns)
        self.excitation[gap_edges] = gap_sign * mesh.edge_len[gap_edges]
        self.len = mesh.edge_len
        # distance to the nearer neighbouring grid cut (inf on a side that has none)
        k = np.searchsorted(grid_cuts, s)
        back = s - grid_cuts[np.maximum(k - 1, 0)]
        ahead = grid_cuts[np.minimum(k + 1, grid_cuts.size - 1)] - s
        half = 0.5 * np.minimum(np.where(back > 0, back, np.inf), np.where(ahead > 0, ahead, np.inf))
        both_sides = np.stack([s - half, s + half], 1)  # (Ns, 2)
        pts = port.point(both_sides[:, :, None], self.FRACTIONS * port.width)  # (Ns, 2, 4, 2)
        self.vpts = pts.reshape(-1, 2)
        self.nper = 2 * self.FRACTIONS.size


@dataclass
class SweepResult:
    freqs: np.ndarray
    S: np.ndarray  # (F,P,P), referenced to each port's line impedance z0
    z0: np.ndarray  # (F,P)
    gamma: np.ndarray  # (F,P)
    z0_line: np.ndarray  # (F,P)
    fit_residual: np.ndarray  # (F,P)
    port_names: list
    currents: list = None  # per frequency: (N, P) coefficients (keep_currents=True)
    waves: np.ndarray = None  # (F, P, P) incident current-wave amplitudes A [port, excitation]
    info: dict = None

    @property
    def eeff(self):
        k0 = 2 * np.pi * self.freqs / C0
        return (self.gamma.imag / k0[:, None]) ** 2

    def renormalize(self, zref=50.0):
        """S-parameters referenced to a common real impedance zref."""
        out = np.empty_like(self.S)
        eye = np.eye(self.S.shape[1])
        for f, S in enumerate(self.S):
            sq = np.diag(np.sqrt(self.z0[f]))
            Zm = sq @ (eye + S) @ np.linalg.inv(eye - S) @ sq
            out[f] = (Zm - zref * eye) @ np.linalg.inv(Zm + zref * eye)
        return out

    def matched_currents(self, fi, port):
        """Coefficients at frequency index fi for a unit incident current wave
        on `port`, the other ports terminated in their line impedance: the
        delta-gap solutions combined by the inverse of the wave amplitudes
        (Engine/mom25d/solver.py:685-694)."""
        if self.currents is None or self.waves is None:
            raise ValueError("run sweep(..., keep_currents=True)")
        e = np.zeros(self.waves.shape[1])
        e[port] = 1.0
        return self.currents[fi] @ np.linalg.solve(self.waves[fi], e)

    def wave_currents(self, fi, a50, z0=50.0):
        """Coefficients at frequency index fi for incident power waves a50
        (one per port, reference z0) at the ports (solver.py:740-750)."""
        if self.currents is None or self.waves is None:
            raise ValueError("run sweep(..., keep_currents=True)")
        a = np.asarray(a50, complex)
        b = self.renormalize(z0)[fi] @ a
        V = np.sqrt(z0) * (a + b)  # port voltage and current into the layout
        I = (a - b) / np.sqrt(z0)
        A = 0.5 * (I + V / self.z0[fi])  # incident current waves on the line reference
        return self.currents[fi] @ np.linalg.solve(self.waves[fi], A)

    def connect(self, model, pairs, z0=None, name=None):
        """Join S-parameter blocks to ports of this result (solver.py:711-738).
        model: network.Touchstone or a .sNp path; pairs: [(port name or
        index, block port 1..n), ...]; z0: common reference (default the
        block's). Returns a network.Network on the remaining ports: the
        layout's, then the block's free ports named '<name>.<k>'."""
        from .network import Network, Touchstone, connect

        if isinstance(model, str):
            model = Touchstone(model)
        z0 = z0 or getattr(model, "z0", 50.0)
        name = name or getattr(model, "path", "block").rsplit("/", 1)[-1].rsplit(".", 1)[0]
        SA = self.renormalize(z0)
        SB = np.array([model.s(f) for f in self.freqs])
        na = SA.shape[-1]
        pa = [(self.port_names.index(a) if isinstance(a, str) else int(a), int(b) - 1) for a, b in pairs]
        S, idx = connect(SA, SB, pa)
        names = [self.port_names[i] if i < na else f"{name}.{i - na + 1}" for i in idx]
        net = Network(self.freqs, S, names, z0)
        net._source = (self, model, pa, idx, z0)
        return net

    def db(self, i, j, S=None):
        S = self.S if S is None else S
        return 20 * np.log10(np.abs(S[:, i, j]))

    def write_touchstone(self, path, zref=50.0):
        S = self.S if zref is None else self.renormalize(zref)
        z = zref if zref is not None else float(np.mean(self.z0))
        n = S.shape[1]
        with open(path, "w") as fh:
            fh.write(f"! mom25d_gb300 2.5D MoM. ports: {', '.join(self.port_names)}\n")
            fh.write(f"# HZ S RI R {z:g}\n")
            for f, Sf in zip(self.freqs, S):
                vals = Sf.T.ravel() if n == 2 else Sf.ravel()
                fh.write(f"{f:.9e} " + " ".join(f"{v.real:.9e} {v.imag:.9e}" for v in vals) + "\n")


PRECISIONS = {"fp64": E.M25_FP64, "mixed": E.M25_MIXED, "mixed_fill32": E.M25_MIXED_FILL32}


class Solver:
    """mom25d.Solver on the GB300 engine.

    mesh      : a Mesh with RWG data, via segments and port cuts (this
                package's grid mesher, or mom25d's own Mesh object)
    substrate : Substrate or Stackup (air above or a PEC cover; no inner planes)
    method    : "dense" (Z + LU), "hmatrix" (compressed Z + GMRES,
                mom25d_gb300/hmatrix.py) or "auto": hmatrix above HMATRIX_N
                unknowns (where the dense working set no longer fits beside
                other work on one GPU), else dense
    precision : "fp64" (fill + LU in fp64), "mixed" (fill with fp64 singular
                parts and fp32 elsewhere, complex64 LU, fp64 GMRES refinement
                to the normwise backward error refine_tol) or "mixed_fill32"
                (fp32 fill throughout: larger error in S at low frequency)
    refine_tol: backward-error target of the mixed refinement. The mixed
                fill already moves Z by ~1e-7 relative; at the 1e-12 default
                the solve adds nothing measurable to S (LPF, N = 5943:
                max |dS| against the fp64 path 7.8e-7 at 1e-12 and 7.7e-7 at
                1e-14; 1.0e-5 at 1e-9). A point whose refinement stops
                above the target is recomputed on the fp64 path
                (refine_steps -1, listed in the sweep's info["fp64_fallback"])
    """

    # "auto": the compressed solver above this many unknowns (mom25d switches at 7000,
    # Engine/mom25d/solver.py:1037, to fit host memory; one GB300 holds the mixed
    # path's dense planes of N = 60000 in about 90 GB)
    HMATRIX_N = 60000

    def __init__(self, mesh, substrate, z0=None, verbose=True, method="dense", v_weight=None, precision="fp64",
                 device=0, refine_tol=1e-12, max_refine=60):
        if method not in ("auto", "dense", "hmatrix"):
            raise ValueError("method must be 'auto', 'dense' or 'hmatrix'")
        if precision not in PRECISIONS:
            raise ValueError("precision must be 'fp64', 'mixed' or 'mixed_fill32'")
        self.mesh = mesh
        self.sub = substrate
        self.stack = st = substrate if hasattr(substrate, "layers") else substrate.to_stackup()
        missing = [n for n in mesh.layer_names if n not in st.metals]
        if missing:
            raise ValueError(f"mesh layers {missing} are not metal levels of the stackup {list(st.metals)}")
        if getattr(mesh, "n_frills", 0) or getattr(mesh, "n_ap", 0) or getattr(mesh, "n_walls", 0):
            raise ValueError("antipads, plane apertures and thick metal are not part of this engine")
        if st.top == "pec" and len(getattr(mesh, "via_segments", [])):
            raise ValueError("vias under a PEC cover (a closed section: parallel-plate via modes, "
                             "mom25d solver.py:181-188) are not part of this engine")
        self.single = len(st.layers) == 1 and st.top == "air" and list(mesh.layer_names) == ["top"]
        self.zl = np.array([st.level_z(n) for n in mesh.layer_names])
        order = sorted(list(mesh.layer_names), key=st.level_z)
        if getattr(mesh, "level_order", None) != order:
            mesh.assign_levels(order)
        self.ports = mesh.layout.ports
        # internal ports (gap and via ports): S-parameter ports of fixed
        # reference impedance, excited and terminated across a delta gap
        self.iports = list(getattr(mesh.layout, "internal_ports", []))
        if not self.ports:
            raise ValueError("layout has no feed ports (this engine de-embeds at least one feed)")
        # lumped components across delta gaps (one-port values and multi-port
        # blocks): loaded after the solve (Woodbury); via ports add their
        # columns after the lumped gaps (a gap port is a lumped gap)
        self.lumped = list(getattr(mesh.layout, "lumped", []))
        self.components = list(getattr(mesh.layout, "components", []))
        self.Lm = mesh.lumped_vectors() if self.lumped else None
        self.iport_index = []  # column of each internal port in Lm
        if self.iports:
            names = [q.name for q in self.lumped]
            vecs = mesh.internal_port_vectors()
            vias = [k for k, ip in enumerate(self.iports) if ip["kind"] == "via"]
            if vias:
                self.Lm = vecs[:, vias] if self.Lm is None else np.hstack([self.Lm, vecs[:, vias]])
            col = {k: len(names) + i for i, k in enumerate(vias)}
            self.iport_index = [names.index(ip["name"]) if ip["kind"] == "gap" else col[k]
                                for k, ip in enumerate(self.iports)]
        self.values = {}  # per-sweep overrides of lumped values
        if method == "auto":
            method = "hmatrix" if mesh.n_unknowns > self.HMATRIX_N else "dense"
        self.method = method
        self._hop = None
        self.hmatrix_options = {}  # HMatrix keyword arguments (leaf, eta, tol, kcap, prec_block)
        self.gmres_rtol = 1e-6  # relative residual of the compressed solve (mom25d: 1e-6, hmatrix.py:563)
        self.precision = precision
        self.refine_tol, self.max_refine = refine_tol, max_refine
        self.z0_fixed = None if z0 is None else np.asarray(z0, float)
        v = mesh.nodes
        self.rho_max = 1.02 * np.hypot(*(v.max(0) - v.min(0)))
        self.verbose = verbose
        self.surrogate = None  # a GreensSurrogate (mom25d_gb300.surrogate) for the Green's tables
        # the engine's knobs of a mixed-precision sweep: "table" -> by N from the table measured
        # on the device (mom25d_gb300/tuning.json, autotune.py), a Tuning, or None (process defaults)
        self.tuning = "table"
        self.v_weight = 1.0 if v_weight is None else float(v_weight)
        self.pm = [PortModel(mesh, p, st.level_h(p.layer)) for p in self.ports]
        self.groups = {}
        for p, port in enumerate(self.ports):
            hp = st.level_h(port.layer)
            key = (round(port.width / hp, 9), port.layer,
                   port.ground.key(hp) if port.ground is not None else None, port.z0_from)
            self.groups.setdefault(key, []).append(p)
        self.device = device
        self.ctx = E.Context(device)
        self._geom = None
        self._ports = None
        self._siblings = []  # further engine contexts for concurrent points (sweep(workers=...))
        self._sib_lock = threading.Lock()
        self._blocks_host = None  # test blocks (host), shared with the siblings

    # ----------------------------------------------------------- device data
    def geometry(self):
        """Device copy of the mesh + near/mid/far classes + closed-form near integrals."""
        if self._geom is not None:
            return self._geom
        m, st = self.mesh, self.stack
        if self._blocks_host is None:
            self._blocks_host = test_blocks(m)
        blocks = self._blocks_host
        nt, nb = len(m.tris), m.n_basis
        segs = m.via_segments
        nv = len(segs)
        lev = {n: i for i, n in enumerate(m.layer_names)}
        zmap = {n: st.level_z(n) for n in m.layer_names}
        zmap["gnd"] = 0.0
        arrs = dict(verts=E.f64(m.verts), tb=E.i32(m.tri_basis), ts=E.f64(m.tri_sign), el=E.f64(m.edge_len),
                    tl=E.i32(m.tri_layer), lz=E.f64(self.zl), et=E.i32(np.stack([m.tp, m.tm], 1)),
                    eloc=E.i32(np.stack([m.vp, m.vm], 1)), blocks=E.i32(blocks))
        if nv:
            tris = [g[e] for g in segs for e in ("top_tris", "bottom_tris") if g[e] is not None]
            pad = np.unique(np.concatenate(tris))
            pos = -np.ones(nt, int)
            pos[pad] = np.arange(pad.size)
            off, ent, w, endlev, span, xy, drill = [0], [], [], [], [], [], []
            for g in segs:
                for key, sg in (("top_tris", 1.0), ("bottom_tris", -1.0)):
                    t = g[key]
                    if t is not None:
                        a = m.area[t].sum()
                        ent += list(pos[t])
                        w += [sg / a] * len(t)
                off.append(len(ent))
                endlev.append([m.tri_layer[g["top_tris"][0]] if g["top_tris"] is not None else -1,
                               m.tri_layer[g["bottom_tris"][0]] if g["bottom_tris"] is not None else -1])
                span.append([zmap[g["bottom"]], zmap[g["top"]]])
                v = m.vias[g["via"]]
                xy.append(v.xy)
                drill.append(v.drill)
            arrs.update(pad=E.i32(pad), off=E.i32(off), ent=E.i32(ent), w=E.f64(w), endlev=E.i32(endlev),
                        span=E.f64(span), xy=E.f64(xy), drill=E.f64(drill))
        g = lambda k, t=C.c_double: E.ptr(arrs[k], t) if k in arrs else None  # noqa: E731
        i = C.c_int32
        d = E.MeshDesc(nt, nb, len(m.layer_names), g("verts"), g("tb", i), g("ts"), g("el"), g("tl", i), g("lz"),
                       g("et", i), g("eloc", i), blocks.shape[0], g("blocks", i), nv,
                       int(arrs["pad"].size) if nv else 0, g("pad", i), g("off", i), g("ent", i), g("w"),
                       g("endlev", i), g("span"), g("xy"), g("drill"), 3.0, 10.0)
        h = C.c_void_p()
        E.check(self.ctx.lib.m25_geometry_create(self.ctx.h, C.byref(d), C.byref(h)))
        self._geom = E.Handle(self.ctx, h, self.ctx.lib.m25_geometry_destroy)
        return self._geom

    def geometry_stats(self):
        out = (C.c_int64 * 4)()
        E.check(self.ctx.lib.m25_geometry_stats(self.geometry().h, out))
        return dict(near_pairs=out[0], mid_pairs=out[1], far_pairs=out[2], near_bytes=out[3])

    def port_data(self):
        if self._ports is not None:
            return self._ports
        m = self.mesh
        groups = list(self.groups.values())
        gid = np.zeros(len(self.ports), int)
        for k, mem in enumerate(groups):
            gid[mem] = k
        cut_off, cut_edge, cut_w = [0], [], []
        for pm in self.pm:
            for idx, sg in pm.cuts:
                cut_edge += list(idx)
                cut_w += list(sg * m.edge_len[idx])
                cut_off.append(len(cut_edge))
        lev = [m.layer_names.index(p.layer) for p in self.ports]
        arrs = dict(gid=E.i32(gid), lev=E.i32(lev), ns=E.i32([pm.s.size for pm in self.pm]),
                    s=E.f64(np.concatenate([pm.s for pm in self.pm])), off=E.i32(cut_off), edge=E.i32(cut_edge),
                    w=E.f64(cut_w), nvpt=E.i32([len(pm.vpts) for pm in self.pm]),
                    vpts=E.f64(np.concatenate([pm.vpts for pm in self.pm])),
                    exc=E.f64(np.stack([pm.excitation for pm in self.pm])))
        # a lossless stack fits gamma = j beta, beta / |beta0| searched in
        # (0.7, 1.3), or (0.7, 1.8) under a dielectric cover (solver.py:1290-1292)
        lossless = bool(self.stack.lossless)
        arrs["bounds"] = E.f64([(0.7, 1.8) if self.stack.covered(self.ports[mem[0]].layer) else (0.7, 1.3)
                                for mem in groups])
        i = C.c_int32
        d = E.PortDesc(len(self.ports), len(groups), E.ptr(arrs["gid"], i), E.ptr(arrs["lev"], i),
                       E.ptr(arrs["ns"], i), E.ptr(arrs["s"]), E.ptr(arrs["off"], i), E.ptr(arrs["edge"], i),
                       E.ptr(arrs["w"]), E.ptr(arrs["nvpt"], i), E.ptr(arrs["vpts"]), None, int(lossless),
                       E.ptr(arrs["bounds"]) if lossless else None, self.v_weight, E.ptr(arrs["exc"]))
        h = C.c_void_p()
        E.check(self.ctx.lib.m25_ports_create(self.ctx.h, self.geometry().h, C.byref(d), C.byref(h)))
        self._ports = E.Handle(self.ctx, h, self.ctx.lib.m25_ports_destroy)
        if self.iports:  # the feeds' fits take the internal ports' excitations too
            E.check(self.ctx.lib.m25_ports_set_excitations(h, len(self.ports) + len(self.iports)))
        return self._ports

    # ---------------------------------------------------------------- path
    def greens(self, freq):
        return Greens(self, freq)

    def surface_impedance(self, freq):
        return self.stack.surface_impedance(freq)

    def beta0(self, f):
        """Kirschning-Jansen phase constant per port group (the fit's start)."""
        out = []
        for members in self.groups.values():
            port = self.ports[members[0]]
            hp = self.stack.level_h(port.layer)
            out.append(float(analytic.beta(port.width, hp, self.stack.eps_below(port.layer), f)))
        return np.array(out)

    def impedance(self, freq, greens=None, precision=None):
        """The MoM impedance matrix at freq as a host array (complex128 for
        fp64, complex64 for mixed)."""
        g = greens or self.greens(freq)
        prec = PRECISIONS[precision or self.precision]
        n = self.mesh.n_unknowns
        Z = np.zeros((n, n), np.complex64 if prec == E.M25_MIXED_FILL32 else np.complex128)
        zs = complex(self.surface_impedance(freq))
        E.check(self.ctx.lib.m25_assemble(self.ctx.h, self.geometry().h, g.h, zs.real, zs.imag, zs.real, zs.imag,
                                          prec, Z.ctypes.data, n, E.M25_ON_HOST))
        return Z

    def port_excitations(self):
        """One column per port: a 1 V delta gap at each feed, then a 1 V
        source (in series with z_ref) at each internal port."""
        cols = [pm.excitation for pm in self.pm] + [self.Lm[:, c] for c in self.iport_index]
        return np.stack(cols, 1)

    def solve_currents(self, freq, excitations=None, greens=None, Z=None):
        """RWG (+ via segment) coefficients (N, Nexc) for the given excitations
        (default: one 1 V delta gap per port)."""
        g = greens or self.greens(freq)
        B = self.port_excitations() if excitations is None else excitations
        if self.method == "hmatrix" and Z is None:
            return self._hmatrix_solve(freq, g, B)
        if Z is None:
            Z = self.impedance(freq, g)
        return dense_solve(Z, B, precision=self.precision, ctx=self.ctx, tol=self.refine_tol,
                           max_iter=self.max_refine)

    def hoperator(self):
        """The compressed operator of this mesh (built once, on this solver's context)."""
        if self._hop is None:
            from .hmatrix import HMatrix

            self._hop = HMatrix(self, **self.hmatrix_options)
        return self._hop

    def _hmatrix_solve(self, freq, g, B):
        """Z^-1 B with the compressed operator assembled at freq; each
        distinct column solved once (Engine/mom25d/solver.py:994-1011)."""
        hop = self.hoperator()
        zs = complex(self.surface_impedance(freq))
        hop.assemble(g, zs, zs)
        B = np.asarray(B, complex).reshape(self.mesh.n_unknowns, -1)
        _, first, inv = np.unique(B.T, axis=0, return_index=True, return_inverse=True)
        X = hop.solve(B[:, first], rtol=self.gmres_rtol)[:, np.ravel(inv)]
        if self.verbose:
            print(f"  f = {freq / 1e9:8.4f} GHz  N = {self.mesh.n_unknowns}  {hop.summary()}", flush=True)
        return X

    OPEN = 1e12  # ohm: an unloaded lumped gap

    def lumped_impedance(self, freq):
        """D (n_lumped, n_lumped): the impedance of the components across the
        lumped gaps (and via ports) at freq: an internal port's z_ref, a
        multi-port block's impedance matrix across its gaps, a one-port value
        on the diagonal, OPEN where none (Engine/mom25d/solver.py:1039-1062)."""
        from .lumped import as_value, parse

        nl = 0 if self.Lm is None else self.Lm.shape[1]
        D = np.zeros((nl, nl), complex)
        names = [q.name for q in self.lumped]
        used = set()
        for ip, c in zip(self.iports, self.iport_index):  # internal ports: terminated in z_ref
            D[c, c] = ip["z_ref"]
            used.add(c)
        for model, gaps in getattr(self, "components", []):
            ix = [names.index(n) for n in gaps]
            D[np.ix_(ix, ix)] = model.z(freq)
            used.update(ix)
        for k, q in enumerate(self.lumped):
            v = self.values.get(q.name, getattr(q, "value", None))
            if k in used and (v is None or k in self.iport_index):
                continue
            if isinstance(v, str):
                v = parse(v)
            D[k, k] = self.OPEN if v is None else as_value(v).z(freq)
        return D

    def _load_lumped(self, Xe, Xi, freq):
        """The solution with the components across the gaps: (Z + L D L^T)^-1 e
        = Xe - Xi D (I + L^T Xi D)^-1 L^T Xe (Woodbury), Xi = Z^-1 L
        (solver.py:1064-1070)."""
        D = self.lumped_impedance(freq)
        M = self.Lm.T @ Xi
        y = self.Lm.T @ Xe
        return Xe - Xi @ (D @ np.linalg.solve(np.eye(len(D)) + M @ D, y))

    def lumped_currents(self, x):
        """Current a -> b through each lumped gap, (n_lumped, Nexc)."""
        return self.Lm.T @ x

    def _lumped_point(self, f, g, Z, keep_currents):
        """A point with lumped loads or internal ports: one solve for the
        port and gap excitations, the loads by Woodbury on the host, then the
        de-embedding of the loaded currents on the device; with internal
        ports the feeds' wave fits take every port's excitation and S is
        assembled here (Engine/mom25d/solver.py:1305-1325)."""
        P, ni = len(self.ports), len(self.iports)
        n = P + ni
        E0 = self.port_excitations()
        B = E0 if self.Lm is None else np.hstack([E0, self.Lm])
        prec = "fp64" if self.precision == "fp64" else "mixed"
        steps = 0
        if Z is None:  # the compressed operator
            X = self._hmatrix_solve(f, g, B)
        else:
            try:
                X = dense_solve(Z, B, precision=prec, ctx=self.ctx, tol=self.refine_tol, max_iter=self.max_refine)
            except E.NumericError:
                if prec == "fp64":
                    raise
                # the mixed refinement stopped above its target: this point in fp64
                X = dense_solve(Z, B, precision="fp64", ctx=self.ctx)
                steps = -1
        x = np.ascontiguousarray(X[:, :n] if self.Lm is None else self._load_lumped(X[:, :n], X[:, n:], f))
        S = np.zeros((P, P), complex)
        z0 = np.zeros(P)
        gam = np.zeros(P, complex)
        zl = np.zeros(P, complex)
        res = np.zeros(P)
        b0 = E.f64(self.beta0(f))
        F = lambda a: E.ptr(a.view(np.float64))  # noqa: E731
        E.check(self.ctx.lib.m25_deembed(self.ctx.h, self.geometry().h, g.h, self.port_data().h, x.ctypes.data,
                                         E.M25_ON_HOST, E.ptr(b0), F(S), E.ptr(z0), F(gam), F(zl), E.ptr(res)))
        self._warn_fit_bounds(f)
        info = dict(refine_steps=steps, fp64_fallback=steps < 0)
        if not ni:
            S, z0 = self._fixed_z0(S, z0)
            info["waves"] = self.last_waves()
            return S, z0, gam, zl, res, (x if keep_currents else None), info
        # internal ports: their rows of the wave amplitudes from the current
        # through each source, V = Vs - z_ref I (current-normalised power waves)
        A, Bc = np.zeros((P, n), complex), np.zeros((P, n), complex)
        E.check(self.ctx.lib.m25_deembed_coefs(self.port_data().h, F(A), F(Bc)))
        zi = np.array([ip["z_ref"] for ip in self.iports], float)
        Ii = self.Lm[:, self.iport_index].T @ x
        Vs = np.zeros((ni, n))
        Vs[:, P:] = np.eye(ni)
        Ac = np.vstack([A, Vs / (2 * zi[:, None])])
        Bc = np.vstack([Bc, -(Vs - 2 * zi[:, None] * Ii) / (2 * zi[:, None])])
        SI = -Bc @ np.linalg.inv(Ac)
        zr = np.zeros(n)
        if self.z0_fixed is None:
            zr[:P] = reciprocal_z0(SI[:P, :P], zl.real, list(self.groups.values()))
            zr[:P] = anchor_z0(SI, zr[:P], zi, list(self.groups.values()))
        else:
            zr[:P] = self.z0_fixed
        zr[P:] = zi
        d = np.sqrt(zr)
        S = d[:, None] * SI / d[None, :]
        info["waves"] = Ac
        return (S, zr, np.r_[gam, np.zeros(ni)], np.r_[zl, zi.astype(complex)], np.r_[res, np.zeros(ni)],
                (x if keep_currents else None), info)

    def point(self, f, keep_currents=False):
        """One frequency of the sweep on the device: (S, z0, gamma, z0_line, residual, x or None, info)."""
        if self.Lm is not None or self.method == "hmatrix":
            # lumped loads, internal ports or the compressed operator: the
            # solve, then the de-embedding of the currents
            g = self.greens(f)
            out = self._lumped_point(f, g, None if self.method == "hmatrix" else self.impedance(f, g), keep_currents)
            g.close()
            return out
        g = self.greens(f)
        P = len(self.ports)
        n = self.mesh.n_unknowns
        S = np.zeros((P, P), complex)
        z0 = np.zeros(P)
        gam = np.zeros(P, complex)
        zl = np.zeros(P, complex)
        res = np.zeros(P)
        x = np.zeros((n, P), complex) if keep_currents else None
        info = np.zeros(2, np.int32)
        zs = complex(self.surface_impedance(f))
        b0 = E.f64(self.beta0(f))
        F = lambda a: E.ptr(a.view(np.float64)) if a is not None else None  # noqa: E731
        E.check(self.ctx.lib.m25_sweep_point(
            self.ctx.h, self.geometry().h, g.h, self.port_data().h, zs.real, zs.imag, zs.real, zs.imag,
            PRECISIONS[self.precision], E.ptr(b0), self.refine_tol, self.max_refine, F(x), F(S), E.ptr(z0), F(gam),
            F(zl), E.ptr(res), E.ptr(info, C.c_int32)))
        g.close()
        self._warn_fit_bounds(f)
        S, z0 = self._fixed_z0(S, z0)
        # refine_steps -1: the mixed refinement did not reach refine_tol and
        # the point was recomputed on the fp64 path
        return S, z0, gam, zl, res, x, dict(refine_steps=int(info[0]), fp64_fallback=bool(info[0] < 0),
                                            waves=self.last_waves())

    def _warn_fit_bounds(self, f):
        """mom25d's warning when a lossless beta fit ends at its search bound
        (Engine/mom25d/solver.py:658-661)."""
        if not self.stack.lossless:
            return
        it = np.zeros(len(self.groups), np.int32)
        E.check(self.ctx.lib.m25_deembed_fit_info(self.port_data().h, E.ptr(it, C.c_int32)))
        if np.any(it < 0):
            import warnings

            warnings.warn(f"beta fit hit its search bound at {f / 1e9:.4g} GHz: gamma, Z0 and S at this frequency "
                          "are unreliable", RuntimeWarning, stacklevel=3)

    def last_waves(self):
        """(P, P) incident current-wave amplitudes A [port, excitation] of the
        last de-embedding on this solver's context (SweepResult.waves)."""
        P = len(self.ports)
        A = np.zeros((P, P), complex)
        E.check(self.ctx.lib.m25_deembed_waves(self.port_data().h, E.ptr(A.view(np.float64))))
        return A

    def _fixed_z0(self, S, z0):
        """S referenced to the fixed port impedances when the solver has them."""
        if self.z0_fixed is not None:
            d0 = np.sqrt(z0)
            SI = S * d0[None, :] / d0[:, None]
            z0 = self.z0_fixed.copy()
            d = np.sqrt(z0)
            S = d[:, None] * SI / d[None, :]
        return S, z0

    def last_deembed(self):
        """Intermediates of the last de-embedding on the device: triangle
        charges q (Nt,P), line voltages phi (M,P), cut currents I and cut
        voltages V (sum Ns, P)."""
        P = len(self.ports)
        M = sum(len(pm.vpts) for pm in self.pm)
        ns = sum(pm.s.size for pm in self.pm)
        q = np.zeros((len(self.mesh.tris), P), complex)
        phi = np.zeros((M, P), complex)
        I = np.zeros((ns, P), complex)
        V = np.zeros((ns, P), complex)
        F = lambda a: E.ptr(a.view(np.float64))  # noqa: E731
        E.check(self.ctx.lib.m25_deembed_debug(self.ctx.h, self.port_data().h, F(phi), F(q), F(I), F(V)))
        return q, phi, I, V

    def _checkpoint_key(self, freqs):
        return checkpoint_key(self.mesh, freqs, values_digest(self.values, self.lumped, self.components))

    _DEVICE_STATE = ("ctx", "_ctx_owner", "_geom", "_geom_owner", "_ports", "_siblings", "_sib_lock", "_hop")

    def _clone(self, ctx=None):
        """A solver sharing this one's host-side set-up (mesh, port models,
        groups, test blocks) and its device geometry (classes, closed-form
        near-pair data: read-only once built, readable from any stream) with
        a fresh engine context of its own (stream, per-point buffers, ports),
        or on the given context (then owned by the caller, who closes it)."""
        s = object.__new__(Solver)
        s.__dict__.update({k: v for k, v in self.__dict__.items() if k not in self._DEVICE_STATE})
        s.verbose = False
        s.ctx = E.Context(self.device) if ctx is None else ctx
        s._ctx_owner = ctx is None
        s._geom = self.geometry()
        s._geom_owner = False  # closed by this solver, after its siblings
        s._ports = None
        s._hop = None
        s._siblings = []
        s._sib_lock = threading.Lock()
        return s

    def _sweep_tuning(self):
        """The knob values of this solver's mixed-precision points (None:
        the process defaults): self.tuning, or the measured table by N."""
        if self.precision != "mixed" or self.tuning is None:
            return None
        if isinstance(self.tuning, str):
            if self.tuning != "table":
                raise ValueError('Solver.tuning must be "table", a Tuning or None')
            from .autotune import load_table

            if not hasattr(Solver, "_table"):
                Solver._table = load_table()
            return Solver._table
        return self.tuning

    # what a caller may change between sweeps; a sweep hands the current values to its workers
    _SETTINGS = ("precision", "method", "refine_tol", "max_refine", "z0_fixed", "v_weight", "surrogate", "tuning",
                 "gmres_rtol")

    def _sibling(self, i):
        """Worker i of a concurrent sweep (0: this solver): the same mesh,
        stack and settings on its own engine context (stream, device data);
        an existing worker takes this solver's current settings."""
        if i == 0:
            return self
        if self._blocks_host is None:
            self._blocks_host = test_blocks(self.mesh)
        with self._sib_lock:
            while len(self._siblings) < i:
                self._siblings.append(self._clone())
            sib = self._siblings[i - 1]
        for k in self._SETTINGS:
            setattr(sib, k, getattr(self, k))
        return sib

    def _worker_bytes(self):
        """Device memory of one more worker: fill scratch, the matrix planes
        and LU copy (or the complex128 Z) and per-point buffers."""
        mesh = self.mesh
        nt, N = int(mesh.tri_layer.size), int(mesh.n_unknowns)
        nv = N - int(mesh.n_basis)
        nblocks = (nt + 31) // 32 + len(mesh.layer_names)
        elem = 16 if self.precision == "fp64" else 8
        b = elem * 3 * nt * nblocks * 96                # fill scratch: H (fp64), H32 (mixed fills)
        if self.precision == "mixed":
            b += b // 4                                 # the near pairs' fp64 values (Hn), a bound
        if self.precision == "fp64":
            b += 16 * N * N                             # Z, factored in place
        else:
            b += 24 * N * (N + 1)                       # Zh, Zl, complex64 LU
            if nv or self.precision == "mixed_fill32":
                b += elem * N * N                       # Z as filled (split after)
        b += 4096 * N                                   # GMRES vectors, LU scratch (the geometry is shared)
        return b

    def _workers_that_fit(self):
        """Workers that fit: those that exist already (this solver and its
        siblings hold their buffers) plus those whose buffers fit in the free
        device memory."""
        free, total = C.c_uint64(), C.c_uint64()
        E.check(self.ctx.lib.m25_ctx_mem_info(self.ctx.h, C.byref(free), C.byref(total)))
        return 1 + len(self._siblings) + int(0.9 * free.value // max(1, self._worker_bytes()))

    def sweep(self, freqs, keep_currents=False, interp=None, values=None, checkpoint=None, wait_memory=None,
              workers=1):
        """S-parameters at freqs. interp: None (default) -> exact fill at
        every frequency; "auto" -> interpolate Z between anchor fills
        (FreqInterp with its defaults) when the sweep has at least twice as
        many frequencies as anchors, else fill every point; a FreqInterp ->
        use it (Engine/mom25d/solver.py:1189-1223). checkpoint: an .npz
        rewritten atomically after every frequency; a restarted sweep with
        the same frequencies and mesh resumes from it. workers: frequency
        points in flight at once on this GPU, each on its own engine context
        and stream, driven by its own host thread (the latency-bound stages of
        one point - LU panels, triangular solves, the wave fit - leave most of
        the GPU to the others); points are handed out in order as workers
        become free. Fewer workers run when their buffers would not fit in
        the free device memory (result.info["workers"]). An interpolated
        sweep fills its anchors first when they all fit on the device
        (FreqInterp resident) and then runs its points like an exact one;
        otherwise it runs on one worker in the order of freqs."""
        freqs = np.atleast_1d(np.asarray(freqs, float))
        self.values.clear()  # shared with the sweep's workers
        self.values.update(values or {})
        if self.method == "hmatrix":
            # FreqInterp stores dense matrices (Engine/mom25d/solver.py:1208-1209); the
            # compressed operator is one per solver: its points run one after another
            interp = None
            workers = 1
        ip = None
        if isinstance(interp, str):
            if interp != "auto":
                raise ValueError("interp must be 'auto', None or a FreqInterp")
            from .freqinterp import FreqInterp

            ip = FreqInterp().setup(self, freqs)
            if len(freqs) < 2 * len(ip.anchors):
                ip = None
        elif interp is not None:
            ip = interp.setup(self, freqs)
        if ip is not None:
            if self.verbose:
                print(f"  FreqInterp: {len(ip.anchors)} anchor fills for {len(freqs)} frequencies "
                      f"(order {ip.order}, k_e = {ip.k_ratio:.3f} k0)")
            ip._device()
            if ip._resident:
                ip.fill_all(freqs)
            if not ip._resident or self.Lm is not None:
                workers = 1
        nf, P = len(freqs), len(self.ports) + len(self.iports)
        S = np.zeros((nf, P, P), complex)
        gam = np.zeros((nf, P), complex)
        zl = np.zeros((nf, P), complex)
        zr = np.zeros((nf, P))
        res = np.zeros((nf, P))
        cur = [None] * nf
        waves = np.zeros((nf, P, P), complex)
        done = np.zeros(nf, bool)
        key = self._checkpoint_key(freqs) if checkpoint else None
        if checkpoint and os.path.exists(checkpoint) and not keep_currents:
            try:
                ck = np.load(checkpoint)
                if ck["key"].shape == key.shape and np.allclose(ck["key"], key, rtol=1e-12, atol=0) \
                        and ck["S"].shape == S.shape:
                    done = ck["done"].astype(bool)
                    S[:], gam[:], zl[:], zr[:], res[:] = (ck[k] for k in ("S", "gam", "zl", "zr", "res"))
                    if "waves" in ck.files:
                        waves[:] = ck["waves"]
            except Exception as exc:  # noqa: BLE001 - unreadable: start afresh
                if self.verbose:
                    print(f" checkpoint: unreadable ({exc}); starting afresh", flush=True)
                done[:] = False
        steps = [None] * nf
        todo = [fi for fi in range(nf) if not done[fi]]
        workers = max(1, min(int(workers), len(todo) or 1, self._workers_that_fit()))
        tun = self._sweep_tuning()
        if workers > 1:
            self.geometry()  # built once here, shared by the workers' contexts
        lock = threading.Lock()
        nxt = [0]
        errors = []

        def work(w):
            try:  # each worker sets up its own context's device data
                sol = self._sibling(w)
                if tun is not None:
                    tun.apply(sol.ctx, self.mesh.n_unknowns)
                sol.geometry()
                sol.port_data()
            except Exception as exc:  # noqa: BLE001 - re-raised below in the caller's thread
                with lock:
                    errors.append(exc)
                return
            while True:
                with lock:
                    if errors or nxt[0] >= len(todo):
                        return
                    fi = todo[nxt[0]]
                    nxt[0] += 1
                try:
                    if ip is not None:
                        out = ip.point(freqs[fi], keep_currents, solver=sol)
                    else:
                        out = sol.point(freqs[fi], keep_currents)
                except Exception as exc:  # noqa: BLE001 - re-raised below in the caller's thread
                    with lock:
                        errors.append(exc)
                    return
                with lock:
                    S[fi], zr[fi], gam[fi], zl[fi], res[fi], cur[fi], inf = out
                    waves[fi] = inf["waves"]
                    steps[fi] = inf["refine_steps"]
                    done[fi] = True
                    if self.verbose:
                        print(f"PROGRESS {int(done.sum())}/{nf}", flush=True)
                    if checkpoint:
                        tmp = checkpoint + ".tmp.npz"
                        np.savez(tmp, key=key, done=done, S=S, gam=gam, zl=zl, zr=zr, res=res, waves=waves)
                        os.replace(tmp, checkpoint)

        t0 = time.time()
        if workers == 1:
            work(0)
        else:
            th = [threading.Thread(target=work, args=(w,)) for w in range(workers)]
            for t in th:
                t.start()
            for t in th:
                t.join()
        if errors:
            raise errors[0]
        info = dict(seconds=time.time() - t0, refine_steps=[s for s in steps if s is not None], workers=workers,
                    fp64_fallback=[float(freqs[i]) for i, s in enumerate(steps) if s is not None and s < 0])
        if ip is not None:
            info.update(interp_fills=ip.n_fills, interp_anchors=len(ip.anchors), interp_fill_seconds=ip.fill_time)
            if interp is not ip:
                ip.close()  # made here ("auto"); a caller's FreqInterp keeps its anchors
        return SweepResult(freqs, S, zr, gam, zl, res, [p.name for p in self.ports] + [ip["name"] for ip in self.iports],
                           cur if keep_currents else None, waves, info=info)

    def close(self):
        for sib in self._siblings:
            sib.close()
        self._siblings = []
        if getattr(self, "_hop", None) is not None:
            self._hop.close()
            self._hop = None
        if self._ports is not None:
            self._ports.close()
        if self._geom is not None and getattr(self, "_geom_owner", True):
            self._geom.close()
        self._ports = self._geom = None
        if getattr(self, "_ctx_owner", True):
            self.ctx.close()


def reciprocal_z0(SI, zphi, groups, prior=1e-4):
    """Reference impedances of the feeds that make S = D SI D^-1 reciprocal
    (D = diag(sqrt(Z0)): reciprocity fixes Z0_i / Z0_j = |SI_ji / SI_ij|
    between coupled groups), with the scalar-potential estimates zphi as a
    weak prior that sets the level and the groups that barely couple: a
    weighted least-squares fit of log Z0 per group, weights the square of
    the smaller coupling (Engine/mom25d/solver.py:1357-1427). The same fit
    as the device's de-embedding, for S assembled on the host."""
    zphi = np.asarray(zphi, float)
    if len(groups) == 1:
        return zphi.copy()
    gid = np.empty(len(zphi), int)
    for k, members in enumerate(groups):
        gid[members] = k
    rows, rhs, wts = [], [], []
    for i in range(len(gid)):
        for j in range(i + 1, len(gid)):
            w = min(abs(SI[i, j]), abs(SI[j, i])) ** 2
            if gid[i] != gid[j] and w > 0:
                r = np.zeros(len(groups))
                r[gid[i]], r[gid[j]] = 1.0, -1.0
                rows.append(r)
                rhs.append(np.log(abs(SI[j, i] / SI[i, j])))
                wts.append(w)
    for k, members in enumerate(groups):
        r = np.zeros(len(groups))
        r[k] = 1.0
        rows.append(r)
        rhs.append(np.log(np.mean(zphi[members])))
        wts.append(prior)
    sw = np.sqrt(wts)
    logz = np.linalg.lstsq(np.array(rows) * sw[:, None], np.array(rhs) * sw, rcond=None)[0]
    logz += np.mean(np.log(zphi)) - np.mean(logz[gid])  # the scalar-potential level
    return np.exp(logz[gid])


def anchor_z0(SI, zfeed, zi, groups, prior=1e-4):
    """Feed reference impedances refined by reciprocity with the internal
    ports, whose z_ref is exact: per feed group the coupling-weighted mean of
    log(z_i |SI_ij / SI_ji|) over internal ports i and members j, the feed
    estimate as a weak prior (Engine/mom25d/solver.py:1336-1355)."""
    P = len(zfeed)
    z = np.array(zfeed, float)
    for members in groups:
        num, den = prior * np.log(np.mean(z[members])), prior
        for j in members:
            for k, zk in enumerate(zi):
                i = P + k
                w = min(abs(SI[i, j]), abs(SI[j, i])) ** 2
                if w > 0:
                    num += w * np.log(zk * abs(SI[i, j] / SI[j, i]))
                    den += w
        z[members] = np.exp(num / den)
    return z


def values_digest(values, lumped=(), components=()):
    """A digest of what the lumped loads of a sweep are: the per-sweep value
    overrides, the layout's own values and the multi-port blocks (their file
    name, gaps and S data). CRC-32, so that it is the same in every process
    (Python's hash of a string is salted per process)."""
    crc = zlib.crc32(repr(sorted((str(k), repr(v)) for k, v in (values or {}).items())).encode())
    crc = zlib.crc32(repr([(q.name, repr(getattr(q, "value", None))) for q in lumped]).encode(), crc)
    for model, gaps in components:
        crc = zlib.crc32(repr((repr(model), tuple(gaps))).encode(), crc)
        data = getattr(model, "s_data", None)
        if data is not None:
            crc = zlib.crc32(np.ascontiguousarray(data).tobytes(), crc)
    return float(crc)


def checkpoint_key(mesh, freqs, digest=0.0):
    """The key a sweep checkpoint is resumed under (Engine/mom25d/solver.py:
    1183-1187): the frequencies, the mesh's size and node sums, and the
    digest of the lumped loads (values_digest). A checkpoint whose key
    differs is not resumed."""
    m = mesh
    return np.array([len(freqs), float(np.sum(freqs)), float(m.n_unknowns), float(np.sum(m.nodes)),
                     float(np.sum(m.nodes ** 2)), float(len(m.tris)), float(digest)])


def assemble(solver, freq, precision="fp64"):
    """mom25d's assemble(mesh, greens, zs, geom=...) for a Solver's mesh: the
    impedance matrix at freq (host array)."""
    return solver.impedance(freq, precision=precision)


_default_ctx = None


def dense_solve(Z, B, precision="fp64", ctx=None, tol=1e-14, max_iter=60):
    """Z X = B on the GPU (mom25d's _dense_solve): LU with partial pivoting in
    fp64, or ("mixed") a complex64 LU with fp64 GMRES refinement against Z
    (complex128, or complex64 when Z comes from the fp32 fill)."""
    global _default_ctx
    if ctx is None:
        if _default_ctx is None:
            _default_ctx = E.Context(0)
        ctx = _default_ctx
    Z = np.ascontiguousarray(Z)
    n = Z.shape[0]
    B = np.ascontiguousarray(np.asarray(B).reshape(n, -1), np.complex128)
    X = np.zeros_like(B)
    if precision == "fp64":
        prec = E.M25_FP64
        Z = np.ascontiguousarray(Z, np.complex128)
    elif Z.dtype == np.complex64:
        prec = E.M25_MIXED_FILL32
    else:
        prec = E.M25_MIXED
        Z = np.ascontiguousarray(Z, np.complex128)
    info = np.zeros(2, np.int32)
    E.check(ctx.lib.m25_dense_solve(ctx.h, n, B.shape[1], prec, Z.ctypes.data, B.ctypes.data, X.ctypes.data,
                                    E.M25_ON_HOST, tol, max_iter, E.ptr(info, C.c_int32)))
    return X
