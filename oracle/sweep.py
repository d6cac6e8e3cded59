"""ORACLE (test infrastructure only; never imported by the product path).

CPU restatement of mom25d's dense sweep path, used to check the CUDA
engine on the same meshes:

  assembly geometry  mom25d/solver.py:307-426 (Morton blocks of 32 test
                     triangles, near/mid/far classes, closed-form near parts,
                     Gram matrix, via pad maps)
  fill               mom25d/solver.py:265-291, 429-524 (MPIE Galerkin fill,
                     RWG scatter, symmetrisation)
  via blocks         mom25d/solver.py:80-199, 527-566
  dense solve        mom25d/solver.py:11-23 (LAPACK LU via scipy)
  de-embedding       mom25d/solver.py:570-670 (ports, wave fit), 1076-1125
                     (charges, line voltage), 1276-1325, 1357-1427 (S, Z0)

Third-party arithmetic, as mom25d: scipy.linalg lu_factor / lu_solve,
scipy.optimize minimize (Nelder-Mead) and minimize_scalar (bounded),
numpy.linalg.lstsq.
"""

import numpy as np
import scipy.linalg as sla
from scipy.optimize import minimize, minimize_scalar

from . import kernels as K
from .kernels import EPS0, MU0, TRI3_BARY, TRI3_W, TRI7_BARY, TRI7_W, potential_integrals, quad_points


def morton_order(xy):
    q = ((xy - xy.min(0)) / max(np.ptp(xy, 0).max(), 1e-30) * 65535).astype(np.uint64)

    def spread(v):
        for s, m in ((8, 0x00FF00FF), (4, 0x0F0F0F0F), (2, 0x33333333), (1, 0x55555555)):
            v = (v | (v << np.uint64(s))) & np.uint64(m)
        return v

    return np.argsort(spread(q[:, 0]) | (spread(q[:, 1]) << np.uint64(1)), kind="stable")


def stack_info(stack, mesh):
    """(single-slab flag, level heights zl per mesh layer, slab parameters or layer list)."""
    single = len(stack.layers) == 1 and mesh.layer_names == ["top"]
    zl = np.array([stack.level_z(n) for n in mesh.layer_names])
    return single, zl


def make_kernels(stack, mesh, freq, rho_max):
    single, zl = stack_info(stack, mesh)
    zg = stack.surface_impedance(freq) if stack.ground_loss else 0.0
    if single:
        d = stack.layers[0]
        return K.SlabKernels(freq, d.eps_r, d.t, d.tand, rho_max, zs_ground=zg)
    il = [stack.metals[n] for n in mesh.layer_names]
    return K.LayeredKernels(freq, [(d.t, d.eps_r, d.tand) for d in stack.layers], il, zl, rho_max, zs_ground=zg,
                            top=getattr(stack, "top", "air"))


class Geometry:
    """Frequency-independent fill data for one mesh."""

    def __init__(self, mesh, zl, block=32, near=3.0, far=10.0):
        V, A = mesh.verts, mesh.area
        self.nt, self.nb = nt, nb = len(A), mesh.n_basis
        self.V, self.A = V, A
        self.q7 = quad_points(V, TRI7_BARY)
        self.w7 = TRI7_W[None, :] * A[:, None]
        self.q3 = quad_points(V, TRI3_BARY)
        self.w3 = TRI3_W[None, :] * A[:, None]
        self.q1 = mesh.centroid[:, None, :]
        self.w1 = A[:, None]
        size = np.max(np.linalg.norm(V - np.roll(V, 1, axis=1), axis=-1), axis=1)
        cen, tl = mesh.centroid, mesh.tri_layer
        nl = len(mesh.layer_names)
        self.zl = zl
        b = mesh.tri_basis
        lab = np.where(b >= 0, mesh.edge_len[np.maximum(b, 0)], 0.0)
        self.b = b
        self.cA = mesh.tri_sign * lab / (2 * A[:, None])
        self.cV = mesh.tri_sign * lab / A[:, None]
        self.blocks = []
        for lt in range(nl):
            on = np.nonzero(tl == lt)[0]
            if not on.size:
                continue
            order = on[morton_order(cen[on])]
            for p0 in range(0, order.size, block):
                pb = order[p0:p0 + block]
                r = self.q7[pb].reshape(-1, 2)
                groups = []
                for ls in range(nl):
                    src = np.nonzero(tl == ls)[0]
                    if not src.size:
                        continue
                    dz = abs(zl[lt] - zl[ls])
                    dist = np.sqrt(np.linalg.norm(cen[pb][:, None] - cen[None, src], axis=-1) ** 2 + dz ** 2)
                    rel = np.min(dist / np.maximum(size[pb][:, None], size[None, src]), axis=0)
                    cls = np.where(rel < near, 0, np.where(rel < far, 1, 2))
                    for c, (pts, w) in enumerate(((self.q7, self.w7), (self.q3, self.w3), (self.q1, self.w1))):
                        sel = src[cls == c]
                        if not sel.size:
                            continue
                        static = None
                        if c == 0:
                            I0, I1 = potential_integrals(V[sel], r, dz)
                            static = (I0 / (4 * np.pi), (r[None] * I0[..., None] + I1) / (4 * np.pi))
                        groups.append((ls, sel, pts[sel], w[sel], static))
                self.blocks.append((lt, pb, r, groups))
        X = self.q7[:, None] - V[:, :, None]  # (Nt,3,7,2)
        G = np.einsum("tk,tikd,tjkd->tij", self.w7, X, X) * self.cA[:, :, None] * self.cA[:, None, :]
        self.gram = G
        segs = mesh.via_segments
        self.nv = nv = len(segs)
        if nv:
            self.vias = [mesh.vias[g["via"]] for g in segs]
            tris = [g[e] for g in segs for e in ("top_tris", "bottom_tris") if g[e] is not None]
            self.pad_tris = pad = np.unique(np.concatenate(tris))
            self.pad_pos = -np.ones(nt, int)
            self.pad_pos[pad] = np.arange(pad.size)
            self.D = np.zeros((pad.size, nv))
            self.via_ends = []
            for k, g in enumerate(segs):
                ends = []
                if g["top_tris"] is not None:
                    t = g["top_tris"]
                    self.D[self.pad_pos[t], k] += 1 / A[t].sum()
                    ends.append((tl[t[0]], 1.0))
                if g["bottom_tris"] is not None:
                    t = g["bottom_tris"]
                    self.D[self.pad_pos[t], k] -= 1 / A[t].sum()
                    ends.append((tl[t[0]], -1.0))
                self.via_ends.append(ends)
            zmap = {n: z for n, z in zip(mesh.layer_names, zl)}
            zmap["gnd"] = 0.0
            self.spans = np.array([(zmap[g["bottom"]], zmap[g["top"]]) for g in segs])


def filament_mutual_z(a1, a2, b1, b2, d):
    """Partial mutual inductance of parallel z filaments over [a1,a2], [b1,b2]
    at lateral distance d (Grover; mom25d/solver.py:86-90)."""
    f = lambda s: s * np.arcsinh(s / d) - np.sqrt(s * s + d * d)  # noqa: E731
    return MU0 / (4 * np.pi) * (f(a2 - b1) - f(a2 - b2) - f(a1 - b1) + f(a1 - b2))


def via_block_L(vias, spans, z_section):
    """Quasi-static via-segment inductance with images in the ground plane
    for an open (air-topped) stack section [0, h] (mom25d/solver.py:125-199)."""
    xy = np.array([v.xy for v in vias], float)
    rho = np.linalg.norm(xy[:, None] - xy[None], axis=-1)
    rad = np.array([0.5 * v.drill for v in vias])
    rho = np.where(rho < 1e-12, np.minimum(rad[:, None], rad[None, :]), rho)
    np.fill_diagonal(rho, rad)
    zb, zt = z_section
    a1 = np.clip(spans[:, 0], zb, zt) - zb
    a2 = np.clip(spans[:, 1], zb, zt) - zb
    p1, p2, q1, q2 = a1[:, None], a2[:, None], a1[None, :], a2[None, :]
    return filament_mutual_z(p1, p2, q1, q2, rho) + filament_mutual_z(p1, p2, -q2, -q1, rho)


def scatter_blocks(geom, kern, omega, blocks, Z, row_map=None, IVpad=None):
    """Add the Galerkin sums of the given test blocks to Z (mom25d/
    solver.py:429-509): row m of Z receives row_map[m] when row_map is given
    (a partial Z holding only some rows), and IVpad the pad rows' scalar
    potentials when the mesh has vias."""
    b, cA, cV, V = geom.b, geom.cA, geom.cV, geom.V
    jwmu = 1j * omega * MU0
    inv_jwe = 1 / (1j * omega * EPS0)
    for lt, pb, r, groups in blocks:
        npb = pb.size
        rt = r.reshape(npb, 7, 2)
        wo = geom.w7[pb]
        Xt = rt[:, None, :, :] - V[pb][:, :, None, :]  # (npb,3,7,2) test r_k - a_i
        for ls, sel, pts, w, static in groups:
            pr = kern.pair(lt, ls)
            d = rt[:, :, None, None, :] - pts[None, None]  # (npb,7,ns,L,2)
            R = np.hypot(d[..., 0], d[..., 1])
            SA, SV = pr.smooth(R)
            if static is None:
                inv = 1 / (4 * np.pi * np.sqrt(R * R + pr.dz ** 2))
                SA = SA + pr.cA * inv
                SV = SV + pr.cV * inv
                K0A = K1A = K0V = 0.0
            else:
                S0, S1 = static  # (ns, npb*7), (ns, npb*7, 2)
                S0 = S0.reshape(-1, npb, 7).transpose(1, 2, 0)
                S1 = S1.reshape(-1, npb, 7, 2).transpose(1, 2, 0, 3)
                K0A, K1A, K0V = pr.cA * S0, pr.cA * S1, pr.cV * S0
            SAw = SA * w[None, None]
            K0A = K0A + SAw.sum(-1)  # (npb,7,ns)
            K1A = K1A + np.einsum("pksl,sld->pksd", SAw, pts)
            K0V = K0V + np.einsum("pksl,sl->pks", SV, w)
            Vs = V[sel]  # (ns,3,2)
            # IA[p,s,i,j] = sum_k w_k (r_k - a_i) . (K1A_k - b_j K0A_k)
            T1 = np.einsum("pk,pikd,pksd->psi", wo, Xt, K1A)
            T2 = np.einsum("pk,pikd,pks->psid", wo, Xt, K0A)
            IA = T1[..., None] - np.einsum("psid,sjd->psij", T2, Vs)
            IV = np.einsum("pk,pks->ps", wo, K0V)
            vals = (jwmu * cA[pb][:, None, :, None] * cA[sel][None, :, None, :] * IA
                    + inv_jwe * cV[pb][:, None, :, None] * cV[sel][None, :, None, :] * IV[..., None, None])
            rows = np.broadcast_to(b[pb][:, None, :, None], vals.shape)
            cols = np.broadcast_to(b[sel][None, :, None, :], vals.shape)
            ok = (rows >= 0) & (cols >= 0)
            rr = rows[ok] if row_map is None else row_map[rows[ok]]
            np.add.at(Z, (rr, cols[ok]), vals[ok])
            if IVpad is not None:
                pos = geom.pad_pos[pb]
                on = pos >= 0
                if on.any():
                    IVpad[np.ix_(pos[on], sel)] = IV[on]


def block_rows(geom, blocks):
    """The RWG rows the test triangles of `blocks` touch (sorted)."""
    b = np.concatenate([geom.b[pb].ravel() for _, pb, _, _ in blocks]) if blocks else np.zeros(0, int)
    return np.unique(b[b >= 0])


def finish_fill(geom, kern, omega, Z, zs=0.0, zs_via=None, IVpad=None):
    """The parts of the fill after the block sums (mom25d/solver.py:
    510-524): the surface-impedance term, the via rows and the
    symmetrisation."""
    b = geom.b
    nb = geom.nb
    if np.any(zs):
        G = geom.gram
        ii = np.broadcast_to(b[:, :, None], G.shape)
        jj = np.broadcast_to(b[:, None, :], G.shape)
        ok = (ii >= 0) & (jj >= 0)
        np.add.at(Z, (ii[ok], jj[ok]), zs * G[ok])
    if geom.nv:
        zv = zs if zs_via is None else zs_via
        Zvb, Zvv = via_blocks(geom, kern, IVpad, omega, zv)
        Z[nb:, :nb] = Zvb
        Z[nb:, nb:] = Zvv
        Z[:nb, nb:] = Zvb.T
    return 0.5 * (Z + Z.T)


def fill(geom, kern, omega, zs=0.0, zs_via=None):
    """Galerkin MPIE impedance matrix (N x N complex128), symmetrised."""
    nt, nb, nv = geom.nt, geom.nb, geom.nv
    Z = np.zeros((nb + nv, nb + nv), complex)
    IVpad = np.zeros((geom.pad_tris.size, nt), complex) if nv else None
    scatter_blocks(geom, kern, omega, geom.blocks, Z, IVpad=IVpad)
    return finish_fill(geom, kern, omega, Z, zs, zs_via, IVpad)


def via_blocks(geom, kern, IVpad, omega, zs):
    """Via rows of Z (mom25d/solver.py:527-566): charges through gV, the
    Im gV(0) removal, vertical-current inductance, via-wall loss."""
    jwmu = 1j * omega * MU0
    inv_jwe = 1 / (1j * omega * EPS0)
    D = geom.D
    Y = np.zeros((IVpad.shape[0], geom.nb), complex)
    ok = geom.b >= 0
    t_idx, i_idx = np.nonzero(ok)
    np.add.at(Y.T, geom.b[ok], (geom.cV[ok][:, None] * IVpad[:, t_idx].T))
    Zvb = inv_jwe * (D.T @ Y)
    Zvv = inv_jwe * (D.T @ IVpad[:, geom.pad_tris] @ D)
    h = kern.h
    for k, ek in enumerate(geom.via_ends):
        for m, em in enumerate(geom.via_ends):
            acc = 0.0
            for la, sa in ek:
                for lb, sb in em:
                    pr = kern.pair(la, lb)
                    rho = 0.0 if pr.dz else 1e-6 * h
                    acc += sa * sb * pr.gV(np.array([rho]))[0].imag
            Zvv[k, m] -= inv_jwe * 1j * acc
    Zvv += 1j * omega * via_block_L(geom.vias, geom.spans, (0.0, h))
    lengths = geom.spans[:, 1] - geom.spans[:, 0]
    if zs:
        Zvv += np.diag([zs * l / (np.pi * v.drill) for l, v in zip(lengths, geom.vias)])
    return Zvb, Zvv


def dense_solve(Z, B):
    return sla.lu_solve(sla.lu_factor(Z, check_finite=False), B)


# ---------------------------------------------------------------- de-embedding
class PortData:
    """Excitation, fit-window cuts and line-voltage points of one feed
    (mom25d/solver.py:570-610)."""

    def __init__(self, mesh, port, h):
        margin = port.margin if port.margin is not None else max(1.5 * port.width, 4 * h)
        s = mesh.cut_positions(port)
        s = s[(s >= margin - 1e-12) & (s <= port.s_gap - margin + 1e-12)]
        if s.size < 4:
            raise ValueError(f"port {port.name}: feed line too short or mesh too coarse")
        self.s = s
        self.cuts = [mesh.cut_edges(port, si) for si in s]
        idx, sgn = mesh.cut_edges(port, port.s_gap)
        self.excitation = np.zeros(mesh.n_unknowns)
        self.excitation[idx] = sgn * mesh.edge_len[idx]
        self.len = mesh.edge_len
        allcuts = mesh.cut_positions(port)
        k = np.searchsorted(allcuts, s)
        lo = s - allcuts[np.maximum(k - 1, 0)]
        hi = allcuts[np.minimum(k + 1, allcuts.size - 1)] - s
        d = 0.5 * np.minimum(np.where(lo > 0, lo, np.inf), np.where(hi > 0, hi, np.inf))
        frac = np.array([-0.3, -0.1, 0.1, 0.3])
        along = np.stack([s - d, s + d], 1)
        self.vpts = port.point(along[:, :, None], frac * port.width).reshape(-1, 2)
        self.nper = 2 * frac.size

    def currents(self, x):
        return np.array([(sg * self.len[i]) @ x[i] for i, sg in self.cuts])

    def voltages(self, phi):
        return phi.reshape(self.s.size, self.nper, -1).mean(1)


def charges(mesh, x, omega):
    b = mesh.tri_basis
    lab = np.where(b >= 0, mesh.edge_len[np.maximum(b, 0)], 0.0)
    cV = mesh.tri_sign * lab / mesh.area[:, None]
    div = np.einsum("ti,tie->te", cV, np.where((b >= 0)[..., None], x[np.maximum(b, 0)], 0))
    for k, g in enumerate(mesh.via_segments):
        for key, sg in (("top_tris", 1.0), ("bottom_tris", -1.0)):
            t = g[key]
            if t is not None:
                div[t] += sg * x[mesh.n_basis + k] / mesh.area[t].sum()
    return -div / (1j * omega)


def line_voltage(mesh, kern, q, pts, layer):
    li = mesh.layer_names.index(layer)
    out = 0.0
    for ls in range(len(mesh.layer_names)):
        on = np.nonzero(mesh.tri_layer == ls)[0]
        if not on.size:
            continue
        pr = kern.pair(li, ls)
        V = mesh.verts[on]
        qp = quad_points(V, TRI7_BARY)
        qw = TRI7_W[None, :] * mesh.area[on][:, None]
        d = pts[None, :, None, :] - qp[:, None]
        SW = pr.smooth_w(np.hypot(d[..., 0], d[..., 1]))
        K0W = np.einsum("qml,ql->qm", SW, qw)
        if pr.cW:
            I0, _ = potential_integrals(V, pts, pr.dz)
            K0W = K0W + pr.cW * I0 / (4 * np.pi)
        out = out + (K0W.T @ q[on]) / EPS0
    return out


def fit_waves(s_list, I_list, V_list, gamma0, lossless=False, v_weight=1.0, bounds=(0.7, 1.3)):
    """Shared gamma, Z0 and per-dataset (A, B) of I = A e^{gs} + B e^{-gs},
    V = Z0 (A e^{gs} - B e^{-gs}) (mom25d/solver.py:618-670)."""
    scale = abs(gamma0.imag)
    Inrm = sum(np.sum(np.abs(I) ** 2) for I in I_list)
    Vnrm = sum(np.sum(np.abs(V) ** 2) for V in V_list)

    def solve(g):
        coefs, res, Us = [], 0.0, []
        for s, I in zip(s_list, I_list):
            ep, em = np.exp(g * s), np.exp(-g * s)
            M = np.stack([ep, em], 1)
            c = np.linalg.lstsq(M, I, rcond=None)[0]
            coefs.append(c)
            res += np.sum(np.abs(M @ c - I) ** 2) / Inrm
            Us.append(c[0] * ep - c[1] * em)
        U, Vv = np.concatenate(Us), np.concatenate(V_list)
        z0 = np.vdot(U, Vv) / np.vdot(U, U)
        res += v_weight * np.sum(np.abs(Vv - z0 * U) ** 2) / Vnrm
        return coefs, z0, res

    if lossless:
        lo, hi = bounds
        opt = minimize_scalar(lambda bb: solve(1j * scale * bb)[2], bounds=(lo, hi), method="bounded",
                              options=dict(xatol=1e-12))
        g = 1j * scale * opt.x
    else:
        p0 = np.array([gamma0.real, gamma0.imag]) / scale
        opt = minimize(lambda p: solve(scale * (p[0] + 1j * p[1]))[2], p0, method="Nelder-Mead",
                       options=dict(xatol=1e-10, fatol=1e-16, maxiter=4000))
        g = scale * (opt.x[0] + 1j * opt.x[1])
    coefs, z0, res = solve(g)
    return g, z0, coefs, np.sqrt(res)


def voltage_z0(SI, zphi, groups, prior=1e-4):
    """Reciprocity + scalar-potential Z0 over port groups (mom25d/solver.py:1398-1427)."""
    if len(groups) == 1:
        return zphi
    gid = np.empty(len(zphi), int)
    for k, members in enumerate(groups):
        gid[members] = k
    rows, rhs, wts = [], [], []
    for i in range(len(gid)):
        for j in range(i + 1, len(gid)):
            if gid[i] != gid[j]:
                w = min(abs(SI[i, j]), abs(SI[j, i])) ** 2
                if w > 0:
                    r = np.zeros(len(groups))
                    r[gid[i]], r[gid[j]] = 1, -1
                    rows.append(r)
                    rhs.append(np.log(abs(SI[j, i] / SI[i, j])))
                    wts.append(w)
    for k, members in enumerate(groups):
        r = np.zeros(len(groups))
        r[k] = 1
        rows.append(r)
        rhs.append(np.log(np.mean(zphi[members])))
        wts.append(prior)
    sw = np.sqrt(wts)
    logz = np.linalg.lstsq(np.array(rows) * sw[:, None], np.array(rhs) * sw, rcond=None)[0]
    logz += np.mean(np.log(zphi)) - np.mean(logz[gid])
    return np.exp(logz[gid])


def beta0(port, stack, f):
    """Kirschning-Jansen phase constant of the feed (mom25d/analytic.py:14-44)."""
    w, h, er = port.width, stack.level_h(port.layer), stack.eps_below(port.layer)
    u = w / h
    a = 1 + np.log((u ** 4 + (u / 52) ** 2) / (u ** 4 + 0.432)) / 49 + np.log(1 + (u / 18.1) ** 3) / 18.7
    b = 0.564 * ((er - 0.9) / (er + 3)) ** 0.053
    e0 = (er + 1) / 2 + (er - 1) / 2 * (1 + 10 / u) ** (-a * b)
    fn = f * h * 1e-6
    p1 = 0.27488 + (0.6315 + 0.525 / (1 + 0.0157 * fn) ** 20) * u - 0.065683 * np.exp(-8.7513 * u)
    p2 = 0.33622 * (1 - np.exp(-0.03442 * er))
    p3 = 0.0363 * np.exp(-4.6 * u) * (1 - np.exp(-((fn / 38.7) ** 4.97)))
    p4 = 1 + 2.751 * (1 - np.exp(-((er / 15.916) ** 8)))
    p = p1 * p2 * ((0.1844 + p3 * p4) * fn) ** 1.5763
    ee = er - (er - e0) / (1 + p)
    return 2 * np.pi * f / K.C0 * np.sqrt(ee)


class Sweep:
    """Dense sweep of one mesh (interp=None, method='dense')."""

    def __init__(self, mesh, stack):
        if not hasattr(stack, "layers"):
            stack = stack.to_stackup()
        # the levels ordered by height, as Solver.__init__ does before its
        # geometry (mom25d/solver.py:844-846): the via segments' top / bottom
        # pads and the level indices follow this order
        order = sorted(list(mesh.layer_names) + list(getattr(mesh, "planes", [])), key=stack.level_z)
        if getattr(mesh, "level_order", None) != order:
            mesh.assign_levels(order)
        self.mesh, self.stack = mesh, stack
        self.single, self.zl = stack_info(stack, mesh)
        v = mesh.nodes
        self.rho_max = 1.02 * np.hypot(*(v.max(0) - v.min(0)))
        self.geom = Geometry(mesh, self.zl)
        self.ports = mesh.layout.ports
        self.pm = [PortData(mesh, p, stack.level_h(p.layer)) for p in self.ports]
        self.groups = {}
        for p, port in enumerate(self.ports):
            hp = stack.level_h(port.layer)
            key = (round(port.width / hp, 9), port.layer,
                   port.ground.key(hp) if port.ground is not None else None, port.z0_from)
            self.groups.setdefault(key, []).append(p)

    def kernels(self, f):
        return make_kernels(self.stack, self.mesh, f, self.rho_max)

    def impedance(self, f, kern=None):
        kern = kern or self.kernels(f)
        zs = self.stack.surface_impedance(f)
        return fill(self.geom, kern, 2 * np.pi * f, zs, zs)

    def excitations(self):
        return np.stack([pm.excitation for pm in self.pm], 1)

    def point(self, f):
        """(S, z0, gamma, z0_line, residual, x, q, Z) at one frequency."""
        kern = self.kernels(f)
        Z = self.impedance(f, kern)
        x = dense_solve(Z.copy(), self.excitations())
        q = charges(self.mesh, x, kern.omega)
        return self.deembed(f, kern, x, q) + (x, q, Z)

    def deembed(self, f, kern, x, q):
        n = len(self.ports)
        phi = [None] * n
        layers = list(dict.fromkeys(p.layer for p in self.ports))
        for lay in layers:
            ps = [p for p in range(n) if self.ports[p].layer == lay]
            vp = line_voltage(self.mesh, kern, q, np.concatenate([self.pm[p].vpts for p in ps]), lay)
            for p, v in zip(ps, np.split(vp, np.cumsum([len(self.pm[p].vpts) for p in ps])[:-1])):
                phi[p] = v
        A = np.zeros((n, n), complex)
        B = np.zeros((n, n), complex)
        gam = np.zeros(n, complex)
        zl = np.zeros(n, complex)
        res = np.zeros(n)
        for members in self.groups.values():
            port = self.ports[members[0]]
            b0 = beta0(port, self.stack, f)
            bnd = (0.7, 1.3) if not self.stack.covered(port.layer) else (0.7, 1.8)
            s_l, I_l, V_l, keys = [], [], [], []
            for p in members:
                Ip = self.pm[p].currents(x)
                Vp = self.pm[p].voltages(phi[p])
                for e in range(n):
                    s_l.append(self.pm[p].s)
                    I_l.append(Ip[:, e])
                    V_l.append(Vp[:, e])
                    keys.append((p, e))
            g, z0, coefs, r = fit_waves(s_l, I_l, V_l, 1e-3 * b0 + 1j * b0, lossless=self.stack.lossless,
                                        bounds=bnd)
            for (p, e), (a, bb) in zip(keys, coefs):
                A[p, e], B[p, e] = a, bb
            for p in members:
                gam[p], zl[p], res[p] = g, z0, r
        SI = -B @ np.linalg.inv(A)
        z0 = voltage_z0(SI, zl.real, list(self.groups.values()))
        d = np.sqrt(z0)
        S = d[:, None] * SI / d[None, :]
        return S, z0, gam, zl, res

    def sweep(self, freqs):
        out = [self.point(f)[:5] for f in freqs]
        return tuple(np.array([o[k] for o in out]) for k in range(5))


OPEN = 1e12  # ohm: an unloaded lumped gap


def lumped_value(v, f):
    """Z [ohm] of a lumped value at f (mom25d/lumped.py:17-90): an object with
    z(f), a callable, a number, or a string such as 'R 10 + L 0.5n' or
    'C 1p || R 1k'."""
    if isinstance(v, str):
        t = v.strip()
        if "||" in t:
            return 1 / sum(1 / lumped_value(p, f) for p in t.split("||"))
        if "+" in t:
            return sum(lumped_value(p, f) for p in t.split("+"))
        kind, num = t.split()
        mult = dict(f=1e-15, p=1e-12, n=1e-9, u=1e-6, m=1e-3, k=1e3, M=1e6, G=1e9)
        x = float(num[:-1]) * mult[num[-1]] if num[-1] in mult else float(num)
        w = 2 * np.pi * f
        return {"R": complex(x), "L": 1j * w * x, "C": 1 / (1j * w * x)}[kind.upper()]
    if hasattr(v, "z"):
        return complex(v.z(f))
    if callable(v):
        return complex(v(f))
    return complex(v)


def lumped_loads(mesh, f, values=None):
    """D (n_lumped, n_lumped): components across the lumped gaps at f, a
    multi-port block's impedance matrix across its gaps, OPEN where none
    (mom25d/solver.py:1039-1062 without internal ports)."""
    gaps = list(getattr(mesh.layout, "lumped", []))
    names = [q.name for q in gaps]
    D = np.zeros((len(gaps), len(gaps)), complex)
    used = set()
    for model, gn in getattr(mesh.layout, "components", []):
        ix = [names.index(n) for n in gn]
        D[np.ix_(ix, ix)] = model.z(f)
        used.update(ix)
    for k, q in enumerate(gaps):
        v = (values or {}).get(q.name, getattr(q, "value", None))
        if k in used and v is None:
            continue
        D[k, k] = OPEN if v is None else lumped_value(v, f)
    return D


def load_lumped(Lm, D, Xe, Xi):
    """(Z + L D L^T)^-1 e = Xe - Xi D (I + L^T Xi D)^-1 L^T Xe (Woodbury),
    Xi = Z^-1 L (mom25d/solver.py:1064-1070)."""
    M = Lm.T @ Xi
    y = Lm.T @ Xe
    return Xe - Xi @ (D @ np.linalg.solve(np.eye(len(D)) + M @ D, y))


def renormalize(S, z0, zref=50.0):
    out = np.empty_like(S)
    eye = np.eye(S.shape[1])
    for f in range(S.shape[0]):
        sq = np.diag(np.sqrt(z0[f]))
        Zm = sq @ (eye + S[f]) @ np.linalg.inv(eye - S[f]) @ sq
        out[f] = (Zm - zref * eye) @ np.linalg.inv(Zm + zref * eye)
    return out
