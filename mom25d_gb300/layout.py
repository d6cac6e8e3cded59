"""Manhattan layouts (rectangles, microstrip / GCPW port feeds, vias) and the
tensor-grid triangulation with RWG edges that the sweep engine consumes.

This is the input side of the sweep path. The node numbering, the triangle
order, the RWG edge order and the via segment split must be the same as
mom25d's grid mesher (mom25d/mesh.py:696-1097) so that impedance matrices and
currents compare entry by entry; the construction below follows the same
steps (grid lines from rectangle edges plus edge-cell refinement, one cell
split into two triangles with a checkerboard diagonal, RWG edges found by
sorting node-pair keys). Polygons, pours, thick metal, lumped gaps, planes
and apertures are not part of this engine.
"""

from dataclasses import dataclass, field

import numpy as np

_DIRS = {"+x": (1, 0), "-x": (-1, 0), "+y": (0, 1), "-y": (0, -1)}


@dataclass
class CoplanarGround:
    """Side-ground strips of a GCPW feed (mom25d/mesh.py:25-59)."""

    gap: object
    width: object
    via_pitch: float = None
    via_drill: float = 0.3e-3
    via_pad: float = None
    via_to: str = "gnd"
    via_connect: tuple = ()

    def sides(self):
        g = self.gap if isinstance(self.gap, (tuple, list)) else (self.gap, self.gap)
        w = self.width if isinstance(self.width, (tuple, list)) else (self.width, self.width)
        return [(sg, float(gi), float(wi)) for sg, gi, wi in zip((1, -1), g, w) if gi is not None and wi]

    def key(self, scale):
        return tuple((sg, round(gi / scale, 6), round(wi / scale, 6)) for sg, gi, wi in self.sides())


@dataclass
class Port:
    """Axis-aligned feed line with a delta-gap source (mom25d/mesh.py:62-188).

    direction points away from the circuit; the S-parameters are referenced
    to `ref`; the gap sits `gap_from_end` (default: the width) before the
    open end."""

    name: str
    ref: tuple
    direction: str
    width: float
    length: float
    gap_from_end: float = None
    margin: float = None
    layer: str = "top"
    ground: CoplanarGround = None
    z0_from: str = "voltage"

    def __post_init__(self):
        if self.z0_from not in ("voltage", "reciprocity"):
            raise ValueError("z0_from must be 'voltage' or 'reciprocity'")
        if self.direction not in _DIRS:
            raise ValueError(f"direction must be one of {list(_DIRS)} (this engine meshes Manhattan feeds only)")
        self.u = np.array(_DIRS[self.direction], float)
        self.n = np.array([-self.u[1], self.u[0]])
        self.ref = (float(self.ref[0]), float(self.ref[1]))
        if self.gap_from_end is None:
            self.gap_from_end = self.width
        self.aligned = True
        self.axis = 0 if self.direction[1] == "x" else 1
        self.sgn = _DIRS[self.direction][self.axis]

    @property
    def s_gap(self):
        return self.length - self.gap_from_end

    def coord(self, s):
        return self.ref[self.axis] + self.sgn * s

    def point(self, s, t=0.0):
        s, t = np.broadcast_arrays(np.asarray(s, float), np.asarray(t, float))
        return np.asarray(self.ref) + s[..., None] * self.u + t[..., None] * self.n

    def local(self, xy):
        d = np.asarray(xy, float) - np.asarray(self.ref)
        return d @ self.u, d @ self.n

    def rect(self):
        a = self.axis
        c0, c1 = sorted((self.ref[a], self.coord(self.length)))
        t = self.ref[1 - a]
        lo, hi = t - self.width / 2, t + self.width / 2
        return (c0, lo, c1, hi) if a == 0 else (lo, c0, hi, c1)

    def ground_strips(self):
        if self.ground is None:
            return []
        out = []
        for sg, g, w in self.ground.sides():
            t0, t1 = sorted((sg * (self.width / 2 + g), sg * (self.width / 2 + g + w)))
            out.append([tuple(self.point(s, t)) for s, t in
                        ((0, t0), (self.length, t0), (self.length, t1), (0, t1))])
        return out

    def ground_vias(self):
        G = self.ground
        if G is None or not G.via_pitch:
            return []
        n = int(np.floor(self.length / G.via_pitch))
        s = (np.arange(n) + 0.5) * G.via_pitch
        out = []
        for sg, g, w in G.sides():
            pad = min(G.via_pad or 2 * G.via_drill, 0.9 * w)
            if pad < G.via_drill:
                raise ValueError(f"port {self.name}: ground strip too narrow for its fence vias")
            t = sg * (self.width / 2 + g + w / 2)
            out += [Via(tuple(self.point(si, t)), G.via_drill, pad, top=self.layer, bottom=G.via_to,
                        connect=tuple(G.via_connect)) for si in s[s <= self.length - pad / 2]]
        return out


@dataclass
class Via:
    """Plated via between two metal levels ("gnd" = ground plane), mom25d/mesh.py:191-241."""

    xy: tuple
    drill: float
    pad: float = None
    name: str = None
    top: str = "top"
    bottom: str = "gnd"
    connect: tuple = ()
    antipad: float = None

    def __post_init__(self):
        self.xy = (float(self.xy[0]), float(self.xy[1]))
        self.connect = tuple(self.connect)
        if self.pad is None:
            self.pad = 2 * self.drill
        if self.pad < self.drill:
            raise ValueError("via pad smaller than its drill")
        if self.top == self.bottom:
            raise ValueError("via top and bottom layer are the same")
        if self.connect or self.antipad is not None:
            raise ValueError("inner-plane connections and antipads are not part of this engine")

    def pad_layers(self):
        return [n for n in (self.top, self.bottom) if n != "gnd"]


@dataclass
class Layout:
    """Copper rectangles, port feeds and vias on named metal levels."""

    rects: list = field(default_factory=list)
    rect_layers: list = field(default_factory=list)
    ports: list = field(default_factory=list)
    vias: list = field(default_factory=list)
    planes: list = field(default_factory=list)
    lumped: list = field(default_factory=list)
    components: list = field(default_factory=list)  # (model, [gap names]): multi-port blocks across lumped gaps
    internal_ports: list = field(default_factory=list)

    def add_rect(self, x0, y0, x1, y1, layer="top"):
        self.rects.append((min(x0, x1), min(y0, y1), max(x0, x1), max(y0, y1)))
        self.rect_layers.append(layer)
        return self

    def add_port(self, name, ref, direction, width, length, **kw):
        p = Port(name, tuple(ref), direction, width, length, **kw)
        self.ports.append(p)
        self.add_rect(*p.rect(), layer=p.layer)
        for c in p.ground_strips():
            xs, ys = zip(*c)
            self.add_rect(min(xs), min(ys), max(xs), max(ys), layer=p.layer)
        self.vias.extend(p.ground_vias())
        return p

    def add_lumped(self, name, a, b, width, value=None, layer="top"):
        """Lumped component across a delta gap in the middle of a copper
        bridge of `width` from pad point a to pad point b (axis-aligned),
        loaded with `value` (lumped.R / L / C / series / parallel, a number in
        ohm, a callable f -> Z, a string like 'C 1p' or 'R 10 + L 0.5n'; None:
        an open gap); voltage a -> b (mom25d/mesh.py:353-378)."""
        from .lumped import as_value, parse

        a, b = np.asarray(a, float), np.asarray(b, float)
        d = b - a
        length = float(np.hypot(*d))
        if length <= 0:
            raise ValueError("lumped component: a and b coincide")
        if any(q.name == name for q in self.lumped) or any(q.name == name for q in self.ports):
            raise ValueError(f"name {name!r} already used")
        u = d / length
        direction = next((k for k, v in _DIRS.items() if np.allclose(u, v, atol=1e-12)), None)
        if direction is None:
            raise ValueError(f"lumped {name}: oblique bridges need the triangular mesher (not part of this engine)")
        g = Port(name, tuple(a), direction, width, length, gap_from_end=0.5 * length, layer=layer)
        g.value = None if value is None else (parse(value) if isinstance(value, str) else as_value(value))
        self.lumped.append(g)
        self.add_rect(*g.rect(), layer=layer)
        return g

    def add_component(self, model, gaps):
        """Multi-port component (network.Touchstone or a .sNp path) across the
        named lumped gaps, in the model's port order; the gaps are added with
        value=None (mom25d/mesh.py:432-447)."""
        from .network import Touchstone

        if isinstance(model, str):
            model = Touchstone(model)
        names = [q.name for q in self.lumped]
        for n in gaps:
            if n not in names:
                raise ValueError(f"no lumped gap {n!r}")
        if getattr(model, "n", len(gaps)) != len(gaps):
            raise ValueError(f"{model} has {model.n} ports, {len(gaps)} gaps given")
        self.components.append((model, list(gaps)))
        return self

    def add_via(self, x, y, drill=0.3e-3, pad=None, name=None, top="top", bottom="gnd"):
        v = Via((x, y), drill, pad, name, top, bottom)
        self.vias.append(v)
        return v

    def layer_names(self):
        names = list(self.rect_layers) + [n for v in self.vias for n in v.pad_layers()]
        return [n for n in dict.fromkeys(names) if n not in self.planes]

    def all_vias(self):
        return list(self.vias)

    def bbox(self):
        r = [tuple(q) for q in self.rects]
        for v in self.vias:
            r.append((v.xy[0] - v.pad / 2, v.xy[1] - v.pad / 2, v.xy[0] + v.pad / 2, v.xy[1] + v.pad / 2))
        r = np.array(r)
        return r[:, 0].min(), r[:, 1].min(), r[:, 2].max(), r[:, 3].max()

    def contains(self, x, y, layer=None):
        inside = np.zeros(np.broadcast(x, y).shape, bool)
        for (x0, y0, x1, y1), n in zip(self.rects, self.rect_layers):
            if layer is None or n == layer:
                inside |= (x > x0) & (x < x1) & (y > y0) & (y < y1)
        for v in self.vias:  # round pads add copper but no grid lines
            if layer is None or layer in v.pad_layers():
                inside |= (x - v.xy[0]) ** 2 + (y - v.xy[1]) ** 2 < (v.pad / 2) ** 2
        return inside

    def mesh(self, max_cell, edge_cell=None, snap=None, kind="grid"):
        if kind != "grid":
            raise ValueError("this engine meshes with kind='grid' only")
        return Mesh.from_layout(self, max_cell, edge_cell)


def _grid_lines(fixed, refine, lo, hi, max_cell, tol):
    """Sorted grid coordinates: the fixed and refinement lines (merged on a
    `tol` lattice), each interval subdivided evenly to <= max_cell."""
    c = np.unique(np.round(np.concatenate([fixed, refine]) / tol) * tol)
    c = c[(c >= lo - tol) & (c <= hi + tol)]
    out = [c[0]]
    for a, b in zip(c[:-1], c[1:]):
        n = int(np.ceil((b - a) / max_cell - 1e-9))
        out.extend(np.linspace(a, b, n + 1)[1:])
    return np.array(out)


class Mesh:
    """Triangles of all metal levels on one shared tensor grid, RWG edges,
    via segments and port cut look-ups (the arrays mom25d's Mesh exposes)."""

    def __init__(self, nodes, tris, layout, xg, yg, tri_layer, layer_names):
        self.nodes = np.asarray(nodes, float)
        self.tris = np.asarray(tris, int)
        self.layout = layout
        self.xg, self.yg = xg, yg
        self.layer_names = list(layer_names)
        self.tri_layer = np.asarray(tri_layer, int)
        self.twin_layer = -np.ones(len(self.layer_names), int)
        self.planes = list(getattr(layout, "planes", []))
        self._orient()
        self._edges()
        self.edge_layer = self.tri_layer[self.tp]
        self._attach_vias(layout.all_vias())

    @classmethod
    def from_layout(cls, layout, max_cell, edge_cell=None):
        x0, y0, x1, y1 = layout.bbox()
        tol = 1e-9 * max(x1 - x0, y1 - y0)
        fx = [c for r in layout.rects for c in (r[0], r[2])]
        fy = [c for r in layout.rects for c in (r[1], r[3])]
        for p in layout.ports:
            (fx if p.axis == 0 else fy).extend([p.coord(0), p.coord(p.s_gap)])
        for p in layout.lumped:  # a lumped gap and its bridge's ends are grid lines
            (fx if p.axis == 0 else fy).extend([p.coord(0), p.coord(p.s_gap), p.coord(p.length)])
        rx, ry = [], []
        if edge_cell:
            rx = [c + d for c in fx for d in (-edge_cell, edge_cell)]
            ry = [c + d for c in fy for d in (-edge_cell, edge_cell)]
            rx = [c for c in rx if np.min(np.abs(np.array(fx) - c)) > 0.5 * edge_cell]
            ry = [c for c in ry if np.min(np.abs(np.array(fy) - c)) > 0.5 * edge_cell]
        xg = _grid_lines(fx, rx, x0, x1, max_cell, tol)
        yg = _grid_lines(fy, ry, y0, y1, max_cell, tol)
        xc = 0.5 * (xg[1:] + xg[:-1])
        yc = 0.5 * (yg[1:] + yg[:-1])
        XC, YC = np.meshgrid(xc, yc, indexing="ij")
        names = layout.layer_names() or ["top"]
        ny = len(yg)
        nxy = len(xg) * ny
        tris, tl = [], []
        for li, name in enumerate(names):
            ii, jj = np.nonzero(layout.contains(XC, YC, name))
            base = li * nxy
            a = base + ii * ny + jj
            b = base + (ii + 1) * ny + jj
            c = base + (ii + 1) * ny + jj + 1
            d = base + ii * ny + jj + 1
            odd = ((ii + jj) % 2 == 1)[:, None]
            tris.append(np.where(odd, np.stack([a, b, d], 1), np.stack([a, b, c], 1)))
            tris.append(np.where(odd, np.stack([b, c, d], 1), np.stack([a, c, d], 1)))
            tl.append(np.full(2 * ii.size, li))
        tris = np.concatenate(tris)
        used, inv = np.unique(tris, return_inverse=True)
        X, Y = np.meshgrid(xg, yg, indexing="ij")
        nodes = np.stack([np.tile(X.ravel(), len(names))[used], np.tile(Y.ravel(), len(names))[used]], 1)
        return cls(nodes, inv.reshape(tris.shape), layout, xg, yg, np.concatenate(tl), names)

    # ------------------------------------------------------------ geometry
    def _orient(self):
        v = self.nodes[self.tris]
        e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
        cross = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
        cw = cross < 0
        self.tris[cw] = self.tris[cw][:, [0, 2, 1]]
        self.verts = self.nodes[self.tris]
        self.area = 0.5 * np.abs(cross)
        self.centroid = self.verts.mean(1)

    def _edges(self):
        """Interior edges (shared by two triangles) become RWG bases; local
        edge i of a triangle is the one opposite its vertex i."""
        nt = len(self.tris)
        ends = np.concatenate([np.sort(self.tris[:, [1, 2]], 1), np.sort(self.tris[:, [2, 0]], 1),
                               np.sort(self.tris[:, [0, 1]], 1)])
        owner = np.tile(np.arange(nt), 3)
        local = np.repeat(np.arange(3), nt)
        key = ends[:, 0] * len(self.nodes) + ends[:, 1]
        order = np.argsort(key, kind="stable")
        ks = key[order]
        dup = ks[1:] == ks[:-1]
        if np.any(dup[1:] & dup[:-1]):
            raise ValueError("non-manifold edge (more than two triangles)")
        first, second = order[:-1][dup], order[1:][dup]
        self.edge_nodes = ends[first]
        self.tp, self.vp = owner[first], local[first]
        self.tm, self.vm = owner[second], local[second]
        d = self.nodes[self.edge_nodes[:, 1]] - self.nodes[self.edge_nodes[:, 0]]
        self.edge_len = np.hypot(d[:, 0], d[:, 1])
        self.edge_mid = 0.5 * (self.nodes[self.edge_nodes[:, 0]] + self.nodes[self.edge_nodes[:, 1]])
        self.n_basis = len(self.tp)
        self.wall = np.zeros(self.n_basis, bool)
        self.n_walls = 0
        self.tri_basis = -np.ones((nt, 3), int)
        self.tri_sign = np.zeros((nt, 3))
        idx = np.arange(self.n_basis)
        self.tri_basis[self.tp, self.vp] = idx
        self.tri_sign[self.tp, self.vp] = 1.0
        self.tri_basis[self.tm, self.vm] = idx
        self.tri_sign[self.tm, self.vm] = -1.0

    # ---------------------------------------------------------------- vias
    def _cell_tris(self, x, y):
        """Triangles of the grid cell(s) holding (x, y); every cell touching it
        when it lies on a grid line."""
        def span(g, c):
            tol = 1e-6 * (g[-1] - g[0])
            k = np.nonzero(np.abs(g - c) < tol)[0]
            if k.size:
                return g[max(k[0] - 1, 0)], g[min(k[0] + 1, len(g) - 1)]
            i = np.searchsorted(g, c) - 1
            return (g[i], g[i + 1]) if 0 <= i < len(g) - 1 else (c, c)

        (x0, x1), (y0, y1) = span(self.xg, x), span(self.yg, y)
        c = self.centroid
        return np.nonzero((c[:, 0] > x0) & (c[:, 0] < x1) & (c[:, 1] > y0) & (c[:, 1] < y1))[0]

    def _attach_vias(self, vias):
        self.vias = list(vias)
        self.via_attach = []
        c = self.centroid
        for v in self.vias:
            att = {}
            x, y = v.xy
            d2 = (c[:, 0] - x) ** 2 + (c[:, 1] - y) ** 2
            for li, name in enumerate(self.layer_names):
                on = self.tri_layer == li
                t = np.nonzero(on & (d2 < (v.drill / 2) ** 2))[0]
                if t.size == 0:
                    t = self._cell_tris(x, y)
                    t = t[on[t]]
                if t.size:
                    att[name] = t
            for n in v.pad_layers():
                if n in self.layer_names and n not in att:
                    raise ValueError(f"via at ({x * 1e3:.4g}, {y * 1e3:.4g}) mm: no meshed copper on layer {n}")
            self.via_attach.append(att)
        self.assign_levels(self.layer_names + self.planes)

    def assign_levels(self, order):
        """Split every via into vertical segments between the levels it touches
        (top to bottom); unknown n_basis + k is segment k's downward current."""
        rank = {n: i for i, n in enumerate(order)}
        rank["gnd"] = -1
        self.via_segments = []
        for k, (v, att) in enumerate(zip(self.vias, self.via_attach)):
            for n in (v.top, v.bottom):
                if n not in rank:
                    raise ValueError(f"via layer {n!r} is not in the stack order {order}")
            hi, lo = sorted((rank[v.top], rank[v.bottom]), reverse=True)
            mid = sorted([n for n in order if lo < rank[n] < hi and n in att], key=lambda n: -rank[n])
            chain = [order[hi]] + mid + [order[lo] if lo >= 0 else "gnd"]
            for a, b in zip(chain[:-1], chain[1:]):
                self.via_segments.append(dict(via=k, top=a, bottom=b, top_tris=att.get(a), bottom_tris=att.get(b)))
        self.level_order = list(order)
        self.n_vias = len(self.via_segments)
        self.n_frills = 0
        self.n_ap = 0
        self.via_tris = [g["top_tris"] for g in self.via_segments]
        self.n_unknowns = self.n_basis + self.n_vias

    # --------------------------------------------------------------- ports
    def flow_direction(self):
        d = self.centroid[self.tm] - self.centroid[self.tp]
        n = np.linalg.norm(d, axis=1)
        return d / np.where(n > 0, n, 1.0)[:, None]

    def cut_positions(self, port):
        g = self.xg if port.axis == 0 else self.yg
        s = port.sgn * (g - port.ref[port.axis])
        s = s[(s > -1e-12) & (s <= port.length + 1e-12)]
        return np.sort(s)

    def lumped_vectors(self):
        """(N, n_lumped) signed edge lengths of each lumped gap's cut: the
        delta-gap excitation of the gap, and l . x its current a -> b
        (mom25d/mesh.py:1077-1087)."""
        gaps = list(getattr(self.layout, "lumped", []))
        Lm = np.zeros((self.n_unknowns, len(gaps)))
        for k, p in enumerate(gaps):
            idx, sgn = self.cut_edges(p, p.s_gap)
            if idx.size == 0:
                raise ValueError(f"lumped {p.name}: no mesh edges on its gap")
            Lm[idx, k] = -sgn * self.edge_len[idx]
        return Lm

    def cut_edges(self, port, s):
        """RWG edges on the transverse cut at distance s of a feed, signed so
        that positive current flows toward the circuit."""
        # the edges' coordinates in the port frame do not depend on s: once per port
        cache = self.__dict__.setdefault("_cut_frames", {})
        key = id(port)
        if key not in cache or cache[key][0] is not port:
            es, _ = port.local(self.nodes[self.edge_nodes])
            _, tm = port.local(self.edge_mid)
            cand = (np.abs(tm) < port.width / 2) & (self.edge_layer == self.layer_names.index(port.layer))
            idx = np.nonzero(cand)[0]
            cache[key] = (port, es[idx], idx, np.sign(self.flow_direction()[idx] @ -port.u))
        _, es, idx, sign = cache[key]
        tol = 1e-6 * port.width
        on = (np.abs(es[:, 0] - s) < tol) & (np.abs(es[:, 1] - s) < tol)
        return idx[on], sign[on]
