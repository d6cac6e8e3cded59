"""Layouts on named metal levels and their structured triangle mesh: the
input side of the sweep path.

A layout here is what mom25d's grid mesher accepts for the workloads of this
engine: axis-aligned copper rectangles per metal level, feed ports along x or
y (optionally with coplanar side grounds and fence vias), plated round vias
and lumped gaps with their copper bridges. The public names and the meaning
of every argument are mom25d's (Layout / Port / Via / CoplanarGround,
Engine/mom25d/mesh.py:25-460), so a script written for mom25d builds the
same geometry here.

How the mesh is made (`mesh()`):

1. Grid lines. Every rectangle edge, every feed's reference plane and delta
   gap, and every lumped gap and bridge end is a grid line of its axis; with
   an edge cell, lines one edge cell to either side of each of those are
   added unless another fixed line is nearer than half an edge cell. Lines
   closer than 1e-9 of the layout's extent are merged, and each interval is
   cut evenly into cells no longer than max_cell.
2. Cells to triangles. All levels share the grid. A cell whose centre lies
   in copper of a level becomes two triangles of that level, split along the
   diagonal that alternates from cell to cell like a chessboard.
3. Unknowns. Every edge shared by two triangles is an RWG basis (sorted by
   its node pair); then one vertical current per via segment, a via being
   split at every meshed level it passes.

The numbering of nodes, triangles, edges and via segments is the one mom25d
produces for the same layout, because parity with mom25d compares impedance
matrices and currents entry by entry; `tests/test_cpu_mesh_oracle.py` checks
it by hash against meshes made by mom25d. Polygons, pours, thick metal,
inner planes, antipads and apertures are not part of this engine.
"""

from dataclasses import dataclass, field

import numpy as np

# feed direction -> (axis the feed runs along, sign along that axis)
_HEADINGS = {"+x": (0, 1), "-x": (0, -1), "+y": (1, 1), "-y": (1, -1)}


def _heading(name, direction):
    try:
        return _HEADINGS[direction]
    except (KeyError, TypeError):
        raise ValueError(f"{name}: this engine meshes feeds that run along an axis; direction must be one of "
                         f"{sorted(_HEADINGS)}, got {direction!r}") from None


@dataclass
class CoplanarGround:
    """Ground strips beside a feed (a grounded coplanar feed) and the vias
    that tie them down. gap / width: one number for both sides, or a pair
    (left, right) where left is the side at +t, to the left of the feed's
    outward direction; a side whose gap is None or whose width is 0 has no
    strip. via_pitch: spacing of the vias along each strip's centre line
    (None: no vias); via_drill / via_pad: their drill and pad diameters (pad
    default: twice the drill, at most 0.9 of the strip width); via_to: the
    level the vias end on."""

    gap: object
    width: object
    via_pitch: float = None
    via_drill: float = 0.3e-3
    via_pad: float = None
    via_to: str = "gnd"
    via_connect: tuple = ()

    def sides(self):
        """(sign of t, gap, width) for each side that carries a strip, +t first."""
        both = lambda v: tuple(v) if isinstance(v, (tuple, list)) else (v, v)  # noqa: E731
        out = []
        for sign, g, w in zip((1, -1), both(self.gap), both(self.width)):
            if g is not None and w:
                out.append((sign, float(g), float(w)))
        return out

    def key(self, scale):
        """The strips' geometry in units of `scale`, rounded: feeds whose
        keys (and widths and levels) agree share one wave fit."""
        return tuple((sign, round(g / scale, 6), round(w / scale, 6)) for sign, g, w in self.sides())


@dataclass
class Port:
    """A straight feed line with a delta-gap source near its open end.

    The feed starts at the reference plane `ref` (the point on its centre
    line where S is referenced) and runs `length` along `direction`, away
    from the circuit; the gap sits `gap_from_end` (default: the width) short
    of the open end. `margin` keeps the wave fit that far from the reference
    plane and from the gap (default max(1.5 width, 4 h)). Positions along
    the feed are s (0 at the reference plane), across it t (positive to the
    left of the direction)."""

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
            raise ValueError(f"port {self.name}: z0_from is 'voltage' or 'reciprocity', not {self.z0_from!r}")
        self.axis, self.sgn = _heading(f"port {self.name}", self.direction)
        self.ref = (float(self.ref[0]), float(self.ref[1]))
        if self.gap_from_end is None:
            self.gap_from_end = self.width
        # t grows to the left of the direction: +y for +x, -x for +y, ...
        self.side = self.sgn if self.axis == 0 else -self.sgn
        self.u = np.zeros(2)
        self.u[self.axis] = self.sgn
        self.n = np.zeros(2)
        self.n[1 - self.axis] = self.side
        self.aligned = True

    @property
    def s_gap(self):
        """Distance of the delta gap from the reference plane."""
        return self.length - self.gap_from_end

    def coord(self, s):
        """Layout coordinate (along the feed's axis) of the cut at s."""
        return self.ref[self.axis] + self.sgn * s

    def point(self, s, t=0.0):
        """(x, y) of the feed-frame points (s, t); broadcasts."""
        s, t = np.broadcast_arrays(np.asarray(s, float), np.asarray(t, float))
        xy = np.empty(s.shape + (2,))
        xy[..., self.axis] = self.ref[self.axis] + self.sgn * s
        xy[..., 1 - self.axis] = self.ref[1 - self.axis] + self.side * t
        return xy

    def local(self, xy):
        """Feed-frame (s, t) of layout points (..., 2)."""
        xy = np.asarray(xy, float)
        s = self.sgn * (xy[..., self.axis] - self.ref[self.axis])
        t = self.side * (xy[..., 1 - self.axis] - self.ref[1 - self.axis])
        return s, t

    def _box(self, t_lo, t_hi):
        """Layout rectangle over the whole feed length between t_lo < t_hi."""
        a0, a1 = sorted((self.coord(0.0), self.coord(self.length)))
        b0, b1 = sorted((self.ref[1 - self.axis] + self.side * t_lo, self.ref[1 - self.axis] + self.side * t_hi))
        return (a0, b0, a1, b1) if self.axis == 0 else (b0, a0, b1, a1)

    def rect(self):
        """The feed's copper as (x0, y0, x1, y1)."""
        return self._box(-self.width / 2, self.width / 2)

    def ground_rects(self):
        """The side-ground strips' copper, one rectangle per side."""
        if self.ground is None:
            return []
        out = []
        for sign, g, w in self.ground.sides():
            t0, t1 = sorted((sign * (self.width / 2 + g), sign * (self.width / 2 + g + w)))
            out.append(self._box(t0, t1))
        return out

    def ground_vias(self):
        """Fence vias along the centre of each side strip, every via_pitch
        from half a pitch on, while a whole pad fits on the feed."""
        G = self.ground
        if G is None or not G.via_pitch:
            return []
        s = (np.arange(int(np.floor(self.length / G.via_pitch))) + 0.5) * G.via_pitch
        vias = []
        for sign, g, w in G.sides():
            pad = min(G.via_pad or 2 * G.via_drill, 0.9 * w)
            if pad < G.via_drill:
                raise ValueError(f"port {self.name}: a {w * 1e3:g} mm ground strip has no room for "
                                 f"{G.via_drill * 1e3:g} mm fence vias")
            t = sign * (self.width / 2 + g + w / 2)
            for si in s[s <= self.length - pad / 2]:
                vias.append(Via(tuple(self.point(si, t)), G.via_drill, pad, top=self.layer, bottom=G.via_to,
                                connect=tuple(G.via_connect)))
        return vias


@dataclass
class Via:
    """A plated round via from metal level `top` down to `bottom` ("gnd" is
    the ground plane), with a round pad (default twice the drill) on each
    meshed level it ends on."""

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
        where = f"via at ({self.xy[0] * 1e3:g}, {self.xy[1] * 1e3:g}) mm"
        if self.pad < self.drill:
            raise ValueError(f"{where}: its pad ({self.pad * 1e3:g} mm) is narrower than its drill")
        if self.top == self.bottom:
            raise ValueError(f"{where}: it starts and ends on {self.top!r}")
        if self.connect or self.antipad is not None:
            raise ValueError(f"{where}: plane connections and antipads need inner planes, which this engine "
                             "does not model")

    def pad_layers(self):
        """The meshed levels the via has a pad on."""
        return [lv for lv in (self.top, self.bottom) if lv != "gnd"]


@dataclass
class Layout:
    """Copper on named metal levels: rectangles, feed ports, vias, lumped
    gaps and multi-port blocks across them. Every add_* takes the level as
    `layer=` (default "top"); the names are metal levels of the Stackup the
    layout is solved on."""

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
        """A feed port (see Port); its line, side grounds and fence vias
        become copper of the layout."""
        port = Port(name, tuple(ref), direction, width, length, **kw)
        self.ports.append(port)
        for r in [port.rect()] + port.ground_rects():
            self.add_rect(*r, layer=port.layer)
        self.vias.extend(port.ground_vias())
        return port

    def add_lumped(self, name, a, b, width, value=None, layer="top"):
        """A lumped component between pad points a and b (x, y) [m]: a copper
        bridge of `width` from a to b, along x or y, with a delta gap in its
        middle, loaded by `value` (lumped.R / L / C / series / parallel, a
        number in ohm, a callable f -> Z, or text such as 'C 1p' or
        'R 10 + L 0.5n'; None leaves the gap open, e.g. for a port of a
        multi-port block). Its voltage is taken from a to b."""
        from .lumped import as_value, parse

        a, b = np.asarray(a, float), np.asarray(b, float)
        span = b - a
        length = float(np.hypot(*span))
        if length <= 0:
            raise ValueError(f"lumped {name}: its two pad points are the same")
        taken = {q.name for q in self.lumped} | {q.name for q in self.ports}
        if name in taken:
            raise ValueError(f"lumped {name}: the name is already taken by a port or another component")
        heading = next((k for k, (ax, sg) in _HEADINGS.items()
                        if span[ax] * sg > 0 and span[1 - ax] == 0), None)
        if heading is None:
            raise ValueError(f"lumped {name}: bridges run along x or y in this engine")
        gap = Port(name, tuple(a), heading, width, length, gap_from_end=0.5 * length, layer=layer)
        gap.value = None if value is None else (parse(value) if isinstance(value, str) else as_value(value))
        self.lumped.append(gap)
        self.add_rect(*gap.rect(), layer=layer)
        return gap

    def add_gap_port(self, name, a, b, width, layer="top", z_ref=50.0):
        """An internal S-parameter port of reference impedance z_ref across a
        delta gap: a copper bridge of `width` from pad point a to pad point b
        as add_lumped makes it, the port's voltage taken from a to b (e.g. a
        device pin to its ground pad)."""
        gap = self.add_lumped(name, a, b, width, None, layer)
        self.internal_ports.append(dict(kind="gap", name=name, z_ref=float(z_ref)))
        return gap

    def add_via_port(self, name, via, z_ref=50.0):
        """An internal S-parameter port at the bottom of a via that ends on
        the ground plane: a delta gap between the barrel and the plane (the
        via fed through a hole in the ground), voltage barrel to ground, the
        port current flowing down the via. `via`: index into vias, or the
        Via itself."""
        k = via if isinstance(via, (int, np.integer)) else next(
            (i for i, v in enumerate(self.vias) if v is via), None)
        if k is None or not 0 <= k < len(self.vias):
            raise ValueError(f"via port {name}: no such via in the layout")
        if self.vias[k].bottom != "gnd":
            raise ValueError(f"via port {name}: the via must end on the ground plane (bottom 'gnd')")
        taken = {q.name for q in self.lumped} | {q.name for q in self.ports} | {q["name"] for q in self.internal_ports}
        if name in taken:
            raise ValueError(f"via port {name}: the name is already taken")
        self.internal_ports.append(dict(kind="via", name=name, via=int(k), z_ref=float(z_ref)))
        return k

    def add_component(self, model, gaps):
        """A multi-port block (network.Touchstone, or a .sNp path) across the
        named lumped gaps, port k of the model across gaps[k]; add those gaps
        with value=None."""
        from .network import Touchstone

        if isinstance(model, str):
            model = Touchstone(model)
        known = {q.name for q in self.lumped}
        missing = [g for g in gaps if g not in known]
        if missing:
            raise ValueError(f"component {model}: no lumped gaps named {missing}")
        if getattr(model, "n", len(gaps)) != len(gaps):
            raise ValueError(f"component {model}: {model.n} ports but {len(gaps)} gaps")
        self.components.append((model, list(gaps)))
        return self

    def add_via(self, x, y, drill=0.3e-3, pad=None, name=None, top="top", bottom="gnd"):
        v = Via((x, y), drill, pad, name, top, bottom)
        self.vias.append(v)
        return v

    def layer_names(self):
        """Meshed levels in order of first use (rectangles, then via pads)."""
        seen = dict.fromkeys(list(self.rect_layers) + [lv for v in self.vias for lv in v.pad_layers()])
        return [lv for lv in seen if lv not in self.planes]

    def all_vias(self):
        return list(self.vias)

    def bbox(self):
        """(x0, y0, x1, y1) over the rectangles and the via pads."""
        boxes = [tuple(r) for r in self.rects]
        boxes += [(v.xy[0] - v.pad / 2, v.xy[1] - v.pad / 2, v.xy[0] + v.pad / 2, v.xy[1] + v.pad / 2)
                  for v in self.vias]
        b = np.array(boxes)
        return b[:, 0].min(), b[:, 1].min(), b[:, 2].max(), b[:, 3].max()

    def contains(self, x, y, layer=None):
        """Whether the points (x, y) lie strictly inside copper (of `layer`,
        or of any level): a rectangle, or a via's round pad."""
        inside = np.zeros(np.broadcast(x, y).shape, bool)
        for (x0, y0, x1, y1), lv in zip(self.rects, self.rect_layers):
            if layer is None or lv == layer:
                inside |= (x > x0) & (x < x1) & (y > y0) & (y < y1)
        for v in self.vias:  # pads are copper but add no grid lines
            if layer is None or layer in v.pad_layers():
                inside |= (x - v.xy[0]) ** 2 + (y - v.xy[1]) ** 2 < (v.pad / 2) ** 2
        return inside

    def fixed_lines(self):
        """Coordinates that must be grid lines, per axis: rectangle edges,
        every feed's reference plane and gap, every lumped gap and the ends
        of its bridge."""
        lines = ([], [])
        for x0, y0, x1, y1 in self.rects:
            lines[0].extend((x0, x1))
            lines[1].extend((y0, y1))
        for p in self.ports:
            lines[p.axis].extend((p.coord(0), p.coord(p.s_gap)))
        for g in self.lumped:
            lines[g.axis].extend((g.coord(0), g.coord(g.s_gap), g.coord(g.length)))
        return lines

    def mesh(self, max_cell, edge_cell=None, snap=None, kind="grid"):
        if kind != "grid":
            raise ValueError("this engine meshes with kind='grid' only")
        return Mesh.from_layout(self, max_cell, edge_cell)


# ------------------------------------------------------------------ mesher
def axis_lines(fixed, lo, hi, max_cell, edge_cell, tol):
    """Grid coordinates of one axis: the fixed lines, the edge-cell lines
    beside them (those at least half an edge cell from every fixed line),
    merged on a `tol` lattice, clipped to [lo, hi] and cut into cells of at
    most max_cell."""
    fixed = np.asarray(fixed, float)
    lines = fixed
    if edge_cell:
        beside = (fixed[:, None] + np.array([-edge_cell, edge_cell])[None, :]).ravel()
        clear = np.abs(fixed[None, :] - beside[:, None]).min(axis=1) > 0.5 * edge_cell
        lines = np.concatenate([fixed, beside[clear]])
    merged = np.unique(np.round(lines / tol) * tol)
    merged = merged[(merged >= lo - tol) & (merged <= hi + tol)]
    parts = [merged[:1]]
    for a, b in zip(merged[:-1], merged[1:]):
        cells = int(np.ceil((b - a) / max_cell - 1e-9))
        parts.append(np.linspace(a, b, cells + 1)[1:])
    return np.concatenate(parts)


def cell_triangles(layout, xg, yg, levels):
    """Two triangles per copper cell of each level. Node (level, i, j) of
    the grid has the id (level nx + i) ny + j. Per level, the cells in
    row-major (i, j) order give first all their lower triangles, then all
    their upper ones. Returns the triangles (ids) and their levels."""
    nx, ny = len(xg), len(yg)
    XC, YC = np.meshgrid(0.5 * (xg[1:] + xg[:-1]), 0.5 * (yg[1:] + yg[:-1]), indexing="ij")
    tris, level = [], []
    for lv, name in enumerate(levels):
        i, j = np.nonzero(layout.contains(XC, YC, name))
        sw = (lv * nx + i) * ny + j
        se, ne, nw = sw + ny, sw + ny + 1, sw + 1
        odd = ((i + j) % 2 == 1)[:, None]  # the diagonal runs se-nw on odd cells, sw-ne on even ones
        tris.append(np.where(odd, np.stack([sw, se, nw], 1), np.stack([sw, se, ne], 1)))
        tris.append(np.where(odd, np.stack([se, ne, nw], 1), np.stack([sw, ne, nw], 1)))
        level.append(np.full(2 * i.size, lv))
    return np.concatenate(tris), np.concatenate(level)


def shared_edges(tris, n_nodes):
    """Edges shared by two triangles, ordered by their (smaller, larger)
    node pair. Local edge k of a triangle is the one facing its vertex k.
    Returns the node pairs and, per edge, the triangle listed first (local
    edges taken 0 for all triangles, then 1, then 2), its local edge, the
    other triangle and its local edge."""
    nt = len(tris)
    facing = ((1, 2), (2, 0), (0, 1))
    pairs = np.concatenate([np.sort(tris[:, list(f)], axis=1) for f in facing])  # slot = k nt + triangle
    key = pairs[:, 0] * n_nodes + pairs[:, 1]
    slot = np.arange(3 * nt)
    order = np.lexsort((slot, key))
    k_sorted = key[order]
    same = k_sorted[1:] == k_sorted[:-1]
    if np.any(same[1:] & same[:-1]):
        raise ValueError("mesh edge shared by more than two triangles")
    a, b = order[:-1][same], order[1:][same]
    return pairs[a], a % nt, a // nt, b % nt, b // nt


class Mesh:
    """Triangles of all metal levels on one grid, their RWG bases, the via
    segments and the look-ups the port models use (the arrays and methods
    of mom25d's Mesh that the sweep path reads)."""

    def __init__(self, nodes, tris, layout, xg, yg, tri_layer, layer_names):
        self.nodes = np.asarray(nodes, float)
        self.tris = np.asarray(tris, int)
        self.layout = layout
        self.xg, self.yg = xg, yg
        self.layer_names = list(layer_names)
        self.tri_layer = np.asarray(tri_layer, int)
        self.twin_layer = -np.ones(len(self.layer_names), int)
        self.planes = list(getattr(layout, "planes", []))
        self._counter_clockwise()
        self._rwg()
        self.edge_layer = self.tri_layer[self.tp]
        self.vias = layout.all_vias()
        self.via_attach = [self._via_ends(v) for v in self.vias]
        self.assign_levels(self.layer_names + self.planes)

    @classmethod
    def from_layout(cls, layout, max_cell, edge_cell=None):
        x0, y0, x1, y1 = layout.bbox()
        tol = 1e-9 * max(x1 - x0, y1 - y0)
        fx, fy = layout.fixed_lines()
        xg = axis_lines(fx, x0, x1, max_cell, edge_cell, tol)
        yg = axis_lines(fy, y0, y1, max_cell, edge_cell, tol)
        levels = layout.layer_names() or ["top"]
        ids, level = cell_triangles(layout, xg, yg, levels)
        used, local = np.unique(ids, return_inverse=True)  # keep the grid nodes that triangles use
        per_level = used % (len(xg) * len(yg))
        nodes = np.stack([xg[per_level // len(yg)], yg[per_level % len(yg)]], 1)
        return cls(nodes, local.reshape(ids.shape), layout, xg, yg, level, levels)

    # ------------------------------------------------------------ geometry
    def _counter_clockwise(self):
        p = self.nodes[self.tris]
        e1, e2 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]
        twice_area = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
        flip = twice_area < 0
        self.tris[flip] = self.tris[flip][:, [0, 2, 1]]
        self.verts = self.nodes[self.tris]
        self.area = 0.5 * np.abs(twice_area)
        self.centroid = self.verts.mean(1)

    def _rwg(self):
        """One RWG basis per shared edge: + on the triangle listed first, -
        on the other; tri_basis / tri_sign give each triangle's bases by
        local edge (-1 / 0 on boundary edges)."""
        nt = len(self.tris)
        self.edge_nodes, self.tp, self.vp, self.tm, self.vm = shared_edges(self.tris, len(self.nodes))
        a, b = self.nodes[self.edge_nodes[:, 0]], self.nodes[self.edge_nodes[:, 1]]
        self.edge_len = np.hypot((b - a)[:, 0], (b - a)[:, 1])
        self.edge_mid = 0.5 * (a + b)
        self.n_basis = len(self.tp)
        self.wall = np.zeros(self.n_basis, bool)
        self.n_walls = 0
        self.tri_basis = np.full((nt, 3), -1)
        self.tri_sign = np.zeros((nt, 3))
        basis = np.arange(self.n_basis)
        self.tri_basis[self.tp, self.vp] = basis
        self.tri_basis[self.tm, self.vm] = basis
        self.tri_sign[self.tp, self.vp] = 1.0
        self.tri_sign[self.tm, self.vm] = -1.0

    # ---------------------------------------------------------------- vias
    def _cells_at(self, x, y):
        """Triangles whose centroid lies in the grid cell holding (x, y), or
        in any cell touching it when it lies on a grid line."""
        def bounds(g, c):
            on = np.nonzero(np.abs(g - c) < 1e-6 * (g[-1] - g[0]))[0]
            if on.size:
                k = on[0]
                return g[max(k - 1, 0)], g[min(k + 1, len(g) - 1)]
            k = np.searchsorted(g, c) - 1
            return (g[k], g[k + 1]) if 0 <= k < len(g) - 1 else (c, c)

        (xa, xb), (ya, yb) = bounds(self.xg, x), bounds(self.yg, y)
        cx, cy = self.centroid[:, 0], self.centroid[:, 1]
        return np.nonzero((cx > xa) & (cx < xb) & (cy > ya) & (cy < yb))[0]

    def _via_ends(self, via):
        """{level: triangles the via's current enters or leaves by}: those of
        the level whose centroid lies within the drill, else those of the
        grid cell under the via's centre."""
        x, y = via.xy
        r2 = (self.centroid[:, 0] - x) ** 2 + (self.centroid[:, 1] - y) ** 2
        ends = {}
        for lv, name in enumerate(self.layer_names):
            on = self.tri_layer == lv
            t = np.nonzero(on & (r2 < (via.drill / 2) ** 2))[0]
            if t.size == 0:
                t = self._cells_at(x, y)
                t = t[on[t]]
            if t.size:
                ends[name] = t
        bare = [n for n in via.pad_layers() if n in self.layer_names and n not in ends]
        if bare:
            raise ValueError(f"via at ({x * 1e3:.4g}, {y * 1e3:.4g}) mm ends on level {bare[0]} "
                             "where no copper is meshed")
        return ends

    def assign_levels(self, order):
        """Cut every via into vertical segments at each level it passes that
        has copper under it, from its upper to its lower end (order: the
        levels from bottom to top). Unknown n_basis + k is the downward
        current of segment k."""
        height = {name: i for i, name in enumerate(order)}
        height["gnd"] = -1
        self.via_segments = []
        for k, (via, ends) in enumerate(zip(self.vias, self.via_attach)):
            for name in (via.top, via.bottom):
                if name not in height:
                    raise ValueError(f"via ends on {name!r}, which is not one of the levels {order}")
            upper, lower = max(height[via.top], height[via.bottom]), min(height[via.top], height[via.bottom])
            stops = [n for n in sorted(order, key=lambda n: -height[n]) if lower < height[n] < upper and n in ends]
            chain = [order[upper], *stops, order[lower] if lower >= 0 else "gnd"]
            for top, bottom in zip(chain[:-1], chain[1:]):
                self.via_segments.append(dict(via=k, top=top, bottom=bottom, top_tris=ends.get(top),
                                              bottom_tris=ends.get(bottom)))
        self.level_order = list(order)
        self.n_vias = len(self.via_segments)
        self.n_frills = 0
        self.n_ap = 0
        self.via_tris = [seg["top_tris"] for seg in self.via_segments]
        self.n_unknowns = self.n_basis + self.n_vias

    # --------------------------------------------------------------- ports
    def flow_direction(self):
        """Unit vector from each basis' + triangle centroid to its - one."""
        d = self.centroid[self.tm] - self.centroid[self.tp]
        length = np.linalg.norm(d, axis=1)
        return d / np.where(length > 0, length, 1.0)[:, None]

    def cut_positions(self, port):
        """The feed positions s in [0, length] that are grid lines, sorted."""
        grid = self.xg if port.axis == 0 else self.yg
        s = port.sgn * (grid - port.ref[port.axis])
        return np.sort(s[(s > -1e-12) & (s <= port.length + 1e-12)])

    def _feed_edges(self, port):
        """The feed's candidate cut edges (on its level, mid-point within its
        width), the s of both their ends, and the sign that makes a positive
        coefficient a current toward the circuit. Cached per port object."""
        cache = self.__dict__.setdefault("_feed_cache", {})
        hit = cache.get(id(port))
        if hit is None or hit[0] is not port:
            s_ends, _ = port.local(self.nodes[self.edge_nodes])
            _, t_mid = port.local(self.edge_mid)
            idx = np.nonzero((np.abs(t_mid) < port.width / 2)
                             & (self.edge_layer == self.layer_names.index(port.layer)))[0]
            toward = -port.sgn * np.sign(self.flow_direction()[idx, port.axis])
            hit = cache[id(port)] = (port, idx, s_ends[idx], toward)
        return hit[1:]

    def cut_edges(self, port, s):
        """RWG edges lying on the transverse cut at s of a feed, and their
        signs: sum(sign * edge_len * x) over them is the current toward the
        circuit."""
        idx, s_ends, toward = self._feed_edges(port)
        on = np.all(np.abs(s_ends - s) < 1e-6 * port.width, axis=1)
        return idx[on], toward[on]

    def internal_port_vectors(self):
        """(N, n_internal): the delta-gap vector of each internal port of the
        layout, in order: a gap port's column of lumped_vectors (current a ->
        b), a via port's unit vector on the via's segment that ends on the
        ground plane (current flowing down into the plane)."""
        ports = list(getattr(self.layout, "internal_ports", []))
        names = [q.name for q in getattr(self.layout, "lumped", [])]
        Lm = self.lumped_vectors() if names else None
        out = np.zeros((self.n_unknowns, len(ports)))
        for k, ip in enumerate(ports):
            if ip["kind"] == "gap":
                out[:, k] = Lm[:, names.index(ip["name"])]
                continue
            seg = [i for i, g in enumerate(self.via_segments) if g["via"] == ip["via"] and g["bottom"] == "gnd"]
            if len(seg) != 1:
                raise ValueError(f"via port {ip['name']}: its via has no segment ending on the ground plane")
            out[self.n_basis + seg[0], k] = 1.0
        return out

    def lumped_vectors(self):
        """(N, n_lumped): column k holds the signed edge lengths of gap k's
        cut, oriented a -> b; it is the gap's delta-gap excitation, and its
        dot product with the currents the current from a to b."""
        gaps = list(getattr(self.layout, "lumped", []))
        out = np.zeros((self.n_unknowns, len(gaps)))
        for k, gap in enumerate(gaps):
            idx, sign = self.cut_edges(gap, gap.s_gap)
            if idx.size == 0:
                raise ValueError(f"lumped {gap.name}: no mesh edge lies on its gap")
            out[idx, k] = -sign * self.edge_len[idx]
        return out
