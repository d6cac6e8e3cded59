"""Compressed MoM operator (H-matrix) and its iterative solve on the GPU.

mom25d's `method="hmatrix"` (Engine/mom25d/hmatrix.py:145-606): Z is never
formed. The RWG unknowns are grouped in a cluster tree (bisection of their
edge midpoints along the largest extent, at most `leaf` per leaf); pairs of
clusters that are well separated (max diameter <= eta x box distance, and the
distance >= 5 triangle sizes) are far blocks held as low-rank products U V^T
built by adaptive cross approximation (ACA, partial pivoting) from entries of
the 3-point rule on both sides (the centroid rule once the clusters are 10
triangle sizes apart), each unordered pair once; the remaining leaf pairs
are near blocks with the exact entries of the dense fill; the via unknowns
stay dense. The system is solved by GMRES with a preconditioner.

Here (the host part; the device part is csrc/hmatrix.cu):
- the tree and the partition follow hmatrix.py:40-97 (`_tree`, `_partition`:
  the same split axis, halving, admissibility and tie-break by cluster id),
  built in the unknowns' tree order, so that every cluster is one range of
  positions and every block a contiguous row range x column range;
- the near blocks are the dense fill's own values (the same triangle-pair
  classes and integration as `Solver.impedance`), computed by the fill kernel
  for the listed (test block, source triangle) pairs only;
- far blocks: ACA on the device, one CTA per block, with mom25d's stopping
  rule (hmatrix.py:100-136); blocks with a side <= 64 and blocks that are not
  low rank within min(m, n) / 3 terms (or `kcap` terms, the storage bound)
  are stored as they are. The ACA factors are not recompressed (QR + SVD,
  hmatrix.py:137-142): that would lower their rank, not their error;
- preconditioner: restricted additive Schwarz in place of mom25d's sparse
  LU of the nearest entries (hmatrix.py:523-560): the largest clusters of
  at most `prec_block` unknowns, each extended by the leaves its own leaves
  are near-coupled to (the most coupled first) and by the vias whose pads
  those hold, up to `prec_max` unknowns; each block of the compressed operator is scaled to a unit
  diagonal and inverted in complex64, so that applying the preconditioner
  is one batched matrix-vector product, and each block writes only its own
  unknowns (overlap=False: block Jacobi); GMRES (restart 200, at most 3 restarts,
  relative residual 1e-6) is flexible: it keeps M^-1 v_j for every basis
  vector, so the preconditioner's precision does not enter the solution.
"""

import ctypes as C
import warnings

import numpy as np

from . import engine as E

ADM_SIZES = 5.0  # far blocks are also this many triangle sizes apart (hmatrix.py:60)
SMALL = 64       # far blocks with a side <= SMALL are stored dense (hmatrix.py:148)
CEN = 10.0       # centroid rule for far blocks this many triangle sizes apart (hmatrix.py:149)
ACCEPT = 1.0     # a stalled GMRES solve is accepted at residual <= ACCEPT * tol (hmatrix.py:150)

# (barycentric coordinates, weights) of the 3-point rule (Engine/mom25d/integrals.py:16-17)
TRI3_BARY = np.array([[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3]])
TRI3_W = np.full(3, 1 / 3)


class Cluster:
    """A node of the cluster tree: positions [lo, hi) of the tree order."""

    __slots__ = ("id", "lo", "hi", "bmin", "bmax", "lo3", "hi3", "smax", "children", "diam")

    @property
    def size(self):
        return self.hi - self.lo


def cluster_tree(pos, size, leaf):
    """(perm, nodes): the unknowns in tree order (perm[k] = unknown at
    position k) and the clusters in preorder (ids as mom25d numbers them).
    A cluster with more than `leaf` unknowns is split at the middle of its
    unknowns sorted (stably) along the longest side of their bounding box
    (hmatrix.py:52-62)."""
    n = len(pos)
    perm = np.empty(n, np.int64)
    nodes = []
    # explicit stack in the recursion's order: (unknowns in the caller's order, first position, parent slot)
    root = None
    stack = [(np.arange(n), 0, None, 0)]
    while stack:
        idx, lo, parent, slot = stack.pop()
        c = Cluster()
        c.id = len(nodes)
        nodes.append(c)
        c.lo, c.hi = lo, lo + idx.size
        p = pos[idx]
        c.bmin, c.bmax = p.min(0), p.max(0)
        c.lo3, c.hi3 = tuple(float(v) for v in c.bmin), tuple(float(v) for v in c.bmax)
        c.diam = float(np.linalg.norm(c.bmax - c.bmin))  # as mom25d's _Cluster.diam, once
        c.smax = float(size[idx].max())
        c.children = []
        if parent is None:
            root = c
        else:
            parent.children[slot] = c
        if idx.size > leaf:
            ax = int(np.argmax(c.bmax - c.bmin))
            order = idx[np.argsort(pos[idx, ax], kind="stable")]
            h = order.size // 2
            c.children = [None, None]
            # the second child is pushed first: the first child (and its subtree) gets the lower ids
            stack.append((order[h:], lo + h, c, 1))
            stack.append((order[:h], lo, c, 0))
        else:
            perm[lo:lo + idx.size] = idx
    return perm, nodes, root


def _dist(a, b):
    """Distance of the bounding boxes (hmatrix.py:65-67): the gap per axis
    (exact in floats), its norm by numpy as mom25d takes it; overlapping
    boxes at once."""
    gap = [max(0.0, max(x0 - y1, y0 - x1)) for x0, x1, y0, y1 in zip(a.lo3, a.hi3, b.lo3, b.hi3)]
    if gap[0] == 0.0 and gap[1] == 0.0 and gap[2] == 0.0:
        return 0.0
    return float(np.linalg.norm(np.array(gap)))


def partition(root, eta):
    """(far, near): admissible cluster pairs and leaf pairs, in the order of
    mom25d's recursion (hmatrix.py:65-97), which is symmetric: (a, b) and
    (b, a) give mirrored blocks."""
    far, near = [], []
    stack = [(root, root)]
    while stack:
        a, b = stack.pop()
        d = _dist(a, b)
        if max(a.diam, b.diam) <= eta * d and d >= ADM_SIZES * max(a.smax, b.smax):
            far.append((a, b))
        elif not a.children and not b.children:
            near.append((a, b))
        elif a.children and (not b.children or (a.diam, a.id) > (b.diam, b.id)):
            stack.extend((c, b) for c in reversed(a.children))
        else:
            stack.extend((a, c) for c in reversed(b.children))
    return far, near


def unique_far(far):
    """Each unordered far pair once, in the orientation met first (hmatrix.py:200-205)."""
    seen, out = set(), []
    for a, b in far:
        key = (min(a.id, b.id), max(a.id, b.id))
        if key not in seen:
            seen.add(key)
            out.append((a, b))
    return out


def basis_rules(mesh):
    """Per RWG basis, the far-field entry data of both halves (hmatrix.py:168-187):
    3-point rule points P (nb,6,2), w_k cA (r_k - a) (nb,6,2), w_k cV (nb,6); centroids
    (nb,2,2), A cA (c - a) (nb,2,2), A cV (nb,2); and the largest triangle size of each basis."""
    m = mesh
    V, A = m.verts, m.area
    b = m.tri_basis
    lab = np.where(b >= 0, m.edge_len[np.maximum(b, 0)], 0.0)
    cAt = m.tri_sign * lab / (2 * A[:, None])
    cVt = m.tri_sign * lab / A[:, None]
    nb = m.n_basis
    tri = np.stack([m.tp, m.tm], 1)
    loc = np.stack([m.vp, m.vm], 1)
    cA, cV = cAt[tri, loc], cVt[tri, loc]
    P3 = np.einsum("kv,nvd->nkd", TRI3_BARY, V)
    w3 = TRI3_W[None, :] * A[:, None]
    pts = P3[tri].reshape(nb, 6, 2)
    rho = P3[tri] - V[tri, loc][:, :, None, :]
    u6 = (w3[tri][..., None] * cA[:, :, None, None] * rho).reshape(nb, 6, 2)
    q6 = (w3[tri] * cV[:, :, None]).reshape(nb, 6)
    cen = m.centroid[tri]
    u1 = A[tri][..., None] * cA[..., None] * (cen - V[tri, loc])
    q1 = A[tri] * cV
    size = np.max(np.linalg.norm(V - np.roll(V, 1, axis=1), axis=-1), axis=1)
    return pts, u6, q6, cen, u1, q1, size[tri].max(1)


class Plan:
    """The host side of the compressed operator (no device work): the tree,
    the partition and the index lists the device kernels follow."""

    def __init__(self, mesh, zl, blocks, leaf=48, eta=1.0, prec_block=256, overlap=True, prec_max=640):
        m = mesh
        self.nb, self.nv = nb, nv = m.n_basis, len(m.via_segments)
        self.n = nb + nv
        if nb < 2:
            raise ValueError("the compressed operator needs at least two RWG unknowns")
        if nv > 1024:
            raise ValueError("the compressed operator keeps at most 1024 via unknowns in one dense block")
        pts, u6, q6, cen, u1, q1, bsize = basis_rules(m)
        pos = np.c_[m.edge_mid, np.asarray(zl)[m.edge_layer]]
        self.perm, self.nodes, root = cluster_tree(pos, bsize, leaf)
        far, near = partition(root, eta)
        self.far = unique_far(far)
        self.near = near
        perm = self.perm
        # far-field rule data of each basis in tree order (40 values per basis)
        self.rules = np.concatenate([pts.reshape(nb, 12), u6.reshape(nb, 12), q6, cen.reshape(nb, 4),
                                     u1.reshape(nb, 4), q1], 1)[perm]
        self.lev = np.asarray(m.edge_layer)[perm]
        leaves = [c for c in self.nodes if not c.children]
        leaves.sort(key=lambda c: c.lo)
        self.leaves = leaves
        self.leaf_lo = np.array([c.lo for c in leaves] + [nb], np.int32)
        leaf_index = {c.id: k for k, c in enumerate(leaves)}
        self.near_arr = np.array([(a.lo, a.size, b.lo, b.size) for a, b in near], np.int32).reshape(-1, 4)
        self.far_arr = np.array([(a.lo, a.size, b.lo, b.size) for a, b in self.far], np.int32).reshape(-1, 4)
        self.far_cen = np.array([int(_dist(a, b) >= CEN * max(a.smax, b.smax)) for a, b in self.far], np.int32)
        # per leaf: its near pairs (rows), and the far blocks whose rows or columns hold it
        ent = [[] for _ in leaves]
        for p, (a, b) in enumerate(near):
            ent[leaf_index[a.id]].append((0, p, 0, 0))
        lo_sorted = self.leaf_lo[:-1]
        for f, (a, b) in enumerate(self.far):
            for side, c in ((1, a), (2, b)):
                k0 = int(np.searchsorted(lo_sorted, c.lo))
                k1 = int(np.searchsorted(lo_sorted, c.hi))
                for k in range(k0, k1):
                    ent[k].append((side, f, int(self.leaf_lo[k]) - c.lo, 0))
        self.ent_off = np.zeros(len(leaves) + 1, np.int64)
        self.ent_off[1:] = np.cumsum([len(e) for e in ent])
        self.ent = np.array([x for e in ent for x in e], np.int32).reshape(-1, 4)
        # the near field's (test block, source triangle) pairs: the test
        # blocks of a's triangles x the triangles of b, per near pair (a, b)
        nt = len(m.tris)
        self.nt = nt
        self.blk_of = blk_of = np.full(nt, -1, np.int64)
        rows, cols = np.nonzero(blocks >= 0)
        blk_of[blocks[rows, cols]] = rows
        ltri = [np.unique(np.r_[m.tp[perm[c.lo:c.hi]], m.tm[perm[c.lo:c.hi]]]) for c in leaves]
        lblk = [np.unique(blk_of[t]) for t in ltri]
        keys = [np.add.outer(lblk[leaf_index[a.id]] * nt, ltri[leaf_index[b.id]]).ravel() for a, b in near]
        self.keys = np.unique(np.concatenate(keys)) if keys else np.zeros(0, np.int64)
        if self.keys.size >= 2**31 - 1:
            raise MemoryError("too many near-field triangle pairs for the compressed operator")
        self.pblk = np.zeros(0, np.int32)
        if nv:
            segs = m.via_segments
            tris = np.unique(np.concatenate([g[e] for g in segs for e in ("top_tris", "bottom_tris")
                                             if g[e] is not None]))
            self.pblk = np.unique(blk_of[tris]).astype(np.int32)
        # preconditioner: the largest clusters of at most prec_block unknowns,
        # each extended by the leaves its own leaves are near-coupled to
        # (overlap; restricted additive Schwarz: a block writes its own unknowns)
        pcs = []
        stack = [root]
        while stack:
            c = stack.pop()
            if c.size <= prec_block or not c.children:
                pcs.append(c)
            else:
                stack.extend(reversed(c.children))
        pcs.sort(key=lambda c: c.lo)
        nleaf = len(leaves)
        # the source of every (row leaf, column leaf) block: near pair p, or far
        # block f as rows (nnear + 2 f) or as its transpose (nnear + 2 f + 1)
        srcmap = np.full((nleaf, nleaf), -1, np.int64)
        for p, (a, b) in enumerate(near):
            srcmap[leaf_index[a.id], leaf_index[b.id]] = p
        for f, (a, b) in enumerate(self.far):
            r0, r1 = np.searchsorted(lo_sorted, [a.lo, a.hi])
            c0, c1 = np.searchsorted(lo_sorted, [b.lo, b.hi])
            srcmap[r0:r1, c0:c1] = len(near) + 2 * f
            srcmap[c0:c1, r0:r1] = len(near) + 2 * f + 1
        if (srcmap < 0).any():
            raise RuntimeError("the block partition does not cover every leaf pair")
        nbr = [[] for _ in range(nleaf)]
        for a, b in near:
            nbr[leaf_index[a.id]].append(leaf_index[b.id])
        # each via belongs with the RWG unknown of its first pad triangle
        via_pos = np.full(nv, nb - 1, np.int64)
        if nv:
            ipos = np.empty(nb, np.int64)
            ipos[perm] = np.arange(nb)
            for v, g in enumerate(m.via_segments):
                for t in (t for e in ("top_tris", "bottom_tris") if g[e] is not None for t in np.atleast_1d(g[e])):
                    bs = m.tri_basis[t][m.tri_basis[t] >= 0]
                    if bs.size:
                        via_pos[v] = ipos[bs[0]]
                        break
        via_leaf = np.searchsorted(lo_sorted, via_pos, side="right") - 1
        leaf_size = np.diff(self.leaf_lo).astype(np.int64)
        gidx, own, items, offs, ioffs, sizes, overl = [], [], [], [0], [0], [], []
        nvia_leaf = np.bincount(via_leaf, minlength=nleaf) if nv else np.zeros(nleaf, np.int64)
        for c in pcs:
            k0, k1 = np.searchsorted(lo_sorted, [c.lo, c.hi])
            mine = list(range(k0, k1))
            size = int(leaf_size[mine].sum() + nvia_leaf[mine].sum())
            if size > 1024:
                raise ValueError("a preconditioner block with its vias exceeds 1024 unknowns (lower prec_block)")
            ext = set(mine)
            if overlap:  # the halo: near-coupled leaves, the most coupled first, up to prec_max unknowns
                cnt = {}
                for k in mine:
                    for b in nbr[k]:
                        if b not in ext:
                            cnt[b] = cnt.get(b, 0) + 1
                for b in sorted(cnt, key=lambda b: (-cnt[b], b)):
                    add = int(leaf_size[b] + nvia_leaf[b])
                    if size + add <= prec_max:
                        ext.add(b)
                        size += add
            ext = sorted(ext)
            vias = np.nonzero(np.isin(via_leaf, ext))[0] if nv else np.zeros(0, np.int64)
            ext = np.array(ext, np.int64)
            lstart = np.concatenate([[0], np.cumsum(leaf_size[ext])])[:-1]
            g = np.concatenate([np.arange(self.leaf_lo[k], self.leaf_lo[k + 1]) for k in ext] + [nb + vias])
            o = np.concatenate([np.full(leaf_size[k], k0 <= k < k1) for k in ext] +
                               [(via_leaf[vias] >= k0) & (via_leaf[vias] < k1)])
            I, J = np.meshgrid(np.arange(ext.size), np.arange(ext.size), indexing="ij")
            it = np.stack([srcmap[ext[I], ext[J]].ravel(), ext[I].ravel(), ext[J].ravel(),
                           lstart[I].ravel(), lstart[J].ravel()], 1)
            gidx.append(g)
            own.append(o)
            items.append(it)
            offs.append(offs[-1] + g.size)
            ioffs.append(ioffs[-1] + it.shape[0])
            sizes.append(size)
            overl.append(size - int(o.sum()))
        self.pc_off = np.array(offs, np.int64)
        self.pc_gidx = np.concatenate(gidx).astype(np.int32)
        self.pc_own = np.concatenate(own).astype(np.int8)
        self.pc_item_off = np.array(ioffs, np.int64)
        self.pc_items = np.concatenate(items).astype(np.int32)
        self.prec_sizes = np.array(sizes)
        self.prec_overlap = np.array(overl)
        self.npc = len(pcs)
        self.stats = dict(clusters=len(self.nodes), leaves=len(leaves), near_pairs=len(near),
                          far_blocks=len(self.far), near_field_pairs=int(self.keys.size), prec_blocks=len(pcs),
                          prec_size_max=int(self.prec_sizes.max()), prec_overlap_mean=float(self.prec_overlap.mean()))


class HMatrix:
    """The compressed operator of a Solver's mesh on the solver's engine
    context. assemble(greens, zs) at a frequency, then matvec / solve."""

    def __init__(self, solver, leaf=48, eta=1.0, tol=1e-4, kcap=96, prec_block=256, overlap=True, prec_max=640):
        if solver._blocks_host is None:
            solver.geometry()
        P = self.plan = Plan(solver.mesh, solver.zl, solver._blocks_host, leaf, eta, prec_block, overlap, prec_max)
        self.solver, self.tol = solver, tol
        self.nb, self.nv, self.n = P.nb, P.nv, P.n
        self._arrs = arrs = dict(
            perm=E.i32(P.perm), rules=E.f64(P.rules), lev=E.i32(P.lev), leaf_lo=E.i32(P.leaf_lo),
            near=E.i32(P.near_arr), far=E.i32(P.far_arr), far_cen=E.i32(P.far_cen),
            ent_off=np.ascontiguousarray(P.ent_off, np.int64), ent=E.i32(P.ent),
            keys=np.ascontiguousarray(P.keys, np.int64), pblk=E.i32(P.pblk),
            pc_off=np.ascontiguousarray(P.pc_off, np.int64), pc_gidx=E.i32(P.pc_gidx),
            pc_own=np.ascontiguousarray(P.pc_own, np.int8), pc_item_off=np.ascontiguousarray(P.pc_item_off, np.int64),
            pc_items=E.i32(P.pc_items))
        i32, i64, i8 = C.c_int32, C.c_int64, C.c_int8
        d = E.HmatDesc(P.nb, P.nv, E.ptr(arrs["perm"], i32), E.ptr(arrs["rules"]), E.ptr(arrs["lev"], i32),
                       len(P.leaves), E.ptr(arrs["leaf_lo"], i32), len(P.near), E.ptr(arrs["near"], i32),
                       len(P.far), E.ptr(arrs["far"], i32), E.ptr(arrs["far_cen"], i32),
                       E.ptr(arrs["ent_off"], i64), E.ptr(arrs["ent"], i32), int(P.keys.size),
                       E.ptr(arrs["keys"], i64), int(P.pblk.size), E.ptr(arrs["pblk"], i32), P.npc,
                       E.ptr(arrs["pc_off"], i64), E.ptr(arrs["pc_gidx"], i32), E.ptr(arrs["pc_own"], i8),
                       E.ptr(arrs["pc_item_off"], i64), E.ptr(arrs["pc_items"], i32), float(tol), int(kcap))
        self.ctx = solver.ctx
        h = C.c_void_p()
        E.check(self.ctx.lib.m25_hmat_create(self.ctx.h, solver.geometry().h, C.byref(d), C.byref(h)))
        self._h = E.Handle(self.ctx, h, self.ctx.lib.m25_hmat_destroy)
        self.stats = dict(P.stats)

    STAT_KEYS = ("near_entries", "lowrank_blocks", "dense_far_blocks", "far_entries", "max_rank", "rank_sum",
                 "not_low_rank")

    def assemble(self, greens, zs=0.0, zsv=None):
        """Near blocks, far blocks (ACA) and via blocks at greens' frequency;
        zs: the conductors' surface impedance (zsv: the via walls', default zs)."""
        zs = complex(zs)
        zsv = zs if zsv is None else complex(zsv)
        st = np.zeros(8, np.int64)
        E.check(self.ctx.lib.m25_hmat_assemble(self._h.h, greens.h, zs.real, zs.imag, zsv.real, zsv.imag,
                                               E.ptr(st, C.c_int64)))
        self.stats.update({k: int(v) for k, v in zip(self.STAT_KEYS, st)})
        return self

    def matvec(self, x):
        """Z x with the compressed operator (x: (n,) or (n, k) complex)."""
        x = np.asarray(x, np.complex128)
        X = np.ascontiguousarray(x.reshape(self.n, -1).T)
        Y = np.zeros_like(X)
        for k in range(X.shape[0]):
            E.check(self.ctx.lib.m25_hmat_matvec(self._h.h, E.ptr(X[k].view(np.float64)),
                                                 E.ptr(Y[k].view(np.float64))))
        return Y.T.reshape(x.shape)

    def solve(self, B, rtol=1e-6, restart=200, maxiter=3):
        """Z^-1 B by preconditioned GMRES, one column at a time, on the
        symmetrically scaled system W Z W (W = |Z_ii|^-1/2: the via unknowns'
        diagonal entries are ~1e10 times the RWG unknowns'), whose relative
        residual is the stopping test. A column that stops above rtol is
        accepted when its residual is within the compression's accuracy
        (ACCEPT x tol, with a warning), else RuntimeError (hmatrix.py:563-597)."""
        B = np.asarray(B, np.complex128)
        Bm = np.ascontiguousarray(B.reshape(self.n, -1))
        X = np.zeros_like(Bm)
        k = Bm.shape[1]
        its = np.zeros(k, np.int32)
        res = np.zeros(k)
        E.check(self.ctx.lib.m25_hmat_solve(self._h.h, k, E.ptr(Bm.view(np.float64)), E.ptr(X.view(np.float64)),
                                            rtol, restart, maxiter, E.ptr(its, C.c_int32), E.ptr(res)))
        self.stats["gmres_iterations"] = its.tolist()
        self.stats["gmres_residuals"] = res.tolist()
        for c in range(k):
            if res[c] > rtol:
                if res[c] > ACCEPT * self.tol:
                    raise RuntimeError(f"GMRES did not converge ({its[c]} iterations, rhs {c}, "
                                       f"residual {res[c]:.1e})")
                warnings.warn(f"GMRES stopped at residual {res[c]:.1e} (target {rtol:g}) after {its[c]} "
                              f"iterations, rhs {c}: accepted (H-matrix tolerance {self.tol:g})",
                              RuntimeWarning, stacklevel=2)
        return X.reshape(B.shape)

    def summary(self):
        s = self.stats
        dense = self.n ** 2
        return (f"H-matrix: {s['leaves']} leaves, {s['near_pairs']} near pairs, {s['far_blocks']} far blocks "
                f"({s.get('lowrank_blocks', 0)} low rank, max rank {s.get('max_rank', 0)}); "
                f"{100 * (s.get('near_entries', 0) + s.get('far_entries', 0)) / dense:.1f} % of dense entries; "
                f"GMRES its {s.get('gmres_iterations', '')}")

    def close(self):
        self._h.close()
