"""Host side of the compressed operator (mom25d_gb300/hmatrix.py): the
cluster tree and block partition against mom25d's own (tests/golden/
hmatrix.npz, made by make_hmatrix_golden.py), and the index lists that the
device kernels follow (near-field pairs, per-leaf row items, preconditioner
blocks), checked entry by entry on small meshes."""

import os

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import hmatrix as H
from mom25d_gb300 import workloads
from mom25d_gb300.solver import test_blocks as morton_blocks

from conftest import GOLDEN


def _cover(nodes_far_near, n):
    far, near = nodes_far_near
    cover = np.zeros((n, n), int)
    for a, b in near:
        cover[a.lo:a.hi, b.lo:b.hi] += 1
    for a, b in H.unique_far(far):
        cover[a.lo:a.hi, b.lo:b.hi] += 1
        cover[b.lo:b.hi, a.lo:a.hi] += 1
    return cover


def test_partition_covers_every_entry_once():
    """Near leaf pairs plus far blocks (each unordered pair once, applied with
    its transpose) tile the matrix exactly: random points and a regular grid
    (equal cluster diameters, where the tie-break by id keeps the partition
    symmetric)."""
    for pos in (np.random.default_rng(3).random((400, 3)),
                np.c_[np.mgrid[0:20, 0:20].reshape(2, -1).T * 1.0, np.zeros(400)]):
        perm, nodes, root = H.cluster_tree(pos, np.full(len(pos), 0.01), 16)
        assert np.array_equal(np.sort(perm), np.arange(len(pos)))
        far, near = H.partition(root, 1.0)
        assert far and np.all(_cover((far, near), len(pos)) == 1)


def _golden():
    path = os.path.join(GOLDEN, "hmatrix.npz")
    if not os.path.exists(path):
        pytest.skip("no hmatrix.npz fixture")
    return np.load(path)


@pytest.mark.parametrize("prefix", ["rand_", "grid_", "via_"])
def test_tree_and_partition_equal_mom25d(prefix):
    """The clusters (as sets of unknowns, in mom25d's preorder numbering) and
    the near / far cluster pairs, in mom25d's order, equal those of mom25d's
    _tree / _partition on the same points."""
    g = _golden()
    pos, size, leaf = g[prefix + "pos"], g[prefix + "size"], int(g[prefix + "leaf"])
    perm, nodes, root = H.cluster_tree(pos, size, leaf)
    idx = [perm[c.lo:c.hi].astype(np.int64) for c in nodes]
    assert len(nodes) == len(g[prefix + "cl_n"])
    assert np.array_equal([i.size for i in idx], g[prefix + "cl_n"])
    assert np.array_equal([i.sum() for i in idx], g[prefix + "cl_s1"])
    assert np.array_equal([(i * i).sum() for i in idx], g[prefix + "cl_s2"])
    far, near = H.partition(root, 1.0)
    assert np.array_equal(np.array([(a.id, b.id) for a, b in near]), g[prefix + "near"])
    assert np.array_equal(np.array([(a.id, b.id) for a, b in far]), g[prefix + "far"])


def _plan(name, **kw):
    lay, st, m, _ = workloads.build(G, name)
    st = st if hasattr(st, "layers") else st.to_stackup()
    zl = np.array([st.level_z(n) for n in m.layer_names])
    return m, H.Plan(m, zl, morton_blocks(m), **kw)


@pytest.mark.parametrize("name", ["tee", "via"])
def test_plan_index_lists(name):
    """What the kernels read is complete and consistent:
    - every triangle pair a near entry sums (test block of t_m, source t_n)
      is among the listed near-field pairs;
    - every row's items (near pairs, far blocks as rows, far blocks as
      columns) cover each column exactly once;
    - every unknown is written by one preconditioner block, and each block's
      items tile its RWG part exactly once from blocks that hold them;
    - the pad blocks hold every via pad triangle."""
    m, P = _plan(name)
    nb, nt = P.nb, P.nt
    keys = set(P.keys.tolist())
    perm = P.perm
    for a0, am, b0, bn in P.near_arr:
        rows, cols = perm[a0:a0 + am], perm[b0:b0 + bn]
        tm = np.r_[m.tp[rows], m.tm[rows]]
        tn = np.unique(np.r_[m.tp[cols], m.tm[cols]])
        need = np.add.outer(np.unique(P.blk_of[tm]) * nt, tn).ravel()
        assert all(int(k) in keys for k in need)
    for k in range(len(P.leaves)):
        lo, hi = P.leaf_lo[k], P.leaf_lo[k + 1]
        cnt = np.zeros(nb, int)
        for t, i, off, _ in P.ent[P.ent_off[k]:P.ent_off[k + 1]]:
            if t == 0:
                a0, am, b0, bn = P.near_arr[i]
                assert a0 == lo and am == hi - lo
                cnt[b0:b0 + bn] += 1
            else:
                r0, mm, c0, nn = P.far_arr[i]
                if t == 1:
                    assert r0 + off == lo and off + (hi - lo) <= mm
                    cnt[c0:c0 + nn] += 1
                else:
                    assert c0 + off == lo and off + (hi - lo) <= nn
                    cnt[r0:r0 + mm] += 1
        assert np.all(cnt == 1), (k, np.unique(cnt))
    # preconditioner blocks: every unknown written by exactly one block; a
    # block's (row leaf, column leaf) items tile its RWG part exactly once,
    # each from a source block that holds it; its vias follow its RWG unknowns
    owned = np.zeros(P.n, int)
    np.add.at(owned, P.pc_gidx[P.pc_own == 1], 1)
    assert np.all(owned == 1)
    lsz = np.diff(P.leaf_lo)
    nnear = len(P.near_arr)
    for k in range(P.npc):
        g = P.pc_gidx[P.pc_off[k]:P.pc_off[k + 1]]
        R = int((g < nb).sum())
        assert np.all(g[:R] < nb) and np.all(g[R:] >= nb) and g.size <= 1024
        cnt = np.zeros((R, R), int)
        for src, li, lj, lr0, lc0 in P.pc_items[P.pc_item_off[k]:P.pc_item_off[k + 1]]:
            assert np.array_equal(g[lr0:lr0 + lsz[li]], np.arange(P.leaf_lo[li], P.leaf_lo[li + 1]))
            assert np.array_equal(g[lc0:lc0 + lsz[lj]], np.arange(P.leaf_lo[lj], P.leaf_lo[lj + 1]))
            cnt[lr0:lr0 + lsz[li], lc0:lc0 + lsz[lj]] += 1
            a0, b0 = P.leaf_lo[li], P.leaf_lo[lj]
            if src < nnear:
                assert tuple(P.near_arr[src]) == (a0, lsz[li], b0, lsz[lj])
            else:
                f, o = divmod(src - nnear, 2)
                r0, mm, c0, nn = P.far_arr[f]
                if o:
                    r0, mm, c0, nn = c0, nn, r0, mm
                assert r0 <= a0 and a0 + lsz[li] <= r0 + mm and c0 <= b0 and b0 + lsz[lj] <= c0 + nn
        assert np.all(cnt == 1)
    assert P.prec_sizes.max() <= 1024
    if P.nv:
        pads = np.unique(np.concatenate([g[e] for g in m.via_segments for e in ("top_tris", "bottom_tris")
                                         if g[e] is not None]))
        assert set(P.blk_of[pads].tolist()) <= set(P.pblk.tolist())


def test_plan_rules_match_mesh():
    """The far-field rule data: the 3-point points of both halves average to
    the triangle centroids, and the weights w cV of a basis' two halves sum
    to zero (the divergence integrates to zero over the basis)."""
    m, P = _plan("tee")
    r = P.rules
    perm = P.perm
    pts = r[:, :12].reshape(-1, 2, 3, 2).mean(2)
    cen = np.stack([m.centroid[m.tp[perm]], m.centroid[m.tm[perm]]], 1)
    assert np.allclose(pts, cen, rtol=0, atol=1e-15)
    assert np.allclose(r[:, 24:30].sum(1), 0, atol=1e-12 * np.abs(r[:, 24:30]).max())
    assert np.allclose(r[:, 38:40].sum(1), 0, atol=1e-12 * np.abs(r[:, 38:40]).max())


def test_plan_block_jacobi_and_overlap_cap():
    """overlap=False: each preconditioner block holds exactly its own leaves
    (and vias) and writes all of them; with overlap every block stays within
    prec_max unknowns unless its own part is larger, and grows by whole
    near-coupled leaves only."""
    m, P = _plan("via", overlap=False)
    assert np.all(P.pc_own == 1)
    m, P2 = _plan("via", prec_max=400)
    own = [int(P2.pc_own[P2.pc_off[k]:P2.pc_off[k + 1]].sum()) for k in range(P2.npc)]
    for k in range(P2.npc):
        assert P2.prec_sizes[k] <= max(400, own[k])
        g = P2.pc_gidx[P2.pc_off[k]:P2.pc_off[k + 1]]
        g = g[g < P2.nb]
        starts = set(P2.leaf_lo[:-1].tolist())
        # whole leaves: every run of consecutive positions starts at a leaf start
        runs = np.r_[0, np.nonzero(np.diff(g) != 1)[0] + 1]
        assert all(int(g[r]) in starts for r in runs)
    assert P2.prec_sizes.max() <= P.prec_sizes.max() + 400


class _FakeLib:
    """Stands in for the engine's m25_hmat_solve: X = B, with the given
    iterations and residuals per column."""

    def __init__(self, resid):
        self.resid = resid

    def m25_hmat_solve(self, h, k, B, X, rtol, restart, maxiter, its, res):
        import ctypes

        n2 = 2 * k * self.n
        ctypes.memmove(X, B, 8 * n2)
        for c in range(k):
            its[c] = 600
            res[c] = self.resid[c]
        return 0


def _fake_hmatrix(resid, n=6, tol=1e-4):
    from types import SimpleNamespace

    hm = object.__new__(H.HMatrix)
    lib = _FakeLib(resid)
    lib.n = n
    hm.ctx = SimpleNamespace(lib=lib)
    hm._h = SimpleNamespace(h=None)
    hm.n, hm.tol, hm.stats = n, tol, {}
    return hm


def test_stalled_gmres_accepted_within_the_compression_tolerance():
    """mom25d's acceptance (hmatrix.py:583-591): a column that stops above
    rtol is accepted with a RuntimeWarning when its residual is within
    ACCEPT x tol, and raises RuntimeError above it."""
    B = np.arange(12.0).reshape(6, 2) + 1j
    hm = _fake_hmatrix([1e-7, 1e-7])
    X = hm.solve(B, rtol=1e-6)
    assert np.array_equal(X, B) and hm.stats["gmres_iterations"] == [600, 600]
    hm = _fake_hmatrix([5e-5, 1e-7])
    with pytest.warns(RuntimeWarning, match="accepted"):
        hm.solve(B, rtol=1e-6)
    hm = _fake_hmatrix([1e-7, 2e-4])
    with pytest.raises(RuntimeError, match="did not converge"):
        hm.solve(B, rtol=1e-6)
    assert hm.stats["gmres_residuals"] == [1e-7, 2e-4]
