"""Generate tests/golden/hmatrix.npz by running mom25d's compressed operator
(Engine/mom25d/hmatrix.py) itself.

    MOM25D_SRC=<mom25d checkout>/Engine python tests/golden/make_hmatrix_golden.py

Recorded:
- the cluster tree and block partition of mom25d's `_tree` / `_partition`
  on two point sets (seeded random points in a box, a regular grid, leaf 16)
  and on the RWG edge midpoints of the via-transition mesh (leaf 48): per
  cluster its size and the sum and sum of squares of its unknowns, and the
  near / far cluster-id pairs in the order mom25d lists them;
- S of the tee (N = 1085) at 3 and 9 GHz and of the LPF (N = 5943) at 3
  and 6 GHz from mom25d's `method="hmatrix"` sweep (ACA, sparse-LU-
  preconditioned GMRES) and from its dense sweep, with the GMRES iteration
  counts.
"""

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "..", ".."))

import make_golden  # noqa: E402
from mom25d_gb300 import workloads  # noqa: E402


def tree_record(prefix, pos, size, leaf, hm):
    nodes = []
    root = hm._tree(np.arange(len(pos)), pos, size, leaf, nodes)
    far, near = [], []
    hm._partition(root, root, 1.0, far, near)
    idx = [np.asarray(c.idx, np.int64) for c in nodes]
    return {prefix + "pos": pos, prefix + "size": size, prefix + "leaf": leaf,
            prefix + "cl_n": np.array([i.size for i in idx]), prefix + "cl_s1": np.array([i.sum() for i in idx]),
            prefix + "cl_s2": np.array([(i * i).sum() for i in idx]),
            prefix + "near": np.array([(a.id, b.id) for a, b in near]),
            prefix + "far": np.array([(a.id, b.id) for a, b in far])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MOM25D_SRC"))
    args = ap.parse_args()
    make_golden.import_reference(args.ref)
    ref = make_golden.ref
    from mom25d import hmatrix as hm

    out = {}
    rng = np.random.default_rng(7)
    out.update(tree_record("rand_", rng.random((500, 3)), np.full(500, 0.01), 16, hm))
    grid = np.c_[np.mgrid[0:24, 0:24].reshape(2, -1).T * 1.0, np.zeros(576)]
    out.update(tree_record("grid_", grid, np.full(576, 0.01), 16, hm))
    lay, stack, mkw, _ = workloads.BUILDERS["via"](ref)
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="hmatrix")
    # the basis sizes of hmatrix.py:186: the larger triangle's longest edge
    V = m.verts
    size = np.max(np.linalg.norm(V - np.roll(V, 1, axis=1), axis=-1), axis=1)
    bsize = size[np.stack([m.tp, m.tm], 1)].max(1)
    pos = np.c_[m.edge_mid, sol.zl[m.edge_layer]]
    out.update(tree_record("via_", pos, bsize, 48, hm))
    # S by the compressed operator and by the dense solve (mom25d's GMRES stalls
    # at 2e-3 on the via-transition mesh: its sparse-LU preconditioner is not
    # enough there, so these cases have no via)
    for name, freqs in (("tee", np.array([3e9, 9e9])), ("lpf", np.array([3e9, 6e9]))):
        lay, stack, mkw, _ = workloads.BUILDERS[name](ref)
        m = lay.mesh(**mkw)
        sol = ref.Solver(m, stack, verbose=False, method="hmatrix")
        t = time.time()
        rh = sol.sweep(freqs)
        th = time.time() - t
        its = sol._hop.stats.get("gmres_iterations", [])
        t = time.time()
        rd = ref.Solver(m, stack, verbose=False, method="dense").sweep(freqs, interp=None)
        td = time.time() - t
        out.update({f"{name}_freqs": freqs, f"{name}_S_hmatrix": rh.S, f"{name}_S_dense": rd.S,
                    f"{name}_N": m.n_unknowns, f"{name}_mesh_sha": make_golden.mesh_digest(m),
                    f"{name}_gmres_its": np.array(its), f"{name}_seconds": np.array([th, td])})
        print(f"{name}: N = {m.n_unknowns}, hmatrix sweep {th:.1f} s, dense {td:.1f} s, "
              f"max |S_h - S_d| = {np.abs(rh.S - rd.S).max():.2e}, GMRES its {its}", flush=True)
    np.savez_compressed(os.path.join(HERE, "hmatrix.npz"), **out)


if __name__ == "__main__":
    main()
