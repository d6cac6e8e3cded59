"""ORACLE (test and measurement infrastructure; never imported by the
product path): the oracle's dense sweep point on all host cores, the CPU
baseline that bench.py times beside the GPU.

mom25d fills Z in one Python process and factors it with multi-threaded
LAPACK (Engine/mom25d/solver.py:11-23, 429-524, 1259-1333). Here the fill's
test blocks are shared out to worker processes (started with `spawn`, one
per host core, one BLAS thread each), each summing its blocks into the rows
of Z they touch (oracle.sweep.scatter_blocks); the parent adds the rows,
finishes the fill (surface impedance, via rows, symmetrisation), factors and
solves with LAPACK on all host threads, and de-embeds. The result is the
oracle's point up to the order in which block sums are added. Every point is
computed in full: nothing is sampled or scaled.
"""

import multiprocessing as mp
import os
import time

import numpy as np

_STATE = {}


def _start(workload, kw):
    """Worker set-up (once per process): the workload's mesh and the
    oracle's assembly geometry."""
    import mom25d_gb300 as G
    from mom25d_gb300 import workloads

    from . import sweep as O

    lay, st, mesh, freqs = workloads.build(G, workload, **kw)
    _STATE["sweep"] = O.Sweep(mesh, st)
    _STATE["kern"] = (None, None)


def _rows(task):
    """Block sums of blocks [a, b) at frequency f: (rows, Z rows)."""
    from . import sweep as O

    f, a, b = task
    sw = _STATE["sweep"]
    fk, kern = _STATE["kern"]
    if fk != f:
        kern = sw.kernels(f)
        _STATE["kern"] = (f, kern)
    geo = sw.geom
    blocks = geo.blocks[a:b]
    rows = O.block_rows(geo, blocks)
    row_map = -np.ones(geo.nb + geo.nv, np.int64)
    row_map[rows] = np.arange(rows.size)
    Z = np.zeros((rows.size, geo.nb + geo.nv), complex)
    O.scatter_blocks(geo, kern, 2 * np.pi * f, blocks, Z, row_map=row_map)
    return rows, Z


class ParallelPoint:
    """Full oracle points of one workload on `procs` worker processes (all
    host cores by default) plus LAPACK on all host threads in this process.

    with ParallelPoint("lpf") as pp:
        S, seconds = pp.point(f)
    """

    def __init__(self, workload, procs=None, chunks_per_proc=4, **kw):
        import mom25d_gb300 as G
        from mom25d_gb300 import workloads

        from . import sweep as O

        self.procs = procs or os.cpu_count() or 1
        lay, st, mesh, freqs = workloads.build(G, workload, **kw)
        self.sweep = O.Sweep(mesh, st)
        if self.sweep.geom.nv:
            raise ValueError("the parallel oracle fill handles meshes without vias")
        nblk = len(self.sweep.geom.blocks)
        edges = np.linspace(0, nblk, min(nblk, self.procs * chunks_per_proc) + 1).round().astype(int)
        self.ranges = [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]
        # workers: spawned (no fork of a process that may hold a CUDA
        # context), one BLAS thread each (the block sums are not BLAS work)
        saved = os.environ.get("OPENBLAS_NUM_THREADS")
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(self.procs, initializer=_start, initargs=(workload, kw))
            self.pool.map(_noop, range(self.procs))  # every worker has built its geometry
        finally:
            if saved is None:
                os.environ.pop("OPENBLAS_NUM_THREADS", None)
            else:
                os.environ["OPENBLAS_NUM_THREADS"] = saved

    def impedance(self, f, kern=None):
        from . import sweep as O

        sw = self.sweep
        geo = sw.geom
        kern = kern or sw.kernels(f)
        Z = np.zeros((geo.nb + geo.nv, geo.nb + geo.nv), complex)
        for rows, part in self.pool.imap_unordered(_rows, [(f, a, b) for a, b in self.ranges]):
            Z[rows] += part
        zs = sw.stack.surface_impedance(f)
        return O.finish_fill(geo, kern, 2 * np.pi * f, Z, zs, zs)

    def point(self, f):
        """(S, seconds) of one full point: tables, fill, LU + solve,
        charges and de-embedding."""
        from . import sweep as O

        sw = self.sweep
        t0 = time.perf_counter()
        kern = sw.kernels(f)
        Z = self.impedance(f, kern)
        x = O.dense_solve(Z, sw.excitations())
        q = O.charges(sw.mesh, x, kern.omega)
        S = sw.deembed(f, kern, x, q)[0]
        return S, time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _noop(_):
    return 0


def serial_point(workload, f, **kw):
    """Seconds of one oracle point the way mom25d runs it: the fill in this
    one process, LAPACK with this process's BLAS threads. Run it in a
    process whose OPENBLAS_NUM_THREADS was set before numpy loaded."""
    import mom25d_gb300 as G
    from mom25d_gb300 import workloads

    from . import sweep as O

    lay, st, mesh, freqs = workloads.build(G, workload, **kw)
    sw = O.Sweep(mesh, st)
    t0 = time.perf_counter()
    S = sw.point(f)[0]
    return S, time.perf_counter() - t0
