"""Batched sweeps over geometry variants of uneven N.

mom25d sweeps one layout at a time, one frequency after another
(Engine/mom25d/solver.py:1189-1335): a family of variants (the 16 coupled-
line band-pass filters, N 1524 to 4972) is a loop over independent sweeps.
Here every (variant, frequency) point of the family goes through one work
queue onto K worker threads, each owning ONE engine context (stream and
workspace) that serves every variant: the device buffers of a context grow
to the largest N once and are reused by the points of every smaller variant,
each variant's device geometry is built once and shared by all workers, and
points of different N run side by side on the GPU. Points are handed out
longest first (dense LU cost N^3, then frequency order), which keeps the
last points of the batch short and the GPU full to the end.

Per point, the engine's tuning knobs (smallest cluster of the LU panel, CTA
cap of the triangular solves, the tensor-core update's TMEM accumulation
chunk) are set on the worker's context from the table that autotune.py
measures and writes (tuning.json beside this file), by the point's N.
"""

import threading
import time

import numpy as np

from . import engine as E
from .solver import SweepResult


def point_order(sizes, nfreq):
    """The order in which (variant, frequency index) points are handed out:
    largest N first (LPT on the N^3 cost of the dense LU), then variant,
    then frequency."""
    items = [(v, fi) for v in range(len(sizes)) for fi in range(nfreq[v])]
    return sorted(items, key=lambda it: (-int(sizes[it[0]]), it[0], it[1]))


class VariantBatch:
    """Sweeps of several solvers (variants: their own meshes, one stack or
    several) as one batch of points on this GPU.

    batch = VariantBatch([Solver(m, st, precision="mixed") for m in meshes])
    results = batch.sweep(freqs, workers=8)   # one SweepResult per variant
    """

    def __init__(self, solvers, tuning=None):
        if not solvers:
            raise ValueError("a batch needs at least one solver")
        devices = {s.device for s in solvers}
        if len(devices) != 1:
            raise ValueError("the solvers of a batch run on one device")
        self.solvers = list(solvers)
        self.device = devices.pop()
        self.sizes = [int(s.mesh.n_unknowns) for s in self.solvers]
        # worker contexts and the variants' solvers on them, kept between
        # sweeps (their buffers, port data and kernel set-up are reused)
        self._ctxs = []
        self._views = []
        if tuning is None:
            from .autotune import load_table

            tuning = load_table()
        self.tuning = tuning

    def _workers_that_fit(self, wanted):
        """Workers whose buffers (sized by the largest variant) fit in 90 %
        of the free device memory, on top of every variant's geometry."""
        big = self.solvers[int(np.argmax(self.sizes))]
        for s in self.solvers:
            s.geometry()  # built before measuring what is left
        free, total = E.C.c_uint64(), E.C.c_uint64()
        E.check(big.ctx.lib.m25_ctx_mem_info(big.ctx.h, E.C.byref(free), E.C.byref(total)))
        return max(1, min(int(wanted), int(0.9 * free.value // max(1, big._worker_bytes()))))

    def sweep(self, freqs, workers=8, keep_currents=False):
        """S-parameters of every variant at freqs (one array for all, or one
        per variant). Returns one SweepResult per variant, in order; each
        carries info["batch"] with the batch's wall time, worker count and
        points per second."""
        V = len(self.solvers)
        if len(freqs) == V and all(np.ndim(f) == 1 for f in freqs):
            fl = [np.asarray(f, float) for f in freqs]
        else:
            fl = [np.atleast_1d(np.asarray(freqs, float))] * V
        for s in self.solvers:
            s.values.clear()
        order = point_order(self.sizes, [len(f) for f in fl])
        # the worker pool is sized by the first sweep (what fits in device
        # memory then); later sweeps use at most that many
        pool = len(self._ctxs) or self._workers_that_fit(workers)
        K = max(1, min(len(order), int(workers), pool))
        while len(self._ctxs) < K:
            self._ctxs.append(E.Context(self.device))
            self._views.append([None] * V)
        ctxs, views = self._ctxs, self._views
        def arrays(s, f):
            n = len(s.ports) + len(s.iports)
            return dict(S=np.zeros((len(f), n, n), complex), z0=np.zeros((len(f), n)),
                        gamma=np.zeros((len(f), n), complex), z0_line=np.zeros((len(f), n), complex),
                        res=np.zeros((len(f), n)), waves=np.zeros((len(f), n, n), complex), cur=[None] * len(f),
                        steps=[None] * len(f))

        out = [arrays(s, f) for s, f in zip(self.solvers, fl)]
        lock = threading.Lock()
        nxt = [0]
        errors = []

        def view(w, v):
            if views[w][v] is None:
                views[w][v] = self.solvers[v]._clone(ctx=ctxs[w])
            for k in self.solvers[v]._SETTINGS:  # the variant's settings as they are now
                setattr(views[w][v], k, getattr(self.solvers[v], k))
            return views[w][v]

        def work(w):
            while True:
                with lock:
                    if errors or nxt[0] >= len(order):
                        return
                    v, fi = order[nxt[0]]
                    nxt[0] += 1
                try:
                    sol = view(w, v)
                    if self.tuning is not None:
                        self.tuning.apply(ctxs[w], self.sizes[v])
                    S, z0, gam, zl, res, x, info = sol.point(float(fl[v][fi]), keep_currents)
                except Exception as exc:  # noqa: BLE001 - re-raised in the caller's thread
                    with lock:
                        errors.append(exc)
                    return
                o = out[v]
                with lock:
                    o["S"][fi], o["z0"][fi], o["gamma"][fi], o["z0_line"][fi], o["res"][fi] = S, z0, gam, zl, res
                    o["waves"][fi] = info["waves"]
                    o["cur"][fi] = x
                    o["steps"][fi] = info["refine_steps"]

        t0 = time.time()
        for s in self.solvers:
            s.geometry()
        th = [threading.Thread(target=work, args=(w,)) for w in range(K)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errors:
            raise errors[0]
        dt = time.time() - t0
        batch = dict(seconds=dt, workers=K, points=len(order), points_per_s=len(order) / dt)
        res = []
        for s, f, o in zip(self.solvers, fl, out):
            info = dict(refine_steps=o["steps"], workers=K, batch=batch,
                        fp64_fallback=[float(f[i]) for i, st in enumerate(o["steps"]) if st is not None and st < 0])
            names = [p.name for p in s.ports] + [ip["name"] for ip in s.iports]
            res.append(SweepResult(f, o["S"], o["z0"], o["gamma"], o["z0_line"], o["res"], names,
                                   o["cur"] if keep_currents else None, o["waves"], info=info))
        return res

    def close(self):
        """Release the worker contexts (the variants' own solvers stay open)."""
        for row in self._views:
            for sv in row:
                if sv is not None:
                    sv.close()
        for c in self._ctxs:
            c.close()
        self._ctxs, self._views = [], []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
