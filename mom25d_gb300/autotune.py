"""The engine's per-context tuning knobs, chosen by problem size N from a
table measured on the device (mom25d has no such knobs: its LU is LAPACK's).

Knobs (m25_ctx_set_tuning): the smallest cluster (4, 8 or 16 CTAs) the LU
panel runs on, the CTA cap of the triangular solves (0: one CTA per 64-row
block), the number of k-blocks the tensor-core update accumulates in TMEM
before adding into fp32 registers, and the tile shape of that update (N of
128 or 192 real columns; 0: by the update's width). The best values depend
on N: how many rows the panel's cluster holds, how long the wavefront is,
how much of the GPU the points running beside each other leave free.

`run()` measures, for probe workloads spread over the sizes of the sweeps
(band-pass variants of N 1524 to 4972, the LPF at 5943), the points per
second of a concurrent mixed-precision sweep under every candidate
combination, and writes the best per probe to tuning.json beside this file;
each probe covers N up to the midpoint to the next one. batch.VariantBatch
sets the knobs of each point from that table.

    python -m mom25d_gb300.autotune [--points 64] [--workers 8]     (on a GPU)
"""

import argparse
import itertools
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning.json")
KNOBS = ("panel_cluster_min", "wave_ctas", "tc_chunk", "tc_tile_n")
CANDIDATES = dict(panel_cluster_min=(4, 8, 16), wave_ctas=(0, 16), tc_chunk=(1, 2), tc_tile_n=(0, 128))
PROBES = (("bandpass", dict(k=0)), ("bandpass", dict(k=6)), ("bandpass", dict(k=11)), ("bandpass", dict(k=14)),
          ("lpf", {}))


class Tuning:
    """Knob values by N: rows sorted by n_max, the first row whose n_max is
    at least N applies (the last one beyond)."""

    def __init__(self, rows):
        if not rows:
            raise ValueError("a tuning table needs at least one row")
        for r in rows:
            missing = [k for k in KNOBS[:3] + ("n_max",) if k not in r]
            if missing:
                raise ValueError(f"tuning row {r} lacks {missing}")
        # a row without a tile shape leaves it to the engine (0)
        self.rows = sorted(({"tc_tile_n": 0, **r} for r in rows), key=lambda r: r["n_max"])

    def knobs(self, n):
        for r in self.rows:
            if n <= r["n_max"]:
                return tuple(int(r[k]) for k in KNOBS)
        return tuple(int(self.rows[-1][k]) for k in KNOBS)

    def apply(self, ctx, n):
        """Set the knobs for a point of N unknowns on an engine context."""
        from . import engine as E

        E.check(ctx.lib.m25_ctx_set_tuning(ctx.h, *self.knobs(n)))

    @classmethod
    def fixed(cls, **knobs):
        """One row for every N (unset knobs: 0, the process default)."""
        row = {k: int(knobs.get(k, 0)) for k in KNOBS}
        row["n_max"] = math.inf
        return cls([row])


def load_table(path=TABLE):
    """The measured table, or None when none has been written."""
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        data = json.load(fh)
    rows = [dict(r, n_max=math.inf if r["n_max"] is None else r["n_max"]) for r in data["rows"]]
    return Tuning(rows)


def measure(workload, kw, knobs, freqs, workers, device=0, repeats=2):
    """Points per second of a concurrent mixed-precision sweep of one
    workload with the given knob values: the best of `repeats` timed sweeps
    after one untimed one."""
    import mom25d_gb300 as G

    from . import workloads
    from .batch import VariantBatch
    from .solver import Solver

    lay, st, mesh, _ = workloads.build(G, workload, **kw)
    sol = Solver(mesh, st, verbose=False, precision="mixed", device=device)
    try:
        with VariantBatch([sol], tuning=Tuning.fixed(**knobs)) as batch:
            batch.sweep(freqs[:workers], workers=workers)
            best = max(batch.sweep(freqs, workers=workers)[0].info["batch"]["points_per_s"] for _ in range(repeats))
        return best, mesh.n_unknowns
    finally:
        sol.close()


def run(points=64, workers=8, path=TABLE, log=print):
    """Measure every candidate on every probe and write the table."""
    import mom25d_gb300 as G

    from . import workloads

    probes = []
    for workload, kw in PROBES:
        freqs = workloads.BUILDERS[workload](G, **kw)[3]
        fr = freqs[np.linspace(0, len(freqs) - 1, points).round().astype(int)]
        best = None
        for combo in itertools.product(*(CANDIDATES[k] for k in KNOBS)):
            knobs = dict(zip(KNOBS, combo))
            pps, n = measure(workload, kw, knobs, fr, workers)
            log(f"{workload} {kw} N={n} {knobs}: {pps:.2f} points/s")
            if best is None or pps > best[0]:
                best = (pps, knobs, n)
        probes.append(dict(workload=workload, kw=kw, n=best[2], points_per_s=round(best[0], 3), **best[1]))
    probes.sort(key=lambda p: p["n"])
    rows = []
    for i, p in enumerate(probes):
        n_max = (p["n"] + probes[i + 1]["n"]) // 2 if i + 1 < len(probes) else None
        rows.append(dict({k: p[k] for k in KNOBS}, n_max=n_max, probe_n=p["n"], probe=f"{p['workload']} {p['kw']}",
                         points_per_s=p["points_per_s"]))
    data = dict(how=f"mixed-precision concurrent sweep, {workers} workers, {points} frequencies per probe, "
                    "points/s: best of two timed sweeps after an untimed one; candidates " + json.dumps(CANDIDATES),
                rows=rows)
    with open(path, "w") as fh:
        json.dump(data, fh, indent=1)
    return load_table(path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=64)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--out", default=TABLE)
    args = ap.parse_args()
    run(args.points, args.workers, args.out, log=lambda s: print(s, flush=True))


if __name__ == "__main__":
    main()
