"""Multi-GPU sweeps: frequency points (and geometry variants) shard across
ranks with no exchange during the points.

mom25d sweeps one frequency after another in one process
(Engine/mom25d/solver.py:1189-1335); every point is independent, so on N GPUs
each rank takes a share of the (variant, frequency) points, sized by the
dense-LU cost N^3 of its variant, runs them on its own GPU with its own
geometry and Green's tables, and the S / z0 / gamma / fit results (F x P^2
values) come back to rank 0 as host objects through torch.distributed
(gloo or nccl). One process per GPU, launched by torchrun.
"""

import numpy as np


def point_cost(n_unknowns):
    """Relative cost of one frequency point: the dense LU, O(N^3)."""
    return float(n_unknowns) ** 3


def partition(costs, world):
    """Split work items with the given costs over `world` ranks: greedy
    longest-processing-time first (ties to the lower index and rank). Returns
    one list of item indices per rank, each in increasing order; every item
    appears exactly once."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    loads = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += float(costs[i])
    return [sorted(p) for p in parts]


def sharded_map(items, costs, fn, rank=0, world=1, group=None):
    """Evaluate fn(item) for this rank's share of items; on rank 0 return the
    results of all items in input order, on the other ranks None. The only
    communication is one gather of host objects to rank 0 at the end."""
    parts = partition(costs, world)
    local = [(i, fn(items[i])) for i in parts[rank]]
    if world == 1:
        out = [None] * len(items)
        for i, r in local:
            out[i] = r
        return out
    import torch.distributed as dist

    gathered = [None] * world if rank == 0 else None
    dist.gather_object(local, gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * len(items)
    for part in gathered:
        for i, r in part:
            out[i] = r
    return out


def sweep_sharded(solver, freqs, rank=0, world=1, group=None, values=None):
    """Solver.sweep over ranks: rank r runs its share of freqs on its own GPU
    (the solver of each rank holds the same mesh and stack), rank 0 returns
    the SweepResult of all frequencies in order, the other ranks None.
    values: {lumped name: value} overrides, set on every rank's solver before
    its points run, as Solver.sweep(values=...) does."""
    freqs = np.asarray(freqs, float)
    solver.values.clear()
    solver.values.update(values or {})
    cost = point_cost(solver.mesh.n_unknowns)

    def one(f):
        S, z0, gam, zl, res, _, info = solver.point(float(f))
        return S, z0, gam, zl, res, info

    rows = sharded_map(list(freqs), [cost] * len(freqs), one, rank, world, group)
    if rows is None:
        return None
    return assemble_result(freqs, rows, [p.name for p in solver.ports], world)


def assemble_result(freqs, rows, port_names, world=1):
    """The SweepResult of a sharded sweep from its rows in frequency order:
    per frequency (S, z0, gamma, z0_line, residual, info)."""
    from .solver import SweepResult

    return SweepResult(freqs=np.asarray(freqs, float), S=np.array([r[0] for r in rows]),
                       z0=np.array([r[1] for r in rows]), gamma=np.array([r[2] for r in rows]),
                       z0_line=np.array([r[3] for r in rows]), fit_residual=np.array([r[4] for r in rows]),
                       port_names=list(port_names),
                       waves=np.array([r[5]["waves"] for r in rows]) if rows and "waves" in rows[0][5] else None,
                       info=dict(refine_steps=[r[5]["refine_steps"] for r in rows], ranks=world))
