"""Small, self-contained runs of single engine stages, for profiler captures.

    python -m mom25d_gb300.profile_cases fill  --workload bandpass --precision fp64 [--reps 2]
    python -m mom25d_gb300.profile_cases point --workload lpf --precision mixed [--reps 1]
    python -m mom25d_gb300.profile_cases lu --n 4096 [--simt] [--reps 1]
    python -m mom25d_gb300.profile_cases batch [--variants 16] [--nfreq 128] [--workers 8]
    python -m mom25d_gb300.profile_cases hmatrix --workload gcpw [--freq 10e9] [--reps 2]

`fill` builds the mesh geometry and one frequency's Green's tables, then
runs the impedance fill `reps` times (device output, no host copy);
`point` runs `reps` full frequency points (tables, fill, LU + solve,
de-embedding); `lu` factors a seeded random n x n complex64 matrix on the
device (tensor-core trailing updates unless --simt); `batch` sweeps the
band-pass variants 0 .. variants - 1 at nfreq frequencies 1-12 GHz (mixed
precision) once variant by variant (each a concurrent sweep on `workers`
contexts) and once as one VariantBatch, and prints the points per second of
both; `hmatrix` runs `reps` points with the compressed operator (method
"hmatrix") and one with the dense mixed path, and prints the stage times,
the operator's size and GMRES iterations, and the largest |dS| between the
two. Each exits non-zero on any engine error.
"""

import argparse
import ctypes as C

import numpy as np

from . import engine as E
from . import workloads
from .solver import PRECISIONS, Solver


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["fill", "point", "lu", "batch", "hmatrix"])
    ap.add_argument("--variants", type=int, default=16, help="batch mode: band-pass variants")
    ap.add_argument("--nfreq", type=int, default=128, help="batch mode: frequencies per variant")
    ap.add_argument("--workers", type=int, default=8, help="batch mode: points in flight")
    ap.add_argument("--n", type=int, default=4096, help="matrix size of the lu mode")
    ap.add_argument("--simt", action="store_true", help="lu mode: SIMT trailing updates")
    ap.add_argument("--timing", action="store_true", help="lu mode: print the stage times (CUDA events)")
    ap.add_argument("--workload", default="bandpass")
    ap.add_argument("--precision", default="fp64", choices=list(PRECISIONS))
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--freq", type=float, default=None, help="Hz (default: the workload's middle frequency)")
    ap.add_argument("--prec-block", type=int, default=256, help="hmatrix mode: preconditioner block size")
    ap.add_argument("--restart", type=int, default=200, help="hmatrix mode: GMRES restart length")
    ap.add_argument("--maxiter", type=int, default=3, help="hmatrix mode: GMRES restarts")
    args = ap.parse_args()
    if args.mode == "lu":
        return lu_case(args)
    if args.mode == "batch":
        return batch_case(args)
    if args.mode == "hmatrix":
        return hmatrix_case(args)
    import mom25d_gb300 as G

    kw = {"k": 0} if args.workload == "bandpass" else {}
    lay, st, mesh, freqs = workloads.build(G, args.workload, **kw)
    f = args.freq or float(freqs[len(freqs) // 2])
    sol = Solver(mesh, st, verbose=False, precision=args.precision)
    if args.mode == "fill":
        import torch

        n = mesh.n_unknowns
        dtype = torch.complex64 if args.precision == "mixed_fill32" else torch.complex128
        Z = torch.empty((n, n), dtype=dtype, device="cuda")
        g = sol.greens(f)
        zs = complex(sol.surface_impedance(f))
        for _ in range(args.reps):
            E.check(sol.ctx.lib.m25_assemble(sol.ctx.h, sol.geometry().h, g.h, zs.real, zs.imag, zs.real, zs.imag,
                                             PRECISIONS[args.precision], C.c_void_p(Z.data_ptr()), n,
                                             E.M25_ON_DEVICE))
        sol.ctx.synchronize()
        print(f"fill ok: N={n} |Z|max={float(Z.abs().max()):.3e}")
    else:
        for _ in range(args.reps):
            S = sol.point(f)[0]
        print(f"point ok: N={mesh.n_unknowns} S11={np.round(S[0, 0], 6)}")
    sol.close()


def hmatrix_case(args):
    import json
    import time

    import mom25d_gb300 as G

    kw = {"k": 0} if args.workload == "bandpass" else {}
    lay, st, mesh, freqs = workloads.build(G, args.workload, **kw)
    f = args.freq or float(freqs[len(freqs) // 2])
    sol = Solver(mesh, st, verbose=False, method="hmatrix")
    sol.hmatrix_options = dict(prec_block=args.prec_block)
    t = time.perf_counter()
    hop = sol.hoperator()
    t_plan = time.perf_counter() - t
    times = []
    for _ in range(max(1, args.reps)):
        t = time.perf_counter()
        g = sol.greens(f)
        zs = complex(sol.surface_impedance(f))
        hop.assemble(g, zs, zs)
        sol.ctx.synchronize()
        t1 = time.perf_counter()
        try:
            hop.solve(sol.port_excitations(), restart=args.restart, maxiter=args.maxiter)
        except RuntimeError as exc:  # not converged: report and go on
            print(f"hmatrix: {exc}", flush=True)
        t2 = time.perf_counter()
        g.close()
        times.append((t1 - t, t2 - t1))
    try:
        S_h = sol.point(f)[0]
    except RuntimeError:
        S_h = np.full((len(sol.ports), len(sol.ports)), np.nan, complex)
    sol.close()
    dense = Solver(mesh, st, verbose=False, precision="mixed")
    dense.point(f)
    t = time.perf_counter()
    S_d = dense.point(f)[0]
    t_dense = time.perf_counter() - t
    dense.close()
    s = dict(hop.stats)
    out = dict(workload=args.workload, N=mesh.n_unknowns, freq=f, prec_block=args.prec_block, plan_s=round(t_plan, 3),
               assemble_s=round(min(a for a, _ in times), 4), solve_s=round(min(b for _, b in times), 4),
               hmatrix_point_s=round(min(a + b for a, b in times), 4), dense_mixed_point_s=round(t_dense, 4),
               entries_vs_dense=round((s["near_entries"] + s["far_entries"]) / mesh.n_unknowns ** 2, 4),
               max_dS_vs_dense_mixed=float(np.abs(S_h - S_d).max()),
               **{k: s[k] for k in ("leaves", "near_pairs", "far_blocks", "lowrank_blocks", "dense_far_blocks",
                                    "max_rank", "not_low_rank", "near_field_pairs", "gmres_iterations", "gmres_residuals")})
    print(json.dumps(out))


def lu_case(args):
    import torch

    n = args.n
    ctx = E.Context(0)
    g = torch.Generator(device="cuda").manual_seed(0)
    A0 = torch.randn((n, n), dtype=torch.complex64, device="cuda", generator=g)
    piv = torch.empty(n, dtype=torch.int32, device="cuda")
    info = np.zeros(1, np.int32)
    flags = E.M25_LU_NO_TENSOR_CORES if args.simt else 0
    ms = (C.c_double * 11)()
    if args.timing:
        E.check(ctx.lib.m25_ctx_timing(ctx.h, 1, None, None))
    for _ in range(args.reps):
        A = A0.clone()
        # the engine works on its own stream: torch's copy must have landed
        torch.cuda.synchronize()
        E.check(ctx.lib.m25_lu_factor(ctx.h, n, E.M25_MIXED, C.c_void_p(A.data_ptr()), n,
                                      C.cast(C.c_void_p(piv.data_ptr()), C.POINTER(C.c_int32)), E.M25_ON_DEVICE, flags,
                                      E.ptr(info, C.c_int32)))
    ctx.synchronize()
    if args.timing:
        E.check(ctx.lib.m25_ctx_timing(ctx.h, 0, ms, None))
        names = ["greens", "fill", "gather", "via", "panel", "pack", "swap_trsm", "update", "trsv", "refine",
                 "deembed"]
        print("stage ms per factorisation:", {k: round(v / args.reps, 3) for k, v in zip(names, ms) if v})
    print(f"lu ok: n={n} info={int(info[0])} tensor_cores={not args.simt}")
    ctx.close()


def batch_case(args):
    import json
    import time

    import mom25d_gb300 as G

    from .batch import VariantBatch

    sols, sizes = [], []
    for k in range(args.variants):
        lay, st, mesh, _ = workloads.build(G, "bandpass", k=k)
        sols.append(Solver(mesh, st, verbose=False, precision="mixed"))
        sizes.append(mesh.n_unknowns)
    f = np.linspace(1, 12, args.nfreq) * 1e9
    for s in sols:  # geometry, contexts and buffers of every variant, untimed
        s.sweep(f[:args.workers], workers=args.workers)
    t0 = time.time()
    seq = [s.sweep(f, workers=args.workers) for s in sols]
    t_seq = time.time() - t0
    batch = VariantBatch(sols)
    batch.sweep(f[:args.workers], workers=args.workers)  # the worker contexts' set-up, untimed
    res = batch.sweep(f, workers=args.workers)
    info = res[0].info["batch"]
    dS = max(float(np.abs(a.S - b.S).max()) for a, b in zip(res, seq))
    out = dict(variants=args.variants, N=sizes, freqs=args.nfreq, workers=args.workers, points=info["points"],
               variant_by_variant_points_per_s=round(info["points"] / t_seq, 2),
               batch_points_per_s=round(info["points_per_s"], 2), batch_workers=info["workers"],
               max_dS_batch_vs_separate=dS, tuning=batch.tuning is not None)
    print(json.dumps(out))
    batch.close()
    for s in sols:
        s.close()


if __name__ == "__main__":
    main()
