"""Frequency points per second of the mom25d sweep path on GB300.

Workload: the 7-section stepped-impedance low-pass (eps_r 3.55, h 0.508 mm,
widths 4.0/0.3 mm, lengths from default_rng(0), mesh 0.35/0.05 mm ->
N = 5943 unknowns), its 101 frequencies 0.5-8 GHz taken in turn. One step =
one frequency point of Solver.sweep: Green's tables, impedance fill, LU +
solve of the 2 port excitations, de-embedding to S, all on the GPU.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64] [--impl reference]

value: points/s with the mesh, test blocks and port data already on the
device (the `mixed` path: fp64 fill, complex64 LU with tensor-core trailing
updates, GMRES refinement to fp64 accuracy), --workers points in flight on
the GPU (one engine context and stream each); timed with CUDA events around
a device-wide synchronisation on both sides. e2e: the same through the
public API (Solver construction + sweep(workers=...), host arrays in, S and
the currents back on the host). Under torchrun each rank sweeps its
own share of the frequencies (shard.partition; weak scaling, no collective
in the path). --impl reference times the CPU oracle (numpy restatement of
mom25d's own path) on full points: the fill's test blocks on one worker
process per host core, LAPACK on all host threads (oracle/parallel.py), plus
one point run as mom25d runs it (one process, 4 BLAS threads).
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "freq points/s at N~6k (mixed + fp64 refinement vs plain fp64), |dS| <= 1e-5"
UNIT = "points/s"
WORKLOAD = {"workload": "stepped-impedance LPF, 7 sections, eps_r 3.55 h 0.508 mm, mesh 0.35/0.05 mm",
            "N": 5943, "triangles": 4134, "ports": 2, "freqs": "101 points 0.5-8 GHz, taken in turn"}


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def build_workload(api):
    from mom25d_gb300 import workloads

    return workloads.build(api, "lpf")


def update_flops(n):
    """Algorithmic real flops of the tensor-core updates of one complex64 LU
    of order n in super-blocks of 256 columns (mom25d_gb300/csrc/lu.cu): per
    super-block at k0 (width SW = min(256, n - k0), blocks a = min(128, SW)
    and b = SW - a) each block's rank-64 update of its second panel's
    columns, block a's rank-128 update of block b's columns, L_ba U_a on
    block b's rows of the trailing columns and the rank-256 update of the
    trailing matrix; 8 real flops per complex multiply-add. The sum is the
    update work of any right-looking complex LU (about 8/3 n^3)."""
    tot = 0.0
    for k0 in range(0, n, 256):
        SW = min(256, n - k0)
        wa = min(128, SW)
        wb = SW - wa
        for c0, W in ((k0, wa), (k0 + wa, wb)):
            w1 = min(64, W)
            tot += 8.0 * (n - c0 - w1) * (W - w1) * w1
        ra = k0 + wa
        if ra >= n:
            break
        tot += 8.0 * (n - ra) * wb * wa
        nt = n - k0 - SW
        if nt > 0:
            tot += 8.0 * wb * nt * wa + 8.0 * nt * nt * SW
    return tot


def lu_flops(n, nrhs=2):
    """Complex LU (8/3 n^3 real flops) + the two triangular solves (8 n^2 nrhs)."""
    return 8.0 / 3.0 * n ** 3 + 8.0 * n * n * nrhs


def run_ours(args, rank, world, local):
    import torch

    import mom25d_gb300 as G
    from mom25d_gb300 import engine as E
    from mom25d_gb300.solver import Solver

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lay, st, mesh, freqs = build_workload(G)
    n = mesh.n_unknowns
    # every rank sweeps its share of world * steps points (equal costs: the
    # same mesh), after `warmup` untimed ones
    from mom25d_gb300.shard import partition, point_cost

    everything = [freqs[(args.warmup + i) % len(freqs)] for i in range(world * args.steps)]
    mine = partition([point_cost(n)] * len(everything), world)[rank]
    my = [freqs[i % len(freqs)] for i in range(args.warmup)] + [everything[i] for i in mine]

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident: geometry, ports uploaded before the timed region;
    # K workers = K engine contexts (streams), points handed out in order;
    # at least three timed points per worker, so that the pipeline's ramp and
    # tail stay a small part of the timed region
    K = max(1, min(args.workers, args.steps // 3))
    tol_kw = {} if args.refine_tol is None else {"refine_tol": args.refine_tol}
    sol = Solver(mesh, st, verbose=False, precision=args.precision, device=local, **tol_kw)
    sols = [sol._sibling(w) for w in range(K)]
    tun = sol._sweep_tuning()  # the engine's knobs by N, as Solver.sweep sets them
    for s_ in sols:
        if tun is not None:
            tun.apply(s_.ctx, n)
        s_.geometry()
        s_.port_data()
    warm = my[:args.warmup]
    for w, s_ in enumerate(sols):
        for f in warm[w::K] or warm[:1]:
            s_.point(f)
    import ctypes as C

    # stage slots of the engine's timers (the row interchanges are timed with the U12 solve they are fused
    # into; lu_pack = the tensor-core update's operand packing, lu_gemm = the update itself)
    STAGES = ["greens", "fill", "gather", "via", "lu_panel", "lu_pack", "lu_swap_trsm", "lu_gemm", "trsv", "refine",
              "deembed"]
    pts = my[args.warmup:]

    def run_points(per_worker):
        lock = threading.Lock()
        nxt = [0]
        errors = []

        def worker(w):
            try:
                while True:
                    with lock:
                        if nxt[0] >= len(pts) or errors:
                            return
                        f = pts[nxt[0]]
                        nxt[0] += 1
                    sols[w].point(f)
                    per_worker[w] += 1
            except Exception as exc:  # noqa: BLE001 - re-raised in the main thread
                with lock:
                    errors.append(exc)

        th = [threading.Thread(target=worker, args=(w,)) for w in range(K)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errors:
            raise errors[0]

    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record()
        run_points([0] * K)
        barrier()  # every worker's stream drained
        ev1.record()
        ev1.synchronize()
    dt = ev0.elapsed_time(ev1) * 1e-3
    # the same points again with the engine's stage timers (CUDA events around
    # every stage, which cost host time: kept out of the timed region above);
    # stage times of worker 0's points, overlapped with the other workers'
    ms = [(C.c_double * 11)() for _ in sols]
    cnt = [(C.c_longlong * 11)() for _ in sols]
    for s_, m_, c_ in zip(sols, ms, cnt):
        E.check(s_.ctx.lib.m25_ctx_timing(s_.ctx.h, 1, m_, c_))  # reset + enable the stage timers
    per_worker = [0] * K
    run_points(per_worker)
    barrier()
    for s_, m_, c_ in zip(sols, ms, cnt):
        E.check(s_.ctx.lib.m25_ctx_timing(s_.ctx.h, 0, m_, c_))
    n0 = max(1, per_worker[0])
    stages = {k: round(v / n0, 4) for k, v in zip(STAGES, ms[0])}
    launches = sum(int(c) for c_ in cnt for c in c_)
    # the tensor-core update of a point with the GPU to itself (after the
    # timed region): CUDA events around its launches, for the roofline
    iso = (C.c_double * 11)()
    E.check(sols[0].ctx.lib.m25_ctx_timing(sols[0].ctx.h, 1, None, None))
    for f in my[:2]:
        sols[0].point(f)
    E.check(sols[0].ctx.lib.m25_ctx_timing(sols[0].ctx.h, 0, iso, None))
    iso_ms = {k: v / 2 for k, v in zip(STAGES, iso)}
    geo = sol.geometry_stats()
    sol.close()
    # ---- e2e through the public API: host arrays in, S + currents out; the
    # Solver and its workers (contexts, buffers) made and warmed on the
    # warm-up frequencies before the timed sweep, as the timed region of the
    # device arm and the reference arm's steps start after their warm-up
    sol2 = Solver(mesh, st, verbose=False, precision=args.precision, device=local, **tol_kw)
    sol2.sweep(warm if len(warm) >= K else my[:K], workers=K)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    r = sol2.sweep(my[args.warmup:], keep_currents=True, workers=K)
    torch.cuda.synchronize()
    barrier()
    dt_e2e = time.perf_counter() - t0
    sol2.close()
    # the engine's fp64 path (fp64 fill + LU) on the same worker count over
    # every 4th timed point: its points/s, and the largest |dS| of the mixed
    # sweep above against it at those frequencies
    t64 = max_dS = None
    n64 = 0
    if args.precision != "fp64" and args.fp64_points > 0:
        step = max(1, len(pts) // args.fp64_points)
        idx = list(range(0, len(pts), step))[:args.fp64_points]
        sub = [pts[i] for i in idx]
        s64 = Solver(mesh, st, verbose=False, precision="fp64", device=local)
        s64.sweep(sub[:K], workers=K)  # the workers' contexts and buffers, untimed
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r64 = s64.sweep(sub, workers=K)
        torch.cuda.synchronize()
        t64 = (time.perf_counter() - t0) / len(sub)
        n64 = len(sub)
        max_dS = float(np.abs(r.S[idx] - r64.S).max())
        s64.close()
    # the learned remainder (mixed + surrogate): a network trained on this
    # stack's Sommerfeld remainders over the workload's band before the timed
    # sweep (its training time reported, not in the points/s), then the same
    # points through Solver.sweep like e2e, S against the fp64 path
    sur_arm = None
    if args.precision == "mixed" and world == 1 and not args.no_surrogate:
        from mom25d_gb300.solver import Greens
        from mom25d_gb300.surrogate import GreensSurrogate

        s3 = Solver(mesh, st, verbose=False, precision="mixed", device=local, **tol_kw)
        t0 = time.perf_counter()
        sur = GreensSurrogate(s3, float(min(freqs)), float(max(freqs)), nfreq=256, nrad=512, steps=20000)
        t_train = time.perf_counter() - t0
        s3.surrogate = sur
        s3.sweep(warm if len(warm) >= K else my[:K], workers=K)  # the workers' contexts and buffers, untimed
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r3 = s3.sweep(pts, workers=K)
        torch.cuda.synchronize()
        dt3 = time.perf_counter() - t0
        used = []
        for f in pts[::max(1, len(pts) // 16)]:
            g = Greens(s3, f)
            info = g.remainder()[1]
            used.append((info[0], info[2], g.rho.size))
            g.close()
        sur_arm = {"value": round(len(pts) / dt3, 4), "unit": UNIT,
                   "timing": "Solver.sweep with the learned remainder attached: the same points, workers, warm-up, "
                             "host arrays in and S out as e2e",
                   "e2e_without": round(world * args.steps / dt_e2e, 4),
                   "train_seconds": round(t_train, 2), "samples": sur.nsamples,
                   "tables_learned": f"{sum(u for u, _, _ in used)} of {len(used)} sampled frequencies",
                   "sommerfeld_radii": f"{sum(k for _, k, _ in used)} of {sum(m for _, _, m in used)}",
                   "max_dS_vs_mixed": float(np.abs(r3.S - r.S).max())}
        if args.fp64_points > 0 and max_dS is not None:
            sur_arm["max_dS_vs_fp64"] = float(np.abs(r3.S[idx] - r64.S).max())
        sur.close()
        s3.close()
    # the compressed operator (method="hmatrix") on the same mesh: one point
    # at the band's middle frequency after one untimed point (its tree,
    # partition and index lists built then), against the mixed path's S there
    hm_arm = None
    if world == 1 and not args.no_hmatrix:
        fm = float(freqs[len(freqs) // 2])
        sh = Solver(mesh, st, verbose=False, method="hmatrix", device=local)
        sh.point(fm)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Sh = sh.point(fm)[0]
        torch.cuda.synchronize()
        th = time.perf_counter() - t0
        hs = sh.hoperator().stats
        sm = Solver(mesh, st, verbose=False, precision="mixed", device=local, **tol_kw)
        Sm = sm.point(fm)[0]
        hm_arm = {"value": round(1.0 / th, 4), "unit": UNIT, "freq": fm,
                  "timing": "one Solver.point with method='hmatrix' (tables, near field, ACA, preconditioner, "
                            "GMRES on both port columns, de-embedding), after one untimed point",
                  "gmres_iterations": hs["gmres_iterations"], "entries_vs_dense":
                      round((hs["near_entries"] + hs["far_entries"]) / mesh.n_unknowns ** 2, 4),
                  "lowrank_blocks": hs["lowrank_blocks"], "max_rank": hs["max_rank"],
                  "max_dS_vs_mixed": float(np.abs(Sh - Sm).max())}
        sm.close()
        sh.close()
    # max over ranks
    tt = torch.tensor([dt, dt_e2e], dtype=torch.float64, device="cuda")
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    dt, dt_e2e = float(tt[0]), float(tt[1])
    if rank != 0:
        return None
    value = world * args.steps / dt
    step_ms = dt / args.steps * 1e3
    # roofline: the LU trailing update (tensor path) or, on the SIMT path,
    # the fill; algorithmic flops per step over the stage's event time
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    lu_ms = iso_ms["lu_gemm"]  # per point: the update kernels of one LU, GPU to themselves
    gemm_flops = update_flops(n)
    achieved = gemm_flops / (lu_ms * 1e-3) / 1e12 if lu_ms else None
    bf16 = peaks.get("bf16_tflops") or 1900.0  # burst: the kernel is timed alone
    # DRAM traffic of the updates per flop, from the ncu capture of all 78
    # update launches of an n = 4096 factorisation in super-blocks of 256
    # columns (1.553 GB for 1.769e11 flops):
    # the rank-256 updates, which carry nearly all of it, read and write C
    # and their operands in proportion to their flops
    traffic = 1.553e9 / 1.769e11 * gemm_flops
    roof = {"kernel": "tc_gemm_kernel: LU trailing update (tcgen05 3xTF32, complex64), all launches of one point",
            "bound": "tensor", "achieved": round(achieved, 2) if achieved else None, "peak": bf16, "unit": "TFLOP/s",
            "frac": round(achieved / bf16, 4) if achieved else None, "traffic": round(traffic),
            "algorithmic_flops": gemm_flops,
            # 3xTF32 executes three tf32 products per algorithmic one, on a pipe
            # with half the bf16 rate
            "tf32_executed_tflops": round(3 * achieved, 1) if achieved else None,
            "tf32_peak_tflops": round(bf16 / 2, 1),
            "tf32_frac": round(3 * achieved / (bf16 / 2), 4) if achieved else None,
            "timing": "CUDA events around the update launches of 2 points run on one worker alone after the "
                      "timed region (in the timed region: stages_ms_per_point_worker0.lu_gemm, shared with the "
                      "other workers)",
            "peak_source": "MEASURED_PEAKS.json bf16 burst" if peaks else "fallback 1.9 PFLOP/s"}
    h2d = (mesh.verts.nbytes + mesh.tri_basis.nbytes // 2 + mesh.tri_sign.nbytes + mesh.edge_len.nbytes) / args.steps
    d2h = n * 2 * 16 + 4 * 16
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64+c128" if args.precision == "mixed" else "c128", "data": "synthetic",
        "config": dict(WORKLOAD, precision=args.precision, l2="inputs > L2 (Z 283 MB, fill scratch 1.4 GB per step)"),
        "e2e": {"value": round(world * args.steps / dt_e2e, 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "workers": K, "stages_ms_per_point_worker0": stages, "gpu_launches": int(launches),
        "fp64_ms_per_point": round(t64 * 1e3, 2) if t64 else None,
        "fp64_points": n64,
        "speedup_vs_fp64": round(t64 / (dt / args.steps), 2) if t64 else None,
        "max_dS_vs_fp64": max_dS,
        "roofline": roof, "clocks": clk.summary(), "geometry": geo,
        "refine_steps": r.info["refine_steps"][:4] if r.info else None,
    }
    if sur_arm is not None:
        out["surrogate"] = sur_arm
    if hm_arm is not None:
        out["hmatrix"] = hm_arm
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline()
    return out


def cpu_baseline(points=2):
    """The oracle's full LPF points on all host cores (oracle/parallel.py):
    one untimed point, then `points` timed ones."""
    import mom25d_gb300 as G
    from oracle.parallel import ParallelPoint

    lay, st, mesh, freqs = build_workload(G)
    with ParallelPoint("lpf") as pp:
        pp.point(freqs[49])
        ts = [pp.point(freqs[50 + i])[1] for i in range(points)]
        procs = pp.procs
    sec = float(np.mean(ts))
    return {"value": round(1.0 / sec, 5), "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{points} full point(s) of the workload after one untimed one (Green's tables, fill, LU + "
                      f"solve, de-embedding; nothing scaled): the fill's test blocks on {procs} worker processes, "
                      "LAPACK (OpenBLAS) on all host threads"}


def serial_reference_point(f, blas_threads=4):
    """Seconds of one oracle point run as mom25d runs it (the fill in one
    Python process, LAPACK with mom25d's default of 4 OpenBLAS threads), in
    a child process whose BLAS thread count is set before numpy loads."""
    code = ("import sys, json; sys.path.insert(0, %r); from oracle.parallel import serial_point; "
            "S, t = serial_point('lpf', %r); print(json.dumps(t))") % (HERE, float(f))
    env = dict(os.environ, OPENBLAS_NUM_THREADS=str(blas_threads), OMP_NUM_THREADS=str(blas_threads))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, check=True)
    return float(out.stdout.strip().splitlines()[-1])


def run_reference(args, rank, world):
    if rank != 0:
        return None
    import mom25d_gb300 as G
    from oracle.parallel import ParallelPoint

    lay, st, mesh, freqs = build_workload(G)
    with ParallelPoint("lpf") as pp:
        for i in range(args.warmup):
            pp.point(freqs[i % len(freqs)])
        ts = [pp.point(freqs[(args.warmup + i) % len(freqs)])[1] for i in range(args.steps)]
        procs = pp.procs
    sec = float(np.sum(ts))
    value = args.steps / sec
    out = {"metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(sec / args.steps * 1e3, 1), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic", "impl": "reference",
           "config": dict(WORKLOAD, precision="fp64 (numpy / scipy LAPACK)"),
           "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": procs, "kind": "port",
                            "sample": "every step one full frequency point (Green's tables, fill, LU + solve, "
                                      f"de-embedding; nothing sampled or scaled): the fill's test blocks on {procs} "
                                      "worker processes, LAPACK (OpenBLAS) on all host threads"},
           "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.serial_points > 0:
        # as mom25d runs by default: one process, 4 BLAS threads
        tser = [serial_reference_point(freqs[(args.warmup + i) % len(freqs)]) for i in range(args.serial_points)]
        out["as_shipped"] = {"s_per_point": round(float(np.mean(tser)), 2), "points": args.serial_points,
                             "processes": 1, "blas_threads": 4,
                             "note": "the oracle point as mom25d runs it: fill in one process, OpenBLAS 4 threads"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-points", type=int, default=16,
                    help="timed points also run on the fp64 path (same workers): its points/s and max |dS|")
    ap.add_argument("--workers", type=int, default=8, help="frequency points in flight on the GPU")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the mixed + learned-remainder arm")
    ap.add_argument("--no-hmatrix", action="store_true", help="skip the compressed-operator point")
    ap.add_argument("--refine-tol", type=float, default=None, help="mixed path: backward-error target of the refinement")
    ap.add_argument("--serial-points", type=int, default=1,
                    help="reference arm: points also timed as mom25d runs them (one process, 4 BLAS threads)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world, local)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
