"""Generate the golden fixtures of this directory by running mom25d itself.

Run where the mom25d sources are importable: pass the directory that holds
mom25d's `mom25d` package (its `Engine` directory) with --ref or in the
environment variable MOM25D_SRC. The fixtures are committed so that tests on
machines without mom25d compare against them:

    MOM25D_SRC=<mom25d checkout>/Engine python tests/golden/make_golden.py [--quick]

Every case uses the sweep settings the parity tests assume: method="dense"
(dense LU) and interp=None (an exact fill at every frequency), except the
*_interp fixtures (--interp), which record mom25d's FreqInterp.
"""

import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from mom25d_gb300 import workloads  # noqa: E402

ref = ref_solver = potential_integrals = None


def import_reference(src):
    """Import mom25d from the directory `src` (the one holding its package)."""
    global ref, ref_solver, potential_integrals
    if not src or not os.path.isdir(os.path.join(src, "mom25d")):
        raise SystemExit("give mom25d's source directory (the one holding the mom25d package) "
                         "with --ref or MOM25D_SRC")
    sys.path.insert(0, src)
    import mom25d
    from mom25d import solver
    from mom25d.integrals import potential_integrals as pint

    ref, ref_solver, potential_integrals = mom25d, solver, pint


def mesh_digest(m):
    h = hashlib.sha256()
    for a in (m.nodes, m.tris, m.tri_basis, m.tri_sign, m.edge_len, m.tri_layer):
        h.update(np.ascontiguousarray(a).tobytes())
    for s in m.via_segments:
        h.update(repr((s["via"], s["top"], s["bottom"])).encode())
        for k in ("top_tris", "bottom_tris"):
            if s[k] is not None:
                h.update(np.asarray(s[k], np.int64).tobytes())
    return h.hexdigest()


def cache_points(sol):
    """Wrap a mom25d Solver's greens / solve_currents so that a frequency's
    tables and currents are computed once: the sweep then reuses the point
    computed step by step for the stage fixtures (and the floor runs redo
    only the de-embedding)."""
    cache = {}
    greens, solve = sol.greens, sol.solve_currents

    def cached_greens(f):
        if ("g", f) not in cache:
            cache[("g", f)] = greens(f)
        return cache[("g", f)]

    def cached_solve(f, excitations=None, greens=None, Z=None, interp=None):
        if excitations is not None or interp is not None:
            return solve(f, excitations=excitations, greens=greens, Z=Z, interp=interp)
        if ("x", f) not in cache:
            cache[("x", f)] = solve(f, greens=greens, Z=Z)
        return cache[("x", f)]

    sol.greens, sol.solve_currents = cached_greens, cached_solve
    return cache


def solve_point(sol, f):
    """Everything the sweep computes at one frequency, step by step."""
    g = sol.greens(f)
    Z = sol.impedance(f, g)
    x = sol.solve_currents(f, greens=g, Z=Z.copy())
    q = sol.charges(x, g.omega)
    return g, Z, x, q


def stage_arrays(sol, g, x, q):
    """The de-embedding's inputs at one frequency as mom25d's sweep forms them
    (Engine/mom25d/solver.py:1276-1301): line voltages phi at every port's
    voltage points (ports in order, (M, P)), cut currents I and cut voltages
    V of every port ((sum Ns, P))."""
    npt = len(sol.ports)
    phi = [None] * npt
    for lay in dict.fromkeys(p.layer for p in sol.ports):
        ps = [p for p in range(npt) if sol.ports[p].layer == lay]
        vp = sol.line_voltage(g, q, np.concatenate([sol.pm[p].vpts for p in ps]), lay)
        for p, v in zip(ps, np.split(vp, np.cumsum([len(sol.pm[p].vpts) for p in ps])[:-1])):
            phi[p] = v
    I = np.concatenate([sol.pm[p].currents(x) for p in range(npt)])
    V = np.concatenate([sol.pm[p].voltages(phi[p]) for p in range(npt)])
    return dict(phi=np.concatenate(phi), I=I, V=V)


def sweep(sol, freqs):
    t = time.time()
    r = sol.sweep(freqs, interp=None)
    return r, time.time() - t


def result_arrays(r, prefix=""):
    return {prefix + "S": r.S, prefix + "z0": r.z0, prefix + "gamma": r.gamma, prefix + "z0_line": r.z0_line,
            prefix + "fit_residual": r.fit_residual, prefix + "S50": r.renormalize(50)}


def fixture_name(name, kw):
    return f"{name}{'_' + str(kw['k']) if kw and 'k' in kw else ''}"


def case(name, freqs_full=None, zfull=False, zrows=None, sweep_freqs=None, kw=None, tables=True):
    lay, stack, mkw, freqs = workloads.BUILDERS[name](ref, **(kw or {}))
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    cache_points(sol)
    out = dict(N=m.n_unknowns, Nt=len(m.tris), mesh_sha=mesh_digest(m), rho_max=sol.rho_max)
    f0 = freqs[0] if sweep_freqs is None else sweep_freqs[0]
    t = time.time()
    g, Z, x, q = solve_point(sol, f0)
    out["f0"] = f0
    if zfull:
        out["Z"] = Z
    if zrows is not None:
        rows = np.unique(np.r_[zrows, m.n_unknowns - 1])
        out["Z_rows_idx"] = rows
        out["Z_rows"] = Z[rows]
        out["Z_diag"] = np.diag(Z).copy()
    del Z
    out["x"] = x
    out["q"] = q
    out.update(stage_arrays(sol, g, x, q))
    print(f"{name}: first point {time.time() - t:.1f} s", flush=True)
    if sol.single and tables:
        out["rho_tab"] = g.rho_tab
        out["SA_tab"], out["SV_tab"], out["SW_tab"] = g.SA_tab, g.SV_tab, g.SW_tab
        out["spl_c"], out["splw_c"] = g._spl.c, g._splw.c
        out["cv"] = g.cv
    elif tables:
        out["rho_tab"] = g.rho_tab
        L = len(g.levels)
        for i in range(L):
            for j in range(L):
                p = g.pair(i, j)
                out[f"pair{i}{j}_c"] = np.array([p.cA, p.cV, p.cW], complex)
                out[f"pair{i}{j}_dz"] = p.dz
                out[f"pair{i}{j}_spl_c"] = p._spl.c
                out[f"pair{i}{j}_splw_c"] = p._splw.c
    sf = freqs if sweep_freqs is None else np.asarray(sweep_freqs)
    r, dt = sweep(sol, sf)
    out["freqs"] = sf
    out["sweep_seconds"] = dt
    out.update(result_arrays(r))
    np.savez_compressed(os.path.join(HERE, fixture_name(name, kw) + ".npz"), **out)
    print(f"{name}: N={m.n_unknowns} Nt={len(m.tris)} {len(sf)} freqs {dt:.1f} s ({dt / len(sf):.2f} s/pt)", flush=True)


FLOOR_EPS = (1e-15, 1e-14, 1e-13, 1e-12, 1e-11, 1e-10)


def floor_case(name, sweep_freqs, seeds=4, kw=None):
    """The reference's own reproducibility floor: mom25d's sweep at the same
    frequencies with (a) the inputs of its wave fit (cut currents I and
    voltages V, Engine/mom25d/solver.py:618-670) and (b) its RWG currents x
    multiplied by 1 + eps (n1 + j n2), n standard normal, seeded, for eps in
    FLOOR_EPS. Stored: per eps, the largest |S - S0| over the seeds at each
    frequency, and the largest relative change of gamma. A re-implementation
    whose fit inputs differ from mom25d's by eps cannot be expected to match
    mom25d's S closer than this."""
    lay, stack, mkw, _ = workloads.BUILDERS[name](ref, **(kw or {}))
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    cache = cache_points(sol)
    freqs = np.asarray(sweep_freqs, float)
    r0 = sol.sweep(freqs, interp=None)
    fit0 = ref_solver.fit_waves
    cached = sol.solve_currents
    out = dict(freqs=freqs, eps=np.array(FLOOR_EPS), S=r0.S, gamma=r0.gamma, N=m.n_unknowns)
    for mode in ("fit", "x"):
        dS = np.zeros((len(FLOOR_EPS), len(freqs)))
        dg = np.zeros((len(FLOOR_EPS), len(freqs)))
        for ie, eps in enumerate(FLOOR_EPS):
            for seed in range(seeds):
                rng = np.random.default_rng(1000 * ie + seed)

                def noisy(a):
                    return a * (1 + eps * (rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape)))

                def fit(s_list, I_list, V_list, gamma0, **k):
                    return fit0(s_list, [noisy(I) for I in I_list], [noisy(V) for V in V_list], gamma0, **k)

                def solve(f, **k):
                    return noisy(cached(f, **k))

                try:
                    if mode == "fit":
                        ref_solver.fit_waves = fit
                    else:
                        sol.solve_currents = solve
                    r = sol.sweep(freqs, interp=None)
                finally:
                    ref_solver.fit_waves = fit0
                    sol.solve_currents = cached
                dS[ie] = np.maximum(dS[ie], np.abs(r.S - r0.S).max(axis=(1, 2)))
                dg[ie] = np.maximum(dg[ie], (np.abs(r.gamma - r0.gamma) / np.abs(r0.gamma)).max(axis=1))
        out[f"dS_{mode}"], out[f"dgamma_{mode}"] = dS, dg
        print(f"floor {name} {mode}: max |dS| per eps", dS.max(1), flush=True)
    del cache
    return out


FLOOR_CASES = dict(line=("line", [2e9, 7e9], None), tee=("tee", np.linspace(1, 10, 37)[[0, 12, 24, 36]] * 1e9, None),
                   via=("via", [2e9, 10e9, 18e9], None), bandpass_0=("bandpass", [3e9, 9e9], dict(k=0)),
                   lpf=("lpf", [0.5e9, 4e9, 8e9], None), line_lossless=("line_lossless", [2e9, 5e9, 7e9], None))


def floor_all(only=None):
    """fit_floor.npz for FLOOR_CASES (only: those keys, merged into the
    existing file)."""
    path = os.path.join(HERE, "fit_floor.npz")
    out, done = {}, []
    if only and os.path.exists(path):
        old = np.load(path)
        done = [str(c) for c in old["cases"] if str(c) not in only]
        out = {k: old[k] for k in old.files if k != "cases" and any(k.startswith(c + "_") for c in done)}
    for key, (name, fr, kw) in FLOOR_CASES.items():
        if only and key not in only:
            continue
        for k, v in floor_case(name, fr, kw=kw).items():
            out[f"{key}_{k}"] = v
        done.append(key)
    np.savez_compressed(path, cases=np.array(done), **out)
    print("fit floor: done", flush=True)


def x_floor_case(name, f, kw=None, eps=1e-13, seeds=2):
    """The conditioning floor of every stage of a point: mom25d's currents x
    from its Z at f, and from the same Z with every entry multiplied by
    1 + eps (n1 + j n2) (n standard normal, seeded), then the charges q,
    line voltages phi, cut currents I and voltages V and S of each (its own
    de-embedding). Returns {stage: max over the seeds of max |d| / max |.|}
    (S: max |dS|). An implementation whose Z agrees with mom25d's to eps
    cannot be expected to agree closer than this."""
    lay, stack, mkw, _ = workloads.BUILDERS[name](ref, **(kw or {}))
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    cache = cache_points(sol)
    g = sol.greens(f)
    Z = sol.impedance(f, g)
    B = sol.port_excitations()
    solve = sol.solve_currents

    def stages(x):
        q = sol.charges(x, g.omega)
        st = stage_arrays(sol, g, x, q)
        sol.solve_currents = lambda fr, **k: x
        try:
            S = sol.sweep([f], interp=None).S[0]
        finally:
            sol.solve_currents = solve
        return dict(x=x, q=q, phi=st["phi"], I=st["I"], V=st["V"], S=S)

    base = stages(ref_solver._dense_solve(Z.copy(), B))
    worst = {k: 0.0 for k in base}
    for seed in range(seeds):
        rng = np.random.default_rng(seed)
        Zp = Z * (1 + eps * (rng.standard_normal(Z.shape) + 1j * rng.standard_normal(Z.shape)))
        other = stages(ref_solver._dense_solve(Zp, B))
        del Zp
        for k in base:
            d = float(np.abs(other[k] - base[k]).max())
            worst[k] = max(worst[k], d if k == "S" else d / float(np.abs(base[k]).max()))
    del cache
    print(f"stage floors {name} {kw or ''}: " + ", ".join(f"{k} {v:.1e}" for k, v in worst.items()), flush=True)
    return worst


def x_floor_all(names):
    """x_floor.npz: the conditioning floors of x (key: the fixture's name)
    and of each stage (key: name_stage) at each fixture's f0."""
    path = os.path.join(HERE, "x_floor.npz")
    for key in names:
        g = np.load(os.path.join(HERE, key + ".npz"))
        base, kw = (("bandpass", dict(k=int(key.split("_")[1]))) if key.startswith("bandpass_") else (key, None))
        floors = x_floor_case(base, float(g["f0"]), kw)
        # read the file again just before writing: other runs may have added cases
        out = dict(np.load(path)) if os.path.exists(path) else {}
        out["eps"] = np.array(1e-13)
        out[key] = np.array(floors["x"])
        for k, v in floors.items():
            out[f"{key}_{k}"] = np.array(v)
        np.savez_compressed(path, **out)


def interp_case(name, interp_kw=None, nfreq=None, zrows=None):
    """FreqInterp (Engine/mom25d/freqinterp.py) on a case: the anchors, phase
    ratio, step, basis centres, window and weights of every frequency, rows
    of the interpolated Z at an off-anchor frequency and the S of the
    interpolated sweep."""
    from mom25d.freqinterp import FreqInterp

    lay, stack, mkw, freqs = workloads.BUILDERS[name](ref)
    if nfreq is not None:
        freqs = np.linspace(min(freqs), max(freqs), nfreq)
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    ip = FreqInterp(**(interp_kw or {})).setup(sol, freqs)
    out = dict(N=m.n_unknowns, mesh_sha=mesh_digest(m), freqs=np.asarray(freqs), anchors=ip.anchors,
               k_ratio=ip.k_ratio, step=ip.step, order=ip.order, pos=ip.pos, nb=ip.nb)
    out["windows"] = np.array([ip._window(f) for f in freqs])
    out["weights"] = np.array([ip.weights(f, ip._window(f)) for f in freqs])
    # the off-anchor frequency farthest from every anchor
    fm = max(freqs, key=lambda f: np.min(np.abs(ip.anchors - f)))
    Zi = ip.impedance(fm)
    rows = np.unique(np.r_[zrows if zrows is not None else [0], m.n_unknowns - 1])
    out.update(f_mid=fm, Z_rows_idx=rows, Zi_rows=Zi[rows])
    t = time.time()
    r = sol.sweep(freqs, interp=FreqInterp(**(interp_kw or {})))
    dt = time.time() - t
    out["sweep_seconds"] = dt
    out.update(result_arrays(r))
    np.savez_compressed(os.path.join(HERE, f"{name}_interp.npz"), **out)
    print(f"{name} interp: N={m.n_unknowns} {len(freqs)} freqs, {len(ip.anchors)} anchors, {dt:.1f} s", flush=True)


def iport_case(name):
    """Internal ports (Layout.add_gap_port / add_via_port): mom25d's sweep with
    the internal ports' excitations, loads and S extension
    (Engine/mom25d/solver.py:1029-1070, 1305-1356)."""
    lay, stack, mkw, freqs = workloads.BUILDERS[name](ref)
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    r = sol.sweep(freqs, interp=None, keep_currents=True)
    out = dict(N=m.n_unknowns, mesh_sha=mesh_digest(m), freqs=freqs, iport_vectors=m.internal_port_vectors(),
               Lm=sol.Lm, iport_index=np.array(sol.iport_index), port_names=np.array(r.port_names),
               x0=r.currents[0], waves=r.waves)
    out.update(result_arrays(r))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: N={m.n_unknowns} ports {r.port_names}", flush=True)


def write_block(path, freqs):
    """A synthetic 2-port (attenuator with a phase delay, slightly unmatched)
    as a Touchstone v1 file in MA format with a GHz axis, 50 ohm."""
    with open(path, "w") as fh:
        fh.write("! synthetic 2-port block for the network tests\n# GHZ S MA R 50\n")
        for f in freqs:
            ph = -360.0 * f / 4e9
            s11, s21 = 0.08 * (1 + f / 20e9), 0.7 - 0.01 * f / 1e9
            # Touchstone v1 2-port order: S11 S21 S12 S22
            fh.write(f"{f / 1e9:.6f} {s11:.6f} {ph / 3:.4f} {s21:.6f} {ph:.4f} {s21:.6f} {ph:.4f} "
                     f"{s11 * 1.1:.6f} {ph / 2:.4f}\n")


def lumped_case():
    """A lumped component across a gap (Layout.add_lumped, Solver._load_lumped):
    gap vectors, loads, loaded currents and gap currents at the first
    frequency, the sweep, and a sweep with the value overridden."""
    lay, stack, mkw, freqs = workloads.BUILDERS["lumped_line"](ref)
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    f0 = freqs[0]
    g = sol.greens(f0)
    x = sol.solve_currents(f0, greens=g)
    out = dict(N=m.n_unknowns, mesh_sha=mesh_digest(m), freqs=freqs, Lm=sol.Lm, D0=sol.lumped_impedance(f0),
               x=x, I_gap=sol.lumped_currents(x))
    r = sol.sweep(freqs, interp=None)
    out.update(result_arrays(r))
    r2 = sol.sweep(freqs, interp=None, values={"Z1": "C 1p"})
    out.update(result_arrays(r2, "C1p_"))
    r3 = sol.sweep(freqs, interp=None, values={"Z1": None})
    out.update(result_arrays(r3, "open_"))
    np.savez_compressed(os.path.join(HERE, "lumped_line.npz"), **out)
    print(f"lumped_line: N={m.n_unknowns}", flush=True)
    # a 2-port block (block.s2p, written by network_case) across two open gaps
    lay, stack, mkw, freqs = workloads.BUILDERS["component_line"](ref, block=os.path.join(HERE, "block.s2p"))
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    out = dict(N=m.n_unknowns, mesh_sha=mesh_digest(m), freqs=freqs, Lm=sol.Lm, D0=sol.lumped_impedance(freqs[0]))
    r = sol.sweep(freqs, interp=None)
    out.update(result_arrays(r))
    np.savez_compressed(os.path.join(HERE, "component_line.npz"), **out)
    print(f"component_line: N={m.n_unknowns}", flush=True)


def network_case():
    """SweepResult waves, matched / wave currents and connect (Engine/mom25d/
    solver.py:673-765, network.py) on the line case with a synthetic block."""
    lay, stack, mkw, freqs = workloads.BUILDERS["line"](ref)
    m = lay.mesh(**mkw)
    sol = ref.Solver(m, stack, verbose=False, method="dense")
    g = np.load(os.path.join(HERE, "line.npz"))
    fr = g["freqs"]
    r = sol.sweep(fr, interp=None, keep_currents=True)
    block = os.path.join(HERE, "block.s2p")
    write_block(block, np.linspace(0.5 * fr.min(), 1.5 * fr.max(), 9))
    net = r.connect(block, [(1, 1)])
    out = dict(freqs=fr, S=r.S, z0=r.z0, gamma=r.gamma, z0_line=r.z0_line, fit_residual=r.fit_residual,
               waves=r.waves, x0=r.currents[0], port_names=np.array(r.port_names), matched0=r.matched_currents(0, 0),
               wave0=r.wave_currents(0, [1.0, 0.5j]), net_S=net.S, net_names=np.array(net.names),
               net_currents0=net.currents(0, 0))
    np.savez_compressed(os.path.join(HERE, "line_network.npz"), **out)
    print("network: done", flush=True)


def kernels():
    """Known-answer vectors for the closed-form integrals and the slab kernels."""
    rng = np.random.default_rng(1)
    V = rng.uniform(-1e-3, 1e-3, (6, 3, 2))
    e1, e2 = V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]
    cw = (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]) < 0
    V[cw] = V[cw][:, [0, 2, 1]]
    r = rng.uniform(-2e-3, 2e-3, (9, 2))
    r[0] = V[0, 0]  # observer on a vertex
    r[1] = 0.5 * (V[1, 0] + V[1, 1])  # on an edge
    out = dict(V=V, r=r)
    for d in (0.0, 0.254e-3):
        I0, I1 = potential_integrals(V, r, d)
        out[f"I0_{d:g}"], out[f"I1_{d:g}"] = I0, I1
    g = ref.GroundedSlabGreens(5e9, 3.55, 0.508e-3, 0.0027, rho_max=0.03, zs_ground=0.02 + 0.02j)
    R = np.geomspace(1e-6, 0.03, 40)
    out["slab_R"] = R
    out["slab_gA"], out["slab_gV"], out["slab_gW"] = g.gA(R), g.gV(R), g.gW(R)
    out["slab_rho_tab"] = g.rho_tab
    out["slab_SA"], out["slab_SV"], out["slab_SW"] = g.SA_tab, g.SV_tab, g.SW_tab
    L = ref_solver.via_inductance([ref.Via((0, 0), 0.3e-3), ref.Via((1e-3, 0.2e-3), 0.2e-3)], 0.508e-3)
    out["via_L"] = L
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **out)
    print("kernels: done", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MOM25D_SRC"),
                    help="directory holding mom25d's package (default: $MOM25D_SRC)")
    ap.add_argument("--quick", action="store_true", help="small cases only")
    ap.add_argument("--interp", action="store_true", help="only the FreqInterp fixtures")
    ap.add_argument("--network", action="store_true", help="only the network / waves fixture")
    ap.add_argument("--lumped", action="store_true", help="only the lumped-component fixture")
    ap.add_argument("--floor", nargs="*", default=None, metavar="CASE",
                    help="only the wave-fit floor fixture (of the given FLOOR_CASES keys, merged into the file)")
    ap.add_argument("--xfloor", nargs="+", default=None, metavar="FIXTURE",
                    help="only the conditioning floor of x at the f0 of the given fixtures")
    ap.add_argument("--variants", action="store_true", help="only band-pass variants 3, 7, 11 and 14")
    ap.add_argument("--lossless", action="store_true", help="only the lossless line (mom25d's bounded beta fit)")
    ap.add_argument("--iports", action="store_true", help="only the internal-port cases (gap port, via port)")
    ap.add_argument("--stripline", action="store_true", help="only the stripline under a PEC cover")
    ap.add_argument("--gcpw", action="store_true",
                    help="only the grounded CPW (N = 25284: ~30 GB of memory, ~20 min per frequency)")
    args = ap.parse_args()
    import_reference(args.ref)
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "4")
    if args.network:
        network_case()
        return
    if args.lumped:
        lumped_case()
        return
    if args.interp:
        interp_case("tee", zrows=np.arange(0, 1085, 97))
        interp_case("shunt_via", interp_kw=dict(step=1.5e9), nfreq=25, zrows=np.arange(0, 492, 41))
        return
    if args.floor is not None:
        floor_all(args.floor or None)
        return
    if args.xfloor:
        x_floor_all(args.xfloor)
        return
    fb = np.linspace(1, 12, 128) * 1e9
    if args.iports:
        iport_case("gap_port_line")
        iport_case("via_port_line")
        return
    if args.lossless:
        case("line_lossless", zrows=np.arange(0, 546, 37), sweep_freqs=[2e9, 5e9, 7e9])
        return
    if args.stripline:
        case("stripline", zrows=np.arange(0, 200, 23))
        return
    if args.variants:
        for k in (3, 7, 11, 14):
            n = workloads.BANDPASS_N[k]
            case("bandpass", kw=dict(k=k), zrows=np.arange(0, n, n // 7), sweep_freqs=fb[[10, 60, 115]],
                 tables=False)
        return
    if args.gcpw:
        fg = np.linspace(1, 20, 64) * 1e9
        case("gcpw", zrows=np.arange(0, 25284, 4214), sweep_freqs=[fg[0], fg[31]], tables=False)
        return
    kernels()
    case("line", zrows=np.arange(0, 546, 37))
    case("shunt_via", zrows=np.arange(0, 492, 41))
    case("line_lossless", zrows=np.arange(0, 546, 37), sweep_freqs=[2e9, 5e9, 7e9])
    if args.quick:
        return
    case("tee", zrows=np.arange(0, 1085, 97))
    case("via", zrows=np.arange(0, 3789, 379), sweep_freqs=[2e9, 10e9, 18e9])
    case("bandpass", kw=dict(k=0), zrows=np.arange(0, 1524, 211), sweep_freqs=[3e9, 9e9])
    # 11 of the 101 frequencies, 0.5 GHz (the hardest for the mixed refinement) to 8 GHz
    case("lpf", zrows=np.arange(0, 5943, 743), sweep_freqs=np.linspace(0.5, 8, 101)[::10] * 1e9)


if __name__ == "__main__":
    main()
