"""CPU tests of lumped components (Layout.add_lumped, mom25d_gb300/lumped.py,
Solver.lumped_impedance / _load_lumped) against mom25d's own run of the
lumped_line workload (tests/golden/lumped_line.npz; make_golden.py
--lumped): the mesh and gap vectors, the loads, and the loaded currents from
the oracle's fill."""

import hashlib
import os
from types import SimpleNamespace

import numpy as np

import mom25d_gb300 as G
from mom25d_gb300 import lumped as LP
from mom25d_gb300 import workloads
from mom25d_gb300.solver import Solver
from oracle import sweep as O

from conftest import golden


def digest(m):
    h = hashlib.sha256()
    for a in (m.nodes, m.tris, m.tri_basis, m.tri_sign, m.edge_len, m.tri_layer):
        h.update(np.ascontiguousarray(a).tobytes())
    for s in m.via_segments:
        h.update(repr((s["via"], s["top"], s["bottom"])).encode())
        for k in ("top_tris", "bottom_tris"):
            if s[k] is not None:
                h.update(np.asarray(s[k], np.int64).tobytes())
    return h.hexdigest()


def host_solver(m):
    """What Solver.lumped_impedance and _load_lumped read, without a device."""
    return SimpleNamespace(lumped=list(m.layout.lumped), values={}, OPEN=Solver.OPEN, Lm=m.lumped_vectors(),
                           iports=[], iport_index=[])


def test_mesh_and_gap_vectors_match_reference():
    g = golden("lumped_line")
    lay, st, m, _ = workloads.build(G, "lumped_line")
    assert digest(m) == str(g["mesh_sha"])
    np.testing.assert_array_equal(m.lumped_vectors(), g["Lm"])


def test_values_and_loads():
    f = 3.3e9
    assert LP.parse("R 20 + L 0.5n").z(f) == 20 + 2j * np.pi * f * 0.5e-9
    assert abs(LP.parse("C 1p || R 1k").z(f) - 1 / (2j * np.pi * f * 1e-12 + 1e-3)) < 1e-9
    assert LP.as_value(50).z(f) == 50
    g = golden("lumped_line")
    lay, st, m, _ = workloads.build(G, "lumped_line")
    sol = host_solver(m)
    np.testing.assert_allclose(Solver.lumped_impedance(sol, float(g["freqs"][0])), g["D0"], rtol=1e-15)
    sol.values["Z1"] = None
    assert Solver.lumped_impedance(sol, 1e9)[0, 0] == Solver.OPEN


def test_loaded_currents_from_oracle_fill():
    """The oracle's fill, one solve for the port and gap excitations and the
    Woodbury loading give mom25d's loaded currents and gap current."""
    g = golden("lumped_line")
    lay, st, m, _ = workloads.build(G, "lumped_line")
    sw = O.Sweep(m, st)
    f0 = float(g["freqs"][0])
    Z = sw.impedance(f0)
    sol = host_solver(m)
    sol.lumped_impedance = lambda f: Solver.lumped_impedance(sol, f)
    E0 = sw.excitations()
    X = O.dense_solve(Z.copy(), np.hstack([E0, sol.Lm]))
    P = E0.shape[1]
    x = Solver._load_lumped(sol, X[:, :P], X[:, P:], f0)
    assert np.abs(x - g["x"]).max() <= 1e-8 * np.abs(g["x"]).max()
    np.testing.assert_allclose(sol.Lm.T @ x, g["I_gap"], rtol=1e-8)


def test_component_mesh_and_loads_match_reference():
    """A 2-port S-parameter block across two open gaps (Layout.add_component):
    the mesh, the gap vectors and the block's impedance matrix in D."""
    import os

    from conftest import GOLDEN

    g = golden("component_line")
    lay, st, m, _ = workloads.build(G, "component_line", block=os.path.join(GOLDEN, "block.s2p"))
    assert digest(m) == str(g["mesh_sha"])
    np.testing.assert_array_equal(m.lumped_vectors(), g["Lm"])
    sol = host_solver(m)
    sol.components = list(m.layout.components)
    np.testing.assert_allclose(Solver.lumped_impedance(sol, float(g["freqs"][0])), g["D0"], rtol=1e-13)


def test_oracle_lumped_sweeps_match_reference():
    """The oracle's sweep with the loads (its fill, one solve for the port and
    gap excitations, Woodbury, de-embedding) against mom25d's S for the
    series R + L, a 1 pF override and an open gap, and a 2-port block across
    two gaps."""
    import os

    from conftest import GOLDEN

    cases = [("lumped_line", {}, [("S", None), ("C1p_S", {"Z1": "C 1p"}), ("open_S", {"Z1": None})]),
             ("component_line", {"block": os.path.join(GOLDEN, "block.s2p")}, [("S", None)])]
    for name, kw, variants in cases:
        g = golden(name)
        lay, st, m, _ = workloads.build(G, name, **kw)
        sw = O.Sweep(m, st)
        Lm = m.lumped_vectors()
        E0 = sw.excitations()
        P = E0.shape[1]
        got = {key: [] for key, _ in variants}
        for f in g["freqs"]:
            kern = sw.kernels(f)
            Z = sw.impedance(f, kern)
            X = O.dense_solve(Z.copy(), np.hstack([E0, Lm]))
            for key, values in variants:
                x = O.load_lumped(Lm, O.lumped_loads(m, f, values), X[:, :P], X[:, P:])
                q = O.charges(m, x, kern.omega)
                got[key].append(sw.deembed(f, kern, x, q)[0])
        for key, _ in variants:
            assert np.abs(np.array(got[key]) - g[key]).max() < 1e-6, (name, key)


def test_checkpoint_key_depends_on_the_lumped_values():
    """A checkpoint written under one set of lumped values is not resumed
    under another: the key's last field is a process-independent digest of
    the overrides, the layout's values and the multi-port blocks."""
    import subprocess
    import sys

    from mom25d_gb300 import workloads
    from mom25d_gb300.solver import checkpoint_key, values_digest

    lay, st, m, freqs = workloads.build(G, "lumped_line")
    lumped = list(m.layout.lumped)
    k0 = checkpoint_key(m, freqs, values_digest({}, lumped))
    k1 = checkpoint_key(m, freqs, values_digest({"Z1": "C 1p"}, lumped))
    k2 = checkpoint_key(m, freqs, values_digest({"Z1": None}, lumped))
    k1b = checkpoint_key(m, freqs, values_digest({"Z1": "C 1p"}, lumped))
    assert not np.allclose(k0, k1, rtol=1e-12, atol=0)
    assert not np.allclose(k1, k2, rtol=1e-12, atol=0)
    assert not np.allclose(k0, k2, rtol=1e-12, atol=0)
    np.testing.assert_array_equal(k1, k1b)
    # the same digest in a fresh interpreter (string hashing is salted per process)
    code = ("from mom25d_gb300 import workloads; import mom25d_gb300 as G; "
            "from mom25d_gb300.solver import values_digest; "
            "lay, st, m, f = workloads.build(G, 'lumped_line'); "
            "print(repr(values_digest({'Z1': 'C 1p'}, list(m.layout.lumped))))")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True,
                         cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    assert float(out.stdout.strip()) == k1[-1]
