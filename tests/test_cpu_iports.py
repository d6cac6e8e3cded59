"""Internal S-parameter ports (Layout.add_gap_port / add_via_port) on the CPU:
the mesh, the ports' delta-gap vectors, the load matrix and the host-side
reference-impedance algebra against mom25d's own run of the gap-port and
via-port lines (tests/golden/*_port_line.npz, make_golden.py --iports)."""

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import workloads
from mom25d_gb300.solver import anchor_z0, reciprocal_z0

from conftest import golden
from test_cpu_mesh_oracle import mesh_digest

CASES = ["gap_port_line", "via_port_line"]


@pytest.mark.parametrize("name", CASES)
def test_internal_port_mesh_and_vectors_match_reference(name):
    g = golden(name)
    lay, st, m, _ = workloads.build(G, name)
    m.assign_levels(sorted(m.layer_names, key=st.to_stackup().level_z))
    assert m.n_unknowns == int(g["N"])
    assert mesh_digest(m) == str(g["mesh_sha"])
    np.testing.assert_array_equal(m.internal_port_vectors(), g["iport_vectors"])


@pytest.mark.parametrize("name", CASES)
def test_reference_impedances_of_internal_ports(name):
    """From mom25d's S, z0 and line impedances: SI = D^-1 S D; the feeds'
    reciprocity fit followed by the anchoring to the internal ports' exact
    z_ref gives mom25d's z0 (the same algebra as mom25d's sweep)."""
    g = golden(name)
    lay, st, m, _ = workloads.build(G, name)
    P = len(lay.ports)
    zi = np.array([ip["z_ref"] for ip in lay.internal_ports])
    groups = [[0, 1]]  # the two feeds share a line (same width and level)
    for fi in range(len(g["freqs"])):
        d = np.sqrt(g["z0"][fi])
        SI = g["S"][fi] * d[None, :] / d[:, None]
        zf = reciprocal_z0(SI[:P, :P], g["z0_line"][fi, :P].real, groups)
        z = anchor_z0(SI, zf, zi, groups)
        np.testing.assert_allclose(z, g["z0"][fi, :P], rtol=1e-12)
        np.testing.assert_array_equal(g["z0"][fi, P:], zi)


def test_reciprocal_z0_of_uncoupled_groups_keeps_the_potential_estimate():
    """Groups that do not couple keep their scalar-potential estimates; one
    group keeps them as they are."""
    SI = np.eye(3, dtype=complex)
    z = reciprocal_z0(SI, np.array([48.0, 52.0, 75.0]), [[0, 1], [2]])
    np.testing.assert_allclose(z[2] / z[0], 75.0 / 50.0, rtol=1e-9)
    np.testing.assert_array_equal(reciprocal_z0(SI, np.array([48.0, 52.0, 75.0]), [[0, 1, 2]]), [48.0, 52.0, 75.0])
