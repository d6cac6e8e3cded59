"""CPU tests of the C ABI and the host-side preparation (no GPU calls)."""

import ctypes as C
import os
import re

import numpy as np
import pytest

import mom25d_gb300 as G
from mom25d_gb300 import engine, workloads
from mom25d_gb300 import solver as S
from oracle import kernels as K
from oracle import sweep as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "m25.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(m25_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = engine.load()
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(engine.EXPORTS)
    assert lib.m25_version() == 1


def test_struct_layouts_match_header():
    # the ctypes mirrors follow the C structs field by field
    txt = open(os.path.join(ROOT, "include", "m25.h")).read()
    for cls, name in ((engine.MeshDesc, "m25_mesh_desc"), (engine.GreensDesc, "m25_greens_desc"),
                      (engine.PortDesc, "m25_port_desc"), (engine.HmatDesc, "m25_hmat_desc")):
        body = re.search(r"typedef struct \{([^}]*)\}\s*" + name, txt, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            names = decl.split(None, 1)[1] if not decl.startswith("const") else decl.split(None, 2)[2]
            fields += [n.strip().lstrip("*").strip() for n in names.split(",")]
        assert [f[0] for f in cls._fields_] == fields, name


def test_no_device_is_an_error_not_a_crash():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises((RuntimeError, ValueError)):
        engine.Context(0)


def test_morton_blocks_equal_oracle_blocks():
    for name in ("tee", "via"):
        lay, st, m, _ = workloads.build(G, name)
        stack = st if hasattr(st, "layers") else st.to_stackup()
        zl = np.array([stack.level_z(n) for n in m.layer_names])
        blocks = S.test_blocks(m)
        geo = O.Geometry(m, zl)
        ref = [pb for _, pb, _, _ in geo.blocks]
        assert len(ref) == blocks.shape[0]
        for row, pb in zip(blocks, ref):
            np.testing.assert_array_equal(row[:pb.size], pb)
            assert np.all(row[pb.size:] == -1)


def test_path_and_radii_equal_oracle():
    for f in (0.5e9, 7e9, 20e9):
        k0 = 2 * np.pi * f / K.C0
        k1 = abs(k0 * np.sqrt(3.55 * (1 - 0.0027j)))
        a = S.sommerfeld_path(k0, k1, 0.508e-3, 0.04)
        b = K.lifted_path(k0, k1, 0.508e-3, 0.04)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(S.tabulation_radii(0.04, 2 * np.pi / k1, 0.508e-3),
                                      K.rho_grid(0.04, 2 * np.pi / k1, 0.508e-3))


def test_port_models_equal_oracle():
    lay, st, m, _ = workloads.build(G, "tee")
    for p in lay.ports:
        a = S.PortModel(m, p, 0.508e-3)
        b = O.PortData(m, p, 0.508e-3)
        np.testing.assert_array_equal(a.s, b.s)
        np.testing.assert_array_equal(a.vpts, b.vpts)
        np.testing.assert_array_equal(a.excitation, b.excitation)
        for (i1, s1), (i2, s2) in zip(a.cuts, b.cuts):
            np.testing.assert_array_equal(i1, i2)
            np.testing.assert_array_equal(s1, s2)


def test_short_feed_raises_value_error():
    lay = G.Layout()
    W = 1.137e-3
    lay.add_rect(0, -W / 2, 2e-3, W / 2)
    lay.add_port("P1", (0, 0), "-x", W, 3e-3)
    m = lay.mesh(0.5e-3, 0.1e-3)
    with pytest.raises(ValueError):
        S.PortModel(m, lay.ports[0], 0.508e-3)


def test_layout_rejects_unsupported_features():
    with pytest.raises(ValueError):
        G.Port("P", (0, 0), "+z", 1e-3, 1e-3)
    with pytest.raises(ValueError):
        G.Stackup([G.Dielectric(1e-3, 3.0)], top="pec")
    with pytest.raises(ValueError):
        G.Via((0, 0), 0.3e-3, pad=0.1e-3)
