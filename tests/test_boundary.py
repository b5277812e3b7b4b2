"""The C-ABI boundary and the host flattener (CPU only, no compute calls).

* libsprgb300.so loads and exports every function include/spr_gb300.h declares;
* the flattened apf::makeMdsBox numbering (coordinates, element vertices in
  getDownward order, edge vertices) is bitwise the numbering of the oracle's
  MDS-semantics builder, which replays BoxBuilder + apf::buildElement +
  mds find-or-create (mds/apfBox.cc, apf/apfMesh2.cc, mds/mds.c);
* entity counts follow the box formulas.
"""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "spr_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sprg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from core_gb300 import build
    build.build()
    import core_gb300
    return core_gb300.load()


def test_library_exports_every_declared_symbol(lib):
    import ctypes
    names = declared_symbols()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
        assert isinstance(getattr(lib, n), ctypes._CFuncPtr)
    from core_gb300 import _lib
    assert sorted(_lib.EXPORTS) == names


@pytest.mark.parametrize("shape", [(8, 8, 8), (3, 5, 2), (1, 1, 1), (7, 2, 5), (4, 3, 0), (16, 16, 0), (1, 9, 0)])
def test_box_numbering_matches_mds(lib, oracle_lib, shape):
    import core_gb300 as cg
    nx, ny, nz = shape
    m = cg.makeMdsBox(nx, ny, nz, 1.0, 2.0, 0.5)
    o = oracle_lib.OracleMesh.box(nx, ny, nz, 1.0, 2.0, 0.5)
    assert (m.n_verts, m.n_elems, m.n_edges) == (o.V, o.T, o.E)
    assert np.array_equal(m.coords, o.coords)
    assert np.array_equal(m.elem_verts, o.elem_verts)
    assert np.array_equal(m.edge_verts, o.edge_verts)


def test_box_counts_formulas(lib):
    import core_gb300 as cg
    for n in (8, 128, 160):
        V, T, E = cg.box_counts(n, n, n)
        assert V == (n + 1) ** 3 and T == 6 * n ** 3
        assert E == 3 * n * (n + 1) ** 2 + 3 * n ** 2 * (n + 1) + n ** 3
    assert cg.box_counts(160, 160, 160) == (4173281, 24576000, 28902880)
    assert cg.box_counts(4096, 4096, 0) == (16785409, 33554432, 50339840)


def test_oracle_adjacency_is_mds_get_up_order(oracle_lib):
    """getAdjacent(v, 3) on the 1^3 box: union over v's edges (newest
    first), their faces (newest first), then tets, as mds get_up does."""
    o = oracle_lib.OracleMesh.box(1, 1, 1)
    off, adj = o.v2e_off, o.v2e
    # the ends of the cube diagonal (grid vertices 0 and 7) touch all six Kuhn tets
    assert off[1] - off[0] == 6 and off[8] - off[7] == 6
    for v in range(8):
        s = adj[off[v]:off[v + 1]]
        assert len(set(s.tolist())) == len(s)
        ev = o.elem_verts
        assert set(s.tolist()) == {t for t in range(6) if v in ev[t]}
