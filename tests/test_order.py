"""Locality renumbering of flattened meshes (sprg_locality_order, host-only;
core_gb300.mesh.reorder), the flat-array counterpart of apf::reorderMdsMesh
(mds/mds_order.c:127-176): breadth-first vertex numbering, then elements and
edges in the order the renumbered vertices reach them."""
import numpy as np
import pytest

from refcases import shuffled_box


@pytest.fixture(scope="module")
def lib():
    from core_gb300 import build
    build.build()
    import core_gb300
    return core_gb300.load()


def shuffled_mesh(oracle_lib, n, seed):
    from core_gb300.mesh import Mesh
    c, e, f, t = shuffled_box(oracle_lib, n, seed)
    o = oracle_lib.OracleMesh.from_down(3, c, e, f, t)
    return Mesh(3, o.coords.copy(), o.elem_verts, o.edge_verts, v2e_off=o.v2e_off, v2e=o.v2e)


def edge_span(m):
    return float(np.mean(np.abs(m.edge_verts[:, 0].astype(np.int64) - m.edge_verts[:, 1])))


@pytest.mark.parametrize("n,seed", [(5, 1), (9, 2)])
def test_renumbering_is_a_permutation_with_local_rows(lib, oracle_lib, n, seed):
    from core_gb300.mesh import reorder
    m = shuffled_mesh(oracle_lib, n, seed)
    m2, vn, tn, en = reorder(m)
    for p, k in ((vn, m.n_verts), (tn, m.n_elems), (en, m.n_edges)):
        assert np.array_equal(np.sort(p), np.arange(k))
    # rows moved, ids mapped, each element's and edge's vertex order kept
    assert np.array_equal(m2.coords[vn], m.coords)
    assert np.array_equal(m2.elem_verts[tn], vn[m.elem_verts])
    assert np.array_equal(m2.edge_verts[en], vn[m.edge_verts])
    # the averaging adjacency keeps each vertex's element order
    for v in range(0, m.n_verts, 7):
        a = m.v2e[m.v2e_off[v]:m.v2e_off[v + 1]]
        b = m2.v2e[m2.v2e_off[vn[v]]:m2.v2e_off[vn[v] + 1]]
        assert np.array_equal(b, tn[a])
    assert edge_span(m2) < 0.3 * edge_span(m)


def test_breadth_first_vertex_order(lib, oracle_lib):
    """Every vertex but the seed has a neighbour numbered before it, and the
    numbering visits whole breadth-first layers in order."""
    from core_gb300.mesh import reorder
    m = shuffled_mesh(oracle_lib, 6, 3)
    m2, vn, _, _ = reorder(m)
    V = m2.n_verts
    nb = [[] for _ in range(V)]
    for a, b in m2.edge_verts:
        nb[a].append(b)
        nb[b].append(a)
    depth = np.full(V, -1)
    depth[0] = 0
    for v in range(V):  # BFS numbering: vertex v's depth is known before it is reached
        assert depth[v] >= 0
        for w in nb[v]:
            if depth[w] < 0:
                depth[w] = depth[v] + 1
    assert np.all(np.diff(depth) >= 0)
    assert min(len(x) for x in nb) == len(nb[0])  # the seed has the smallest degree


def test_renumbering_is_deterministic_and_refuses_bad_views(lib, oracle_lib):
    import ctypes
    from core_gb300 import _lib
    from core_gb300.mesh import locality_order
    m = shuffled_mesh(oracle_lib, 4, 5)
    a = locality_order(m)
    b = locality_order(m)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    v = m.view()
    out = [np.empty(k, np.int32) for k in (m.n_verts, m.n_elems, m.n_edges)]
    bad = m.elem_verts.copy()
    bad[3, 1] = m.n_verts
    v.elem_verts = bad.ctypes.data
    assert lib.sprg_locality_order(ctypes.byref(v), *(o.ctypes.data for o in out)) == _lib.SPRG_EINVAL
    assert lib.sprg_locality_order(None, *(o.ctypes.data for o in out)) == _lib.SPRG_EINVAL
