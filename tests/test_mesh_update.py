"""Incremental update after host topology changes (sprg_update_mesh): a
context updated from mesh A to mesh B gives bitwise the results of a fresh
context on B, in every form, for moved vertices, grown and shrunk meshes;
bad deltas are refused before anything changes."""
import numpy as np
import pytest


def moved(m, frac, seed):
    """A copy of m with a fraction of its interior vertices moved."""
    from core_gb300.mesh import Mesh
    rng = np.random.Generator(np.random.PCG64(seed))
    x = m.coords.copy()
    inner = np.nonzero(~np.isin(np.arange(m.n_verts), m.boundary_vertices()))[0]
    pick = rng.choice(inner, size=max(1, int(frac * len(inner))), replace=False)
    h = 1.0 / 8
    x[pick, :m.dim] += rng.uniform(-0.1 * h, 0.1 * h, size=(len(pick), m.dim))
    return Mesh(m.dim, x, m.elem_verts.copy(), m.edge_verts.copy())


def apply_delta(old, d, counts):
    """numpy restatement of the update rule: kept rows, listed rows, truncation."""
    out = []
    for a, ids, vals, n in ((old.coords, d["vert_ids"], d["coords"], counts[0]),
                            (old.elem_verts, d["elem_ids"], d["elem_verts"], counts[1]),
                            (old.edge_verts, d["edge_ids"], d["edge_verts"], counts[2])):
        b = np.zeros((n,) + a.shape[1:], a.dtype)
        k = min(n, a.shape[0])
        b[:k] = a[:k]
        b[ids] = vals
        out.append(b)
    return out


@pytest.mark.parametrize("na,nb", [(5, 5), (4, 6), (6, 4)])
def test_delta_rows_reproduce_the_new_mesh(na, nb):
    from core_gb300 import mesh_delta, workload
    a = workload.box(na, jitter=0.2, seed=1)
    b = workload.box(nb, jitter=0.2, seed=2) if na != nb else moved(a, 0.3, 3)
    d = mesh_delta(a, b)
    x, ev, ed = apply_delta(a, d, (b.n_verts, b.n_elems, b.n_edges))
    assert np.array_equal(x, b.coords) and np.array_equal(ev, b.elem_verts) and np.array_equal(ed, b.edge_verts)
    if na == nb:
        assert 0 < len(d["vert_ids"]) < b.n_verts and len(d["elem_ids"]) == 0 and len(d["edge_ids"]) == 0


# ---------------------------------------------------------------------------
def results(ctx, m, u, precision):
    ctx.set_precision(precision)
    size, flags, ns, nc, info = ctx.estimate_and_mark(u, 0.05)
    return size, flags, ns, nc


def check_same(a, b):
    assert np.array_equal(a[0], b[0], equal_nan=True)
    assert np.array_equal(a[1], b[1]) and a[2:] == b[2:]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32", "learned"])
def test_updated_context_equals_fresh(gpu_lib, precision):
    import core_gb300 as cg
    from core_gb300 import workload
    a = workload.box(10, jitter=0.2, seed=4)
    steps = [moved(a, 0.2, 5), workload.box(12, jitter=0.2, seed=6), workload.box(9, jitter=0.2, seed=7)]
    with cg.Context(a) as ctx:
        results(ctx, a, workload.bump_field(a.coords, seed=4), precision)  # per-mesh state of A
        for b in steps:
            u = workload.bump_field(b.coords, seed=4)
            ctx.update_mesh(b)
            got = results(ctx, b, u, precision)
            with cg.Context(b) as fresh:
                want = results(fresh, b, u, precision)
            check_same(got, want)
            assert got[2] + got[3] > 0


@pytest.mark.gpu
def test_updated_triangle_context_mixed_aniso(gpu_lib):
    """The mixed anisotropic pass rebuilds its per-mesh operator after an update."""
    import torch
    import core_gb300 as cg
    from core_gb300 import workload
    a, u_a, (eps, hmin, hmax) = workload.aniso2d(40)
    b, u_b, _ = workload.aniso2d(48)

    def run(ctx, m, u):
        nw = (m.n_edges + 31) // 32
        bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
        d_u = torch.from_numpy(u).cuda()
        ctx.aniso_estimate_and_mark_resident(d_u.data_ptr(), eps, hmin, hmax, bits.data_ptr(),
                                             bits.data_ptr() + 4 * nw)
        torch.cuda.synchronize()
        return bits.cpu().numpy()
    with cg.Context(a, precision="fp32") as ctx:
        run(ctx, a, u_a)
        ctx.update_mesh(b)
        got = run(ctx, b, u_b)
    with cg.Context(b, precision="fp32") as fresh:
        want = run(fresh, b, u_b)
    assert np.array_equal(got, want) and got.any()


@pytest.mark.gpu
def test_bad_deltas_are_refused_and_leave_the_context(gpu_lib):
    import ctypes
    import core_gb300 as cg
    from core_gb300 import _lib as K, workload
    a = workload.box(6, jitter=0.2, seed=8)
    u = workload.bump_field(a.coords, seed=8)
    with cg.Context(a) as ctx:
        before = results(ctx, a, u, "fp64")

        def refuse(**kw):
            f = dict(n_verts=a.n_verts, n_elems=a.n_elems, n_edges=a.n_edges)
            f.update(kw)
            d = K.MeshDelta(**f)
            rc = ctx._lib.sprg_update_mesh(ctx.h, ctypes.byref(d))
            assert rc == K.SPRG_EINVAL
        # a new vertex row that is not listed
        refuse(n_verts=a.n_verts + 1)
        # an element naming a vertex beyond the count
        ids = np.array([0], np.int32)
        ev = np.array([[0, 1, 2, a.n_verts]], np.int32)
        refuse(n_elem_rows=1, elem_ids=ids.ctypes.data, elem_verts=ev.ctypes.data)
        # kept elements naming vertices beyond a shrunk count
        refuse(n_verts=a.n_verts - 5)
        # row ids out of range
        bad = np.array([a.n_edges], np.int32)
        e2 = np.array([[0, 1]], np.int32)
        refuse(n_edge_rows=1, edge_ids=bad.ctypes.data, edge_verts=e2.ctypes.data)
        check_same(results(ctx, a, u, "fp64"), before)
