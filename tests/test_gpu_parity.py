"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances (FP64 mode):
  * element/edge arithmetic that follows the reference's operation order
    (integration-point gradients, metric edge lengths, qualities given the
    same size field) must be bitwise equal;
  * recovered fields, size fields: max |gpu - oracle| <= 1e-10 * max |oracle|
    per component (the patch QR and the two global sums use a different
    reduction order, which moves results by a few ulps);
  * split/collapse marks: identical on every edge.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


def relerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim == 1:
        a = a[:, None]
        b = b[:, None]
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return float((np.abs(a - b).max(axis=0) / scale).max())


def make_pair(oracle_mod, n, nz=None, jitter=0.0, seed=0, mds_order=True):
    from core_gb300 import workload
    nz = n if nz is None else nz
    m = workload.box(n, nz=nz, jitter=jitter, seed=seed)
    o = oracle_mod.OracleMesh.box(n, n, nz)
    o.set_coords(m.coords)
    if mds_order:
        m.v2e_off = o.v2e_off
        m.v2e = o.v2e
    return m, o


CASES = [
    ("box8", 8, None, 0.0),
    ("jbox10", 10, None, 0.2),
    ("jbox6x", 6, 3, 0.2),
    ("tri16", 16, 0, 0.0),
    ("jtri20", 20, 0, 0.15),
]


def field_for(m, name):
    from core_gb300 import workload
    if name == "box8":
        return workload.sine_field(m.coords)
    return workload.bump_field(m.coords, seed=5 if m.dim == 2 else 2)


@pytest.mark.parametrize("name,n,nz,jit", CASES)
def test_estimate_chain_fp64(gpu_lib, oracle_lib, name, n, nz, jit):
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, n, nz, jit, seed=3)
    u = field_for(m, name)
    with cg.Context(m) as ctx:
        ip = ctx.getGradIPField(u)
        ip_o = o.grad_ip(u)
        assert np.array_equal(ip, ip_o), "integration-point gradients must be bitwise equal"
        rec = ctx.recoverField(ip)
        rc, rec_o, nexp, fail = o.recover(ip_o)
        assert rc == 0
        assert relerr(rec, rec_o) <= TOL
        size, info = ctx.getSPRSizeField(ip, 0.1)
        rc, size_o, _, esize_o, err_o, info_o = o.size_field(ip_o, 0.1)
        assert rc == 0
        assert relerr(size, size_o) <= TOL
        assert info["n_expanded"] == info_o["n_expanded"]
        assert abs(info["size_factor"] - info_o["size_factor"]) <= TOL * abs(info_o["size_factor"])
        # ma measure / quality given the oracle's size field: bitwise
        L = ctx.measure_edges(size_o)
        L_o = o.measure(size_o)
        assert np.array_equal(L, L_o)
        q = ctx.measureQuality(size_o)
        assert np.array_equal(q, o.quality(size_o))


@pytest.mark.parametrize("name,n,nz,jit", CASES)
def test_marks_identical(gpu_lib, oracle_lib, name, n, nz, jit):
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, n, nz, jit, seed=4)
    u = field_for(m, name)
    rc, size_o, L_o, flags_o, ns_o, nc_o, _ = o.estimate_and_mark(u, 0.1)
    assert rc == 0
    with cg.Context(m) as ctx:
        size, flags, ns, nc, info = ctx.estimate_and_mark(u, 0.1)
    near = np.sum((np.abs(L_o - 1.5) < 1e-9) | (np.abs(L_o - 0.5) < 1e-9))
    assert near == 0, "near-tie edges present; marks could legitimately differ"
    assert np.array_equal(flags, flags_o)
    assert (ns, nc) == (ns_o, nc_o)
    assert relerr(size, size_o) <= TOL


def test_ascending_adjacency_order(gpu_lib, oracle_lib):
    """Without the caller's getAdjacent order the vertex average sums in
    ascending element order: sizes within tolerance, marks identical."""
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, 9, None, 0.2, seed=8, mds_order=False)
    u = field_for(m, "jbox")
    rc, size_o, L_o, flags_o, *_ = o.estimate_and_mark(u, 0.1)
    with cg.Context(m) as ctx:
        size, flags, *_ = ctx.estimate_and_mark(u, 0.1)
    assert relerr(size, size_o) <= TOL
    assert np.array_equal(flags, flags_o)


def test_target_size_field(gpu_lib, oracle_lib):
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, 8, None, 0.2, seed=9)
    u = field_for(m, "jbox")
    ip = o.grad_ip(u)
    with cg.Context(m) as ctx:
        for target, a, b in [(5000, 0.25, 2.0), (100, 0.5, 1.5), (10 ** 6, 0.25, 2.0)]:
            size, info = ctx.getTargetSPRSizeField(ip, target, a, b)
            rc, size_o, *_ = o.size_field(ip, target=target, alpha=a, beta=b)
            assert rc == 0
            assert relerr(size, size_o) <= TOL


def test_vector_field_matrix_ip(gpu_lib, oracle_lib):
    """getGradIPField of a VECTOR field gives a MATRIX (9-component) ip field."""
    import core_gb300 as cg
    for n, nz in [(7, None), (12, 0)]:
        m, o = make_pair(oracle_lib, n, nz, 0.2, seed=10)
        x = m.coords
        f = np.stack([np.sin(3 * x[:, 0]) * x[:, 1], np.cos(2 * x[:, 1]) + x[:, 2] ** 2,
                      x[:, 0] * x[:, 1] * x[:, 2] + np.exp(x[:, 0])], axis=1)
        with cg.Context(m) as ctx:
            ip = ctx.getGradIPField(f)
            ip_o = o.grad_ip(f)
            assert ip.shape[1] == 9 and np.array_equal(ip, ip_o)
            rec = ctx.recoverField(ip)
            rc, rec_o, *_ = o.recover(ip_o)
            assert rc == 0 and relerr(rec, rec_o) <= TOL


@pytest.mark.parametrize("n,jit,vector", [(16, 0.0, False), (20, 0.15, False), (12, 0.2, True)])
def test_triangle_recovery_bitwise(gpu_lib, oracle_lib, n, jit, vector):
    """On triangles the thread-per-vertex QR follows the reference's operation
    order (explicit Q, ascending sums): every patch that needs no growth
    recovers bitwise the oracle's values, for 3- and 9-component fields."""
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, n, 0, jit, seed=6)
    x = m.coords
    if vector:
        f = np.stack([np.sin(3 * x[:, 0]) * x[:, 1], np.cos(2 * x[:, 1]), np.exp(x[:, 0]) * x[:, 1]], axis=1)
    else:
        f = workload_field(m)
    with cg.Context(m) as ctx:
        ip = ctx.getGradIPField(f)
        rec = ctx.recoverField(ip)
    rc, rec_o, nexp, _ = o.recover(o.grad_ip(f))
    assert rc == 0
    exact = np.all(rec == rec_o, axis=1)
    assert exact.sum() >= m.n_verts - nexp
    assert relerr(rec, rec_o) <= TOL


def workload_field(m):
    from core_gb300 import workload
    return workload.bump_field(m.coords, seed=5)


def random_frames(V, seed, dim):
    rng = np.random.Generator(np.random.PCG64(seed))
    F = np.empty((V, 9))
    for v in range(V):
        if dim == 3:
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        else:
            t = rng.uniform(0, np.pi)
            q = np.array([[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1.0]])
        F[v] = q.reshape(9)
    sizes = np.exp(rng.uniform(np.log(0.01), np.log(0.3), size=(V, 3)))
    return sizes, F


@pytest.mark.parametrize("n,nz", [(6, None), (14, 0)])
def test_aniso_measure_quality_bitwise(gpu_lib, oracle_lib, n, nz):
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, n, nz, 0.15, seed=12)
    sizes, frames = random_frames(m.n_verts, 13, m.dim)
    with cg.Context(m) as ctx:
        L = ctx.measure_edges_aniso(sizes, frames)
        assert np.array_equal(L, o.measure(sizes=sizes, frames=frames))
        q = ctx.measureQuality(sizes=sizes, frames=frames)
        assert np.array_equal(q, o.quality(sizes=sizes, frames=frames))


def test_mark_semantics_and_errors(gpu_lib, oracle_lib):
    import core_gb300 as cg
    from core_gb300 import _lib as K
    m, o = make_pair(oracle_lib, 8, None, 0.2, seed=14)
    u = field_for(m, "jbox")
    rng = np.random.Generator(np.random.PCG64(15))
    with cg.Context(m) as ctx:
        ip = ctx.getGradIPField(u)
        size, _ = ctx.getSPRSizeField(ip, 0.3)
        L = ctx.measure_edges(size)
        pre = rng.choice(np.array([0, K.DONT_SPLIT, K.DONT_COLLAPSE, K.NEED_NOT_SPLIT, K.NEED_NOT_COLLAPSE, 1 << 9],
                                  np.int32), size=m.n_edges)
        for which in (K.MARK_COLLAPSE, K.MARK_SPLIT):
            f_gpu = pre.copy()
            f_cpu = pre.copy()
            n_gpu = ctx._mark(which, f_gpu)
            rc, n_cpu = oracle_lib.mark_edges(L, which, f_cpu)
            assert rc == 0 and n_gpu == n_cpu and np.array_equal(f_gpu, f_cpu)
        bad = pre.copy()
        bad[5] |= K.SPLIT  # markEntities asserts the true flag is clear
        with pytest.raises(cg.SprgError) as e:
            ctx.markEdgesToSplit(bad)
        assert e.value.code == K.SPRG_EFLAGS


def test_patch_failure_reports_epatch(gpu_lib, oracle_lib):
    """A single tet: the vertex patch cannot grow ("all hope is lost")."""
    import core_gb300 as cg
    from core_gb300 import _lib as K
    from core_gb300.mesh import Mesh
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    ev = np.array([[0, 1, 2, 3]], np.int32)
    ed = np.array([[0, 1], [1, 2], [2, 0], [0, 3], [1, 3], [2, 3]], np.int32)
    m = Mesh(3, xyz, ev, ed)
    with cg.Context(m) as ctx:
        ip = ctx.getGradIPField(xyz[:, 0] + 2 * xyz[:, 1])
        with pytest.raises(cg.SprgError) as e:
            ctx.recoverField(ip)
        assert e.value.code == K.SPRG_EPATCH
        # the context stays usable after the error
        ip2 = ctx.getGradIPField(xyz[:, 2])
        assert np.allclose(ip2, [[0, 0, 1]])


def test_linear_field_patch_test(gpu_lib):
    """SPR reproduces the gradient of a linear field exactly (patch test)."""
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(9, jitter=0.2, seed=16)
    g = np.array([0.3, -1.7, 2.2])
    u = m.coords @ g + 0.5
    with cg.Context(m) as ctx:
        ip = ctx.getGradIPField(u)
        assert np.abs(ip - g).max() < 1e-10
        rec = ctx.recoverField(ip)
        assert np.abs(rec - g).max() < 1e-9


def test_resident_bitmaps_and_determinism(gpu_lib, oracle_lib):
    import torch
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, 11, None, 0.2, seed=17)
    u = field_for(m, "jbox")
    rc, size_o, L_o, flags_o, *_ = o.estimate_and_mark(u, 0.1)
    E = m.n_edges
    nw = (E + 31) // 32
    d_u = torch.from_numpy(u).cuda()
    bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
    with cg.Context(m) as ctx:
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        ctx.set_stream(stream.cuda_stream)
        outs = []
        for _ in range(2):
            bits.zero_()
            ctx.estimate_and_mark_resident(d_u.data_ptr(), 0.1, bits.data_ptr(), bits.data_ptr() + 4 * nw)
            torch.cuda.synchronize()
            outs.append(bits.cpu().numpy().view(np.uint32).copy())
        assert ctx.last_launch_count > 0
    assert np.array_equal(outs[0], outs[1])
    b = outs[0]
    split = ((b[:nw][np.arange(E) >> 5] >> (np.arange(E) & 31)) & 1).astype(bool)
    coll = ((b[nw:][np.arange(E) >> 5] >> (np.arange(E) & 31)) & 1).astype(bool)
    assert np.array_equal(split, L_o > 1.5)
    assert np.array_equal(coll, L_o < 0.5)
    # host write-back reproduces markEntities
    flags = np.zeros(E, np.int32)
    cg.apply_marks(b[:nw], b[nw:], flags)
    assert np.array_equal(flags, flags_o)
