"""The 2D anisotropic workload: nodal Hessian by two SPR recoveries, the
metric from it, AnisoSizeField measure, marks and triangle quality.

Parity (FP64 path against the oracle, on a jittered square with the
boundary-layer field): Hessian within 1e-10 relative of its largest entry;
the metric kernel on the same Hessian equal to the numpy restatement to
1e-14 (2D closed form) and 1e-12 (3D Jacobi); metric edge lengths within
1e-12 and identical split/collapse marks; qualities within 1e-12.
"""
import numpy as np
import pytest

from oracle import aniso_oracle as ao


def test_metric_restatement_diagonal():
    H = np.zeros((3, 9))
    H[0, 0], H[0, 4] = 4.0, -1.0      # |lambda| ordered: x first
    H[1, 0], H[1, 4] = 1.0, 9.0       # y first
    H[2, 0], H[2, 4] = 0.0, 0.0       # flat: h_max
    s, f = ao.metric_2d(H, eps=1.0, hmin=0.01, hmax=10.0)
    assert np.allclose(s[0], [0.5, 1.0, 10.0]) and np.allclose(f[0], np.eye(3).ravel())
    assert np.allclose(s[1], [1.0 / 3, 1.0, 10.0]) and np.allclose(f[1], [0, -1, 0, 1, 0, 0, 0, 0, 1])
    assert np.allclose(s[2], [10.0, 10.0, 10.0])


def test_metric_restatement_3d_reconstructs():
    rng = np.random.Generator(np.random.PCG64(1))
    Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    lam = np.array([5.0, -2.0, 0.5])
    A = Q @ np.diag(lam) @ Q.T
    s, f = ao.metric_3d(A.reshape(1, 9), eps=1.0, hmin=1e-3, hmax=1e3)
    R = f.reshape(3, 3)
    assert np.allclose(R.T @ R, np.eye(3), atol=1e-12)
    assert np.allclose(s[0], np.sqrt(1.0 / np.abs(lam)))
    assert np.allclose(R @ np.diag([5.0, -2.0, 0.5]) @ R.T, A, atol=1e-12)


def test_metric_restatement_tiny_and_huge_hessians():
    """A Hessian scaled by a power of two has the same frames (the metric
    prescales it by a power of two before the eigen-decomposition): even at
    1e-160 scale, where the squares of its entries underflow, and at 1e+150."""
    rng = np.random.Generator(np.random.PCG64(3))
    H = np.zeros((50, 9))
    H[:, [0, 1, 3, 4]] = rng.normal(size=(50, 4))
    H[:, 3] = H[:, 1]
    _, f = ao.metric_2d(H, 1.0, 1e-3, 1e3)
    for k in (-560, -531, 498):
        s, fk = ao.metric_2d(np.ldexp(H, k), 1.0, 1e-3, 1e3)
        assert np.all(np.isfinite(fk)) and np.array_equal(fk, f)
    A = rng.normal(size=(20, 3, 3))
    A = (A + A.transpose(0, 2, 1)).reshape(20, 9)
    s3, f3 = ao.metric_3d(A, 1.0, 1e-3, 1e3)
    for k in (-560, 498):
        sk, fk = ao.metric_3d(np.ldexp(A, k), 1.0, 1e-3, 1e3)
        assert np.array_equal(fk, f3)


def case(n=48):
    from core_gb300 import workload
    return workload.aniso2d(n)


@pytest.mark.gpu
def test_hessian_and_metric_match_oracle(gpu_lib, oracle_lib):
    import core_gb300 as cg
    m, u, (eps, hmin, hmax) = case()
    om = oracle_lib.OracleMesh.box(48, 48, 0)
    om.set_coords(m.coords)
    H_ref = ao.hessian(om, u)
    with cg.Context(m) as c:
        g = c.recoverField(c.getGradIPField(u))
        H = c.recoverField(c.getGradIPField(g))
        sizes, frames = c.hessian_metric(H_ref, eps, hmin, hmax)
    assert np.abs(H - H_ref).max() <= 1e-10 * np.abs(H_ref).max()
    s_ref, f_ref = ao.metric_2d(H_ref, eps, hmin, hmax)
    assert np.abs(sizes - s_ref).max() <= 1e-14 * s_ref.max()
    assert np.abs(frames - f_ref).max() <= 1e-14


@pytest.mark.gpu
def test_metric_3d_matches_restatement(gpu_lib):
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(3)
    rng = np.random.Generator(np.random.PCG64(2))
    V = m.n_verts
    H = np.empty((V, 9))
    for v in range(V):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        lam = rng.choice([-1, 1], 3) * rng.uniform(0.1, 10, 3)
        H[v] = (Q @ np.diag(lam) @ Q.T).ravel()
    with cg.Context(m) as c:
        sizes, frames = c.hessian_metric(H, 0.5, 1e-3, 1e3)
    s_ref, f_ref = ao.metric_3d(H, 0.5, 1e-3, 1e3)
    assert np.abs(sizes - s_ref).max() <= 1e-12 * s_ref.max()
    assert np.abs(frames - f_ref).max() <= 1e-10


@pytest.mark.gpu
def test_aniso_pass_matches_oracle(gpu_lib, oracle_lib):
    import torch
    import core_gb300 as cg
    n = 48
    m, u, (eps, hmin, hmax) = case(n)
    om = oracle_lib.OracleMesh.box(n, n, 0)
    om.set_coords(m.coords)
    s_ref, f_ref = ao.metric_2d(ao.hessian(om, u), eps, hmin, hmax)
    L_ref = om.measure(sizes=s_ref, frames=f_ref)
    q_ref = om.quality(sizes=s_ref, frames=f_ref)
    E, T = m.n_edges, m.n_elems
    nw = (E + 31) // 32
    with cg.Context(m) as c:
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        c.set_stream(stream.cuda_stream)
        d_u = torch.from_numpy(u).cuda()
        bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
        q = torch.zeros(T, dtype=torch.float64, device="cuda")
        c.aniso_estimate_and_mark_resident(d_u.data_ptr(), eps, hmin, hmax, bits.data_ptr(),
                                           bits.data_ptr() + 4 * nw, q.data_ptr())
        torch.cuda.synchronize()
        L = c.debug_read("L", np.float64, E)
        b = bits.cpu().numpy().view(np.uint32)
        q = q.cpu().numpy()
    idx = np.arange(E)
    split = ((b[:nw][idx >> 5] >> (idx & 31)) & 1).astype(bool)
    coll = ((b[nw:][idx >> 5] >> (idx & 31)) & 1).astype(bool)
    assert np.abs(L - L_ref).max() <= 1e-12 * L_ref.max()
    near = (np.abs(L_ref - 1.5) < 1e-12) | (np.abs(L_ref - 0.5) < 1e-12)
    assert not near.any()
    assert np.array_equal(split, L_ref > 1.5) and np.array_equal(coll, L_ref < 0.5)
    assert split.any() and coll.any()
    assert np.abs(q - q_ref).max() <= 1e-12


def run_aniso(m, u, eps, hmin, hmax, precision):
    """Resident anisotropic pass; returns (split, collapse, quality, metric
    tensors R diag(1/h^2) R^T, nodal Hessians, guarded edges).  The FP64 pass
    keeps its FP64 metric; the mixed pass its FP32 metric records (on
    triangles it stores no FP64 metric)."""
    import torch
    import core_gb300 as cg
    E, T, V = m.n_edges, m.n_elems, m.n_verts
    nw = (E + 31) // 32
    with cg.Context(m) as c:
        c.set_precision(precision)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        c.set_stream(stream.cuda_stream)
        d_u = torch.from_numpy(u).cuda()
        bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
        q = torch.zeros(T, dtype=torch.float64, device="cuda")
        for _ in range(2):  # the second pass runs on the per-mesh caches
            c.aniso_estimate_and_mark_resident(d_u.data_ptr(), eps, hmin, hmax, bits.data_ptr(),
                                               bits.data_ptr() + 4 * nw, q.data_ptr())
        torch.cuda.synchronize()
        if precision == "fp32":
            rec = c.debug_read("met32", np.float32, 12 * V).reshape(V, 12).astype(np.float64)
            sizes, frames = rec[:, :3], rec[:, 3:]
            hess = c.debug_read("rec9" if m.dim == 2 else "rec", np.float64, 9 * V).reshape(V, 9)
        else:
            sizes = c.debug_read("sizes3", np.float64, 3 * V).reshape(V, 3)
            frames = c.debug_read("frames9", np.float64, 9 * V).reshape(V, 9)
            hess = c.debug_read("rec", np.float64, 9 * V).reshape(V, 9)
        guard = int(c.debug_read("agcount", np.int32, 1)[0]) if precision == "fp32" else 0
        b = bits.cpu().numpy().view(np.uint32)
        q = q.cpu().numpy()
    idx = np.arange(E)
    split = ((b[:nw][idx >> 5] >> (idx & 31)) & 1).astype(bool)
    coll = ((b[nw:][idx >> 5] >> (idx & 31)) & 1).astype(bool)
    R = frames.reshape(-1, 3, 3)
    tensors = np.einsum("vij,vj,vkj->vik", R, 1.0 / sizes ** 2, R)
    return split, coll, q, tensors, hess, guard


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_aniso_pass_matches_fp64(gpu_lib, dim):
    """SPRG_FP32 on the anisotropic pass: recoveries from cached FP64 patch
    weights (triangles), the metric's decisions in FP64, FP32 metric records,
    FP32 measure with the FP64 guard band, FP32 qualities.  Marks identical
    to the FP64 pass, the Hessians within 1e-9 relative (the weights sum the
    patch in another order than the QR), the FP32 metric tensors within 1e-5
    relative of the FP64 ones (frames alone rotate freely where two sizes
    coincide, so tensors are compared), qualities within 1e-4 relative."""
    from core_gb300 import workload
    if dim == 2:
        m, u, (eps, hmin, hmax) = case(96)
    else:
        m = workload.box(12, jitter=0.2, seed=5)
        u = np.tanh((m.coords[:, 1] - 0.5) / 0.05) + 0.1 * np.sin(4 * np.pi * m.coords[:, 0])
        eps, hmin, hmax = 0.02, 1.0 / 48, 0.5
    s64, c64, q64, M64, H64, _ = run_aniso(m, u, eps, hmin, hmax, "fp64")
    s32, c32, q32, M32, H32, guard = run_aniso(m, u, eps, hmin, hmax, "fp32")
    assert np.array_equal(s32, s64) and np.array_equal(c32, c64)
    assert s64.any() and c64.any()
    # symmetric parts (the metric's input; the mixed operator stores the
    # Hessian transposed)
    def sym(H):
        H = H.reshape(-1, 3, 3)
        return 0.5 * (H + H.transpose(0, 2, 1))
    S64, S32 = sym(H64), sym(H32)
    hs = np.abs(S64).reshape(len(S64), -1).max(axis=1)
    ok = hs > 0
    assert (np.abs(S32 - S64).reshape(len(S64), -1).max(axis=1)[ok] / hs[ok]).max() <= 1e-9
    scale = np.abs(M64).reshape(len(M64), -1).max(axis=1)
    assert (np.abs(M32 - M64).reshape(len(M64), -1).max(axis=1) / scale).max() <= 1e-5
    assert np.abs(q32 - q64).max() <= 1e-4 * np.abs(q64).max()
    assert np.median(np.abs(q32 - q64) / np.abs(q64)) <= 1e-6
    assert guard < 0.01 * m.n_edges


@pytest.mark.gpu
def test_metric_on_tiny_hessians_matches_restatement(gpu_lib):
    """The device metric (FP64 function and the mixed pass's records) on
    Hessians at 1e-160 and 1e-170 scale: finite frames, those of the
    restatement (whose power-of-two prescaling it shares)."""
    import core_gb300 as cg
    m, u, (eps, hmin, hmax) = case(8)
    rng = np.random.Generator(np.random.PCG64(5))
    H = np.zeros((m.n_verts, 9))
    H[:, [0, 1, 4]] = rng.normal(size=(m.n_verts, 3))
    H[:, 3] = H[:, 1]
    H = np.ldexp(H, np.where(np.arange(m.n_verts) % 2 == 0, -531, -565)[:, None])
    with cg.Context(m) as c:
        sizes, frames = c.hessian_metric(H, eps, hmin, hmax)
    s_ref, f_ref = ao.metric_2d(H, eps, hmin, hmax)
    assert np.all(np.isfinite(frames)) and np.array_equal(frames, f_ref)
    assert np.array_equal(sizes, s_ref)


@pytest.mark.gpu
def test_batch_of_squares_matches_per_mesh_passes(gpu_lib):
    """The batched form of the anisotropic pass: uneven triangle meshes with
    their own fields in one context (a disjoint union).  The pass has no
    reduction across vertices (the metric comes from each vertex's Hessian),
    so every mesh gets exactly its own pass's result: FP64 marks and
    qualities bitwise, mixed (SPRG_FP32) marks identical to the mesh's own
    mixed pass and to the FP64 batch."""
    from core_gb300 import workload
    from core_gb300.mesh import Mesh
    m, u, voff, eoff, doff, ns = workload.batch_squares(6, seed=7, lo=8, hi=48)
    eps, hmin, hmax = workload.aniso2d_params(24)
    s64, c64, q64, *_ = run_aniso(m, u, eps, hmin, hmax, "fp64")
    s32, c32, q32, *_ = run_aniso(m, u, eps, hmin, hmax, "fp32")
    assert np.array_equal(s32, s64) and np.array_equal(c32, c64)
    assert s64.any() and c64.any()
    for k in range(len(ns)):
        mk = Mesh(2, m.coords[voff[k]:voff[k + 1]], m.elem_verts[eoff[k]:eoff[k + 1]] - voff[k],
                  m.edge_verts[doff[k]:doff[k + 1]] - voff[k])
        uk = u[voff[k]:voff[k + 1]]
        e, t = slice(doff[k], doff[k + 1]), slice(eoff[k], eoff[k + 1])
        a64, b64, r64, *_ = run_aniso(mk, uk, eps, hmin, hmax, "fp64")
        assert np.array_equal(s64[e], a64) and np.array_equal(c64[e], b64), k
        assert np.array_equal(q64[t], r64), k
        a32, b32, r32, *_ = run_aniso(mk, uk, eps, hmin, hmax, "fp32")
        assert np.array_equal(s32[e], a32) and np.array_equal(c32[e], b32), k
        assert np.abs(q32[t] - r64).max() <= 1e-4 * np.abs(r64).max(), k


@pytest.mark.gpu
def test_isotropic_fp32_pass_rejects_triangles(gpu_lib):
    import core_gb300 as cg
    from core_gb300 import _lib as K, workload
    m = workload.box(8, nz=0, jitter=0.1, seed=1)
    with cg.Context(m, precision="fp32") as c:
        with pytest.raises(K.SprgError) as ei:
            c.estimate_and_mark(workload.bump_field(m.coords, seed=1), 0.1)
        assert ei.value.code == K.SPRG_EINVAL


# Fields whose Hessians hit the metric's special cases: b = 0 with a != c
# (axis-aligned), a = c with b = 0 (isotropic: the frame comes from the
# a >= c branch), a = c = 0 with b != 0 (pure shear), negative eigenvalues
# (the |lambda| swap and the sign convention), and a linear field (zero
# Hessian: both sizes h_max).  The mixed pass takes those decisions with
# integer tests on the FP64 bits; marks and qualities must still be the
# FP64 pass's.
SPECIAL_FIELDS = {
    "axis": lambda x, y: 3.0 * x * x - 0.5 * y * y,
    "isotropic": lambda x, y: x * x + y * y,
    "shear": lambda x, y: 4.0 * x * y,
    "negative": lambda x, y: -(x * x + 3.0 * y * y) + 0.2 * x * y,
    "linear": lambda x, y: 2.0 * x - y,
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SPECIAL_FIELDS))
def test_mixed_metric_special_hessians(gpu_lib, name):
    from core_gb300 import workload
    m = workload.box(40, nz=0, jitter=0.15, seed=11)
    x, y = m.coords[:, 0], m.coords[:, 1]
    u = SPECIAL_FIELDS[name](x, y)
    eps, hmin, hmax = 2e-3, 1.0 / 160, 0.2
    s64, c64, q64, M64, _, _ = run_aniso(m, u, eps, hmin, hmax, "fp64")
    s32, c32, q32, M32, _, guard = run_aniso(m, u, eps, hmin, hmax, "fp32")
    assert np.array_equal(s32, s64) and np.array_equal(c32, c64)
    assert np.abs(q32 - q64).max() <= 1e-4 * np.abs(q64).max()
    scale = np.abs(M64).reshape(len(M64), -1).max(axis=1)
    assert (np.abs(M32 - M64).reshape(len(M64), -1).max(axis=1) / scale).max() <= 1e-5


@pytest.mark.gpu
def test_mixed_aniso_pass_off_plane(gpu_lib):
    """A triangle mesh in the plane z = 0.25 (not z = 0) keeps three
    operator components per slot; its marks equal the FP64 pass's and the
    same mesh in z = 0 (two components)."""
    from core_gb300.mesh import Mesh
    m, u, (eps, hmin, hmax) = case(64)
    x = m.coords.copy()
    x[:, 2] = 0.25
    lifted = Mesh(m.dim, x, m.elem_verts, m.edge_verts)
    s0, c0, q0, _, _, _ = run_aniso(m, u, eps, hmin, hmax, "fp32")
    s1, c1, q1, _, _, _ = run_aniso(lifted, u, eps, hmin, hmax, "fp32")
    s64, c64, _, _, _, _ = run_aniso(lifted, u, eps, hmin, hmax, "fp64")
    assert np.array_equal(s1, s64) and np.array_equal(c1, c64)
    assert np.array_equal(s1, s0) and np.array_equal(c1, c0)
    assert np.abs(q1 - q0).max() <= 1e-5 * np.abs(q0).max()
