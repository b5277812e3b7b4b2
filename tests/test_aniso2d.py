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
