"""LogAnisoSizeField (makeSizeField(m, sizes, frames, true), the default of
ma::configure): per-vertex log-metrics f diag(log(1/h^2)) f^T, interpolated
and eigen-decomposed by mth::eigenQR at every evaluation point.

The oracle's eigenQR is pinned bitwise to the reference's compiled
mth::eigenQR / apf::eigen in test_oracle_pinning.py; here the oracle's
log-metric measure is pinned to closed forms (constant metrics, isotropic
geometric interpolation) to 1e-10 relative: the reference's eigen iteration
stops once the off-diagonals fall below 1e-10 absolute, which leaves
eigenvector errors of that order.  The device path is held to the oracle:
lengths and qualities within 1e-10 relative (the device's exp / log may
differ from the host's by an ulp, and the eigen iteration carries such a
difference into its deflation tests), marks identical.
"""
import numpy as np
import pytest

GP = 0.577350269189626


def make_pair(oracle_mod, n, nz, jitter, seed):
    from core_gb300 import workload
    m = workload.box(n, nz=nz, jitter=jitter, seed=seed)
    o = oracle_mod.OracleMesh.box(n, n, n if nz is None else nz)
    o.set_coords(m.coords)
    m.v2e_off, m.v2e = o.v2e_off, o.v2e
    return m, o


def random_metric(V, seed, dim, lo=0.02, hi=0.4):
    rng = np.random.Generator(np.random.PCG64(seed))
    F = np.empty((V, 9))
    for v in range(V):
        if dim == 3:
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        else:
            t = rng.uniform(0, np.pi)
            q = np.array([[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1.0]])
        F[v] = q.reshape(9)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=(V, 3))), F


def test_oracle_log_metric_closed_forms(oracle_lib):
    m, o = make_pair(oracle_lib, 4, None, 0.2, 3)
    V = m.n_verts
    ev = m.edge_verts
    dx = np.linalg.norm(m.coords[ev[:, 1]] - m.coords[ev[:, 0]], axis=1)
    # one constant anisotropic metric everywhere: log and linear interpolation agree
    sizes, frames = random_metric(1, 5, 3)
    S, F = np.repeat(sizes, V, 0), np.repeat(frames, V, 0)
    rc, L_log = o.measure_log(S, F)
    assert rc == 0
    L_lin = o.measure(sizes=S, frames=F)
    assert np.abs(L_log - L_lin).max() <= 1e-10 * L_lin.max()
    # isotropic sizes, identity frames: 1/h interpolates geometrically,
    # 1/h(xi) = h0^-N0 h1^-N1, so L = |dx| / 2 * sum_g h0^-N0(g) h1^-N1(g)
    h = np.random.Generator(np.random.PCG64(6)).uniform(0.05, 0.5, V)
    S = np.repeat(h[:, None], 3, 1)
    F = np.tile(np.eye(3).reshape(1, 9), (V, 1))
    rc, L_log = o.measure_log(S, F)
    assert rc == 0
    h0, h1 = h[ev[:, 0]], h[ev[:, 1]]
    want = np.zeros(len(ev))
    for g in (GP, -GP):
        n0, n1 = (1 - g) / 2, (1 + g) / 2
        want += dx / 2 * h0 ** -n0 * h1 ** -n1
    assert np.abs(L_log - want).max() <= 1e-12 * want.max()
    # the vertex quality transforms are the vertex metrics themselves
    rc, q_log = o.quality_log(S, F)
    assert rc == 0 and np.abs(q_log - o.quality(size=h)).max() <= 1e-10


# ---------------------------------------------------------------------------
CASES = [(6, None, 0.2), (14, 0, 0.15)]


@pytest.mark.gpu
@pytest.mark.parametrize("n,nz,jit", CASES)
def test_log_aniso_matches_oracle(gpu_lib, oracle_lib, n, nz, jit):
    import core_gb300 as cg
    m, o = make_pair(oracle_lib, n, nz, jit, seed=51)
    sizes, frames = random_metric(m.n_verts, 52, m.dim, lo=0.02, hi=1.0)
    rc, L_o = o.measure_log(sizes, frames)
    assert rc == 0
    rc, q_o = o.quality_log(sizes, frames)
    assert rc == 0
    with cg.Context(m) as ctx:
        L = ctx.measure_edges_log_aniso(sizes, frames)
        assert np.abs(L - L_o).max() <= 1e-10 * L_o.max()
        # the lengths stay resident for the marks
        flags = np.zeros(m.n_edges, np.int32)
        ns = ctx.markEdgesToSplit(flags)
        nc = ctx.markEdgesToCollapse(flags)
        assert (ns, nc) == (int(np.sum(L_o > 1.5)), int(np.sum(L_o < 0.5)))
        assert ns > 0 and nc > 0
        q = ctx.measureQualityLog(sizes, frames)
        assert np.abs(q - q_o).max() <= 1e-10
        assert ctx.getMinQuality() == q[np.argmin(q)]
        mx = ctx.getMaximumEdgeLength(sizes=sizes, frames=frames, log=True)
        assert abs(mx - o.max_edge_length(sizes=sizes, frames=frames, log=True)) <= 1e-10 * mx
        pairs = np.random.Generator(np.random.PCG64(53)).integers(0, m.n_verts, size=(300, 2)).astype(np.int32)
        Lp = ctx.measure_vertex_pairs(pairs, sizes=sizes, frames=frames, log=True)
        Lp_o = o.measure_pairs(pairs, sizes=sizes, frames=frames, log=True)
        assert np.abs(Lp - Lp_o).max() <= 1e-10 * Lp_o.max()
    # the log and linear interpolations differ on these metrics
    assert np.abs(L_o - o.measure(sizes=sizes, frames=frames)).max() > 1e-6 * L_o.max()
