"""A second, independent restatement of the gradient at integration points
and of the SPR patch fit, in numpy, against the oracle's C restatement.

Followed here from the reference directly:
* spr/sprGetGradIPField.cc:15-65 - order-1 elements carry one integration
  point, the element's constant gradient of the linear interpolant;
* spr/sprRecoverField.cc:155-192 - a vertex's patch starts as its adjacent
  elements; while it has fewer points than polynomial terms or its
  least-squares matrix is rank-deficient, it takes (from the elements it had
  when growth began) the elements that share a face, then an edge, then a
  vertex with them, testing after each stage, and repeats from the larger
  set (spr/sprRecoverField.cc:365-386);
* spr/sprRecoverField.cc:193-353 - sample points at the element centroids,
  polynomial terms [1, x, y(, z)], the least-squares fit evaluated at the
  vertex.
numpy's lstsq solves the same full-rank systems through another
factorisation, so values agree to rounding (1e-10 relative), and the
growth decisions are checked to sit far from the rank threshold."""
import itertools

import numpy as np
import pytest


def jittered(o, n, nz, seed):
    rng = np.random.default_rng(seed)
    x = o.coords.copy()
    h = np.array([1.0 / n, 1.0 / n, 1.0 / nz if nz else 0.0])
    inner = np.all((x > 1e-12) & (x < 1 - 1e-12), axis=1) if nz else \
        np.all((x[:, :2] > 1e-12) & (x[:, :2] < 1 - 1e-12), axis=1)
    x[inner] += rng.uniform(-0.2, 0.2, (inner.sum(), 3)) * h
    o.set_coords(x)
    return x


def field(x):
    return np.sin(2.1 * x[:, 0]) * np.cos(1.3 * x[:, 1]) + 0.7 * x[:, 2] ** 2 + 0.3 * x[:, 0] * x[:, 1]


def grad_ip_numpy(x, ev, f):
    d = ev.shape[1] - 1
    g = np.empty((ev.shape[0], 3))
    for t, vs in enumerate(ev):
        J = (x[vs[1:]] - x[vs[0]])[:, :d]
        g[t, :d] = np.linalg.solve(J, f[vs[1:]] - f[vs[0]])
        g[t, d:] = 0.0
    return g


class Adjacency:
    """Downward entities of every element as vertex tuples and the elements
    around each entity (the MDS upward adjacency, as sets)."""

    def __init__(self, ev):
        self.ev = ev
        d = ev.shape[1] - 1
        self.down = {k: [] for k in range(d)}
        self.up = {k: {} for k in range(d)}
        for t, vs in enumerate(ev):
            for k in range(d):
                ents = [tuple(sorted(c)) for c in itertools.combinations(vs, k + 1)]
                self.down[k].append(ents)
                for e in ents:
                    self.up[k].setdefault(e, set()).add(t)

    def sharing(self, elems, k):
        out = set()
        for t in elems:
            for e in self.down[k][t]:
                out |= self.up[k][e]
        return out


def fit_matrix(x, elems, ev, d):
    c = x[ev[sorted(elems)]].mean(axis=1)[:, :d]
    return np.hstack([np.ones((len(elems), 1)), c])


def recover_numpy(x, ev, ip):
    d = ev.shape[1] - 1
    nterms = d + 1
    adj = Adjacency(ev)
    out = np.empty((x.shape[0], ip.shape[1]))
    grown = 0
    margins = []

    def enough(elems):
        if len(elems) < nterms:
            return False
        s = np.linalg.svd(fit_matrix(x, elems, ev, d), compute_uv=False)
        margins.append(s[-1])
        return s[-1] > 1e-8

    for v in range(x.shape[0]):
        patch = set(adj.up[0][(v,)])
        if not enough(patch):
            grown += 1
            while True:
                old = set(patch)
                done = False
                for k in range(d - 1, -1, -1):
                    patch |= adj.sharing(old, k)
                    if enough(patch):
                        done = True
                        break
                if done:
                    break
                assert len(patch) > len(old), "no growth possible"
        els = sorted(patch)
        A = fit_matrix(x, patch, ev, d)
        coef, *_ = np.linalg.lstsq(A, ip[els], rcond=None)
        out[v] = np.concatenate([[1.0], x[v, :d]]) @ coef
    return out, grown, np.array(margins)


@pytest.mark.parametrize("n,nz,seed", [(4, 3, 1), (5, 0, 2), (3, 3, 7)])
def test_spr_restated_twice(oracle_lib, n, nz, seed):
    o = oracle_lib.OracleMesh.box(n, n - 1 if nz else n, nz)
    x = jittered(o, n, nz, seed)
    ev = o.elem_verts
    f = field(x)
    ip = o.grad_ip(f)
    ip_np = grad_ip_numpy(x, ev, f)
    scale = np.abs(ip_np).max()
    assert np.abs(ip - ip_np).max() <= 1e-12 * scale
    rc, rec, nexp, fail = o.recover(ip)
    assert rc == 0 and fail == -1
    rec_np, grown, margins = recover_numpy(x, ev, ip_np)
    # every growth decision far from the 1e-10 rank threshold of mth::decomposeQR
    assert not np.any((margins > 1e-13) & (margins < 1e-6))
    assert nexp == grown
    assert np.abs(rec - rec_np).max() <= 1e-10 * np.abs(rec_np).max()


def test_linear_field_is_recovered_exactly_by_both(oracle_lib):
    """SPR's patch test: the gradient of a linear field is constant, so
    both restatements return it at every vertex, grown patches included."""
    o = oracle_lib.OracleMesh.box(3, 3, 2)
    x = jittered(o, 3, 2, 4)
    g = np.array([0.4, -1.1, 2.5])
    f = x @ g - 0.2
    ip = o.grad_ip(f)
    rc, rec, nexp, fail = o.recover(ip)
    rec_np, grown, _ = recover_numpy(x, o.elem_verts, grad_ip_numpy(x, o.elem_verts, f))
    assert rc == 0 and nexp == grown > 0
    assert np.abs(rec - g).max() < 1e-10
    assert np.abs(rec_np - g).max() < 1e-10


def size_field_numpy(x, ev, ip, rec, adapt_ratio):
    """getSPRSizeField (spr/sprEstimateError.cc:98-321) for order-1 fields:
    integration order 1 (one point at the centroid, w dV = the element's
    measure), recovered order p = 1.  Returns (vertex sizes, element sizes,
    ||eps*||^2, sum of err^(2d/(2p+d)), size factor)."""
    d = ev.shape[1] - 1
    p = 1.0
    X = x[ev][:, :, :d]
    J = X[:, 1:] - X[:, :1]
    vol = np.abs(np.linalg.det(J)) / (6.0 if d == 3 else 2.0)
    star_c = rec[ev].mean(axis=1)                       # eps* at the centroid
    self_product = np.sum(np.sum(star_c * star_c, axis=1) * vol)
    e2 = np.sum((ip - star_c) ** 2, axis=1) * vol       # element error integral
    G = np.sum(np.sqrt(e2) ** (2 * d / (2 * p + d)))
    a = adapt_ratio * adapt_ratio * np.sqrt(self_product) ** 2
    factor = (a / G) ** (1.0 / (2.0 * p))
    pairs = list(itertools.combinations(range(d + 1), 2))
    h = np.max([np.linalg.norm(x[ev[:, i]] - x[ev[:, j]], axis=1) for i, j in pairs], axis=0)
    esize = h * np.sqrt(e2) ** (-(2 / (2 * p + d))) * factor
    V = x.shape[0]
    s = np.zeros(V)
    c = np.zeros(V)
    for k in range(d + 1):
        np.add.at(s, ev[:, k], esize)
        np.add.at(c, ev[:, k], 1)
    return s / c, esize, self_product, G, factor


@pytest.mark.parametrize("n,nz,seed,ratio", [(4, 3, 1, 0.1), (6, 0, 2, 0.05), (3, 3, 7, 0.008)])
def test_size_field_restated_twice(oracle_lib, n, nz, seed, ratio):
    o = oracle_lib.OracleMesh.box(n, n - 1 if nz else n, nz)
    x = jittered(o, n, nz, seed)
    ev = o.elem_verts
    f = field(x)
    ip = o.grad_ip(f)
    rc, size, rec, esize, err, info = o.size_field(ip, ratio)
    assert rc == 0
    size_np, esize_np, sp, G, factor = size_field_numpy(x, ev, ip, rec, ratio)
    assert abs(info["eps_star_norm2"] - sp) <= 1e-12 * sp
    assert abs(info["error_sum"] - G) <= 1e-12 * G
    assert abs(info["size_factor"] - factor) <= 1e-12 * factor
    assert np.abs(esize - esize_np).max() <= 1e-11 * np.abs(esize_np).max()
    assert np.abs(size - size_np).max() <= 1e-11 * np.abs(size_np).max()


def target_size_field_numpy(x, ev, ip, rec, target, alpha, beta):
    """getTargetSPRSizeField (spr/sprEstimateTargetError.cc:129-258): size
    factor (G / N)^(1/d), the new element size clamped to [alpha h, beta h],
    then the vertex average."""
    d = ev.shape[1] - 1
    p = 1.0
    X = x[ev][:, :, :d]
    vol = np.abs(np.linalg.det(X[:, 1:] - X[:, :1])) / (6.0 if d == 3 else 2.0)
    e2 = np.sum((ip - rec[ev].mean(axis=1)) ** 2, axis=1) * vol
    G = np.sum(np.sqrt(e2) ** (2 * d / (2 * p + d)))
    factor = (G / target) ** (1.0 / d)
    pairs = list(itertools.combinations(range(d + 1), 2))
    h = np.max([np.linalg.norm(x[ev[:, i]] - x[ev[:, j]], axis=1) for i, j in pairs], axis=0)
    hn = factor * np.sqrt(e2) ** (-2.0 / (2.0 * p + d)) * h
    hn = np.where(hn < alpha * h, alpha * h, hn)
    hn = np.where(hn > beta * h, beta * h, hn)
    s = np.zeros(x.shape[0])
    c = np.zeros(x.shape[0])
    for k in range(d + 1):
        np.add.at(s, ev[:, k], hn)
        np.add.at(c, ev[:, k], 1)
    return s / c, hn, G, factor


@pytest.mark.parametrize("n,nz,seed,target,alpha,beta", [(4, 3, 1, 5000, 0.25, 2.0), (6, 0, 2, 300, 0.5, 1.5),
                                                          (3, 3, 7, 40, 0.25, 2.0)])
def test_target_size_field_restated_twice(oracle_lib, n, nz, seed, target, alpha, beta):
    o = oracle_lib.OracleMesh.box(n, n - 1 if nz else n, nz)
    x = jittered(o, n, nz, seed)
    ev = o.elem_verts
    ip = o.grad_ip(field(x))
    rc, size, rec, esize, err, info = o.size_field(ip, 0.0, target=target, alpha=alpha, beta=beta)
    assert rc == 0
    size_np, esize_np, G, factor = target_size_field_numpy(x, ev, ip, rec, target, alpha, beta)
    assert abs(info["error_sum"] - G) <= 1e-12 * G
    assert abs(info["size_factor"] - factor) <= 1e-12 * factor
    # the cases clamp 7 elements at alpha h (first), 32 at alpha h and 3 at
    # beta h (second), 11 at beta h (third)
    assert np.abs(esize - esize_np).max() <= 1e-11 * np.abs(esize_np).max()
    assert np.abs(size - size_np).max() <= 1e-11 * np.abs(size_np).max()


def iso_lengths_numpy(x, ed, size):
    """MetricSizeField::measure of an edge under an isotropic size field
    (ma/maSize.cc:208-216, 140-196): apf's edge rule of accuracy 3 (two
    points at +-0.577350269189626, weight 1, apf/apfIntegrate.cc:41-52) of
    |dx/dxi| / h(xi), h interpolated linearly along the edge."""
    a, b = ed[:, 0], ed[:, 1]
    half = np.linalg.norm(x[b] - x[a], axis=1) / 2.0
    out = np.zeros(ed.shape[0])
    for xi in (0.577350269189626, -0.577350269189626):
        h = size[a] * (1 - xi) / 2 + size[b] * (1 + xi) / 2
        out += 1.0 * half / h
    return out


@pytest.mark.parametrize("n,nz,seed", [(4, 3, 1), (6, 0, 2)])
def test_iso_edge_lengths_and_marks_restated_twice(oracle_lib, n, nz, seed):
    o = oracle_lib.OracleMesh.box(n, n - 1 if nz else n, nz)
    x = jittered(o, n, nz, seed)
    rng = np.random.default_rng(seed)
    size = rng.uniform(0.05, 0.6, o.V)
    L = o.measure(size=size)
    L_np = iso_lengths_numpy(x, o.edge_verts, size)
    assert np.abs(L - L_np).max() <= 1e-13 * L_np.max()
    # markEdgesToSplit / markEdgesToCollapse: > 1.5 and < 0.5 (ma/maSize.h:26-27)
    flags = np.zeros(o.E, np.int32)
    rc, ns = oracle_lib.mark_edges(L, 0, flags)
    assert rc == 0 and ns == int(np.sum(L_np > 1.5))
    rc, nc = oracle_lib.mark_edges(L, 1, flags)
    assert rc == 0 and nc == int(np.sum(L_np < 0.5))


def iso_quality_numpy(x, ev, size):
    """measureTetQuality / measureTriQuality with useMax = true under an
    isotropic size field (ma/maQuality.cc:83-167): the metric of the element
    vertex with the largest det Q (the smallest h), edge lengths and measure
    in it; 15552 V^2 / (sum l^2)^3 with V's sign for tets, 48 A^2 / (sum
    l^2)^2 for triangles."""
    d = ev.shape[1] - 1
    h = size[ev].min(axis=1)
    X = x[ev]
    pairs = list(itertools.combinations(range(d + 1), 2))
    s = sum(np.sum((X[:, j] - X[:, i]) ** 2, axis=1) for i, j in pairs) / h ** 2
    if d == 3:
        V = np.linalg.det(X[:, 1:] - X[:, :1]) / 6.0 / h ** 3
        return np.sign(V) * 15552.0 * V * V / (s * s * s)
    e1, e2 = X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]
    A = 0.5 * np.linalg.norm(np.cross(e1, e2), axis=1) / h ** 2
    return 48.0 * A * A / (s * s)


@pytest.mark.parametrize("n,nz,seed", [(4, 3, 1), (6, 0, 2), (3, 2, 5)])
def test_iso_quality_restated_twice(oracle_lib, n, nz, seed):
    o = oracle_lib.OracleMesh.box(n, n - 1 if nz else n, nz)
    x = jittered(o, n, nz, seed)
    rng = np.random.default_rng(seed + 10)
    size = rng.uniform(0.05, 0.6, o.V)
    q = o.quality(size=size)
    q_np = iso_quality_numpy(x, o.elem_verts, size)
    assert np.all(q > 0) and np.all(q <= 1 + 1e-12)
    assert np.abs(q - q_np).max() <= 1e-12


def aniso_lengths_numpy(x, ed, sizes, frames):
    """AnisoSizeField::measure of an edge (ma/maSize.cc:94-121, 364-412):
    at each point of the two-point rule the sizes and the frame R are
    interpolated linearly, R is re-orthogonalised (first column normalised,
    second made orthogonal to it and normalised, third their cross
    product), Q = R diag(1/h), and the edge's tangent row dx/dxi times Q
    gives the length element."""
    a, b = ed[:, 0], ed[:, 1]
    g = (x[b] - x[a]) / 2.0
    Ra, Rb = frames[a].reshape(-1, 3, 3), frames[b].reshape(-1, 3, 3)
    out = np.zeros(ed.shape[0])
    for xi in (0.577350269189626, -0.577350269189626):
        wa, wb = (1 - xi) / 2, (1 + xi) / 2
        h = sizes[a] * wa + sizes[b] * wb
        RT = np.transpose(Ra * wa + Rb * wb, (0, 2, 1))
        r0 = RT[:, 0] / np.linalg.norm(RT[:, 0], axis=1)[:, None]
        r1 = RT[:, 1] - r0 * np.sum(r0 * RT[:, 1], axis=1)[:, None]
        r1 = r1 / np.linalg.norm(r1, axis=1)[:, None]
        r2 = np.cross(r0, r1)
        R = np.stack([r0, r1, r2], axis=2)              # columns: the directions
        gq = np.einsum("ei,eik->ek", g, R) / h
        out += np.linalg.norm(gq, axis=1)
    return out


def random_frames(rng, V, spread):
    """Rotations near a common one, so neighbouring frames interpolate to a
    usable frame."""
    base = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    F = np.empty((V, 3, 3))
    for v in range(V):
        w = rng.normal(size=3) * spread
        K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
        F[v] = base @ (np.eye(3) + K + K @ K / 2)     # close to a rotation
        F[v] = np.linalg.qr(F[v])[0]
    return F.reshape(V, 9)


@pytest.mark.parametrize("n,nz,seed", [(4, 3, 1), (5, 0, 2)])
def test_aniso_edge_lengths_restated_twice(oracle_lib, n, nz, seed):
    o = oracle_lib.OracleMesh.box(n, n - 1 if nz else n, nz)
    x = jittered(o, n, nz, seed)
    rng = np.random.default_rng(seed + 20)
    sizes = rng.uniform(0.05, 0.6, (o.V, 3))
    frames = random_frames(rng, o.V, 0.3)
    L = o.measure(sizes=sizes, frames=frames)
    L_np = aniso_lengths_numpy(x, o.edge_verts, sizes, frames)
    assert np.abs(L - L_np).max() <= 1e-12 * L_np.max()
