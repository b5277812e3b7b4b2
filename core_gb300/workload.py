"""Seeded synthetic workloads (meshes and fields) of the benchmark configs.

The reference publishes no benchmark inputs; these generators stand in for
them with the shapes, sizes and value distributions the configs name:
jittered unit boxes (interior vertices moved by U(-a h, a h) per axis,
boundary vertices fixed), Gaussian-bump plus ramp fields, and the 2D
boundary-layer field.  numpy's PCG64 makes them identical on every host.
"""
import numpy as np

from .mesh import makeMdsBox


def box(n, nz=None, jitter=0.0, seed=0):
    """n^3 unit box (or n x n square when nz == 0) with interior jitter."""
    nz = n if nz is None else nz
    m = makeMdsBox(n, n, nz, 1.0, 1.0, 1.0)
    if jitter:
        rng = np.random.Generator(np.random.PCG64(seed))
        h = 1.0 / n
        d = rng.uniform(-jitter * h, jitter * h, size=m.coords.shape)
        if not nz:
            d[:, 2] = 0.0
        d[m.boundary_vertices()] = 0.0
        m.coords = m.coords + d
    return m


def sine_field(coords):
    """u = sin(2 pi x) sin(2 pi y) sin(2 pi z) (the 8^3 CPU config)."""
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    return np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)


def bump_field(coords, seed, n_bumps=4, width=(0.05, 0.2), amplitudes=None, ramp=(0.3, -0.2, 0.1)):
    """Sum of Gaussian bumps (centres uniform in the unit cube, widths uniform
    in `width`) plus a linear ramp."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.0, 1.0, size=(n_bumps, 3))
    w = rng.uniform(width[0], width[1], size=n_bumps)
    a = np.ones(n_bumps) if amplitudes is None else amplitudes
    u = coords @ np.asarray(ramp, np.float64)
    for k in range(n_bumps):
        r2 = ((coords - c[k]) ** 2).sum(axis=1)
        u = u + a[k] * np.exp(-r2 / (2 * w[k] ** 2))
    return u


def batched_field(coords, seed):
    """1-8 Gaussian bumps, widths U[0.02, 0.3], amplitudes N(0,1), no ramp."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nb = int(rng.integers(1, 9))
    amps = rng.normal(0.0, 1.0, size=nb)
    return bump_field(coords, seed + 1_000_003, n_bumps=nb, width=(0.02, 0.3), amplitudes=amps, ramp=(0, 0, 0))


def boundary_layer_field(coords):
    """u = tanh((y - 0.5) / 1e-3) + 0.1 sin(8 pi x) (the 2D anisotropic config)."""
    x, y = coords[:, 0], coords[:, 1]
    return np.tanh((y - 0.5) / 1e-3) + 0.1 * np.sin(8 * np.pi * x)


def aniso2d_params(n):
    """Metric constants of the 2D anisotropic workload on an n x n square:
    eps = 63 (2/n)^2 (twice the cell size where |u_xx| = 0.1 (8 pi)^2),
    h_min = 1 / (4 n), h_max = 0.05."""
    return 63.0 * (2.0 / n) ** 2, 1.0 / (4 * n), 0.05


def aniso2d(n, seed=5):
    """(mesh, u, (eps, h_min, h_max)): n x n square, interior jitter +-0.15h,
    boundary-layer field."""
    m = box(n, nz=0, jitter=0.15, seed=seed)
    return m, boundary_layer_field(m.coords), aniso2d_params(n)


def batch_boxes(n_meshes, seed=3, lo=4, hi=40, jitter=0.0):
    """The batched workload: n_meshes unit tet boxes with n per side
    log-uniform in [lo, hi] (seeded), each with its own field of 1-8 Gaussian
    bumps (batched_field), flattened into one disjoint union.  Returns
    (mesh, u, vert_offsets, elem_offsets, edge_offsets, ns)."""
    from .mesh import Mesh
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), n_meshes))).astype(int)
    parts, us = [], []
    for k, n in enumerate(ns):
        m = box(int(n), jitter=jitter, seed=seed * 1_000_003 + k)
        parts.append(m)
        us.append(batched_field(m.coords, seed * 1_000_003 + k))
    voff = np.concatenate([[0], np.cumsum([p.n_verts for p in parts])]).astype(np.int64)
    eoff = np.concatenate([[0], np.cumsum([p.n_elems for p in parts])]).astype(np.int64)
    doff = np.concatenate([[0], np.cumsum([p.n_edges for p in parts])]).astype(np.int64)
    coords = np.concatenate([p.coords for p in parts])
    ev = np.concatenate([p.elem_verts + np.int32(voff[k]) for k, p in enumerate(parts)])
    ed = np.concatenate([p.edge_verts + np.int32(voff[k]) for k, p in enumerate(parts)])
    return Mesh(3, coords, ev, ed), np.concatenate(us), voff, eoff, doff, ns


def batch_squares(n_meshes, seed=5, lo=8, hi=64, jitter=0.15):
    """A batch of triangle meshes for the anisotropic pass: n_meshes unit
    squares of n x n cells (n log-uniform in [lo, hi], seeded, interior
    jitter), each with its own field of Gaussian bumps (batched_field),
    flattened into one disjoint union.  Returns (mesh, u, vert_offsets,
    elem_offsets, edge_offsets, ns)."""
    from .mesh import Mesh
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), n_meshes))).astype(int)
    parts, us = [], []
    for k, n in enumerate(ns):
        m = box(int(n), nz=0, jitter=jitter, seed=seed * 1_000_003 + k)
        parts.append(m)
        us.append(batched_field(m.coords, seed * 1_000_003 + k))
    voff = np.concatenate([[0], np.cumsum([p.n_verts for p in parts])]).astype(np.int64)
    eoff = np.concatenate([[0], np.cumsum([p.n_elems for p in parts])]).astype(np.int64)
    doff = np.concatenate([[0], np.cumsum([p.n_edges for p in parts])]).astype(np.int64)
    coords = np.concatenate([p.coords for p in parts])
    ev = np.concatenate([p.elem_verts + np.int32(voff[k]) for k, p in enumerate(parts)])
    ed = np.concatenate([p.edge_verts + np.int32(voff[k]) for k, p in enumerate(parts)])
    return Mesh(2, coords, ev, ed), np.concatenate(us), voff, eoff, doff, ns


def config(name):
    """(mesh, field, adapt_ratio) of a named workload."""
    if name == "box8":
        m = box(8)
        return m, sine_field(m.coords), 0.1
    if name.startswith("jbox"):
        n = int(name[4:])
        m = box(n, jitter=0.2, seed=2)
        return m, bump_field(m.coords, seed=2), 0.1
    raise KeyError(name)
