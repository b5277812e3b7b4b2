"""Shared inputs of the reference-pinning tests and fixtures (no test here).

Seeded meshes and fields restated with numpy only (no product code), so the
reference, the oracle and the GPU path all see the same numbers:
jittered boxes, the bump and boundary-layer fields, random anisotropic
metrics, a box with shuffled numbering, the case list that
tests/golden/make_ref_golden.py runs through the reference, and the mask of
vertices whose FP64 size is well conditioned.
"""
import numpy as np


def jitter_coords(x, n, nz, jitter, seed):
    """Interior vertices moved by U(-jitter h, jitter h) per axis (the seeded
    jitter of core_gb300.workload.box, restated without the product)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = 1.0 / n
    d = rng.uniform(-jitter * h, jitter * h, size=x.shape)
    bnd = np.any((x == 0.0) | (x == 1.0), axis=1) if nz else np.any((x[:, :2] == 0.0) | (x[:, :2] == 1.0), axis=1)
    if not nz:
        d[:, 2] = 0.0
    d[bnd] = 0.0
    return x + d


def bump(x, seed, n_bumps=4, width=(0.05, 0.2), ramp=(0.3, -0.2, 0.1)):
    """Gaussian bumps (centres uniform in the unit cube) plus a linear ramp."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.0, 1.0, size=(n_bumps, 3))
    w = rng.uniform(width[0], width[1], size=n_bumps)
    u = x @ np.asarray(ramp, np.float64)
    for k in range(n_bumps):
        u = u + np.exp(-((x - c[k]) ** 2).sum(axis=1) / (2 * w[k] ** 2))
    return u


def layer(x, width=0.05):
    """tanh((y - 0.5) / width) + 0.1 sin(8 pi x)."""
    return np.tanh((x[:, 1] - 0.5) / width) + 0.1 * np.sin(8 * np.pi * x[:, 0])


def sine(x):
    return np.sin(2 * np.pi * x[:, 0]) * np.sin(2 * np.pi * x[:, 1]) * np.sin(2 * np.pi * x[:, 2])


def random_metric(V, seed, dim, lo=0.04, hi=0.5):
    """Per-vertex sizes (log-uniform in [lo, hi]) and orthonormal frames
    (row-major 3 x 3; in 2D a rotation about z)."""
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


def shuffled_box(oracle_mod, n, seed):
    """A jittered n^3 tet box as downward adjacency with every entity kind's
    numbering randomly permuted (mesh order far from local, as in meshes from
    other generators): (coords, edges E x 2, faces F x 3, tets T x 4)."""
    o = oracle_mod.OracleMesh.box(n, n, n)
    x = jitter_coords(o.coords.copy(), n, n, 0.2, seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    f, t = o.down(2), o.down(3)
    pv, pe, pf, pt = (rng.permutation(k) for k in (o.V, o.E, len(f), o.T))
    coords = np.empty_like(x)
    coords[pv] = x
    edges = np.empty((o.E, 2), np.int32)
    edges[pe] = pv[o.down(1)]
    faces = np.empty_like(f)
    faces[pf] = pe[f]
    tets = np.empty_like(t)
    tets[pt] = pf[t]
    return coords, edges, faces, tets


def shuffled_box_smb(oracle_mod, path, n, seed):
    """shuffled_box written as a one-part .smb file; returns its arrays."""
    from test_smb import write_smb
    coords, edges, faces, tets = shuffled_box(oracle_mod, n, seed)
    write_smb(path, 3, coords, edges, faces, tets)
    return coords, edges, faces, tets


# Cases of the reference-output fixture (tests/golden/ref_path.npz):
# name -> (kind, parameters).  "iso": box n x n x nz, jitter, seed, field,
# adapt ratio (target set: getTargetSPRSizeField); "aniso": box with a random
# metric, log interpolation or not; "shuffled": shuffled_box.
REF_CASES = {
    "box8": ("iso", dict(n=8, nz=8, jitter=0.0, seed=0, field="sine", ratio=0.1)),
    "jbox10": ("iso", dict(n=10, nz=10, jitter=0.2, seed=4, field="bump", ratio=0.1)),
    "tri24": ("iso", dict(n=24, nz=0, jitter=0.15, seed=5, field="layer", ratio=0.02)),
    "target10": ("iso", dict(n=10, nz=10, jitter=0.2, seed=7, field="bump", ratio=0.0, target=0.5)),
    "shuf6": ("shuffled", dict(n=6, seed=13, field="bump", ratio=0.1)),
    "aniso5": ("aniso", dict(n=5, nz=5, jitter=0.2, seed=9, log=False)),
    "loganiso5": ("aniso", dict(n=5, nz=5, jitter=0.2, seed=9, log=True)),
    "aniso12tri": ("aniso", dict(n=12, nz=0, jitter=0.2, seed=9, log=False)),
}


def field(name, x, seed):
    if name == "sine":
        return sine(x)
    if name == "layer":
        return layer(x)
    return bump(x, seed)


def conditioned(n_verts, elem_verts, ip, rec, rel=1e-7):
    """Vertices whose size is well conditioned in FP64: every adjacent
    element's deviation |eps_t - eps*(IP)| is above `rel` of the largest
    gradient.  Where a patch is linear to the rounding level, the element
    error is rounding noise and err^(-1/5) turns a 1e-16 change of the
    recovered field into an O(1) change of that element's size, in the
    reference as in any other summation order."""
    d = ip - rec[elem_verts].mean(axis=1)
    good_el = np.linalg.norm(d, axis=1) > rel * np.abs(ip).max()
    bad_v = np.zeros(n_verts, bool)
    bad_v[elem_verts[~good_el].reshape(-1)] = True
    return ~bad_v
