"""CPU restatement of the learned form -- TEST INFRASTRUCTURE ONLY.

numpy FP64 versions of (a) the network (forward and backward, BF16 rounding
at the points where the GPU kernels store BF16: weights, inputs and hidden
activations) and (b) the per-vertex features.  The learned form has no
reference counterpart: SCOREC/core recovers gradients with SPR only
(spr/sprRecoverField.cc); these restate this project's own network so that
the GPU forward/backward kernels and the feature kernel can be checked
against an independent FP64 computation.  Only tests/ import this module.
"""
import numpy as np
from scipy.special import erf

N_IN, N_HID, N_OUT = 128, 64, 3
ONE_SIDED = 0.3  # neighbour centroid offset / r_v beyond which a patch takes plain SPR
N_PARAMS = N_HID * N_IN + N_HID + N_HID * N_HID + N_HID + N_OUT * N_HID + N_OUT


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    bits = a32.view(np.uint32).astype(np.uint64)
    r = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits_to_f64(bits):
    b = np.ascontiguousarray(bits, dtype=np.uint16).astype(np.uint32) << 16
    return b.view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_HID * N_IN].reshape(N_HID, N_IN); o += N_HID * N_IN
    b1 = p[o:o + N_HID]; o += N_HID
    W2 = p[o:o + N_HID * N_HID].reshape(N_HID, N_HID); o += N_HID * N_HID
    b2 = p[o:o + N_HID]; o += N_HID
    W3 = p[o:o + N_OUT * N_HID].reshape(N_OUT, N_HID); o += N_OUT * N_HID
    b3 = p[o:o + N_OUT]
    return W1, b1, W2, b2, W3, b3


def forward(p, x, rounding=True):
    """Layer values for inputs x [n][128] (float64)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(p)
    W1, W2, W3 = r(W1), r(W2), r(W3)
    X = r(x)
    Z1 = X @ W1.T + b1
    H1 = r(gelu(Z1))
    Z2 = H1 @ W2.T + b2
    H2 = r(gelu(Z2))
    Z3 = H2 @ W3.T + b3
    return {"X": X, "W1": W1, "W2": W2, "W3": W3, "Z1": Z1, "H1": H1, "Z2": Z2, "H2": H2, "Z3": Z3}


def grad(p, x, y, rounding=True):
    """(gradient of the mean squared error, sum of squared errors)."""
    f = forward(p, x, rounding)
    n = x.shape[0]
    d = f["Z3"] - y
    dY = 2.0 * d / (N_OUT * n)
    dW3 = dY.T @ f["H2"]
    db3 = dY.sum(0)
    dZ2 = (dY @ f["W3"]) * gelu_grad(f["Z2"])
    dW2 = dZ2.T @ f["H1"]
    db2 = dZ2.sum(0)
    dZ1 = (dZ2 @ f["W2"]) * gelu_grad(f["Z1"])
    dW1 = dZ1.T @ f["X"]
    db1 = dZ1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return g, float((d * d).sum())


def mse(p, x, y, rounding=False):
    z = forward(p, x, rounding)["Z3"]
    return float(((z - y) ** 2).mean())


# ---------------------------------------------------------------------------
# features
# ---------------------------------------------------------------------------
def neighbours(n_verts, edge_verts):
    """Vertex -> neighbour CSR from the edges, ascending ids."""
    e = np.asarray(edge_verts, np.int64)
    a = np.concatenate([e[:, 0], e[:, 1]])
    b = np.concatenate([e[:, 1], e[:, 0]])
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    off = np.zeros(n_verts + 1, np.int64)
    np.add.at(off, a + 1, 1)
    return np.cumsum(off), b


def truncate_f32(u):
    """u truncated to 24 significant bits (the kernel's integer conversion)."""
    bits = np.ascontiguousarray(u, np.float64).view(np.uint64) & ~np.uint64((1 << 29) - 1)
    return bits.view(np.float64)


def features(coords, u, edge_verts, listed, slots=32):
    """(x [V][128] float64 before BF16 rounding, aux [V][5]) in FP64 from the
    kernel's FP32 inputs: coordinates rounded to FP32, u truncated."""
    V = coords.shape[0]
    off, nb = neighbours(V, edge_verts)
    xyz = np.asarray(coords, np.float32).astype(np.float64)
    uu = truncate_f32(u)
    cnt = np.diff(off)
    n = np.where(cnt <= slots, cnt, 0)
    idx = np.full((V, slots), -1, np.int64)
    for j in range(slots):
        has = j < n
        idx[has, j] = nb[off[:-1][has] + j]
    valid = idx >= 0
    safe = np.where(valid, idx, np.arange(V)[:, None])
    d = xyz[safe] - xyz[:, None, :]
    du = uu[safe] - uu[:, None]
    d[~valid] = 0.0
    du[~valid] = 0.0
    r = np.sqrt((d * d).sum(2).max(1))
    ir = np.where(r > 0, 1.0 / np.where(r > 0, r, 1.0), 0.0)
    A = np.einsum("vji,vjk->vik", d, d) * (ir * ir)[:, None, None]
    b = np.einsum("vji,vj->vi", d, du) * ir[:, None]
    det = np.linalg.det(A)
    tr = np.trace(A, axis1=1, axis2=2)
    msum = d.sum(1)
    one_sided = (msum * msum).sum(1) * ir * ir > (ONE_SIDED * np.maximum(n, 1)) ** 2
    flag = (cnt < 4) | (cnt > slots) | np.asarray(listed, bool) | ~(det > 1e-6 * tr ** 3) | one_sided
    ok = det > 0
    g = np.zeros((V, 3))
    g[ok] = np.linalg.solve(A[ok], b[ok][:, :, None])[:, :, 0] * ir[ok, None]
    rho = du - np.einsum("vji,vi->vj", d, g)
    rho[~valid] = 0.0
    s = np.sqrt((rho * rho).sum(1) / np.maximum(n, 1))
    is_ = np.where(s > 0, 1.0 / np.where(s > 0, s, 1.0), 0.0)
    x = np.concatenate([d * ir[:, None, None], (rho * is_[:, None])[:, :, None]], axis=2)
    x[~valid] = 0.0
    aux = np.column_stack([g, s * ir, flag.astype(np.float64)])
    return x.reshape(V, 4 * slots), aux
