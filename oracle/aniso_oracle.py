"""CPU restatement of the anisotropic metric -- TEST INFRASTRUCTURE ONLY.

numpy FP64 version of the metric the 2D anisotropic workload derives from a
nodal Hessian (sizes h_i = clamp(sqrt(eps / |lambda_i|), h_min, h_max),
frames = principal directions as columns), with the same eigen-decomposition,
ordering and sign convention as the device kernel (closed form in 2D, fixed
8-sweep cyclic Jacobi in 3D).  The reference's drivers build this metric
with apf::eigen (apf/apfMatrix.cc:68-82, mth::eigenQR); it then feeds
ma::makeSizeField(m, sizes, frames, false) (ma/maSize.cc:618), whose measure
the C oracle (spr_oracle.c) restates.  Only tests/ import this module.
"""
import numpy as np


def _size(lam, eps, hmin, hmax):
    a = np.abs(lam)
    with np.errstate(divide="ignore", invalid="ignore"):
        h = np.minimum(np.maximum(np.sqrt(eps / np.where(a > 0, a, 1.0)), hmin), hmax)
    return np.where(a > 0, h, hmax)


def _bexp(x):
    return ((np.asarray(x, np.float64).view(np.int64) >> 52) & 0x7FF).astype(np.int64)


def _scale_exp(E):
    """The metric's power-of-two prescaling of a Hessian, from the largest
    biased exponent E of its entries: none while the largest entry lies in
    [2^-400, 2^401) or an entry is not finite, else 2^-(E - 1022) (2^1022
    when every entry is zero or subnormal)."""
    E = np.asarray(E)
    keep = (E == 2047) | ((E >= 623) & (E <= 1423))
    return np.where(keep, 0, np.where(E == 0, -1022, E - 1022))


def _times_pow2(x, k):
    """x 2^k (two factors where 2^k is outside the normal range)."""
    k = np.asarray(k)
    h = k // 2
    return x * np.ldexp(1.0, h) * np.ldexp(1.0, k - h)


def metric_2d(H, eps, hmin, hmax):
    H = np.asarray(H, np.float64).reshape(-1, 9)
    b0 = 0.5 * (H[:, 1] + H[:, 3])
    es = _scale_exp(np.maximum(np.maximum(_bexp(H[:, 0]), _bexp(H[:, 4])), _bexp(b0)))
    a, b, c = _times_pow2(H[:, 0], -es), _times_pow2(b0, -es), _times_pow2(H[:, 4], -es)
    mid, hd = 0.5 * (a + c), 0.5 * (a - c)
    d = np.sqrt(hd * hd + b * b)
    l1, l2 = mid + d, mid - d
    zero_b = b == 0.0
    ge = a >= c
    x = np.where(zero_b, np.where(ge, 1.0, 0.0), np.where(ge, l1 - c, b))
    y = np.where(zero_b, np.where(ge, 0.0, 1.0), np.where(ge, b, l1 - a))
    n = np.sqrt(x * x + y * y)
    x, y = x / n, y / n
    sw = np.abs(l2) > np.abs(l1)
    l1, l2 = np.where(sw, l2, l1), np.where(sw, l1, l2)
    x, y = np.where(sw, -y, x), np.where(sw, x, y)
    neg = (x < 0) | ((x == 0) & (y < 0))
    x, y = np.where(neg, -x, x), np.where(neg, -y, y)
    l1, l2 = _times_pow2(l1, es), _times_pow2(l2, es)
    V = H.shape[0]
    R = np.zeros((V, 3, 3))
    R[:, 0, 0], R[:, 0, 1] = x, -y
    R[:, 1, 0], R[:, 1, 1] = y, x
    R[:, 2, 2] = 1.0
    sizes = np.column_stack([_size(l1, eps, hmin, hmax), _size(l2, eps, hmin, hmax), np.full(V, hmax)])
    return sizes, R.reshape(V, 9)


def _jacobi(A):
    with np.errstate(over="ignore"):  # theta^2 may overflow: t = 0, as on the device
        return _jacobi_sweeps(A)


def _jacobi_sweeps(A):
    A = A.copy()
    Vm = np.eye(3)
    for _ in range(8):
        for p in range(2):
            for q in range(p + 1, 3):
                apq = A[p, q]
                if apq == 0.0:
                    continue
                theta = (A[q, q] - A[p, p]) / (2.0 * apq)
                t = (1.0 if theta >= 0 else -1.0) / (abs(theta) + np.sqrt(theta * theta + 1.0))
                c = 1.0 / np.sqrt(t * t + 1.0)
                s = t * c
                for k in range(3):
                    akp, akq = A[k, p], A[k, q]
                    A[k, p], A[k, q] = c * akp - s * akq, s * akp + c * akq
                for k in range(3):
                    apk, aqk = A[p, k], A[q, k]
                    A[p, k], A[q, k] = c * apk - s * aqk, s * apk + c * aqk
                for k in range(3):
                    vkp, vkq = Vm[k, p], Vm[k, q]
                    Vm[k, p], Vm[k, q] = c * vkp - s * vkq, s * vkp + c * vkq
    return np.diag(A).copy(), Vm


def metric_3d(H, eps, hmin, hmax):
    H = np.asarray(H, np.float64).reshape(-1, 3, 3)
    V = H.shape[0]
    sizes = np.empty((V, 3))
    frames = np.empty((V, 3, 3))
    for v in range(V):
        A = 0.5 * (H[v] + H[v].T)
        es = int(_scale_exp(_bexp(A).max()))
        lam, Vm = _jacobi(_times_pow2(A, -es))
        lam = _times_pow2(lam, es)
        order = [0, 1, 2]
        for i in range(3):
            for j in range(i + 1, 3):
                if abs(lam[order[j]]) > abs(lam[order[i]]):
                    order[i], order[j] = order[j], order[i]
        R = np.zeros((3, 3))
        for k in range(2):
            col = Vm[:, order[k]]
            im = int(np.argmax(np.abs(col)))
            # first maximum, as the device scan keeps the first strictly larger
            im = min(i for i in range(3) if abs(col[i]) == abs(col[im]))
            R[:, k] = -col if col[im] < 0 else col
            sizes[v, k] = _size(lam[order[k]], eps, hmin, hmax)
        R[0, 2] = R[1, 0] * R[2, 1] - R[2, 0] * R[1, 1]
        R[1, 2] = R[2, 0] * R[0, 1] - R[0, 0] * R[2, 1]
        R[2, 2] = R[0, 0] * R[1, 1] - R[1, 0] * R[0, 1]
        sizes[v, 2] = _size(lam[order[2]], eps, hmin, hmax)
        frames[v] = R
    return sizes, frames.reshape(V, 9)


def hessian(om, u):
    """Nodal Hessian through the C oracle: recover(grad(recover(grad(u))))."""
    rc, g, _, _ = om.recover(om.grad_ip(u))
    assert rc == 0
    rc, H, _, _ = om.recover(om.grad_ip(g))
    assert rc == 0
    return H
