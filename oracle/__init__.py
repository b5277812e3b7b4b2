"""CPU oracle of the estimate-and-mark path -- TEST INFRASTRUCTURE ONLY.

Python binding of oracle/liboracle.so (oracle/spr_oracle.c, a plain-C
restatement of the reference algorithms).  Only tests/, __graft_entry__.smoke()
and bench.py's cpu_baseline / --impl reference legs may import this package,
and only as the checker or the timed CPU baseline; the product never does.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_QR_PATH = os.path.join(HERE, "_ref", "libmthqr_ref.so")

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_lib = None


class SizeInfo(ctypes.Structure):
    _fields_ = [("eps_star_norm2", _D), ("error_sum", _D), ("size_factor", _D), ("n_expanded", _I),
                ("fail_vertex", _I)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} missing: run `make -C oracle`")
    L = ctypes.CDLL(LIB_PATH)
    L.orc_box.argtypes = [_I, _I, _I, _D, _D, _D, ctypes.POINTER(_P)]
    L.orc_from_down.argtypes = [_I, _I, _P, _I, _P, _I, _P, _I, _P, ctypes.POINTER(_P)]
    L.orc_mesh_free.argtypes = [_P]
    L.orc_count.argtypes = [_P, _I]
    L.orc_dim.argtypes = [_P]
    for f in ["orc_coords", "orc_elem_verts", "orc_elem_edges", "orc_edge_verts", "orc_v2e_off", "orc_v2e"]:
        getattr(L, f).argtypes = [_P]
        getattr(L, f).restype = _P
    L.orc_down.argtypes = [_P, _I]
    L.orc_down.restype = _P
    L.orc_grad_ip.argtypes = [_P, _P, _I, _P]
    L.orc_recover.argtypes = [_P, _P, _I, _P, ctypes.POINTER(_I), ctypes.POINTER(_I)]
    L.orc_size_field.argtypes = [_P, _P, _I, _I, _D, _D, _D, _D, _P, _P, _P, _P, ctypes.POINTER(SizeInfo)]
    L.orc_measure_edges.argtypes = [_P, _P, _P, _P, _P]
    L.orc_mark_edges.argtypes = [_I, _P, _I, _P, ctypes.POINTER(ctypes.c_long)]
    L.orc_quality.argtypes = [_P, _P, _P, _P, _P]
    L.orc_estimate_and_mark.argtypes = [_P, _P, _D, _P, _P, _P, ctypes.POINTER(ctypes.c_long),
                                        ctypes.POINTER(ctypes.c_long), ctypes.POINTER(SizeInfo)]
    L.orc_qr_decompose.argtypes = [_I, _I, _P, _P, _P, _P]
    L.orc_qr_solve.argtypes = [_I, _I, _P, _P, _P]
    L.orc_set_threads.argtypes = [_I]
    L.orc_measure_pairs.argtypes = [_P, _I, _P, _P, _P, ctypes.c_long, _P, _P]
    L.orc_max_edge_length.argtypes = [_P, _I, _P, _P, _P]
    L.orc_max_edge_length.restype = _D
    L.orc_average_edge_length.argtypes = [_P]
    L.orc_average_edge_length.restype = _D
    L.orc_max_iterations.argtypes = [_D]
    L.orc_mark_bad_quality.argtypes = [_I, _P, _D, _P, ctypes.POINTER(ctypes.c_long)]
    L.orc_min_quality.argtypes = [_I, _P]
    L.orc_min_quality.restype = _D
    L.orc_eigen_qr3.argtypes = [_P, _P, _P, _I]
    L.orc_log_metric.argtypes = [_P, _P, _P, _P]
    L.orc_measure_edges_log.argtypes = [_P, _P, _P, _P]
    L.orc_quality_log.argtypes = [_P, _P, _P, _P]
    _lib = L
    return L


def set_threads(n):
    """OpenMP threads for the oracle's parallel loops; returns the count in use."""
    return load().orc_set_threads(int(n))


def _arr(ptr, shape, dtype):
    ct = {np.float64: ctypes.c_double, np.int32: ctypes.c_int}[dtype]
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), shape)


class OracleMesh:
    """MDS-semantics mesh built by the oracle (mds/mds.c, mds/apfBox.cc)."""

    def __init__(self, handle):
        self.L = load()
        self.h = handle
        self.dim = self.L.orc_dim(self.h)
        self.V = self.L.orc_count(self.h, 0)
        self.E = self.L.orc_count(self.h, 1)
        self.T = self.L.orc_count(self.h, self.dim)

    @classmethod
    def box(cls, nx, ny, nz, wx=1.0, wy=1.0, wz=1.0):
        h = _P()
        rc = load().orc_box(nx, ny, nz, wx, wy, wz if nz else 0.0, ctypes.byref(h))
        if rc:
            raise RuntimeError(f"orc_box failed: {rc}")
        return cls(h)

    def __del__(self):
        try:
            if self.h:
                self.L.orc_mesh_free(self.h)
        except Exception:
            pass

    @property
    def coords(self):
        """Writable view of the oracle's coordinates (V x 3)."""
        return _arr(self.L.orc_coords(self.h), (self.V, 3), np.float64)

    def set_coords(self, xyz):
        self.coords[:] = np.asarray(xyz, np.float64)

    @classmethod
    def from_down(cls, dim, coords, edges, faces, tets=None):
        """MDS mesh from downward adjacency: edges (E x 2 vertices), faces
        (F x 3 edges), tets (T x 4 faces, 3D)."""
        L = load()
        x = np.ascontiguousarray(coords, np.float64)
        e = np.ascontiguousarray(edges, np.int32)
        f = np.ascontiguousarray(faces, np.int32)
        t = np.ascontiguousarray(tets if tets is not None else np.zeros((0, 4)), np.int32)
        h = _P()
        rc = L.orc_from_down(dim, x.shape[0], x.ctypes.data, e.shape[0], e.ctypes.data, f.shape[0], f.ctypes.data,
                             t.shape[0], t.ctypes.data, ctypes.byref(h))
        if rc:
            raise RuntimeError(f"orc_from_down failed: {rc}")
        return cls(h)

    def down(self, d):
        """Stored downward adjacency of dimension d (one dimension down)."""
        n = self.L.orc_count(self.h, d)
        deg = {1: 2, 2: 3, 3: 4}[d]
        return _arr(self.L.orc_down(self.h, d), (n, deg), np.int32).copy()

    @property
    def elem_verts(self):
        return _arr(self.L.orc_elem_verts(self.h), (self.T, self.dim + 1), np.int32).copy()

    @property
    def elem_edges(self):
        return _arr(self.L.orc_elem_edges(self.h), (self.T, 6 if self.dim == 3 else 3), np.int32).copy()

    @property
    def edge_verts(self):
        return _arr(self.L.orc_edge_verts(self.h), (self.E, 2), np.int32).copy()

    @property
    def v2e_off(self):
        return _arr(self.L.orc_v2e_off(self.h), (self.V + 1,), np.int32).copy()

    @property
    def v2e(self):
        off = self.v2e_off
        return _arr(self.L.orc_v2e(self.h), (int(off[-1]),), np.int32).copy()

    # -- the path ---------------------------------------------------------
    def grad_ip(self, f):
        f = np.ascontiguousarray(f, np.float64)
        ncin = 1 if f.ndim == 1 else f.shape[1]
        out = np.empty((self.T, 3 * ncin), np.float64)
        rc = self.L.orc_grad_ip(self.h, f.ctypes.data, ncin, out.ctypes.data)
        assert rc == 0
        return out

    def recover(self, ip):
        ip = np.ascontiguousarray(ip, np.float64)
        out = np.empty((self.V, ip.shape[1]), np.float64)
        nexp, fail = _I(), _I()
        rc = self.L.orc_recover(self.h, ip.ctypes.data, ip.shape[1], out.ctypes.data, ctypes.byref(nexp),
                                ctypes.byref(fail))
        return rc, out, nexp.value, fail.value

    def size_field(self, ip, adapt_ratio=0.1, target=None, alpha=0.25, beta=2.0):
        """getSPRSizeField (target None) or getTargetSPRSizeField.  Returns
        (rc, size, rec, esize, err, info)."""
        ip = np.ascontiguousarray(ip, np.float64)
        nc = ip.shape[1]
        size = np.empty(self.V, np.float64)
        rec = np.empty((self.V, nc), np.float64)
        esize = np.empty(self.T, np.float64)
        err = np.empty(self.T, np.float64)
        info = SizeInfo()
        mode = 0 if target is None else 1
        rc = self.L.orc_size_field(self.h, ip.ctypes.data, nc, mode, float(adapt_ratio),
                                   float(target or 0), float(alpha), float(beta), size.ctypes.data,
                                   rec.ctypes.data, esize.ctypes.data, err.ctypes.data, ctypes.byref(info))
        return rc, size, rec, esize, err, info.as_dict()

    def measure(self, size=None, sizes=None, frames=None):
        L = np.empty(self.E, np.float64)
        s = None if size is None else np.ascontiguousarray(size, np.float64)
        ss = None if sizes is None else np.ascontiguousarray(sizes, np.float64)
        ff = None if frames is None else np.ascontiguousarray(frames, np.float64)
        self.L.orc_measure_edges(self.h, None if s is None else s.ctypes.data, None if ss is None else ss.ctypes.data,
                                 None if ff is None else ff.ctypes.data, L.ctypes.data)
        return L

    def quality(self, size=None, sizes=None, frames=None):
        q = np.empty(self.T, np.float64)
        s = None if size is None else np.ascontiguousarray(size, np.float64)
        ss = None if sizes is None else np.ascontiguousarray(sizes, np.float64)
        ff = None if frames is None else np.ascontiguousarray(frames, np.float64)
        self.L.orc_quality(self.h, None if s is None else s.ctypes.data, None if ss is None else ss.ctypes.data,
                           None if ff is None else ff.ctypes.data, q.ctypes.data)
        return q

    @staticmethod
    def _sf(size, sizes, frames, identity, log=False):
        """(kind, size, sizes, frames) arrays of a size field argument set."""
        c = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        if identity:
            return 0, None, None, None
        if sizes is not None:
            return (3 if log else 2), None, c(sizes), c(frames)
        return 1, c(size), None, None

    @staticmethod
    def _p(a):
        return None if a is None else a.ctypes.data

    def measure_pairs(self, pairs, size=None, sizes=None, frames=None, identity=False, log=False):
        kind, s, ss, ff = self._sf(size, sizes, frames, identity, log)
        pr = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        L = np.empty(pr.shape[0], np.float64)
        rc = self.L.orc_measure_pairs(self.h, kind, self._p(s), self._p(ss), self._p(ff), pr.shape[0],
                                      pr.ctypes.data, L.ctypes.data)
        if rc:
            raise ValueError("vertex id out of range")
        return L

    def log_metric(self, sizes, frames):
        """Per-vertex log-metric f diag(log(1/h^2)) f^T (V x 9)."""
        out = np.empty((self.V, 9))
        self.L.orc_log_metric(self.h, np.ascontiguousarray(sizes, np.float64).ctypes.data,
                              np.ascontiguousarray(frames, np.float64).ctypes.data, out.ctypes.data)
        return out

    def measure_log(self, sizes, frames):
        """Edge lengths under makeSizeField(m, sizes, frames, true); (rc, L)."""
        L = np.empty(self.E)
        rc = self.L.orc_measure_edges_log(self.h, np.ascontiguousarray(sizes, np.float64).ctypes.data,
                                          np.ascontiguousarray(frames, np.float64).ctypes.data, L.ctypes.data)
        return rc, L

    def quality_log(self, sizes, frames):
        q = np.empty(self.T)
        rc = self.L.orc_quality_log(self.h, np.ascontiguousarray(sizes, np.float64).ctypes.data,
                                    np.ascontiguousarray(frames, np.float64).ctypes.data, q.ctypes.data)
        return rc, q

    def max_edge_length(self, size=None, sizes=None, frames=None, identity=False, log=False):
        kind, s, ss, ff = self._sf(size, sizes, frames, identity, log)
        return self.L.orc_max_edge_length(self.h, kind, self._p(s), self._p(ss), self._p(ff))

    def average_edge_length(self):
        return self.L.orc_average_edge_length(self.h)

    def estimate_and_mark(self, u, adapt_ratio):
        """Returns (rc, size, L, flags, n_split, n_collapse, info)."""
        u = np.ascontiguousarray(u, np.float64)
        size = np.empty(self.V, np.float64)
        L = np.empty(self.E, np.float64)
        flags = np.zeros(self.E, np.int32)
        ns, nc = ctypes.c_long(), ctypes.c_long()
        info = SizeInfo()
        rc = self.L.orc_estimate_and_mark(self.h, u.ctypes.data, float(adapt_ratio), size.ctypes.data,
                                          L.ctypes.data, flags.ctypes.data, ctypes.byref(ns), ctypes.byref(nc),
                                          ctypes.byref(info))
        return rc, size, L, flags, ns.value, nc.value, info.as_dict()


def eigen_qr3(A, max_iters=100):
    """mth::eigenQR restated: (converged, L, Q); converged -1 when the
    Wilkinson shift's denominator vanishes (the reference asserts)."""
    A9 = np.ascontiguousarray(A, np.float64).reshape(9)
    L9, Q9 = np.empty(9), np.empty(9)
    rc = load().orc_eigen_qr3(A9.ctypes.data, L9.ctypes.data, Q9.ctypes.data, int(max_iters))
    return rc, L9.reshape(3, 3), Q9.reshape(3, 3)


def max_iterations(max_metric_length):
    return int(load().orc_max_iterations(float(max_metric_length)))


def mark_bad_quality(q, good, flags):
    """markBadQuality on given qualities; returns (rc, count); flags updated in place."""
    qa = np.ascontiguousarray(q, np.float64)
    c = ctypes.c_long()
    rc = load().orc_mark_bad_quality(qa.shape[0], qa.ctypes.data, float(good), flags.ctypes.data, ctypes.byref(c))
    return rc, c.value


def min_quality(q):
    qa = np.ascontiguousarray(q, np.float64)
    return load().orc_min_quality(qa.shape[0], qa.ctypes.data)


def mark_edges(L, which, flags):
    """markEntities on given lengths; returns (rc, count); flags updated in place."""
    Lh = load()
    Larr = np.ascontiguousarray(L, np.float64)
    c = ctypes.c_long()
    rc = Lh.orc_mark_edges(Larr.shape[0], Larr.ctypes.data, which, flags.ctypes.data, ctypes.byref(c))
    return rc, c.value


def qr_decompose(A):
    A = np.ascontiguousarray(A, np.float64)
    m, n = A.shape
    Q = np.empty((m, m)); R = np.empty((m, n)); v = np.empty(m)
    rank = load().orc_qr_decompose(m, n, A.ctypes.data, Q.ctypes.data, R.ctypes.data, v.ctypes.data)
    return rank, Q, R


def qr_solve(A, b):
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    m, n = A.shape
    x = np.zeros(n)
    rank = load().orc_qr_solve(m, n, A.ctypes.data, b.ctypes.data, x.ctypes.data)
    return rank, x


def ref_qr():
    """The reference's own mth QR compiled from source (oracle/_ref), or None."""
    if not os.path.exists(REF_QR_PATH):
        return None
    L = ctypes.CDLL(REF_QR_PATH)
    L.ref_qr_decompose.argtypes = [_I, _I, _P, _P, _P]
    L.ref_qr_solve.argtypes = [_I, _I, _P, _P, _P]
    L.ref_eigen_qr3.argtypes = [_P, _P, _P, _I]
    L.ref_apf_eigen.argtypes = [_P, _P, _P]
    return L
