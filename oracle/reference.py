"""The reference's own estimate-and-mark path -- TEST INFRASTRUCTURE ONLY.

Python binding of oracle/_ref/libspr_ref.so: SCOREC/core's pcu, gmi, apf,
mds, spr and ma compiled from their sources by ``make -C oracle refall
REF=<tree>`` and linked with oracle/ref_driver.cc.  It exists only where the
reference tree was present at build time (not on the GPU host).  Tests use it
to pin the oracle restatement and to generate the golden fixtures the GPU
tests compare against; bench.py may time it as the reference's CPU baseline.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libspr_ref.so")
TREE_FILE = os.path.join(HERE, "_ref", "REF_TREE")

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_D = ctypes.c_double
_lib = None


def available():
    return os.path.exists(LIB_PATH)


def tree():
    """The reference source tree the library was built from, or None."""
    try:
        with open(TREE_FILE) as f:
            t = f.read().strip()
        return t if os.path.isdir(t) else None
    except OSError:
        return None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not available():
        raise ImportError(f"{LIB_PATH} missing: run `make -C oracle refall REF=<SCOREC/core tree>`")
    L = ctypes.CDLL(LIB_PATH)
    L.refd_box.argtypes = [_I, _I, _I]
    L.refd_box.restype = _P
    L.refd_load.argtypes = [ctypes.c_char_p]
    L.refd_load.restype = _P
    L.refd_free.argtypes = [_P]
    L.refd_dim.argtypes = [_P]
    L.refd_count.argtypes = [_P, _I]
    L.refd_count.restype = _L
    L.refd_mesh.argtypes = [_P, _P, _P, _P]
    L.refd_vert_elems.argtypes = [_P, _P, _P]
    L.refd_set_coords.argtypes = [_P, _P]
    L.refd_spr.argtypes = [_P, _P, _I, _D, _L, _D, _D, _P, _P, _P, _P]
    L.refd_mark_iso.argtypes = [_P, _P, _P, _P, ctypes.POINTER(_L), ctypes.POINTER(_L), _P, _P]
    L.refd_mark_aniso.argtypes = [_P, _P, _P, _I, _P, _P, ctypes.POINTER(_L), ctypes.POINTER(_L), _P]
    L.refd_pass.argtypes = [_P, _P, _D, _P, _P, ctypes.POINTER(_L), ctypes.POINTER(_L), _P]
    _lib = L
    return L


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype)


def _p(a):
    return None if a is None else a.ctypes.data


class RefMesh:
    """An apf::Mesh2 built by the reference (apf::makeMdsBox or
    apf::loadMdsMesh), addressed by MDS index."""

    def __init__(self, handle):
        self.L = load()
        self.h = handle
        self.dim = self.L.refd_dim(self.h)
        self.V = self.L.refd_count(self.h, 0)
        self.E = self.L.refd_count(self.h, 1)
        self.T = self.L.refd_count(self.h, self.dim)

    @classmethod
    def box(cls, nx, ny, nz):
        """apf::makeMdsBox(nx, ny, nz, 1, 1, 1 (0 when nz = 0), true)."""
        return cls(load().refd_box(nx, ny, nz))

    @classmethod
    def load_smb(cls, path):
        return cls(load().refd_load(os.fsencode(path)))

    def __del__(self):
        try:
            if self.h:
                self.L.refd_free(self.h)
                self.h = None
        except Exception:
            pass

    def mesh(self):
        """(coords V x 3, elem_verts T x (dim + 1), edge_verts E x 2)."""
        x = np.empty((self.V, 3))
        ev = np.empty((self.T, self.dim + 1), np.int32)
        ed = np.empty((self.E, 2), np.int32)
        self.L.refd_mesh(self.h, x.ctypes.data, ev.ctypes.data, ed.ctypes.data)
        return x, ev, ed

    def vert_elems(self):
        """getAdjacent(v, dim) of every vertex as CSR (offsets, elements)."""
        off = np.empty(self.V + 1, np.int32)
        adj = np.empty(self.T * (self.dim + 1), np.int32)
        self.L.refd_vert_elems(self.h, off.ctypes.data, adj.ctypes.data)
        return off, adj[: off[-1]].copy()

    def set_coords(self, xyz):
        x = _c(xyz)
        assert x.shape == (self.V, 3)
        self.L.refd_set_coords(self.h, x.ctypes.data)

    def spr(self, u, adapt_ratio=0.1, target=None, alpha=0.25, beta=2.0, ip=True, rec=True, size=True):
        """getGradIPField(u) -> [recoverField] -> getSPRSizeField (target
        None) or getTargetSPRSizeField.  Returns a dict of the outputs asked
        for plus 'seconds' (gradient, recovery, size field)."""
        ua = _c(u)
        out = {}
        ip_o = np.empty((self.T, 3)) if ip else None
        rec_o = np.empty((self.V, 3)) if rec else None
        size_o = np.empty(self.V) if size else None
        sec = np.zeros(3)
        mode = 0 if target is None else 1
        rc = self.L.refd_spr(self.h, ua.ctypes.data, mode, float(adapt_ratio), int(target or 0), float(alpha),
                             float(beta), _p(ip_o), _p(rec_o), _p(size_o), sec.ctypes.data)
        assert rc == 0
        if ip:
            out["ip"] = ip_o
        if rec:
            out["rec"] = rec_o
        if size:
            out["size"] = size_o
        out["seconds"] = sec
        return out

    def mark_iso(self, size, quality=True):
        """configure(m, size) -> markEdgesToCollapse -> markEdgesToSplit.
        Returns (lengths, flags, n_split, n_collapse, quality or None)."""
        s = _c(size)
        Lg = np.empty(self.E)
        fl = np.empty(self.E, np.int32)
        q = np.empty(self.T) if quality else None
        ns, nc = _L(), _L()
        sec = np.zeros(4)
        self.L.refd_mark_iso(self.h, s.ctypes.data, Lg.ctypes.data, fl.ctypes.data, ctypes.byref(ns),
                             ctypes.byref(nc), _p(q), sec.ctypes.data)
        return Lg, fl, ns.value, nc.value, q

    def mark_aniso(self, sizes, frames, log=False, quality=True):
        """configure(m, sizes, frames, 0, log) -> the marks; as mark_iso."""
        s = _c(sizes)
        f = _c(frames)
        Lg = np.empty(self.E)
        fl = np.empty(self.E, np.int32)
        q = np.empty(self.T) if quality else None
        ns, nc = _L(), _L()
        self.L.refd_mark_aniso(self.h, s.ctypes.data, f.ctypes.data, 1 if log else 0, Lg.ctypes.data,
                               fl.ctypes.data, ctypes.byref(ns), ctypes.byref(nc), _p(q))
        return Lg, fl, ns.value, nc.value, q

    def estimate_and_mark(self, u, adapt_ratio):
        """The timed pass: (size, flags, n_split, n_collapse, seconds[4]:
        gradient, size field, configure, marks)."""
        ua = _c(u)
        size = np.empty(self.V)
        fl = np.empty(self.E, np.int32)
        ns, nc = _L(), _L()
        sec = np.zeros(4)
        self.L.refd_pass(self.h, ua.ctypes.data, float(adapt_ratio), size.ctypes.data, fl.ctypes.data,
                         ctypes.byref(ns), ctypes.byref(nc), sec.ctypes.data)
        return size, fl, ns.value, nc.value, sec
