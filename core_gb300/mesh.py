"""Flattened simplex meshes in MDS numbering (the host side of the flattener).

A :class:`Mesh` holds exactly what ``sprg_mesh_view`` carries: coordinates,
element vertices in ``getDownward(e, 0)`` order and edge vertices, all in
MDS index order, plus an optional vertex-to-element adjacency in the
reference's ``getAdjacent`` order.
"""
import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib


@dataclass
class Mesh:
    dim: int
    coords: np.ndarray            # V x 3 float64
    elem_verts: np.ndarray        # T x (dim+1) int32
    edge_verts: np.ndarray        # E x 2 int32
    v2e_off: Optional[np.ndarray] = None   # V+1 int32 (getAdjacent order), optional
    v2e: Optional[np.ndarray] = None
    grid: Optional[tuple] = None  # (nx, ny, nz) for boxes

    @property
    def n_verts(self):
        return self.coords.shape[0]

    @property
    def n_elems(self):
        return self.elem_verts.shape[0]

    @property
    def n_edges(self):
        return self.edge_verts.shape[0]

    def view(self):
        """A sprg_mesh_view over this mesh's arrays (kept alive by the mesh)."""
        self.coords = np.ascontiguousarray(self.coords, dtype=np.float64)
        self.elem_verts = np.ascontiguousarray(self.elem_verts, dtype=np.int32)
        self.edge_verts = np.ascontiguousarray(self.edge_verts, dtype=np.int32)
        v = _lib.MeshView()
        v.dim = self.dim
        v.n_verts = self.n_verts
        v.n_elems = self.n_elems
        v.n_edges = self.n_edges
        v.coords = self.coords.ctypes.data
        v.elem_verts = self.elem_verts.ctypes.data
        v.edge_verts = self.edge_verts.ctypes.data
        if self.v2e_off is not None:
            self.v2e_off = np.ascontiguousarray(self.v2e_off, dtype=np.int32)
            self.v2e = np.ascontiguousarray(self.v2e, dtype=np.int32)
            v.vert_elem_offsets = self.v2e_off.ctypes.data
            v.vert_elems = self.v2e.ctypes.data
        return v

    def boundary_vertices(self):
        """Boolean mask of vertices on the box boundary (boxes only)."""
        nx, ny, nz = self.grid
        V = self.n_verts
        i = np.arange(V)
        x = i % (nx + 1)
        y = (i // (nx + 1)) % (ny + 1)
        b = (x == 0) | (x == nx) | (y == 0) | (y == ny)
        if nz:
            z = i // ((nx + 1) * (ny + 1))
            b |= (z == 0) | (z == nz)
        return b


def box_counts(nx, ny, nz):
    lib = _lib.load()
    V, T, E = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    _lib.check(lib.sprg_box_counts(nx, ny, nz, ctypes.byref(V), ctypes.byref(T), ctypes.byref(E)))
    return V.value, T.value, E.value


def makeMdsBox(nx, ny, nz, wx=1.0, wy=1.0, wz=1.0):
    """Flattened apf::makeMdsBox(nx, ny, nz, wx, wy, wz, true) (mds/apfBox.cc:330).
    nz = 0 gives the 2D triangle box."""
    lib = _lib.load()
    V, T, E = box_counts(nx, ny, nz)
    dim = 3 if nz else 2
    coords = np.empty((V, 3), np.float64)
    ev = np.empty((T, dim + 1), np.int32)
    ed = np.empty((E, 2), np.int32)
    _lib.check(lib.sprg_box_fill(nx, ny, nz, float(wx), float(wy), float(wz) if nz else 0.0,
                                 coords.ctypes.data, ev.ctypes.data, ed.ctypes.data))
    return Mesh(dim, coords, ev, ed, grid=(nx, ny, nz))


def read_smb(path):
    """One part of an MDS .smb file (simplex meshes) as a flattened Mesh in
    MDS index order (sprg_smb_read)."""
    lib = _lib.load()
    dim = ctypes.c_int()
    V, T, E = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    p = str(path).encode()
    _lib.check(lib.sprg_smb_counts(p, ctypes.byref(dim), ctypes.byref(V), ctypes.byref(T), ctypes.byref(E)))
    coords = np.empty((V.value, 3), np.float64)
    ev = np.empty((T.value, dim.value + 1), np.int32)
    ed = np.empty((E.value, 2), np.int32)
    _lib.check(lib.sprg_smb_read(p, coords.ctypes.data, ev.ctypes.data, ed.ctypes.data))
    return Mesh(dim.value, coords, ev, ed)


def write_smb(mesh, path):
    """Write a flattened Mesh as one part of an MDS .smb file (sprg_smb_write)."""
    lib = _lib.load()
    view = mesh.view()
    _lib.check(lib.sprg_smb_write(str(path).encode(), ctypes.byref(view)))


def locality_order(mesh):
    """New index of every vertex, element and edge under the locality
    renumbering (sprg_locality_order: apf::reorderMdsMesh's breadth-first
    order on the flattened arrays)."""
    lib = _lib.load()
    vn = np.empty(mesh.n_verts, np.int32)
    tn = np.empty(mesh.n_elems, np.int32)
    en = np.empty(mesh.n_edges, np.int32)
    view = mesh.view()
    _lib.check(lib.sprg_locality_order(ctypes.byref(view), vn.ctypes.data, tn.ctypes.data, en.ctypes.data))
    return vn, tn, en


def reorder(mesh, vert_new=None, elem_new=None, edge_new=None):
    """The mesh renumbered (by default in locality order): rows moved to their
    new indices, ids mapped, every element's and edge's vertex order kept.
    The vertex-element adjacency keeps each vertex's element order (mapped),
    so the size average sums as on the original mesh; without one, the
    original mesh's ascending order is carried over.  Returns (mesh,
    vert_new, elem_new, edge_new); a field f on the original vertices is
    f_new[vert_new] = f, and a result r on the renumbered vertices maps back
    as r[vert_new]."""
    if vert_new is None:
        vert_new, elem_new, edge_new = locality_order(mesh)
    V, T = mesh.n_verts, mesh.n_elems
    coords = np.empty_like(mesh.coords)
    coords[vert_new] = mesh.coords
    ev = np.empty_like(mesh.elem_verts)
    ev[elem_new] = vert_new[mesh.elem_verts]
    ed = np.empty_like(mesh.edge_verts)
    ed[edge_new] = vert_new[mesh.edge_verts]
    if mesh.v2e_off is not None:
        off, adj = mesh.v2e_off, mesh.v2e
    else:
        verts = mesh.elem_verts.reshape(-1)
        elems = np.repeat(np.arange(T, dtype=np.int32), mesh.elem_verts.shape[1])
        o = np.lexsort((elems, verts))
        adj = elems[o].astype(np.int32)
        off = np.zeros(V + 1, np.int32)
        np.cumsum(np.bincount(verts, minlength=V), out=off[1:])
    cnt = np.diff(off)
    old_of = np.empty(V, np.int64)
    old_of[vert_new] = np.arange(V)
    new_cnt = cnt[old_of]
    new_off = np.zeros(V + 1, np.int32)
    np.cumsum(new_cnt, out=new_off[1:])
    rows = np.repeat(old_of, new_cnt)
    pos = np.arange(new_off[-1]) - np.repeat(new_off[:-1], new_cnt)
    new_adj = elem_new[adj[off[rows] + pos]].astype(np.int32)
    return Mesh(mesh.dim, coords, ev, ed, v2e_off=new_off, v2e=new_adj), vert_new, elem_new, edge_new
