"""The reference-side shim (core_gb300/shim/sprGB300.{h,cc}) compiled against
the reference's own headers and libraries (oracle/_ref/libshim_check.so, built
with the reference by `make -C oracle shim REF=<tree>`), on real apf::Mesh2
meshes.  CPU only: the shim's device calls need a GPU, which the hosts that
hold the reference tree lack, so this covers its host half.

* gb300::flatten gives the reference's own numbering (coordinates, element
  and edge vertices) and getAdjacent(v, dim) order, on boxes and on a .smb
  mesh with shuffled numbering;
* the ma_flags round trip of the shim's markEdgesTo* (gb300::readEdgeFlags,
  sprg_apply_marks with the bitmaps of the edge lengths, gb300::writeEdgeFlags)
  leaves exactly the flags and counts of the stock ma::markEdgesToCollapse then
  ma::markEdgesToSplit on an ma::Adapt, with and without prior DONT_* /
  NEED_NOT_* flags.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import reference
from refcases import bump, jitter_coords, shuffled_box_smb

LIB = os.path.join(os.path.dirname(reference.LIB_PATH), "libshim_check.so")
pytestmark = pytest.mark.skipif(not (reference.available() and os.path.exists(LIB)),
                                reason="shim check library not built (the reference tree is absent on this host)")

_P = ctypes.c_void_p


@pytest.fixture(scope="module")
def shim():
    L = ctypes.CDLL(LIB)
    L.shimchk_flatten_box.argtypes = [ctypes.c_int] * 3 + [_P] * 5
    L.shimchk_flatten_smb.argtypes = [ctypes.c_char_p, _P, _P, _P, _P, _P, _P]
    L.shimchk_marks.argtypes = [ctypes.c_int] * 3 + [_P] * 6
    return L


def flat_arrays(V, T, E, nn, nadj):
    return (np.empty((V, 3)), np.empty((T, nn), np.int32), np.empty((E, 2), np.int32),
            np.empty(V + 1, np.int32), np.empty(nadj, np.int32))


@pytest.mark.parametrize("n,nz", [(6, 6), (4, 7), (9, 0)])
def test_flatten_box_is_the_reference_numbering(shim, n, nz):
    r = reference.RefMesh.box(n, n + 1, nz)
    x, ev, ed = r.mesh()
    off, adj = r.vert_elems()
    out = flat_arrays(r.V, r.T, r.E, r.dim + 1, len(adj))
    shim.shimchk_flatten_box(n, n + 1, nz, *(a.ctypes.data for a in out))
    for got, want in zip(out, (x, ev, ed, off, adj)):
        assert np.array_equal(got, want)


def test_flatten_smb_with_shuffled_numbering(shim, oracle_lib, tmp_path):
    shuffled_box_smb(oracle_lib, str(tmp_path / "mesh0.smb"), 5, 17)
    path = str(tmp_path / "mesh.smb").encode()
    counts = np.zeros(5, np.int64)
    shim.shimchk_flatten_smb(path, counts.ctypes.data, None, None, None, None, None)
    dim, V, T, E, nadj = (int(c) for c in counts)
    out = flat_arrays(V, T, E, dim + 1, nadj)
    shim.shimchk_flatten_smb(path, counts.ctypes.data, *(a.ctypes.data for a in out))
    r = reference.RefMesh.load_smb(str(tmp_path / "mesh.smb"))
    x, ev, ed = r.mesh()
    off, adj = r.vert_elems()
    for got, want in zip(out, (x, ev, ed, off, adj)):
        assert np.array_equal(got, want)
    assert not np.array_equal(adj, np.sort(adj))  # the shuffle leaves the adjacency out of ascending order


SPLIT, DONT_SPLIT, COLLAPSE, DONT_COLLAPSE = 1, 2, 4, 8
NEED_NOT_SPLIT, NEED_NOT_COLLAPSE = 1 << 17, 1 << 18


@pytest.mark.parametrize("with_prior", [False, True])
@pytest.mark.parametrize("n,nz,ratio", [(8, 8, 0.1), (10, 10, 0.05), (16, 0, 0.01)])
def test_mark_round_trip_equals_stock_marks(shim, n, nz, ratio, with_prior):
    r = reference.RefMesh.box(n, n, nz)
    x = jitter_coords(r.mesh()[0], n, nz, 0.2, 3)
    r.set_coords(x)
    size = r.spr(bump(x, 3), ratio, ip=False, rec=False)["size"]
    prior = None
    if with_prior:
        rng = np.random.Generator(np.random.PCG64(n))
        prior = rng.choice(np.array([0, 0, 0, DONT_SPLIT, DONT_COLLAPSE, NEED_NOT_SPLIT, NEED_NOT_COLLAPSE,
                                     DONT_SPLIT | DONT_COLLAPSE], np.int32), size=r.E).astype(np.int32)
    fr = np.zeros(r.E, np.int32)
    fs = np.zeros(r.E, np.int32)
    counts = np.zeros(4, np.int64)
    rc = shim.shimchk_marks(n, n, nz, x.ctypes.data, size.ctypes.data, None if prior is None else prior.ctypes.data,
                            fr.ctypes.data, fs.ctypes.data, counts.ctypes.data)
    assert rc == 0
    assert np.array_equal(fs, fr)
    assert tuple(counts[:2]) == tuple(counts[2:])
    assert counts[0] > 0 and counts[1] > 0
