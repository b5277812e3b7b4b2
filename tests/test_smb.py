"""The .smb reader and writer (sprg_smb_counts / sprg_smb_read /
sprg_smb_write, host-only calls).

Files are written here in the layout of mds/mds_smb.c (big-endian, version
4: header, counts, downward connectivity, coordinates, parametric
coordinates, remotes, classification, tags, matches).  Pinning: the
downward adjacency the oracle's MDS box stores, read back, gives exactly the
element vertices of the flattened makeMdsBox; with the face lists of every
tet (and the edge lists of every triangle) shuffled, the element vertices
equal the oracle's independent restatement of MDS's derivation
(orc_from_down).  Mixed-element and malformed files are refused."""
import os
import struct

import numpy as np
import pytest

SMB_TYPES = 8  # vertex, edge, triangle, quad, hex, prism, pyramid, tet


def write_smb(path, dim, coords, edges, faces, tets=None, version=4, quads=0):
    V, E, F = len(coords), len(edges), len(faces)
    T = 0 if tets is None else len(tets)
    u = lambda a: struct.pack(f">{len(a)}I", *[int(x) for x in a])
    d = lambda a: struct.pack(f">{len(a)}d", *[float(x) for x in a])
    counts = [V, E, F, quads, 0, 0, 0, T]
    out = [u([0, version, dim, 1]), u(counts),
           u(np.ravel(edges)), u(np.ravel(faces)), u([0] * (4 * quads)), b"", b"", b"",
           u(np.ravel(tets) if T else []), d(np.ravel(coords))]
    if version >= 2:
        out.append(d([0.0] * (2 * V)))
    out.append(u([0]))                                        # remotes: no peers
    for n in counts:                                          # classification
        out.append(u([0] * (2 * n)))
    out.append(u([0]))                                        # no tags
    for _ in range(SMB_TYPES):
        out.append(b"")                                       # (tag sizes: none)
    for _ in range(SMB_TYPES):
        out.append(u([0]))                                    # matches: no peers
    with open(path, "wb") as f:
        f.write(b"".join(out))


@pytest.fixture(scope="module")
def host_lib():
    """The library (its .smb calls need no GPU)."""
    from core_gb300 import build
    build.build()
    import core_gb300
    return core_gb300.load()


@pytest.mark.parametrize("n,nz", [(3, 3), (4, 2), (5, 0)])
def test_box_read_back_matches_makeMdsBox(host_lib, oracle_lib, tmp_path, n, nz):
    from core_gb300.mesh import makeMdsBox, read_smb
    o = oracle_lib.OracleMesh.box(n, n, nz)
    dim = 3 if nz else 2
    path = tmp_path / "box0.smb"
    write_smb(path, dim, o.coords, o.down(1), o.down(2), o.down(3) if dim == 3 else None)
    m = read_smb(path)
    b = makeMdsBox(n, n, nz)
    assert m.dim == dim
    assert np.array_equal(m.coords, b.coords)
    assert np.array_equal(m.elem_verts, b.elem_verts) and np.array_equal(m.edge_verts, b.edge_verts)


@pytest.mark.parametrize("dim", [3, 2])
def test_shuffled_downward_lists_follow_mds_derivation(host_lib, oracle_lib, tmp_path, dim):
    from core_gb300.mesh import read_smb
    o = oracle_lib.OracleMesh.box(4, 3, 2 if dim == 3 else 0)
    rng = np.random.Generator(np.random.PCG64(3))
    edges, faces = o.down(1), o.down(2)
    tets = o.down(3) if dim == 3 else None
    if dim == 3:
        tets = np.array([rng.permutation(t) for t in tets], np.int32)
    faces = np.array([rng.permutation(f) for f in faces], np.int32)
    edges = np.array([rng.permutation(e) for e in edges], np.int32)
    path = tmp_path / "shuffled0.smb"
    write_smb(path, dim, o.coords, edges, faces, tets)
    m = read_smb(path)
    ref = oracle_lib.OracleMesh.from_down(dim, o.coords, edges, faces, tets)
    assert np.array_equal(m.elem_verts, ref.elem_verts)
    assert np.array_equal(m.edge_verts, edges)
    # the element vertices are still the elements' vertex sets
    assert np.array_equal(np.sort(m.elem_verts, axis=1), np.sort(o.elem_verts, axis=1))


def test_refused_files(host_lib, oracle_lib, tmp_path):
    from core_gb300 import _lib as K
    from core_gb300.mesh import read_smb
    o = oracle_lib.OracleMesh.box(2, 2, 2)
    good = tmp_path / "good0.smb"
    write_smb(good, 3, o.coords, o.down(1), o.down(2), o.down(3))
    read_smb(good)
    raw = good.read_bytes()
    cases = {}
    cases["truncated"] = raw[: len(raw) // 3]
    cases["version"] = raw[:4] + struct.pack(">I", 9) + raw[8:]
    bad_edges = o.down(1).copy()
    bad_edges[0, 0] = o.V  # a vertex id beyond the count
    for name, data in cases.items():
        p = tmp_path / f"{name}0.smb"
        p.write_bytes(data)
        with pytest.raises(K.SprgError) as ei:
            read_smb(p)
        assert ei.value.code == K.SPRG_EINVAL, name
    p = tmp_path / "badid0.smb"
    write_smb(p, 3, o.coords, bad_edges, o.down(2), o.down(3))
    with pytest.raises(K.SprgError):
        read_smb(p)
    p = tmp_path / "mixed0.smb"
    write_smb(p, 3, o.coords, o.down(1), o.down(2), o.down(3), quads=1)
    with pytest.raises(K.SprgError):
        read_smb(p)
    with pytest.raises(K.SprgError):
        read_smb(tmp_path / "missing0.smb")


@pytest.mark.gpu
def test_read_mesh_runs_the_pass(gpu_lib, oracle_lib, tmp_path):
    """A mesh read from a file runs the FP64 pass to the oracle's marks."""
    import core_gb300 as cg
    from core_gb300 import workload
    from core_gb300.mesh import read_smb
    o = oracle_lib.OracleMesh.box(6, 6, 6)
    jit = workload.box(6, jitter=0.2, seed=9).coords
    o.set_coords(jit)
    path = tmp_path / "jbox0.smb"
    write_smb(path, 3, o.coords, o.down(1), o.down(2), o.down(3))
    m = read_smb(path)
    u = workload.bump_field(m.coords, seed=9)
    rc, size_o, L_o, flags_o, ns_o, nc_o, _ = o.estimate_and_mark(u, 0.1)
    assert rc == 0
    with cg.Context(m) as ctx:
        size, flags, ns, nc, _ = ctx.estimate_and_mark(u, 0.1)
    assert np.array_equal(flags, flags_o) and (ns, nc) == (ns_o, nc_o)
    assert np.abs(size - size_o).max() <= 1e-10 * np.abs(size_o).max()


def parse_down(path):
    """The downward arrays of a simplex .smb file, parsed independently here."""
    b = open(path, "rb").read()
    u = lambda off, n: np.frombuffer(b, ">u4", n, off).astype(np.int64)
    _, version, dim, _ = u(0, 4)
    n = u(16, 8)
    off = 48
    edges = u(off, 2 * n[1]).reshape(-1, 2); off += 8 * n[1]
    faces = u(off, 3 * n[2]).reshape(-1, 3); off += 12 * n[2]
    tets = u(off, 4 * n[7]).reshape(-1, 4); off += 16 * n[7]
    coords = np.frombuffer(b, ">f8", 3 * n[0], off).reshape(-1, 3)
    return int(dim), coords, edges, faces, tets


@pytest.mark.parametrize("n,nz,jit", [(4, 3, 0.0), (5, 5, 0.2), (6, 0, 0.15)])
def test_writer_round_trip(host_lib, oracle_lib, tmp_path, n, nz, jit):
    from core_gb300 import workload
    from core_gb300.mesh import read_smb, write_smb
    m = workload.box(n, nz=nz, jitter=jit, seed=5)
    path = tmp_path / "out0.smb"
    write_smb(m, path)
    r = read_smb(path)
    assert r.dim == m.dim
    assert np.array_equal(r.coords, m.coords)
    assert np.array_equal(r.elem_verts, m.elem_verts) and np.array_equal(r.edge_verts, m.edge_verts)
    # the written downward adjacency through the oracle's MDS derivation
    dim, x, e, f, t = parse_down(path)
    o = oracle_lib.OracleMesh.from_down(dim, x, e, f, t if dim == 3 else None)
    assert np.array_equal(o.elem_verts, m.elem_verts)
    # counts: the faces are the element triangles (2D) or the box's triangles (3D)
    if dim == 3:
        nf = 6 * n * n * (n + 1) + 6 * n ** 3 if nz == n else None
        if nf is not None:
            assert len(f) == nf


def test_writer_refuses_inconsistent_meshes(host_lib, tmp_path):
    from core_gb300 import _lib as K, workload
    from core_gb300.mesh import Mesh, write_smb
    m = workload.box(3)
    bad = Mesh(3, m.coords, m.elem_verts, m.edge_verts[1:])  # an element edge missing from the edge list
    with pytest.raises(K.SprgError):
        write_smb(bad, tmp_path / "bad0.smb")
    dup = Mesh(3, m.coords, m.elem_verts, np.vstack([m.edge_verts, m.edge_verts[:1]]))
    with pytest.raises(K.SprgError):
        write_smb(dup, tmp_path / "dup0.smb")


def _required_bytes(o):
    """Header, counts, connectivity and coordinates of a tet file: the part
    the reader needs."""
    E, F, T = len(o.down(1)), len(o.down(2)), len(o.down(3))
    return 16 + 32 + 4 * (2 * E + 3 * F + 4 * T) + 24 * o.V


def test_counts_never_exceed_the_file(host_lib, oracle_lib, tmp_path):
    """A file whose counts announce more entities than it holds is refused
    by sprg_smb_counts, before a caller sizes arrays by them."""
    import ctypes
    from core_gb300 import _lib as K
    o = oracle_lib.OracleMesh.box(2, 2, 2)
    good = tmp_path / "good0.smb"
    write_smb(good, 3, o.coords, o.down(1), o.down(2), o.down(3))
    raw = bytearray(good.read_bytes())
    for slot, value in ((0, 50_000_000), (1, 90_000_000), (2, 7_000_000), (7, 99_999_999), (0, o.V + 1)):
        bad = bytearray(raw)
        bad[16 + 4 * slot: 20 + 4 * slot] = struct.pack(">I", value)
        p = tmp_path / f"count{slot}_{value}0.smb"
        p.write_bytes(bytes(bad))
        dim, V, T, E = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        rc = host_lib.sprg_smb_counts(str(p).encode(), ctypes.byref(dim), ctypes.byref(V), ctypes.byref(T),
                                      ctypes.byref(E))
        if value > 1000:
            assert rc == K.SPRG_EINVAL, (slot, value)
        else:
            # one more vertex than written: the file is still long enough
            # (its tail holds more than 24 bytes), the read must then refuse
            # or return a mesh whose ids stay in range
            assert rc in (K.SPRG_OK, K.SPRG_EINVAL)


def test_truncated_files(host_lib, oracle_lib, tmp_path):
    """Cut anywhere inside the part the reader needs, a file is refused; cut
    after it (parametric coordinates, remotes, classification, tags), it
    reads as the whole file does."""
    from core_gb300 import _lib as K
    from core_gb300.mesh import read_smb
    o = oracle_lib.OracleMesh.box(2, 1, 1)
    good = tmp_path / "good0.smb"
    write_smb(good, 3, o.coords, o.down(1), o.down(2), o.down(3))
    raw = good.read_bytes()
    need = _required_bytes(o)
    want = read_smb(good)
    rng = np.random.default_rng(5)
    cuts = sorted(set([0, 3, 16, 47, 48, need - 1, need, need + 1, len(raw) - 1]
                      + list(rng.integers(0, len(raw), 40))))
    for cut in cuts:
        p = tmp_path / f"cut{cut}0.smb"
        p.write_bytes(raw[:cut])
        if cut < need:
            with pytest.raises(K.SprgError) as ei:
                read_smb(p)
            assert ei.value.code == K.SPRG_EINVAL, cut
        else:
            got = read_smb(p)
            assert np.array_equal(got.elem_verts, want.elem_verts)
            assert np.array_equal(got.coords, want.coords)


def test_damaged_files_are_read_or_refused(host_lib, oracle_lib, tmp_path):
    """Bytes overwritten at random inside the part the reader needs: every
    read either returns an error code or a mesh whose ids stay in range."""
    from core_gb300 import _lib as K
    from core_gb300.mesh import read_smb
    o = oracle_lib.OracleMesh.box(2, 2, 1)
    good = tmp_path / "good0.smb"
    write_smb(good, 3, o.coords, o.down(1), o.down(2), o.down(3))
    raw = good.read_bytes()
    need = _required_bytes(o)
    rng = np.random.default_rng(9)
    refused = accepted = 0
    for trial in range(300):
        bad = bytearray(raw)
        for _ in range(int(rng.integers(1, 6))):
            pos = int(rng.integers(0, need))
            bad[pos] = int(rng.integers(0, 256))
        p = tmp_path / "damaged0.smb"
        p.write_bytes(bytes(bad))
        try:
            m = read_smb(p)
        except K.SprgError as e:
            assert e.code in (K.SPRG_EINVAL, K.SPRG_ENOMEM)
            refused += 1
            continue
        accepted += 1
        assert m.elem_verts.min() >= 0 and m.elem_verts.max() < m.n_verts
        assert m.edge_verts.min() >= 0 and m.edge_verts.max() < m.n_verts
    assert refused > 0 and accepted > 0
