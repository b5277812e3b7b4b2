"""The no-allocation size-field entry point against the allocating one.

sprg_spr_size_from_recovered_noalloc serves callers that cannot allocate
device memory (a code whose memory manager owns the device heap, or a thread
that cannot take the synchronisation an allocation may imply): it keeps its
scratch in a fixed device array instead.  Its sizes must equal those of
sprg_get_spr_size_field on the same integration-point and recovered fields,
on two calls in a row (the shared scratch keeps the previous call's
contents), and meshes above SPRG_NOALLOC_MAX_ELEMS must be rejected.
This file sorts last so a stop-at-first-failure run has run everything else.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


def ascending_adjacency(ev, V):
    """Vertex -> element CSR in ascending element order (what the context builds)."""
    T, nn = ev.shape
    verts = ev.reshape(-1)
    elems = np.repeat(np.arange(T, dtype=np.int32), nn)
    order = np.lexsort((elems, verts))
    off = np.zeros(V + 1, np.int32)
    np.cumsum(np.bincount(verts, minlength=V), out=off[1:])
    return off, elems[order].astype(np.int32)


CASES = [  # (dim, field components in, ip components)
    (3, 1, 3),   # tets, scalar field -> vector ip field
    (2, 1, 3),   # triangles
    (3, 3, 9),   # tets, vector field -> matrix ip field
]


@pytest.mark.parametrize("dim,ncin,ncomp", CASES)
def test_noalloc_size_field_matches_allocating_entry(gpu_lib, dim, ncin, ncomp):
    import torch
    import core_gb300 as cg
    from core_gb300 import _lib, workload
    lib = gpu_lib
    m = workload.box(10 if dim == 3 else 24, nz=None if dim == 3 else 0, jitter=0.2, seed=21)
    u = workload.bump_field(m.coords, seed=21)
    f = u if ncin == 1 else np.stack([u, workload.bump_field(m.coords, seed=22), np.sin(3 * m.coords[:, 0])], 1)
    with cg.Context(m) as ctx:
        ip = ctx.getGradIPField(f)
        assert ip.shape[1] == ncomp
        rec = ctx.recoverField(ip)
        size_ref, info = ctx.getSPRSizeField(ip, 0.1)
    off, adj = ascending_adjacency(m.elem_verts, m.n_verts)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)

    def dput(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    d_xyz, d_ev, d_off, d_adj, d_ip, d_rec = (dput(a) for a in (m.coords, m.elem_verts, off, adj, ip, rec))
    d_size = torch.empty(m.n_verts, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    free = []
    for call in range(2):
        d_size.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        free.append(torch.cuda.mem_get_info(dev)[0])
        sf = ctypes.c_double(0.0)
        rc = lib.sprg_spr_size_from_recovered_noalloc(
            dim, m.n_verts, m.n_elems, d_xyz.data_ptr(), d_ev.data_ptr(), d_off.data_ptr(), d_adj.data_ptr(),
            d_ip.data_ptr(), ncomp, d_rec.data_ptr(), 0.1, d_size.data_ptr(), ctypes.byref(sf),
            ctypes.c_void_p(stream.cuda_stream))
        assert rc == _lib.SPRG_OK, call
        stream.synchronize()
        size = d_size.cpu().numpy()
        assert np.all(np.isfinite(size))
        assert np.abs(size - size_ref).max() <= TOL * np.abs(size_ref).max(), call
        assert abs(sf.value - info["size_factor"]) <= TOL * abs(info["size_factor"]), call
    # the second call commits no device memory (the first one may load the
    # library's module and with it the fixed array)
    torch.cuda.synchronize(dev)
    assert torch.cuda.mem_get_info(dev)[0] == free[1]

    # beyond the fixed scratch: rejected before any device work
    rc = lib.sprg_spr_size_from_recovered_noalloc(
        dim, m.n_verts, _lib.NOALLOC_MAX_ELEMS + 1, d_xyz.data_ptr(), d_ev.data_ptr(), d_off.data_ptr(),
        d_adj.data_ptr(), d_ip.data_ptr(), ncomp, d_rec.data_ptr(), 0.1, d_size.data_ptr(), None, None)
    assert rc == _lib.SPRG_EINVAL
