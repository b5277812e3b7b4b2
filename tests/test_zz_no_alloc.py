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


def test_noalloc_size_field_matches_allocating_entry(gpu_lib):
    import torch
    import core_gb300 as cg
    from core_gb300 import _lib, workload
    lib = gpu_lib
    m = workload.box(10, jitter=0.2, seed=21)
    u = workload.bump_field(m.coords, seed=21)
    with cg.Context(m) as ctx:
        ip = ctx.getGradIPField(u)
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
    for call in range(2):
        d_size.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        sf = ctypes.c_double(0.0)
        rc = lib.sprg_spr_size_from_recovered_noalloc(
            3, m.n_verts, m.n_elems, d_xyz.data_ptr(), d_ev.data_ptr(), d_off.data_ptr(), d_adj.data_ptr(),
            d_ip.data_ptr(), 3, d_rec.data_ptr(), 0.1, d_size.data_ptr(), ctypes.byref(sf),
            ctypes.c_void_p(stream.cuda_stream))
        assert rc == _lib.SPRG_OK, call
        stream.synchronize()
        size = d_size.cpu().numpy()
        assert np.all(np.isfinite(size))
        assert np.abs(size - size_ref).max() <= TOL * np.abs(size_ref).max(), call
        assert abs(sf.value - info["size_factor"]) <= TOL * abs(info["size_factor"]), call

    # beyond the fixed scratch: rejected before any device work
    rc = lib.sprg_spr_size_from_recovered_noalloc(
        3, m.n_verts, _lib.NOALLOC_MAX_ELEMS + 1, d_xyz.data_ptr(), d_ev.data_ptr(), d_off.data_ptr(),
        d_adj.data_ptr(), d_ip.data_ptr(), 3, d_rec.data_ptr(), 0.1, d_size.data_ptr(), None, None)
    assert rc == _lib.SPRG_EINVAL
