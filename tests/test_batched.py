"""The batched workload: many uneven boxes in one context (disjoint union),
per-mesh size factors, FP32 with the FP64 guard band.

Each mesh of the batch gets the marks of its own FP64 pass and of the oracle
(identical) and its own size factor (within 1e-7 relative), and the batch
pass is bitwise repeatable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_per_mesh_passes(gpu_lib):
    import core_gb300 as cg
    from core_gb300 import workload
    from core_gb300.mesh import Mesh
    m, u, voff, eoff, doff, ns = workload.batch_boxes(24, seed=7, lo=4, hi=12)
    K = len(ns)
    ratios = np.full(K, 0.1)
    with cg.Context(m, precision="fp32") as c:
        c.set_batch(voff, eoff, ratios)
        size, flags, ns_, nc_, info = c.estimate_and_mark(u, 0.0 + 1.0)
        per = c.batch_info()
        size2, flags2, *_ = c.estimate_and_mark(u, 1.0)
    assert np.array_equal(flags, flags2) and np.array_equal(size, size2)
    for k in range(K):
        mk = Mesh(3, m.coords[voff[k]:voff[k + 1]], m.elem_verts[eoff[k]:eoff[k + 1]] - voff[k],
                  m.edge_verts[doff[k]:doff[k + 1]] - voff[k])
        with cg.Context(mk, precision="fp64") as c64:
            s64, f64, *_, i64 = c64.estimate_and_mark(u[voff[k]:voff[k + 1]], ratios[k])
        assert np.array_equal(flags[doff[k]:doff[k + 1]], f64), k
        assert abs(per[k, 2] - i64["size_factor"]) <= 1e-7 * i64["size_factor"]
        sk = size[voff[k]:voff[k + 1]]
        fin = np.isfinite(sk) & np.isfinite(s64)
        rel = np.abs(sk[fin] - s64[fin]) / s64[fin]
        assert np.median(rel) <= 1e-6


def test_batch_matches_the_oracle(gpu_lib, oracle_lib):
    """Meshes of a jittered batch against the oracle directly (the oracle is
    pinned to the reference): every mesh's marks identical to the oracle's,
    its size factor within 1e-7, its sizes within the bounds the FP32 path
    carries."""
    import core_gb300 as cg
    from core_gb300 import workload
    m, u, voff, eoff, doff, ns = workload.batch_boxes(12, seed=11, lo=4, hi=16, jitter=0.2)
    K = len(ns)
    ratios = np.linspace(0.02, 0.2, K)
    with cg.Context(m, precision="fp32") as c:
        c.set_batch(voff, eoff, ratios)
        size, flags, *_ = c.estimate_and_mark(u, 1.0)
        per = c.batch_info()
        bound = c.debug_read("sz2", np.float32, 2 * m.n_verts)[1::2].astype(np.float64)
    for k in range(K):
        n = int(ns[k])
        o = oracle_lib.OracleMesh.box(n, n, n)
        o.set_coords(m.coords[voff[k]:voff[k + 1]])
        assert np.array_equal(o.elem_verts, m.elem_verts[eoff[k]:eoff[k + 1]] - voff[k])
        rc, so, Lo, fo, nso, nco, io = o.estimate_and_mark(u[voff[k]:voff[k + 1]], ratios[k])
        assert rc == 0
        assert np.array_equal(flags[doff[k]:doff[k + 1]], fo), k
        assert abs(per[k, 2] - io["size_factor"]) <= 1e-7 * io["size_factor"], k
        sk, bk = size[voff[k]:voff[k + 1]], bound[voff[k]:voff[k + 1]]
        fin = np.isfinite(sk) & np.isfinite(so)
        rel = np.abs(sk[fin] - so[fin]) / so[fin]
        assert np.all(rel <= bk[fin] + 1e-6), k


def test_batch_rejects_bad_offsets(gpu_lib):
    import core_gb300 as cg
    from core_gb300 import workload
    m, u, voff, eoff, doff, ns = workload.batch_boxes(3, seed=1, lo=4, hi=5)
    with cg.Context(m, precision="fp32") as c:
        bad = voff.copy()
        bad[-1] -= 1
        with pytest.raises(cg.SprgError):
            c.set_batch(bad, eoff, np.full(3, 0.1))
    with cg.Context(m, precision="fp64") as c:
        c.set_batch(voff, eoff, np.full(3, 0.1))
        with pytest.raises(cg.SprgError):
            c.estimate_and_mark(u, 0.1)


def test_tilings_give_identical_bits(gpu_lib):
    import core_gb300 as cg
    from core_gb300 import workload
    m, u, voff, eoff, doff, ns = workload.batch_boxes(16, seed=9, lo=4, hi=24, jitter=0.2)
    ratios = np.full(len(ns), 0.05)
    runs = []
    report = None
    # lanes 0: one lane per vertex over the sliced copy of the patch lists
    for cfg in [None, ([4, 4, 4, 4], 256, 8), ([1, 1, 1, 1], 64, 4), ([2, 1, 4, 2], 1024, 16),
                ([0, 0, 0, 0], 256, 8), ([0, 2, 0, 1], 64, 16), ([4, 0, 1, 0], 1024, 4)]:
        with cg.Context(m, precision="fp32") as c:
            c.set_batch(voff, eoff, ratios)
            if cfg is not None:
                c.set_tiling(*cfg)
            size, flags, *_ = c.estimate_and_mark(u, 1.0)
            if cfg is None:
                report = c.tuning_report()
        runs.append((size, flags))
    for size, flags in runs[1:]:
        assert np.array_equal(size, runs[0][0], equal_nan=True) and np.array_equal(flags, runs[0][1])
    assert sum(report["bins"]) > 0 and len(report["lanes"]) == 4 and report["timings"]
    assert set(report["lanes"]) <= {0, 1, 2, 4}
    with cg.Context(m, precision="fp32") as c:
        with pytest.raises(cg.SprgError):
            c.set_tiling([0, 1, 1, 1], 48, 8)  # sliced tiles start on a slice of 32
        with pytest.raises(cg.SprgError):
            c.set_tiling([3, 1, 1, 1], 64, 8)


def test_graph_replay_matches_direct_passes(gpu_lib):
    import torch
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(20, jitter=0.2, seed=3)
    u1 = workload.bump_field(m.coords, seed=3)
    u2 = workload.bump_field(m.coords, seed=5)
    E = m.n_edges
    nw = (E + 31) // 32
    with cg.Context(m, precision="fp32") as c:
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        c.set_stream(stream.cuda_stream)
        d_u = torch.from_numpy(u1).cuda()
        bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
        ps, pc = bits.data_ptr(), bits.data_ptr() + 4 * nw
        direct = []
        for uu in (u1, u2):
            d_u.copy_(torch.from_numpy(uu))
            bits.zero_()
            c.estimate_and_mark_resident(d_u.data_ptr(), 0.001, ps, pc)
            torch.cuda.synchronize()
            direct.append(bits.cpu().numpy().copy())
        d_u.copy_(torch.from_numpy(u1))
        c.graph_capture(d_u.data_ptr(), 0.001, ps, pc)
        for uu, want in zip((u1, u2, u1), (direct[0], direct[1], direct[0])):
            d_u.copy_(torch.from_numpy(uu))
            bits.zero_()
            c.graph_replay()
            torch.cuda.synchronize()
            assert np.array_equal(bits.cpu().numpy(), want)


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["box", "batch"])
def test_bins_are_the_stable_class_order(gpu_lib, which):
    """The recovery's patch-size bins, built on the device (per-block class
    counts, host scan, ballot scatter): every bin (<= 8, <= 16, <= 32, more
    patch elements; listed patches left out) lists its vertices in ascending
    order, as a plain loop over the vertices would."""
    import core_gb300 as cg
    from core_gb300 import workload
    if which == "box":
        m = workload.box(37, jitter=0.2, seed=3)
        u = workload.bump_field(m.coords, seed=3)
    else:
        m, u, *_ = workload.batch_boxes(40, seed=5, lo=3, hi=14, jitter=0.2)
    with cg.Context(m, precision="fp32") as c:
        c.estimate_and_mark(u, 0.05)
        listed = c.debug_read("listed", np.uint8, m.n_verts)
        order = c.debug_read("bverts", np.int32, m.n_verts)
        bins = c.tuning_report()["bins"]
    cnt = np.bincount(m.elem_verts.reshape(-1), minlength=m.n_verts)
    cls = np.where(cnt <= 8, 0, np.where(cnt <= 16, 1, np.where(cnt <= 32, 2, 3)))
    cls[listed != 0] = 4
    want = np.concatenate([np.nonzero(cls == b)[0] for b in range(4)]).astype(np.int32)
    assert list(bins) == [int(np.sum(cls == b)) for b in range(4)]
    assert np.array_equal(order[:len(want)], want)
