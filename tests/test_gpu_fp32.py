"""The FP32 path (SPRG_FP32) against the oracle and the FP64 path.

Stated tolerances of the FP32 path (FP32 arithmetic with compensated
gradient deviations, FP64 global sums per warp, FP64 guard band):
  * size field: median of |s - s_ref| / s_ref <= 1e-6; at every
    vertex the error is within the bound the path carries for it (the
    q-weighted mean of its elements' bounds, large only where |eps - eps*| is
    far below the gradient variation between neighbouring elements); edges
    whose length is within 2e-6 plus their end bounds of 0.5 / 1.5 are
    re-decided in FP64;
  * size factor: relative error <= 1e-7;
  * split/collapse marks: identical to the FP64 result (every edge within
    2e-6 of 0.5 or 1.5 in FP32 is re-decided in FP64 by the guard band);
  * repeated passes are bitwise identical.
Where the field is linear to within rounding over a patch, the element errors
are rounding noise in both precisions and so are the sizes: FP32 may give
+inf (a zero error, as the reference gives for err = 0) where FP64 gives a
large finite value.  Those vertices carry a lower bound of the FP64 size
instead (checked here); their edges are re-decided in FP64 only when that
bound leaves the length's interval touching 0.5 or 1.5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check_sizes(size, ref, bound):
    fin = np.isfinite(size) & np.isfinite(ref)
    rel = np.abs(size[fin] - ref[fin]) / np.abs(ref[fin])
    assert np.median(rel) <= 1e-6
    assert np.all(rel <= bound[fin] + 1e-6)
    # an infinite FP32 size carries the negated lower bound of the FP64 size
    inf = ~np.isfinite(size)
    assert np.all(bound[inf] <= 0) and np.all(ref[inf] >= -bound[inf])
    assert np.mean(fin) > 0.99


def pair(oracle_mod, n, seed):
    from core_gb300 import workload
    m = workload.box(n, jitter=0.2, seed=seed)
    u = workload.bump_field(m.coords, seed=seed)
    o = oracle_mod.OracleMesh.box(n, n, n)
    o.set_coords(m.coords)
    return m, u, o


@pytest.mark.parametrize("n,seed", [(12, 31), (24, 32), (40, 4)])
def test_fp32_against_oracle(gpu_lib, oracle_lib, n, seed):
    import core_gb300 as cg
    m, u, o = pair(oracle_lib, n, seed)
    ratio = 0.008 * n / 160  # the 160^3 workload's length-to-size regime
    rc, size_o, L_o, flags_o, ns_o, nc_o, info_o = o.estimate_and_mark(u, ratio)
    assert rc == 0
    with cg.Context(m, precision="fp32") as ctx:
        size, flags, ns, nc, info = ctx.estimate_and_mark(u, ratio)
        bound = ctx.debug_read("sz2", np.float32, 2 * m.n_verts)[1::2].astype(np.float64)
    check_sizes(size, size_o, bound)
    assert abs(info["size_factor"] - info_o["size_factor"]) <= 1e-7 * info_o["size_factor"]
    assert info["n_guard_unresolved"] == 0 and info["n_rounding_dominated"] == 0
    assert np.array_equal(flags, flags_o)
    assert (ns, nc) == (ns_o, nc_o)


@pytest.mark.parametrize("kind", ["constant", "offset", "zero"])
def test_rounding_dominated_fields_take_the_fp64_pass(gpu_lib, oracle_lib, kind):
    """Fields whose error integral is set by the reference's own FP64
    rounding (a constant field, whose IP gradients sum u_i grad N_i are
    rounding; a bump 1e15 times below its offset) or is zero: the FP32 host
    entry point finds the pass rounding-dominated, leaves the flags alone
    and runs the pass in FP64, so the marks are the reference's (the
    oracle's) all the same.  (An exactly linear field is rounding too, but
    there no summation order other than the reference's reproduces its
    marks, the FP64 recovery included.)"""
    import core_gb300 as cg
    from core_gb300 import workload
    n = 12
    m, u0, o = pair(oracle_lib, n, 3)
    u = {"constant": np.full(m.n_verts, 2.5), "offset": 1e6 + 1e-9 * u0, "zero": np.zeros(m.n_verts)}[kind]
    rc, size_o, L_o, flags_o, ns_o, nc_o, info_o = o.estimate_and_mark(u, 0.1)
    assert rc == 0
    prior = np.zeros(m.n_edges, np.int32)
    prior[::7] = 2  # DONT_SPLIT on some edges: kept through the rerun
    import torch
    with cg.Context(m, precision="fp32") as c:
        size, flags, ns, nc, info = c.estimate_and_mark(u, 0.1, flags=prior.copy())
        # the resident entry leaves the rerun to its caller, who can ask
        nw = (m.n_edges + 31) // 32
        d_u = torch.from_numpy(u).cuda()
        bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        c.estimate_and_mark_resident(d_u.data_ptr(), 0.1, bits.data_ptr(), bits.data_ptr() + 4 * nw)
        assert c.rounding_dominated()
    assert info["n_rounding_dominated"] == 1
    want = prior.copy()
    rc, _ = oracle_lib.mark_edges(L_o, 1, want)
    rc2, _ = oracle_lib.mark_edges(L_o, 0, want)
    assert rc == 0 and rc2 == 0
    assert np.array_equal(flags, want)


def test_fp32_matches_fp64_marks_and_is_deterministic(gpu_lib):
    import torch
    import core_gb300 as cg
    from core_gb300 import workload
    n = 64
    m = workload.box(n, jitter=0.2, seed=33)
    u = workload.bump_field(m.coords, seed=33)
    ratio = 0.008 * n / 160
    with cg.Context(m, precision="fp64") as c64:
        s64, f64, *_ = c64.estimate_and_mark(u, ratio)
    E = m.n_edges
    nw = (E + 31) // 32
    with cg.Context(m, precision="fp32") as c32:
        s32, f32, ns, nc, info = c32.estimate_and_mark(u, ratio)
        d_u = torch.from_numpy(u).cuda()
        bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        c32.set_stream(stream.cuda_stream)
        outs = []
        for _ in range(2):
            bits.zero_()
            c32.estimate_and_mark_resident(d_u.data_ptr(), ratio, bits.data_ptr(), bits.data_ptr() + 4 * nw)
            torch.cuda.synchronize()
            outs.append(bits.cpu().numpy().copy())
        sz2 = c32.debug_read("sz2", np.float32, 2 * m.n_verts)
        s32b, bound = sz2[0::2], sz2[1::2].astype(np.float64)
        assert not c32.rounding_dominated()
    assert info["n_rounding_dominated"] == 0
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(f32, f64)
    check_sizes(s32, s64, bound)
    assert np.array_equal(s32b.astype(np.float64), s32, equal_nan=True)
    assert not np.any(np.isnan(s32))


def test_learned_rejects_triangles(gpu_lib):
    """The learned form covers tets (SPRG_FP32 on triangles is the mixed
    anisotropic pass, tests/test_aniso2d.py)."""
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(8, nz=0)
    with pytest.raises(cg.SprgError):
        cg.Context(m, precision="learned")


def test_fp32_marks_bit_exact_at_128cube(gpu_lib):
    """The 128^3 parity workload: FP32 fits and sweeps with the FP64 guard
    give the FP64 path's marks bit for bit."""
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(128, jitter=0.2, seed=2)
    u = workload.bump_field(m.coords, seed=2)
    ratio = 0.008 * 128 / 160
    with cg.Context(m, precision="fp64") as c64:
        s64, f64, ns64, nc64, _ = c64.estimate_and_mark(u, ratio)
    with cg.Context(m, precision="fp32") as c32:
        s32, f32, ns32, nc32, info = c32.estimate_and_mark(u, ratio)
    assert np.array_equal(f32, f64) and (ns32, nc32) == (ns64, nc64)
    assert ns64 > 0 and nc64 > 0
    assert info["n_guard_unresolved"] == 0
    fin = np.isfinite(s32) & np.isfinite(s64)
    assert np.median(np.abs(s32[fin] - s64[fin]) / s64[fin]) <= 1e-6


def test_config2_against_the_oracle(gpu_lib, oracle_lib):
    """Config 2 at full size: the 128^3 jittered box (12.6M tets), FP64 and
    FP32 passes against the oracle (OpenMP, pinned bitwise to the
    reference): marks identical in both forms; FP64 sizes within 1e-9 where
    they are well conditioned (every adjacent element's deviation above
    1e-7 of the largest gradient; elsewhere the element error is rounding
    noise in any summation order), FP32 sizes within their carried bounds."""
    import os
    import core_gb300 as cg
    from core_gb300 import workload
    oracle_lib.set_threads(os.cpu_count() or 1)
    n = 128
    m, u, o = pair(oracle_lib, n, 2)
    ratio = 0.008 * n / 160
    rc, size_o, L_o, flags_o, ns_o, nc_o, info_o = o.estimate_and_mark(u, ratio)
    assert rc == 0 and ns_o > 0 and nc_o > 0
    with cg.Context(m, precision="fp64") as c64:
        s64, f64, ns64, nc64, _ = c64.estimate_and_mark(u, ratio)
    assert np.array_equal(f64, flags_o) and (ns64, nc64) == (ns_o, nc_o)
    from refcases import conditioned
    ip = o.grad_ip(u)
    rc, rec, _, _ = o.recover(ip)
    ok = conditioned(m.n_verts, m.elem_verts, ip, rec) & np.isfinite(size_o)
    assert ok.mean() > 0.9
    assert np.all(np.abs(s64[ok] - size_o[ok]) <= 1e-9 * size_o[ok])
    with cg.Context(m, precision="fp32") as c32:
        s32, f32, ns32, nc32, info = c32.estimate_and_mark(u, ratio)
        bound = c32.debug_read("sz2", np.float32, 2 * m.n_verts)[1::2].astype(np.float64)
    assert np.array_equal(f32, flags_o) and (ns32, nc32) == (ns_o, nc_o)
    assert info["n_guard_unresolved"] == 0
    check_sizes(s32, size_o, bound)


def test_fp32_flat_regions(gpu_lib, oracle_lib):
    """A narrow bump with no ramp: the field is flat to far below FP32's
    range over most of the box, so the element deviations there are tiny
    (scaled before they are squared) or read as exactly zero (size +inf with
    the negated lower bound of the FP64 size).  Marks identical to the
    oracle's; every finite FP32 size within its carried bound; every
    infinite one's lower bound below the oracle's size."""
    import core_gb300 as cg
    from core_gb300 import workload
    n = 24
    m = workload.box(n, jitter=0.2, seed=8)
    x = m.coords
    u = np.exp(-((x - 0.7) ** 2).sum(axis=1) / (2 * 0.06 ** 2))
    o = oracle_lib.OracleMesh.box(n, n, n)
    o.set_coords(x)
    ratio = 0.05
    rc, size_o, L_o, flags_o, ns_o, nc_o, _ = o.estimate_and_mark(u, ratio)
    assert rc == 0 and np.all(np.isfinite(size_o))
    with cg.Context(m, precision="fp32") as c:
        s, f, ns, nc, info = c.estimate_and_mark(u, ratio)
        bound = c.debug_read("sz2", np.float32, 2 * m.n_verts)[1::2].astype(np.float64)
    assert np.array_equal(f, flags_o) and (ns, nc) == (ns_o, nc_o)
    assert info["n_guard_unresolved"] == 0
    fin = np.isfinite(s)
    rel = np.abs(s[fin] - size_o[fin]) / size_o[fin]
    assert np.all(rel <= bound[fin] + 1e-6)
    inf = ~fin
    assert np.all(s[inf] > 0) and np.all(bound[inf] <= 0) and np.all(size_o[inf] >= -bound[inf])
    # tiny but nonzero deviations (scaled) give finite sizes far above the bump's
    assert np.sum(fin & (size_o > 1e3 * np.median(size_o))) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64", "learned"])
def test_host_entry_graph_replays_follow_the_field(gpu_lib, precision):
    """The host entry point replays its pass from a CUDA graph from the
    third call on; with the field changing between calls every result
    equals a fresh context's (nothing per pass is frozen into the graph)."""
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(24, jitter=0.2, seed=41)
    us = [workload.bump_field(m.coords, seed=s) for s in (41, 42, 43)]
    ratio = 0.008 * 24 / 160
    with cg.Context(m, precision=precision) as ctx:
        got = [ctx.estimate_and_mark(us[i % 3], ratio)[:4] for i in range(7)]
    want = []
    for i in range(3):
        with cg.Context(m, precision=precision) as fresh:
            want.append(fresh.estimate_and_mark(us[i], ratio)[:4])
    for i, g in enumerate(got):
        w = want[i % 3]
        assert np.array_equal(g[0], w[0], equal_nan=True)
        assert np.array_equal(g[1], w[1]) and g[2:] == w[2:]


@pytest.mark.gpu
def test_user_graph_replays_follow_the_field(gpu_lib):
    """sprg_graph_capture / sprg_graph_replay with new field values written
    into the captured input between replays: bits equal direct passes."""
    import torch
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(24, jitter=0.2, seed=44)
    us = [workload.bump_field(m.coords, seed=s) for s in (44, 45)]
    ratio = 0.008 * 24 / 160
    E = m.n_edges
    nw = (E + 31) // 32
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    d_u = torch.from_numpy(us[0]).cuda()
    bits = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
    ref = torch.zeros(2 * nw, dtype=torch.int32, device="cuda")
    with cg.Context(m, precision="fp32") as ctx, cg.Context(m, precision="fp32") as direct:
        ctx.set_stream(stream.cuda_stream)
        direct.set_stream(stream.cuda_stream)
        ctx.graph_capture(d_u.data_ptr(), ratio, bits.data_ptr(), bits.data_ptr() + 4 * nw)
        for i in range(4):
            d_u.copy_(torch.from_numpy(us[i % 2]))
            bits.zero_()
            ctx.graph_replay()
            direct.estimate_and_mark_resident(d_u.data_ptr(), ratio, ref.data_ptr(), ref.data_ptr() + 4 * nw)
            torch.cuda.synchronize()
            assert torch.equal(bits, ref)
    assert ref.any()
