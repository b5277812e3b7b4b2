"""The CUDA path against the reference's own outputs (tests/golden/ref_path.npz,
made from the reference compiled from source; see make_ref_golden.py), through
the C ABI, on the mesh in the reference's numbering and getAdjacent order.

FP64 form: IP gradients, edge lengths and qualities (measured on the
reference's size field) bitwise; recovered field within 1e-10 of its largest
value per component (the patch fits sum in another order); size field within
1e-9 relative at every vertex whose elements' errors are above the rounding
level (see `conditioned`); ma_flags words and counts of the whole pass
identical.  FP32 form (tets): flags identical (FP64 guard band); size within
1e-6 relative at the median vertex and, at every vertex, within the error
bound the path carries for it (plus 1e-6).  Anisotropic cases: lengths and qualities bitwise
(AnisoSizeField) or within 1e-10 (LogAnisoSizeField, device exp / log and
the eigen iteration), marks identical.
"""
import os

import numpy as np
import pytest

import refcases
from refcases import REF_CASES

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_path.npz")
pytestmark = pytest.mark.gpu


def case_mesh(name):
    from core_gb300.mesh import Mesh
    d = np.load(GOLD)
    pre = name + "__"
    g = {k[len(pre):]: d[k] for k in d.files if k.startswith(pre)}
    dim = g["elem_verts"].shape[1] - 1
    m = Mesh(dim, g["coords"], g["elem_verts"], g["edge_verts"], v2e_off=g["v2e_off"], v2e=g["v2e"])
    return m, g


def rel(a, b):
    """max |a - b| over max |b|, per component (the parity tests' measure)."""
    a2, b2 = np.atleast_2d(a.T).T, np.atleast_2d(b.T).T
    scale = np.maximum(np.abs(b2).max(axis=0), 1e-300)
    return float((np.abs(a2 - b2).max(axis=0) / scale).max())


def conditioned(m, g):
    return refcases.conditioned(m.n_verts, g["elem_verts"], g["ip"], g["rec"])


ISO = sorted(k for k, (kind, _) in REF_CASES.items() if kind != "aniso")
ANISO = sorted(k for k, (kind, _) in REF_CASES.items() if kind == "aniso")


@pytest.mark.parametrize("name", ISO)
def test_fp64_pass_matches_reference(gpu_lib, name):
    import core_gb300 as cg
    m, g = case_mesh(name)
    with cg.Context(m, device=0) as ctx:
        ip = ctx.getGradIPField(g["u"])
        assert np.array_equal(ip, g["ip"])
        rec = ctx.recoverField(ip)
        assert rel(rec, g["rec"]) <= 1e-10
        ok = conditioned(m, g)
        if "target" in g:
            size, _ = ctx.getTargetSPRSizeField(ip, int(g["target"]), float(g["alpha"]), float(g["beta"]))
        else:
            size, _ = ctx.getSPRSizeField(ip, float(g["ratio"]))
        r = np.abs(size - g["size"]) / np.abs(g["size"])
        assert np.all(r[ok] <= 1e-9), (r[ok].max(), ok.sum())
        assert ok.mean() > 0.5
        if "target" in g:
            return
        assert np.array_equal(ctx.measure_edges(g["size"]), g["lengths"])
        assert np.array_equal(ctx.measureQuality(size=g["size"]), g["quality"])
        s2, flags, ns, nc, _ = ctx.estimate_and_mark(g["u"], float(g["ratio"]))
        assert np.array_equal(flags, g["flags"])
        assert (ns, nc) == (int(g["n_split"]), int(g["n_collapse"]))


FP32 = [k for k in ISO if REF_CASES[k][1].get("nz", 1) and "target" not in REF_CASES[k][1]]


@pytest.mark.parametrize("name", FP32)
def test_fp32_pass_matches_reference_marks(gpu_lib, name):
    import core_gb300 as cg
    m, g = case_mesh(name)
    with cg.Context(m, device=0, precision="fp32") as ctx:
        for _ in range(2):  # the second call runs on the cached per-mesh data
            size, flags, ns, nc, info = ctx.estimate_and_mark(g["u"], float(g["ratio"]))
            assert np.array_equal(flags, g["flags"])
            assert (ns, nc) == (int(g["n_split"]), int(g["n_collapse"]))
            bound = ctx.debug_read("sz2", np.float32, 2 * m.n_verts)[1::2].astype(np.float64)
            fin = np.isfinite(size)
            r = np.abs(size[fin] - g["size"][fin]) / np.abs(g["size"][fin])
            assert np.median(r) <= 1e-6
            assert np.all(r <= bound[fin] + 1e-6)
            assert np.all(bound[~fin] <= 0) and np.all(g["size"][~fin] >= -bound[~fin])
            assert info["n_guard_unresolved"] == 0


@pytest.mark.parametrize("name", ANISO)
def test_aniso_measure_matches_reference(gpu_lib, name):
    import core_gb300 as cg
    m, g = case_mesh(name)
    with cg.Context(m, device=0) as ctx:
        if int(g["log"]):
            L = ctx.measure_edges_log_aniso(g["sizes"], g["frames"])
            q = ctx.measureQualityLog(g["sizes"], g["frames"])
            assert rel(L, g["lengths"]) <= 1e-10
            assert rel(q, g["quality"]) <= 1e-10
        else:
            L = ctx.measure_edges_aniso(g["sizes"], g["frames"])
            q = ctx.measureQuality(sizes=g["sizes"], frames=g["frames"])
            assert np.array_equal(L, g["lengths"])
            assert np.array_equal(q, g["quality"])
        flags = np.zeros(m.n_edges, np.int32)
        nc = ctx.markEdgesToCollapse(flags)
        ns = ctx.markEdgesToSplit(flags)
        assert np.array_equal(flags, g["flags"])
        assert (ns, nc) == (int(g["n_split"]), int(g["n_collapse"]))
