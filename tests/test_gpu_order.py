"""The pass on a mesh with shuffled numbering and on its locality-renumbered
copy (core_gb300.mesh.reorder): marks identical edge for edge once mapped
back; FP64 sizes within 1e-9 relative wherever the elements' errors are above
the rounding level (the patch fits sum their rows in another order, which
moves rounding-noise errors), FP32 sizes within the stated error."""
import numpy as np
import pytest

from refcases import bump

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_renumbered_pass_gives_the_same_marks(gpu_lib, oracle_lib, precision):
    import core_gb300 as cg
    from core_gb300.mesh import reorder
    from test_gpu_reference import conditioned
    from test_order import shuffled_mesh
    m = shuffled_mesh(oracle_lib, 16, 7)
    u = bump(m.coords, 7)
    m2, vn, tn, en = reorder(m)
    u2 = np.empty_like(u)
    u2[vn] = u
    with cg.Context(m, precision=precision) as c1:
        s1, f1, ns1, nc1, _ = c1.estimate_and_mark(u, 0.1)
    with cg.Context(m) as c64:
        ip = c64.getGradIPField(u)
        g = {"elem_verts": m.elem_verts, "ip": ip, "rec": c64.recoverField(ip)}
    with cg.Context(m2, precision=precision) as c2:
        s2, f2, ns2, nc2, _ = c2.estimate_and_mark(u2, 0.1)
    assert np.array_equal(f2[en], f1)
    assert (ns2, nc2) == (ns1, nc1) and ns1 > 0 and nc1 > 0
    if precision == "fp64":
        ok = conditioned(m, g)
        assert ok.mean() > 0.5
        assert np.all(np.abs(s2[vn] - s1)[ok] <= 1e-9 * s1[ok])
    else:
        assert np.median(np.abs(s2[vn] - s1) / s1) <= 1e-6
