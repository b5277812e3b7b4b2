"""Failure paths, made on the host or by a bounded wait that runs out (no GPU
fault is provoked):

* the learned form's network kernel with its bounded waits cut to one poll:
  the pass returns SPRG_ECUDA after the kernel drained its tensor-core work
  and freed its tensor memory, and the next pass on the same context (limit
  restored) equals a fresh context's;
* a device allocation that fails (injected on the host) part-way through a
  context's first pass: SPRG_ENOMEM, and the next pass recovers;
* fields with NaN or infinite values: every form gives what the reference
  gives (NaN sizes; every edge NEED_NOT_SPLIT | NEED_NOT_COLLAPSE, no marks;
  the reference's own outputs checked by tests/test_reference_pin.py-style
  runs of the oracle), and the context stays usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NEED_NOT_BOTH = (1 << 17) | (1 << 18)


def case(n=10, seed=3):
    from core_gb300 import workload
    m = workload.box(n, jitter=0.2, seed=seed)
    return m, workload.bump_field(m.coords, seed=seed)


def fresh(m, u, precision):
    import core_gb300 as cg
    with cg.Context(m, precision=precision) as c:
        return c.estimate_and_mark(u, 0.1)[:4]


def same(a, b):
    return np.array_equal(a[0], b[0], equal_nan=True) and np.array_equal(a[1], b[1]) and a[2:] == b[2:]


def test_network_wait_that_runs_out(gpu_lib):
    import core_gb300 as cg
    m, u = case()
    with cg.Context(m, precision="learned") as c:
        c.test_hooks(wait_polls=64)
        with pytest.raises(cg.SprgError) as e:
            c.estimate_and_mark(u, 0.1)
        assert e.value.code == 5 and "ran out" in str(e.value)
        c.test_hooks(wait_polls=0)
        got = c.estimate_and_mark(u, 0.1)[:4]
    assert same(got, fresh(m, u, "learned"))


@pytest.mark.parametrize("precision", ["fp64", "fp32", "learned"])
@pytest.mark.parametrize("after", [0, 3, 9])
def test_allocation_failure(gpu_lib, precision, after):
    import core_gb300 as cg
    m, u = case(8)
    with cg.Context(m, precision=precision) as c:
        c.test_hooks(alloc_fail_after=after)
        try:
            c.estimate_and_mark(u, 0.1)
            failed = False
        except cg.SprgError as e:
            assert e.code == 4, e  # SPRG_ENOMEM
            failed = True
        c.test_hooks(alloc_fail_after=-1)
        got = c.estimate_and_mark(u, 0.1)[:4]
    assert failed or after > 0
    assert same(got, fresh(m, u, precision))


@pytest.mark.parametrize("precision", ["fp64", "fp32", "learned"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_nonfinite_field(gpu_lib, oracle_lib, precision, bad):
    import core_gb300 as cg
    m, u = case(6)
    ub = u.copy()
    ub[40] = bad
    o = oracle_lib.OracleMesh.box(6, 6, 6)
    o.set_coords(m.coords)
    rc, so, _, fo, nso, nco, _ = o.estimate_and_mark(ub, 0.1)
    assert rc == 0 and np.all(np.isnan(so)) and np.all(fo == NEED_NOT_BOTH) and (nso, nco) == (0, 0)
    with cg.Context(m, precision=precision) as c:
        s, f, ns, nc, _ = c.estimate_and_mark(ub, 0.1)
        assert np.all(~np.isfinite(s))
        assert np.array_equal(f, fo) and (ns, nc) == (0, 0)
        got = c.estimate_and_mark(u, 0.1)[:4]
    assert same(got, fresh(m, u, precision))
