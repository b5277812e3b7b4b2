"""The C ABI's host-side behaviour, without a GPU: argument validation of
sprg_create before any device call, the null-context answers of every
context entry point, and the host write-back of the edge-mark bitmaps
(sprg_apply_marks) against the oracle's markEntities
(ma/maAdapt.cc:293-324) on given lengths."""
import ctypes

import numpy as np
import pytest

from core_gb300 import _lib
from core_gb300 import workload

SPLIT, DONT_SPLIT, COLLAPSE, DONT_COLLAPSE = 1, 2, 4, 8
NEED_NOT_SPLIT, NEED_NOT_COLLAPSE = 1 << 17, 1 << 18


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def _create(lib, view):
    out = ctypes.c_void_p(12345)
    rc = lib.sprg_create(ctypes.byref(view), 0, ctypes.byref(out))
    return rc, out.value


def _bad_views():
    """(name, mesh arrays kept alive, view) for each malformed input."""
    m = workload.box(2, jitter=0.0, seed=1)
    cases = []

    def add(name, **change):
        v = m.view()
        arrays = {}
        for k, val in change.items():
            if isinstance(val, np.ndarray):
                arrays[k] = val
                setattr(v, k, val.ctypes.data)
            else:
                setattr(v, k, val)
        cases.append((name, (m, arrays), v))

    add("dim 4", dim=4)
    add("dim 1", dim=1)
    add("no vertices", n_verts=0)
    add("no elements", n_elems=0)
    add("no edges", n_edges=0)
    add("null coords", coords=None)
    add("null elements", elem_verts=None)
    add("null edges", edge_verts=None)
    ev = m.elem_verts.copy()
    ev[3, 2] = m.n_verts
    add("element vertex out of range", elem_verts=ev)
    ev = m.elem_verts.copy()
    ev[0, 0] = -1
    add("negative element vertex", elem_verts=ev)
    ed = m.edge_verts.copy()
    ed[-1, 1] = m.n_verts + 7
    add("edge vertex out of range", edge_verts=ed)
    off = np.zeros(m.n_verts + 1, np.int32)
    add("offsets without the element list", vert_elem_offsets=off)
    nn = m.elem_verts.shape[1]
    order = np.argsort(m.elem_verts.ravel(), kind="stable")
    el = (order // nn).astype(np.int32)
    cnt = np.bincount(m.elem_verts.ravel(), minlength=m.n_verts)
    good = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    bad = good.copy()
    bad[-1] -= 1
    add("offsets not ending at T (dim+1)", vert_elem_offsets=bad, vert_elems=el)
    bad = good.copy()
    bad[2], bad[3] = bad[3], bad[2] - 1
    add("decreasing offsets", vert_elem_offsets=bad, vert_elems=el)
    el2 = el.copy()
    el2[5] = m.n_elems
    add("adjacent element out of range", vert_elem_offsets=good, vert_elems=el2)
    add("too many vertices", n_verts=1 << 31)
    return cases


@pytest.mark.parametrize("case", range(len(_bad_views())))
def test_create_rejects_malformed_views_before_any_device_call(lib, case):
    name, keep, view = _bad_views()[case]
    rc, ctx = _create(lib, view)
    assert rc == _lib.SPRG_EINVAL, name
    assert ctx is None, name


def test_create_without_output_pointer(lib):
    m = workload.box(1, jitter=0.0, seed=1)
    v = m.view()
    assert lib.sprg_create(ctypes.byref(v), 0, None) == _lib.SPRG_EINVAL


# every entry point whose first argument is the context
CTX_CALLS = [
    "sprg_set_precision", "sprg_set_stream", "sprg_get_grad_ip_field", "sprg_recover_field",
    "sprg_get_spr_size_field", "sprg_get_target_spr_size_field", "sprg_measure_edges",
    "sprg_measure_edges_aniso", "sprg_mark_edges", "sprg_measure_quality", "sprg_estimate_and_mark",
    "sprg_estimate_and_mark_resident", "sprg_profile_enable", "sprg_profile_flush", "sprg_debug_read",
    "sprg_set_mlp_params", "sprg_set_learned_options", "sprg_learned_features", "sprg_hessian_metric",
    "sprg_aniso_estimate_and_mark_resident", "sprg_set_batch", "sprg_batch_info", "sprg_set_autotune",
    "sprg_graph_capture", "sprg_graph_replay", "sprg_set_tiling", "sprg_measure_vertex_pairs",
    "sprg_get_maximum_edge_length", "sprg_get_average_edge_length", "sprg_mark_bad_quality",
    "sprg_get_min_quality", "sprg_measure_edges_log_aniso", "sprg_measure_quality_log_aniso",
    "sprg_update_mesh", "sprg_e2e_timing", "sprg_test_hooks", "sprg_rounding_dominated",
]


def _zero_args(fn):
    args = []
    for t in fn.argtypes:
        if t in (ctypes.c_int, ctypes.c_int64, ctypes.c_size_t, ctypes.c_long):
            args.append(0)
        elif t in (ctypes.c_double, ctypes.c_float):
            args.append(0.0)
        else:
            args.append(None)
    return args


@pytest.mark.parametrize("name", CTX_CALLS)
def test_null_context_is_einval(lib, name):
    fn = getattr(lib, name)
    assert fn.argtypes and fn.argtypes[0] is ctypes.c_void_p
    assert fn(*_zero_args(fn)) == _lib.SPRG_EINVAL


def test_null_context_queries(lib):
    assert lib.sprg_destroy(None) == _lib.SPRG_OK
    assert lib.sprg_last_error(None) == b"null context"
    assert lib.sprg_last_launch_count(None) == 0
    assert lib.sprg_profile_report(None, 0) == b"{}"
    assert lib.sprg_tuning_report(None) == b""
    assert lib.sprg_e2e_timing_report(None) == b"{}"
    assert lib.sprg_mlp_scratch_bytes(0) == 0
    assert lib.sprg_mlp_scratch_bytes(1000) > 0


def test_ctx_calls_cover_the_header():
    """Every exported symbol is either a context call above or one of the
    context-free entry points."""
    free = {"sprg_create", "sprg_destroy", "sprg_last_error", "sprg_last_launch_count", "sprg_apply_marks",
            "sprg_box_counts", "sprg_box_fill", "sprg_profile_report", "sprg_spr_size_from_recovered_noalloc",
            "sprg_mlp_scratch_bytes", "sprg_mlp_forward", "sprg_mlp_grad", "sprg_mlp_adam",
            "sprg_tuning_report", "sprg_max_iterations_for_length", "sprg_smb_counts", "sprg_smb_read",
            "sprg_smb_write", "sprg_e2e_timing_report", "sprg_locality_order"}
    assert set(CTX_CALLS) | free == set(_lib.EXPORTS)
    assert not set(CTX_CALLS) & free


# ---------------------------------------------------------------------------
# host write-back of the bitmaps
# ---------------------------------------------------------------------------
def _bitmap(mask):
    E = mask.shape[0]
    nw = (E + 31) // 32
    w = np.zeros(nw, np.uint32)
    idx = np.nonzero(mask)[0]
    np.bitwise_or.at(w, idx >> 5, (np.uint32(1) << (idx & 31).astype(np.uint32)))
    return w


def _prior_flags(rng, E):
    """MA flags an edge may carry before marking: the DONT_* and NEED_NOT_*
    bits of earlier passes and unrelated bits (BAD_QUALITY, OK_QUALITY)."""
    f = np.zeros(E, np.int32)
    for bit, p in ((DONT_SPLIT, 0.1), (DONT_COLLAPSE, 0.1), (NEED_NOT_SPLIT, 0.05),
                   (NEED_NOT_COLLAPSE, 0.05), (1 << 5, 0.2), (1 << 6, 0.2)):
        f |= np.where(rng.random(E) < p, bit, 0).astype(np.int32)
    return f


@pytest.mark.parametrize("E", [0, 1, 31, 32, 33, 1000, 4099])
def test_apply_marks_is_mark_entities(lib, oracle_lib, E):
    import core_gb300 as cg
    rng = np.random.default_rng(E + 3)
    L = rng.lognormal(0.0, 0.8, E)
    L[: E // 10] = np.repeat([0.5, 1.5], (E // 10 + 1) // 2)[: E // 10]  # the thresholds themselves
    flags0 = _prior_flags(rng, E)
    flags_o = flags0.copy()
    rc, ns_o = oracle_lib.mark_edges(L, 0, flags_o)
    assert rc == 0
    rc, nc_o = oracle_lib.mark_edges(L, 1, flags_o)
    assert rc == 0
    flags = flags0.copy()
    ns, nc = cg.apply_marks(_bitmap(L > 1.5), _bitmap(L < 0.5), flags)
    assert np.array_equal(flags, flags_o)
    assert (ns, nc) == (ns_o, nc_o)


def test_apply_marks_one_kind(lib, oracle_lib):
    import core_gb300 as cg
    rng = np.random.default_rng(11)
    E = 777
    L = rng.lognormal(0.0, 0.8, E)
    flags0 = _prior_flags(rng, E)
    for which, bits in ((0, (_bitmap(L > 1.5), None)), (1, (None, _bitmap(L < 0.5)))):
        flags_o = flags0.copy()
        rc, n_o = oracle_lib.mark_edges(L, which, flags_o)
        assert rc == 0
        flags = flags0.copy()
        ns, nc = cg.apply_marks(bits[0], bits[1], flags)
        assert np.array_equal(flags, flags_o)
        assert (ns if which == 0 else nc) == n_o and (nc if which == 0 else ns) == 0


@pytest.mark.parametrize("bit", [SPLIT, COLLAPSE])
def test_apply_marks_refuses_a_set_true_flag(lib, bit):
    """markEntities asserts that no edge carries the flag it sets
    (ma/maAdapt.cc:304); the write-back returns EFLAGS and changes nothing."""
    import core_gb300 as cg
    E = 100
    flags = np.zeros(E, np.int32)
    flags[37] = bit
    before = flags.copy()
    w = _bitmap(np.ones(E, bool))
    with pytest.raises(_lib.SprgError) as e:
        cg.apply_marks(w, w, flags)
    assert e.value.code == _lib.SPRG_EFLAGS
    assert np.array_equal(flags, before)


def test_apply_marks_arguments(lib):
    flags = np.zeros(4, np.int32)
    n = ctypes.c_long()
    assert lib.sprg_apply_marks(-1, None, None, flags.ctypes.data, ctypes.byref(n), ctypes.byref(n)) \
        == _lib.SPRG_EINVAL
    assert lib.sprg_apply_marks(4, None, None, None, ctypes.byref(n), ctypes.byref(n)) == _lib.SPRG_EINVAL
    assert lib.sprg_apply_marks(4, None, None, flags.ctypes.data, None, None) == _lib.SPRG_OK
    assert not flags.any()


def test_box_arguments(lib):
    V, T, E = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    for nx, ny, nz in ((0, 1, 1), (1, 0, 1), (1, 1, -1), (-3, 2, 2)):
        assert lib.sprg_box_counts(nx, ny, nz, ctypes.byref(V), ctypes.byref(T), ctypes.byref(E)) \
            == _lib.SPRG_EINVAL
    assert lib.sprg_box_counts(1, 1, 1, None, ctypes.byref(T), ctypes.byref(E)) == _lib.SPRG_EINVAL
    # counts past 32-bit ids are reported but the box is not built
    assert lib.sprg_box_counts(1024, 1024, 1024, ctypes.byref(V), ctypes.byref(T), ctypes.byref(E)) == _lib.SPRG_OK
    assert T.value == 6 * 1024 ** 3
    one = np.zeros(8, np.float64)
    assert lib.sprg_box_fill(1024, 1024, 1024, 1.0, 1.0, 1.0, one.ctypes.data, one.ctypes.data,
                             one.ctypes.data) == _lib.SPRG_EINVAL
    assert lib.sprg_box_fill(1, 1, 1, 1.0, 1.0, 1.0, None, None, None) == _lib.SPRG_EINVAL


def test_max_iterations_rule_host(lib):
    """updateMaxIterBasedOnSize (ma/maInput.cc:174-190): ceil(log2 L) + 1,
    and 10 once ceil(log2 L) reaches 10."""
    import math
    for L in (1.0000001, 1.5, 2.0, 2.5, 7.9, 64.0, 300.0, 511.0, 512.0, 513.0, 1e6):
        c = math.ceil(math.log2(L))
        want = 10 if c >= 10 else c + 1
        assert lib.sprg_max_iterations_for_length(L) == want, L
