"""The oracle against the reference's own outputs stored in
tests/golden/ref_path.npz (made by tests/golden/make_ref_golden.py from the
reference compiled from source).  Runs on any host: the fixture carries the
reference's numbers, so the oracle stays pinned where no reference tree
exists.  Everything must match bitwise: IP gradients, recovered field, size
field, edge lengths, qualities, ma_flags words and counts."""
import os

import numpy as np
import pytest

from refcases import REF_CASES

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_path.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def case_arrays(gold, name):
    pre = name + "__"
    return {k[len(pre):]: gold[k] for k in gold.files if k.startswith(pre)}


def oracle_mesh(oracle_lib, name, g):
    kind, p = REF_CASES[name]
    if kind == "shuffled":
        from refcases import shuffled_box
        coords, edges, faces, tets = shuffled_box(oracle_lib, p["n"], p["seed"])
        assert np.array_equal(coords, g["coords"])
        o = oracle_lib.OracleMesh.from_down(3, coords, edges, faces, tets)
    else:
        o = oracle_lib.OracleMesh.box(p["n"], p["n"], p["nz"])
        o.set_coords(g["coords"])
    assert np.array_equal(o.elem_verts, g["elem_verts"])
    assert np.array_equal(o.edge_verts, g["edge_verts"])
    assert np.array_equal(o.v2e_off, g["v2e_off"]) and np.array_equal(o.v2e, g["v2e"])
    return o


@pytest.mark.parametrize("name", sorted(REF_CASES))
def test_oracle_reproduces_reference_outputs(oracle_lib, gold, name):
    g = case_arrays(gold, name)
    o = oracle_mesh(oracle_lib, name, g)
    flags = np.zeros(o.E, np.int32)
    if REF_CASES[name][0] == "aniso":
        if int(g["log"]):
            rc, L = o.measure_log(g["sizes"], g["frames"])
            assert rc == 0
            rc, q = o.quality_log(g["sizes"], g["frames"])
            assert rc == 0
        else:
            L = o.measure(sizes=g["sizes"], frames=g["frames"])
            q = o.quality(sizes=g["sizes"], frames=g["frames"])
    else:
        ip = o.grad_ip(g["u"])
        assert np.array_equal(ip, g["ip"])
        rc, rec, _, _ = o.recover(ip)
        assert rc == 0 and np.array_equal(rec, g["rec"])
        if "target" in g:
            rc, size, *_ = o.size_field(ip, target=int(g["target"]), alpha=float(g["alpha"]), beta=float(g["beta"]))
        else:
            rc, size, *_ = o.size_field(ip, float(g["ratio"]))
        assert rc == 0 and np.array_equal(size, g["size"])
        L = o.measure(size)
        q = o.quality(size)
    assert np.array_equal(L, g["lengths"])
    assert np.array_equal(q, g["quality"])
    rc, nc = oracle_lib.mark_edges(L, 1, flags)
    rc2, ns = oracle_lib.mark_edges(L, 0, flags)
    assert rc == 0 and rc2 == 0
    assert np.array_equal(flags, g["flags"])
    assert (ns, nc) == (int(g["n_split"]), int(g["n_collapse"]))


def test_oracle_full_size_flags_digest(oracle_lib):
    """The oracle on the 128^3 jittered box (config 2, 12.6M tets) writes the
    reference's ma_flags words (SHA-256 digest and counts from
    tests/golden/ref_full_hashes.json, made by make_ref_hashes.py)."""
    import hashlib
    import json
    from refcases import bump, jitter_coords
    with open(os.path.join(os.path.dirname(__file__), "golden", "ref_full_hashes.json")) as f:
        g = json.load(f)["box128"]
    n = g["n"]
    oracle_lib.set_threads(os.cpu_count() or 1)
    o = oracle_lib.OracleMesh.box(n, n, n)
    x = jitter_coords(o.coords.copy(), n, n, 0.2, g["seed"])
    o.set_coords(x)
    rc, size, L, flags, ns, nc, info = o.estimate_and_mark(bump(x, g["seed"]), g["ratio"])
    assert rc == 0 and (ns, nc) == (g["n_split"], g["n_collapse"])
    assert hashlib.sha256(flags.astype("<i4").tobytes()).hexdigest() == g["flags_sha256"]
