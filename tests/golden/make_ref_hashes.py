"""Generates tests/golden/ref_full_hashes.json: the reference's own marks on
the full-size jittered boxes (128^3, config 2: 12.6M tets; 160^3, the
benchmark box: 24.6M tets), as SHA-256 digests of the ma_flags words (int32,
little endian, MDS edge order) with the split / collapse counts, plus digests
of the inputs (coordinates and field, float64) so a test can check that it
feeds the same numbers.  The reference is the estimate-and-mark path
compiled from the SCOREC/core sources (oracle/_ref/libspr_ref.so, `make -C
oracle refall REF=<tree>`); one pass at 160^3 takes about six minutes on one
core.

Usage: python tests/golden/make_ref_hashes.py   (after building oracle/_ref)
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import reference  # noqa: E402
from refcases import bump, jitter_coords  # noqa: E402

CASES = {"box128": dict(n=128, seed=2, ratio=0.008 * 128 / 160), "box160": dict(n=160, seed=4, ratio=0.008)}


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).astype(np.dtype(a.dtype).newbyteorder("<")).tobytes()).hexdigest()


def main():
    if not reference.available():
        raise SystemExit("oracle/_ref/libspr_ref.so is not built")
    out = {}
    for name, p in CASES.items():
        n = p["n"]
        r = reference.RefMesh.box(n, n, n)
        x = jitter_coords(r.mesh()[0], n, n, 0.2, p["seed"])
        r.set_coords(x)
        u = bump(x, p["seed"])
        t0 = time.perf_counter()
        size, flags, ns, nc, sec = r.estimate_and_mark(u, p["ratio"])
        out[name] = dict(p, coords_sha256=digest(x), u_sha256=digest(u), flags_sha256=digest(flags.astype(np.int32)),
                         n_split=int(ns), n_collapse=int(nc), n_edges=int(flags.shape[0]),
                         size_min=float(np.min(size)), size_max=float(np.max(size)),
                         seconds=round(time.perf_counter() - t0, 1))
        print(name, json.dumps(out[name]), flush=True)
    with open(os.path.join(HERE, "ref_full_hashes.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
