"""Generates tests/golden/ref_path.npz: outputs of the reference's own
estimate-and-mark path (oracle/_ref/libspr_ref.so, compiled from the
SCOREC/core sources by `make -C oracle refall REF=<tree>`) on the cases of
tests/refcases.py:REF_CASES.  The GPU tests compare the CUDA path with these
numbers on a host that has no reference tree.

Per case (keys "<case>__<name>"): the mesh in the reference's MDS numbering
(coords, elem_verts, edge_verts, and v2e_off / v2e: getAdjacent(v, dim) in
the reference's order), the inputs (u and adapt ratio, or target; sizes and
frames for the anisotropic cases) and the outputs: ip (getGradIPField), rec
(recoverField), size (getSPRSizeField / getTargetSPRSizeField), lengths
(SizeField::measure), flags (ma_flags after markEdgesToCollapse then
markEdgesToSplit), n_split / n_collapse, quality (measureElementQuality).

Usage: python tests/golden/make_ref_golden.py   (after building oracle/_ref)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle import reference  # noqa: E402
from refcases import REF_CASES, field, jitter_coords, random_metric, shuffled_box, shuffled_box_smb  # noqa: E402


def run_case(name, kind, p, tmpdir):
    out = {}
    if kind == "shuffled":
        path = os.path.join(tmpdir, "mesh0.smb")
        shuffled_box_smb(oracle, path, p["n"], p["seed"])
        r = reference.RefMesh.load_smb(os.path.join(tmpdir, "mesh.smb"))
        x, ev, ed = r.mesh()
    else:
        r = reference.RefMesh.box(p["n"], p["n"], p["nz"])
        x, ev, ed = r.mesh()
        if p["jitter"]:
            x = jitter_coords(x, p["n"], p["nz"], p["jitter"], p["seed"])
            r.set_coords(x)
    off, v2e = r.vert_elems()
    out.update(coords=x, elem_verts=ev, edge_verts=ed, v2e_off=off, v2e=v2e)
    if kind == "aniso":
        sizes, frames = random_metric(r.V, p["seed"] + p["n"], 3 if p["nz"] else 2, lo=0.3 / p["n"], hi=3.0 / p["n"])
        L, fl, ns, nc, q = r.mark_aniso(sizes, frames, log=p["log"])
        out.update(sizes=sizes, frames=frames, log=int(p["log"]), lengths=L, flags=fl, n_split=ns, n_collapse=nc,
                   quality=q)
        return out
    u = field(p["field"], x, p["seed"])
    target = p.get("target")
    if target is not None:
        t = int(target * r.T)
        res = r.spr(u, target=t)
        out.update(target=t, alpha=0.25, beta=2.0)
    else:
        res = r.spr(u, p["ratio"])
        out.update(ratio=p["ratio"])
    L, fl, ns, nc, q = r.mark_iso(res["size"])
    out.update(u=u, ip=res["ip"], rec=res["rec"], size=res["size"], lengths=L, flags=fl, n_split=ns, n_collapse=nc,
               quality=q)
    return out


def main():
    import tempfile
    if not reference.available():
        sys.exit("oracle/_ref/libspr_ref.so is not built: make -C oracle refall REF=<SCOREC/core tree>")
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (kind, p) in REF_CASES.items():
            for k, v in run_case(name, kind, p, tmp).items():
                arrays[f"{name}__{k}"] = np.asarray(v)
            print(name, "ok")
    dst = os.path.join(HERE, "ref_path.npz")
    np.savez_compressed(dst, **arrays)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
