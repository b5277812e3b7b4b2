"""Generates the golden fixtures under tests/golden/ (run in a tree that has
the reference checkout; the fixtures are committed so nothing at test time
reads the reference).

  qr_kat.json     the 16x10 known-answer system of the reference's own QR
                  test (test/qr.cc:9-44), read from that file as text.
  qr_ref.npz      outputs of the reference's mth::decomposeQR / solveFromQR
                  (mth/mthQR.cc, compiled from source into oracle/_ref by
                  `make -C oracle ref`) on seeded SPR-shaped patch matrices,
                  including exactly rank-deficient ones.
  eigen_ref.npz   outputs of the reference's mth::eigenQR (100 iterations)
                  and apf::eigen (mth/mthQR.cc, apf/apfMatrix.cc compiled
                  from source into oracle/_ref) on seeded symmetric 3x3
                  matrices: log-metrics of random sizes and frames, their
                  edge-midpoint blends, repeated eigenvalues, diagonal ones.
  box8_oracle.npz oracle outputs of the 8^3 sine-field pass (regression
                  fixture of the oracle itself, not a reference output).

Usage: python tests/golden/make_golden.py <SCOREC/core source tree>
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def extract_kat(ref):
    src = open(os.path.join(ref, "test", "qr.cc")).read()
    num = r"[-+]?\d+\.\d+e[-+]\d+"
    a_blk = re.search(r"a_data\[16\]\[10\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    x_blk = re.search(r"x_data\[10\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    a = [float(t) for t in re.findall(num, a_blk)]
    x = [float(t) for t in re.findall(num, x_blk)]
    assert len(a) == 160 and len(x) == 10
    return {"source": "test/qr.cc:9-44 (SCOREC/core)", "tolerance": 1e-15,
            "a": np.array(a).reshape(16, 10).tolist(), "x": x}


def patch_matrices(seed=7):
    """SPR-shaped least-squares systems: rows [1, x, y, z] (or [1, x, y]) at
    integration points of a patch, right-hand sides of 3 components."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cases = []
    for k in range(60):
        n = 4 if k % 3 else 3
        m = int(rng.integers(n, 48))
        h = 10.0 ** rng.uniform(-3, 0)
        c = rng.uniform(0, 1, size=n - 1)
        pts = c + h * rng.uniform(-1, 1, size=(m, n - 1))
        if k % 10 == 0:      # exactly coplanar / collinear points: rank deficient
            pts[:, -1] = c[-1]
        if k % 10 == 5:      # nearly deficient, well above the 1e-10 threshold
            pts[:, -1] = c[-1] + 1e-7 * rng.uniform(-1, 1, size=m)
        A = np.hstack([np.ones((m, 1)), pts])
        b = rng.normal(size=(m, 3))
        cases.append((A, b))
    return cases


def eigen_matrices(seed=9, n=400):
    """Symmetric 3x3 matrices of the kinds a LogAnisoSizeField decomposes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        t = k % 5
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        lam = np.log(1.0 / np.exp(rng.uniform(np.log(1e-4), np.log(0.3), 3)) ** 2)
        if t == 0:
            A = q @ np.diag(lam) @ q.T
        elif t == 1:  # blend of two vertex log-metrics (an edge's Gauss point)
            q2, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            lam2 = np.log(1.0 / rng.uniform(1e-3, 0.2, 3) ** 2)
            w = rng.uniform(0, 1)
            A = w * (q @ np.diag(lam) @ q.T) + (1 - w) * (q2 @ np.diag(lam2) @ q2.T)
        elif t == 2:  # repeated eigenvalue
            lam[1] = lam[0]
            A = q @ np.diag(lam) @ q.T
        elif t == 3:  # 2D frames: rotation about z
            th = rng.uniform(0, np.pi)
            c, s_ = np.cos(th), np.sin(th)
            f = np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1.0]])
            A = f @ np.diag(lam) @ f.T
        else:
            A = np.diag(lam)
        out.append(np.ascontiguousarray(0.5 * (A + A.T)))
    return out


def main(ref):
    import oracle
    os.makedirs(HERE, exist_ok=True)
    kat = extract_kat(ref)
    with open(os.path.join(HERE, "qr_kat.json"), "w") as f:
        json.dump(kat, f)
    L = oracle.ref_qr()
    if L is None:
        raise SystemExit("oracle/_ref/libmthqr_ref.so missing: run `make -C oracle ref`")
    out = {}
    cases = patch_matrices()
    kA = np.array(kat["a"])
    cases.append((kA, (kA @ np.array(kat["x"]))[:, None].repeat(3, axis=1)))
    for i, (A, b) in enumerate(cases):
        m, n = A.shape
        A = np.ascontiguousarray(A)
        Q = np.empty((m, m)); R = np.empty((m, n))
        rank = L.ref_qr_decompose(m, n, A.ctypes.data, Q.ctypes.data, R.ctypes.data)
        X = np.full((3, n), np.nan)
        for c in range(3):
            bc = np.ascontiguousarray(b[:, c])
            x = np.zeros(n)
            if L.ref_qr_solve(m, n, A.ctypes.data, bc.ctypes.data, x.ctypes.data) == n:
                X[c] = x
        out[f"A{i}"] = A; out[f"b{i}"] = b; out[f"Q{i}"] = Q; out[f"R{i}"] = R
        out[f"rank{i}"] = np.array(rank); out[f"x{i}"] = X
    out["n"] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, "qr_ref.npz"), **out)

    mats = eigen_matrices()
    A = np.array(mats)
    Ls, Qs, conv, vecs, vals = [], [], [], [], []
    for M in mats:
        L9, Q9, v9, w3 = np.empty(9), np.empty(9), np.empty(9), np.empty(3)
        conv.append(L.ref_eigen_qr3(M.ctypes.data, L9.ctypes.data, Q9.ctypes.data, 100))
        L.ref_apf_eigen(M.ctypes.data, v9.ctypes.data, w3.ctypes.data)
        Ls.append(L9.reshape(3, 3)); Qs.append(Q9.reshape(3, 3)); vecs.append(v9.reshape(3, 3)); vals.append(w3)
    np.savez_compressed(os.path.join(HERE, "eigen_ref.npz"), A=A, L=np.array(Ls), Q=np.array(Qs),
                        converged=np.array(conv), vecs=np.array(vecs), vals=np.array(vals))

    # oracle regression fixture for the 8^3 sine-field pass (config 1)
    from core_gb300 import workload
    m = oracle.OracleMesh.box(8, 8, 8)
    u = workload.sine_field(m.coords)
    ip = m.grad_ip(u)
    rc, size, rec, esize, err, info = m.size_field(ip, 0.1)
    assert rc == 0
    Lg = m.measure(size)
    flags = np.zeros(m.E, np.int32)
    oracle.mark_edges(Lg, 1, flags)
    oracle.mark_edges(Lg, 0, flags)
    q = m.quality(size)
    np.savez_compressed(os.path.join(HERE, "box8_oracle.npz"), u=u, ip=ip, rec=rec, size=size, esize=esize,
                        err=err, L=Lg, flags=flags, q=q, size_factor=info["size_factor"],
                        n_expanded=info["n_expanded"])
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPRG_REFERENCE_TREE")
    if not tree:
        sys.exit("usage: make_golden.py <SCOREC/core source tree>  (or set SPRG_REFERENCE_TREE)")
    main(tree)
