"""Pins the oracle against the reference's own known answers (CPU only).

* the QR known-answer test of the reference (test/qr.cc:46-61: solveQR on a
  16x10 Octave system, |x - x_known| < 1e-15), from tests/golden/qr_kat.json;
* bitwise equality with the reference's mth::decomposeQR / solveFromQR
  (mth/mthQR.cc compiled from source) on SPR-shaped patch systems, from
  tests/golden/qr_ref.npz, and live against oracle/_ref when it is built;
* the reference's recorded outcome of the 8^3 sine-field pass (every one of
  the 4184 edges marked for split, minimum tet quality 0.432 = mean-ratio
  cubed of the Kuhn tet).
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_qr_known_answer(oracle_lib):
    kat = json.load(open(os.path.join(GOLD, "qr_kat.json")))
    A = np.array(kat["a"])
    x_known = np.array(kat["x"])
    b = np.zeros(A.shape[0])
    for i in range(A.shape[0]):  # mth::multiply order: c(i) = 0; c(i) += a(i,j) b(j)
        s = 0.0
        for j in range(A.shape[1]):
            s += A[i, j] * x_known[j]
        b[i] = s
    rank, x = oracle_lib.qr_solve(A, b)
    assert rank == 10
    assert np.all(np.abs(x_known - x) < kat["tolerance"])


def test_qr_bitwise_against_reference_fixture(oracle_lib):
    d = np.load(os.path.join(GOLD, "qr_ref.npz"))
    n = int(d["n"])
    deficient = 0
    for i in range(n):
        A = d[f"A{i}"]
        rank, Q, R = oracle_lib.qr_decompose(A)
        assert rank == int(d[f"rank{i}"]), i
        assert np.array_equal(Q, d[f"Q{i}"]), i
        assert np.array_equal(R, d[f"R{i}"]), i
        deficient += rank < A.shape[1]
        for c in range(3):
            r, x = oracle_lib.qr_solve(A, d[f"b{i}"][:, c])
            if r == A.shape[1]:
                assert np.array_equal(x, d[f"x{i}"][c]), (i, c)
    assert deficient >= 5  # the fixture exercises the rank test


def test_qr_live_reference_build(oracle_lib):
    L = oracle_lib.ref_qr()
    if L is None:
        pytest.skip("oracle/_ref not built (reference tree absent on this host)")
    rng = np.random.Generator(np.random.PCG64(11))
    for k in range(40):
        m = int(rng.integers(4, 40))
        A = np.hstack([np.ones((m, 1)), rng.uniform(0, 1, (m, 3)) * 10.0 ** rng.uniform(-4, 0)])
        if k % 4 == 0:
            A[:, 3] = 0.25
        A = np.ascontiguousarray(A)
        Q = np.empty((m, m)); R = np.empty((m, 4))
        rr = L.ref_qr_decompose(m, 4, A.ctypes.data, Q.ctypes.data, R.ctypes.data)
        ro, Qo, Ro = oracle_lib.qr_decompose(A)
        assert rr == ro and np.array_equal(Q, Qo) and np.array_equal(R, Ro)


def test_config1_recorded_outcome(oracle_lib):
    from core_gb300 import workload
    m = oracle_lib.OracleMesh.box(8, 8, 8)
    assert (m.V, m.E, m.T) == (729, 4184, 3072)
    u = workload.sine_field(m.coords)
    rc, size, L, flags, n_split, n_collapse, info = m.estimate_and_mark(u, 0.1)
    assert rc == 0
    assert n_split == 4184 and n_collapse == 0
    assert info["n_expanded"] == 8  # 6 too-small + 2 rank-deficient corner patches
    q = m.quality(size)
    assert abs(q.min() - 0.432) < 1e-12 and abs(q.max() - 0.432) < 1e-12


def test_eigen_qr_bitwise_against_reference_fixture(oracle_lib):
    """mth::eigenQR / apf::eigen restated in the oracle equal the reference's
    compiled outputs bit for bit (tests/golden/eigen_ref.npz), and decompose."""
    d = np.load(os.path.join(GOLD, "eigen_ref.npz"))
    for A, L, Q, conv, vecs, vals in zip(d["A"], d["L"], d["Q"], d["converged"], d["vecs"], d["vals"]):
        rc, Lo, Qo = oracle_lib.eigen_qr3(A)
        assert rc == conv == 1
        assert np.array_equal(Lo, L) and np.array_equal(Qo, Q)
        # apf::eigen: eigenvalues on the diagonal, eigenvectors = columns of Q
        assert np.array_equal(np.diag(Lo), vals) and np.array_equal(Qo.T, vecs)
        # off-diagonals below the reference's 1e-10 deflation threshold remain
        assert np.abs(Qo @ np.diag(vals) @ Qo.T - A).max() <= 1e-9 * max(1.0, np.abs(A).max())


def test_eigen_qr_live_reference_build(oracle_lib):
    L = oracle_lib.ref_qr()
    if L is None:
        pytest.skip("oracle/_ref not built (reference tree absent on this host)")
    rng = np.random.Generator(np.random.PCG64(19))
    for k in range(300):
        A = rng.normal(size=(3, 3)) * 10.0 ** rng.uniform(-6, 4)
        A = np.ascontiguousarray(A + A.T)
        if k % 7 == 0:
            A[0, 1] = A[1, 0] = A[0, 2] = A[2, 0] = 0.0
        L9, Q9 = np.empty(9), np.empty(9)
        rr = L.ref_eigen_qr3(A.ctypes.data, L9.ctypes.data, Q9.ctypes.data, 100)
        ro, Lo, Qo = oracle_lib.eigen_qr3(A)
        assert rr == ro and np.array_equal(L9.reshape(3, 3), Lo) and np.array_equal(Q9.reshape(3, 3), Qo)
