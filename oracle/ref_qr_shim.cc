// ref_qr_shim.cc -- C entry points over the reference's own mth QR and
// apf::eigen (mth/mthQR.cc, apf/apfMatrix.cc, compiled from the reference
// sources by oracle/Makefile into oracle/_ref/).  TEST INFRASTRUCTURE ONLY:
// used to generate the golden fixtures that pin the oracle's restatements of
// mth::decomposeQR / mth::solveFromQR (mth/mthQR.cc:106-160) and
// mth::eigenQR / apf::eigen (mth/mthQR.cc:192-297, apf/apfMatrix.cc:68-82).
#include "mthQR.h"
#include "mth_def.h"
#include "apfMatrix.h"

extern "C" {

// A, R: m x n row-major; Q: m x m row-major.  Returns the rank as counted by
// mth::decomposeQR.
int ref_qr_decompose(int m, int n, const double* A, double* Q, double* R) {
  mth::Matrix<double> a(m, n), q, r;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) a(i, j) = A[i * n + j];
  unsigned rank = mth::decomposeQR(a, q, r);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) Q[i * m + j] = q(i, j);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) R[i * n + j] = r(i, j);
  return (int)rank;
}

// Decompose then solveFromQR (the pair spr::preparePolynomialFit /
// runPolynomialFit uses).  x valid only when the returned rank == n.
int ref_qr_solve(int m, int n, const double* A, const double* b, double* x) {
  mth::Matrix<double> a(m, n), q, r;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) a(i, j) = A[i * n + j];
  unsigned rank = mth::decomposeQR(a, q, r);
  if ((int)rank != n) return (int)rank;
  mth::Vector<double> bb(m), xx;
  for (int i = 0; i < m; ++i) bb(i) = b[i];
  mth::solveFromQR(q, r, bb, xx);
  for (int j = 0; j < n; ++j) x[j] = xx(j);
  return (int)rank;
}

// mth::eigenQR on a 3x3 matrix (row-major in and out); returns 1 when it
// converged within max_iters.
int ref_eigen_qr3(const double* A9, double* L9, double* Q9, int max_iters) {
  mth::Matrix<double, 3, 3> a, l, q;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) a(i, j) = A9[3 * i + j];
  bool ok = mth::eigenQR(a, l, q, (unsigned)max_iters);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      L9[3 * i + j] = l(i, j);
      Q9[3 * i + j] = q(i, j);
    }
  return ok ? 1 : 0;
}

// apf::eigen: eigenvectors as rows of vec9, eigenvalues in val3
void ref_apf_eigen(const double* A9, double* vec9, double* val3) {
  apf::Matrix3x3 a;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) a[i][j] = A9[3 * i + j];
  apf::Vector3 vecs[3];
  apf::eigen(a, vecs, val3);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) vec9[3 * i + j] = vecs[i][j];
}

}
