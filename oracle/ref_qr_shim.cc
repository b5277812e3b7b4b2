// ref_qr_shim.cc -- C entry points over the reference's own mth QR
// (mth/mthQR.cc, compiled from the reference sources by oracle/Makefile
// into oracle/_ref/).  TEST INFRASTRUCTURE ONLY: used to generate the
// golden QR fixtures that pin the oracle's restatement of
// mth::decomposeQR / mth::solveFromQR (mth/mthQR.cc:106-160).
#include "mthQR.h"
#include "mth_def.h"

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

}
