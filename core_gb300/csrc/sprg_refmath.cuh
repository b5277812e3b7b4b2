// FP64 element geometry in the reference's evaluation order.
//
// The FP64 ("parity") kernels must round exactly like PUMI's apf/ma code so
// that per-element and per-edge results are bitwise equal.  The operation
// order of each helper follows the operator it stands for:
//   dot / length          apf::Vector::operator*, getLength (apf/apfVector.h:103-111)
//   cross                 apf::cross (apf/apfVector.h:123)
//   matrix product        apf::Matrix::operator* (apf/apfMatrix.h:83-106)
//   determinant           apf::getDeterminant cofactor expansion (apf/apfMatrix.cc:85-125)
//   3x3 inverse           apf::invert (apf/apfMatrix.h:165)
//   pseudo-inverse (2D)   apf::getJacobianInverse (apf/apfElement.cc:43-76)
//   Jacobian              VectorElement::getJacobian / gradHelper (apf/apfVectorElement.cc:44-66)
//   interpolation         Element::getComponents (apf/apfElement.cc:93-112)
// This translation unit is compiled with -fmad=false so no FMA contraction
// changes the rounding.
#pragma once

namespace sprg {
namespace ref {

struct V3 { double v[3]; };
struct M3 { double m[3][3]; };

__device__ __forceinline__ double dot(const V3& a, const V3& b) {
  double r = 0;
  r += a.v[0] * b.v[0];
  r += a.v[1] * b.v[1];
  r += a.v[2] * b.v[2];
  return r;
}
__device__ __forceinline__ double len(const V3& a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ V3 scale(const V3& a, double s) { return V3{{a.v[0] * s, a.v[1] * s, a.v[2] * s}}; }
__device__ __forceinline__ V3 divs(const V3& a, double s) { return V3{{a.v[0] / s, a.v[1] / s, a.v[2] / s}}; }
__device__ __forceinline__ V3 add(const V3& a, const V3& b) { return V3{{a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]}}; }
__device__ __forceinline__ V3 sub(const V3& a, const V3& b) { return V3{{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]}}; }
__device__ __forceinline__ V3 cross(const V3& a, const V3& b) {
  V3 r;
  r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
  r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
  r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
  return r;
}
__device__ __forceinline__ V3 normalize(const V3& a) { return divs(a, len(a)); }
__device__ __forceinline__ V3 row(const M3& a, int i) { return V3{{a.m[i][0], a.m[i][1], a.m[i][2]}}; }
__device__ __forceinline__ void setrow(M3& a, int i, const V3& r) { a.m[i][0] = r.v[0]; a.m[i][1] = r.v[1]; a.m[i][2] = r.v[2]; }
__device__ __forceinline__ M3 transpose(const M3& a) {
  M3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.m[j][i] = a.m[i][j];
  return r;
}
__device__ __forceinline__ M3 mul(const M3& a, const M3& b) {
  M3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double t = a.m[i][0] * b.m[0][j];
      t += a.m[i][1] * b.m[1][j];
      t += a.m[i][2] * b.m[2][j];
      r.m[i][j] = t;
    }
  return r;
}
__device__ __forceinline__ V3 mulv(const M3& a, const V3& b) {
  return V3{{dot(row(a, 0), b), dot(row(a, 1), b), dot(row(a, 2), b)}};
}
__device__ __forceinline__ double det2(double a00, double a01, double a10, double a11) {
  double d = 0;
  d += a00 * (1 * a11);
  d += a10 * (-1 * a01);
  return d;
}
__device__ __forceinline__ double det3(const M3& a) {
  double d = 0;
  d += a.m[0][0] * (1 * det2(a.m[1][1], a.m[1][2], a.m[2][1], a.m[2][2]));
  d += a.m[1][0] * (-1 * det2(a.m[0][1], a.m[0][2], a.m[2][1], a.m[2][2]));
  d += a.m[2][0] * (1 * det2(a.m[0][1], a.m[0][2], a.m[1][1], a.m[1][2]));
  return d;
}
__device__ __forceinline__ M3 invert3(const M3& m) {
  M3 x = transpose(m), r;
  setrow(r, 0, cross(row(x, 1), row(x, 2)));
  setrow(r, 1, cross(row(x, 2), row(x, 0)));
  setrow(r, 2, cross(row(x, 0), row(x, 1)));
  double d = det3(m);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.m[i][j] = r.m[i][j] / d;
  return r;
}
__device__ __forceinline__ M3 jacobian_inverse(const M3& J, int dim) {
  if (dim == 3) return invert3(J);
  double A[2][3], At[3][2], AAt[2][2], inv[2][2];
  for (int j = 0; j < 3; ++j) { A[0][j] = J.m[0][j]; A[1][j] = J.m[1][j]; }
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 3; ++j) At[j][i] = A[i][j];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      double t = A[i][0] * At[0][j];
      t += A[i][1] * At[1][j];
      t += A[i][2] * At[2][j];
      AAt[i][j] = t;
    }
  double d = det2(AAt[0][0], AAt[0][1], AAt[1][0], AAt[1][1]);
  inv[0][0] = AAt[1][1] / d; inv[0][1] = -AAt[0][1] / d;
  inv[1][0] = -AAt[1][0] / d; inv[1][1] = AAt[0][0] / d;
  M3 jinv;
  for (int i = 0; i < 3; ++i) {
    double t0 = At[i][0] * inv[0][0];
    t0 += At[i][1] * inv[1][0];
    double t1 = At[i][0] * inv[0][1];
    t1 += At[i][1] * inv[1][1];
    jinv.m[i][0] = t0;
    jinv.m[i][1] = t1;
    jinv.m[i][2] = 0;
  }
  return jinv;
}
__device__ __forceinline__ double jacobian_det(const M3& J, int dim) {
  if (dim == 3) return det3(J);
  if (dim == 2) return len(cross(row(J, 0), row(J, 1)));
  return len(row(J, 0));
}

// Linear simplex shape gradients (apf/apfShape.cc:139-211) for dim 1/2/3.
__device__ __forceinline__ void shape_grads(int dim, V3* g) {
  for (int i = 0; i < 4; ++i) g[i] = V3{{0, 0, 0}};
  if (dim == 3) {
    g[0] = V3{{-1, -1, -1}}; g[1].v[0] = 1; g[2].v[1] = 1; g[3].v[2] = 1;
  } else if (dim == 2) {
    g[0] = V3{{-1, -1, 0}}; g[1].v[0] = 1; g[2].v[1] = 1;
  } else {
    g[0].v[0] = -0.5; g[1].v[0] = 0.5;
  }
}
// J = sum_i tensorProduct(gradN_i, x_i): row r = sum_i x_i * gradN_i[r]
__device__ __forceinline__ M3 jacobian(const V3* x, int nn, int dim) {
  V3 g[4];
  shape_grads(dim, g);
  M3 J;
  for (int r = 0; r < 3; ++r) setrow(J, r, scale(x[0], g[0].v[r]));
  for (int n = 1; n < nn; ++n)
    for (int r = 0; r < 3; ++r) setrow(J, r, add(row(J, r), scale(x[n], g[n].v[r])));
  return J;
}
// Shape values at the element's order-1 integration point.
__device__ __forceinline__ void ip_shape_values(int dim, double* N) {
  if (dim == 3) {
    double xi = 0.25;
    N[0] = 1 - xi - xi - xi;
    N[1] = xi; N[2] = xi; N[3] = xi;
  } else {
    double xi = 1. / 3.;
    N[0] = 1 - xi - xi;
    N[1] = xi; N[2] = xi; N[3] = 0;
  }
}
__device__ __forceinline__ double ip_weight(int dim) { return dim == 3 ? 1.0 / 6.0 : 1.0 / 2.0; }

// Edge shape values (apf/apfShape.cc:118-123)
__device__ __forceinline__ void edge_shape_values(double xi, double* N) {
  N[0] = (1.0 - xi) / 2.0;
  N[1] = (1.0 + xi) / 2.0;
}

// orthogonalizeR (ma/maSize.cc:94-117)
__device__ __forceinline__ M3 orthogonalize(const M3& R) {
  M3 RT = transpose(R);
  V3 r0 = normalize(row(RT, 0));
  V3 r1 = row(RT, 1);
  r1 = sub(r1, scale(r0, dot(r0, r1)));
  r1 = normalize(r1);
  V3 r2 = cross(r0, r1);
  setrow(RT, 0, r0); setrow(RT, 1, r1); setrow(RT, 2, r2);
  return transpose(RT);
}

// AnisoSizeField::getTransform (ma/maSize.cc:395-412) with nodal h (nn x 3)
// and frames (nn x 9, row-major) interpolated by shape values N.
__device__ __forceinline__ M3 get_transform(const double* hv, const double* Rv, const double* N, int nn) {
  double h[3] = {0, 0, 0}, R9[9];
  for (int k = 0; k < 9; ++k) R9[k] = 0;
  for (int a = 0; a < nn; ++a)
    for (int k = 0; k < 3; ++k) h[k] += hv[3 * a + k] * N[a];
  for (int a = 0; a < nn; ++a)
    for (int k = 0; k < 9; ++k) R9[k] += Rv[9 * a + k] * N[a];
  M3 R;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R.m[i][j] = R9[3 * i + j];
  R = orthogonalize(R);
  M3 S;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) S.m[i][j] = 0;
  S.m[0][0] = 1 / h[0]; S.m[1][1] = 1 / h[1]; S.m[2][2] = 1 / h[2];
  return mul(R, S);
}

// ---- mth::eigenQR on a 3x3 matrix (mth/mthQR.cc:19-297) -------------------
// get_reflector with offset o (mth/mthQR.cc:19-45)
__device__ inline bool eig_reflector(const M3& a, double* v, int k, int o) {
  double cnorm = 0;
  for (int i = k + o; i < 3; ++i) cnorm += a.m[i][k] * a.m[i][k];
  cnorm = sqrt(cnorm);
  if (cnorm < 1e-10) return false;
  for (int i = 0; i < k + o; ++i) v[i] = 0;
  for (int i = k + o; i < 3; ++i) v[i] = a.m[i][k];
  v[k + o] += ((a.m[k + o][k] < 0) ? -1 : 1) * cnorm;
  double rnorm = 0;
  for (int i = k + o; i < 3; ++i) rnorm += v[i] * v[i];
  rnorm = sqrt(rnorm);
  for (int i = k + o; i < 3; ++i) v[i] /= rnorm;
  return true;
}
// reflect_columns / reflect_rows (mth/mthQR.cc:47-79)
__device__ inline void eig_reflect_columns(const double* v, M3& a, int k, int o) {
  for (int j = 0; j < 3; ++j) {
    double d = 0;
    for (int i = k + o; i < 3; ++i) d += a.m[i][j] * v[i];
    for (int i = k + o; i < 3; ++i) a.m[i][j] -= 2 * d * v[i];
  }
}
__device__ inline void eig_reflect_rows(const double* v, M3& q, int k, int o) {
  for (int i = 0; i < 3; ++i) {
    double d = 0;
    for (int j = k + o; j < 3; ++j) d += q.m[i][j] * v[j];
    for (int j = k + o; j < 3; ++j) q.m[i][j] -= 2 * d * v[j];
  }
}
// mth::multiply (mth/mth_def.h:235-248): c(i,j) = 0, then += a(i,l) b(l,j)
__device__ inline M3 eig_mul(const M3& a, const M3& b) {
  M3 c;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      c.m[i][j] = 0;
      for (int l = 0; l < 3; ++l) c.m[i][j] += a.m[i][l] * b.m[l][j];
    }
  return c;
}
__device__ inline void eig_identity(M3& q) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) q.m[i][j] = (double)(i == j);
}
// Hessenberg reduction, then Wilkinson-shifted QR steps with deflation from
// the bottom (at most max_iters).  Returns 1 when converged, 0 when the
// iterations ran out, -1 when the shift's denominator vanished (the
// reference asserts in both failure cases).
__device__ inline int eigen_qr3(const M3& A, M3& L, M3& Q, int max_iters) {
  double v[3];
  eig_identity(Q);
  M3 h = A;
  if (eig_reflector(h, v, 0, 1)) {
    eig_reflect_columns(v, h, 0, 1);
    eig_reflect_rows(v, h, 0, 1);
    eig_reflect_rows(v, Q, 0, 1);
  }
  int red_m = 3, status = 0;
  for (int it = 0; it < max_iters; ++it) {
    bool more = false;
    while (red_m > 1) {
      if (fabs(h.m[red_m - 2][red_m - 1]) < 1e-10 && fabs(h.m[red_m - 1][red_m - 2]) < 1e-10) {
        --red_m;
      } else {
        more = true;
        break;
      }
    }
    if (!more) {
      status = 1;
      break;
    }
    const double amm1 = h.m[red_m - 2][red_m - 2], am = h.m[red_m - 1][red_m - 1], bmm1 = h.m[red_m - 2][red_m - 1];
    const double sig = (amm1 - am) / 2;
    const double denom = (fabs(sig) + sqrt(sig * sig + bmm1 * bmm1));
    if (!(fabs(denom) > 1e-10)) {
      status = -1;
      break;
    }
    const double mu = am - ((((sig < 0) ? -1 : 1) * (bmm1 * bmm1)) / denom);
    for (int i = 0; i < 3; ++i) h.m[i][i] -= mu;
    M3 qk, rk = h;
    eig_identity(qk);
    for (int k = 0; k < 3; ++k)
      if (eig_reflector(rk, v, k, 0)) {
        eig_reflect_columns(v, rk, k, 0);
        eig_reflect_rows(v, qk, k, 0);
      }
    h = eig_mul(rk, qk);
    for (int i = 0; i < 3; ++i) h.m[i][i] -= -mu;
    Q = eig_mul(Q, qk);
  }
  L = h;
  return status;
}

// LogAnisoSizeField::init (ma/maSize.cc:472-503): f diag(log(1/h/h)) f^T
__device__ inline void vertex_logm(const double* h, const double* f9, double* out9) {
  M3 f, S;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      f.m[i][j] = f9[3 * i + j];
      S.m[i][j] = 0;
    }
  S.m[0][0] = log(1 / h[0] / h[0]);
  S.m[1][1] = log(1 / h[1] / h[1]);
  S.m[2][2] = log(1 / h[2] / h[2]);
  const M3 r = mul(mul(f, S), transpose(f));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out9[3 * i + j] = r.m[i][j];
}

// LogAnisoSizeField::getTransform (ma/maSize.cc:508-523): log-metrics of nn
// nodes (nn x 9) interpolated by N, apf::eigen (apf/apfMatrix.cc:68-82),
// orthogonalEigenDecompForSymmetricMatrix (ma/maSize.cc:123-142),
// Q = R diag(sqrt(exp(v))).  *ok = false when the eigen iteration fails.
__device__ inline M3 log_transform(const double* Mv, const double* N, int nn, bool* ok) {
  double M9[9];
  for (int k = 0; k < 9; ++k) M9[k] = 0;
  for (int a = 0; a < nn; ++a)
    for (int k = 0; k < 9; ++k) M9[k] += Mv[9 * a + k] * N[a];
  M3 A, L, Qe;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A.m[i][j] = M9[3 * i + j];
  if (eigen_qr3(A, L, Qe, 100) != 1) *ok = false;
  // eigenvectors: the columns of Qe, as the rows of RT
  M3 RT = transpose(Qe);
  V3 r0 = normalize(row(RT, 0));
  V3 r1 = sub(row(RT, 1), scale(r0, dot(r0, row(RT, 1))));
  r1 = normalize(r1);
  V3 r2 = cross(r0, r1);
  setrow(RT, 0, r0); setrow(RT, 1, r1); setrow(RT, 2, r2);
  M3 S;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) S.m[i][j] = 0;
  S.m[0][0] = sqrt(exp(L.m[0][0]));
  S.m[1][1] = sqrt(exp(L.m[1][1]));
  S.m[2][2] = sqrt(exp(L.m[2][2]));
  return mul(transpose(RT), S);
}

}  // namespace ref
}  // namespace sprg
