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

}  // namespace ref
}  // namespace sprg
