// FP64 ("parity") kernels of the estimate-and-mark pass.
//
// Compiled with -fmad=false: element and edge arithmetic follows the
// reference's operation order (sprg_refmath.cuh), so gradients, element
// errors, sizes, lengths and qualities round like PUMI's apf/spr/ma code.
// Two places differ by design and are stated in the parity tests: the
// patch QR uses warp-tree reductions and applies the reflectors to the
// right-hand side instead of forming Q (mth/mthQR.cc builds an explicit
// m x m Q), and the two global integrals are summed by a fixed tree instead
// of sequentially.  Both move results by a few ulps only.
#include <cub/cub.cuh>
#include <cstring>

#include "sprg_internal.h"
#include "sprg_refmath.cuh"
#include "sprg_reduce.cuh"

namespace sprg {

using ref::M3;
using ref::V3;

namespace {

constexpr int kBlock = 256;
constexpr int kExpandMaxElems = 1024;
constexpr int kExpandHash = 4096;
constexpr int kExpandGrid = 304;  // 2 resident single-warp blocks per SM
constexpr int kExpandSmemRows = 96;  // patches up to this size keep their QR rows in shared memory
constexpr int kTriThreadRows = 8;    // triangle patches up to this size take the thread-per-vertex QR

__device__ __forceinline__ void set_status(DevStatus* st, int code, int where) {
  if (atomicCAS(&st->code, 0, code) == 0) st->where = where;
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__device__ __forceinline__ V3 load_xyz(const double* __restrict__ xyz, int v) {
  return V3{{xyz[3 * (size_t)v], xyz[3 * (size_t)v + 1], xyz[3 * (size_t)v + 2]}};
}

// integration point (mapLocalToGlobal at the order-1 point) of element e,
// in the reference's interpolation order
__device__ __forceinline__ V3 elem_ip_point(const DevMesh& m, int e) {
  double N[4];
  ref::ip_shape_values(m.dim, N);
  V3 p{{0, 0, 0}};
  const int* ev = m.ev + (size_t)e * m.nn;
  for (int a = 0; a < m.nn; ++a) {
    V3 x = load_xyz(m.xyz, ev[a]);
    for (int k = 0; k < 3; ++k) p.v[k] += x.v[k] * N[a];
  }
  return p;
}

// gradient of a scalar P1 field at the order-1 integration point of e
// (ScalarElement::grad, apf/apfScalarElement.cc:18)
__device__ __forceinline__ V3 elem_grad_scalar(const DevMesh& m, int e, const double* __restrict__ f) {
  const int* ev = m.ev + (size_t)e * m.nn;
  V3 x[4];
  for (int a = 0; a < m.nn; ++a) x[a] = load_xyz(m.xyz, ev[a]);
  M3 J = ref::jacobian(x, m.nn, m.dim);
  M3 jinv = ref::jacobian_inverse(J, m.dim);
  V3 lg[4];
  ref::shape_grads(m.dim, lg);
  V3 g = ref::scale(ref::mulv(jinv, lg[0]), f[ev[0]]);
  for (int a = 1; a < m.nn; ++a) g = ref::add(g, ref::scale(ref::mulv(jinv, lg[a]), f[ev[a]]));
  return g;
}

// gradient of component r of a P1 field stored with stride `stride` (a
// VECTOR field's row r of the MATRIX ip value), same operation order
__device__ __forceinline__ V3 elem_grad_component(const DevMesh& m, int e, const double* __restrict__ f, int stride,
                                                  int r) {
  const int* ev = m.ev + (size_t)e * m.nn;
  V3 x[4];
  for (int a = 0; a < m.nn; ++a) x[a] = load_xyz(m.xyz, ev[a]);
  M3 J = ref::jacobian(x, m.nn, m.dim);
  M3 jinv = ref::jacobian_inverse(J, m.dim);
  V3 lg[4];
  ref::shape_grads(m.dim, lg);
  V3 g = ref::scale(ref::mulv(jinv, lg[0]), f[(size_t)ev[0] * stride + r]);
  for (int a = 1; a < m.nn; ++a) g = ref::add(g, ref::scale(ref::mulv(jinv, lg[a]), f[(size_t)ev[a] * stride + r]));
  return g;
}

// ---------------------------------------------------------------------
// spr::getGradIPField
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_grad_ip(DevMesh m, const double* __restrict__ f, int ncin,
                                                    double* __restrict__ ip) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.T) return;
  const int* ev = m.ev + (size_t)e * m.nn;
  V3 x[4];
  for (int a = 0; a < m.nn; ++a) x[a] = load_xyz(m.xyz, ev[a]);
  M3 J = ref::jacobian(x, m.nn, m.dim);
  M3 jinv = ref::jacobian_inverse(J, m.dim);
  V3 lg[4], gg[4];
  ref::shape_grads(m.dim, lg);
  for (int a = 0; a < m.nn; ++a) gg[a] = ref::mulv(jinv, lg[a]);
  if (ncin == 1) {
    V3 g = ref::scale(gg[0], f[ev[0]]);
    for (int a = 1; a < m.nn; ++a) g = ref::add(g, ref::scale(gg[a], f[ev[a]]));
    for (int k = 0; k < 3; ++k) ip[(size_t)e * 3 + k] = g.v[k];
  } else {
    M3 g;
    for (int a = 0; a < m.nn; ++a) {
      V3 u{{f[3 * (size_t)ev[a]], f[3 * (size_t)ev[a] + 1], f[3 * (size_t)ev[a] + 2]}};
      for (int r = 0; r < 3; ++r) {
        V3 rw = ref::scale(u, gg[a].v[r]);
        if (a == 0) ref::setrow(g, r, rw);
        else ref::setrow(g, r, ref::add(ref::row(g, r), rw));
      }
    }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) ip[(size_t)e * 9 + 3 * r + c] = g.m[r][c];
  }
}

// ---------------------------------------------------------------------
// spr::recoverField -- register path: one warp per vertex, RPL rows per
// lane.  Patches that are too small, rank deficient or larger than 32*RPL
// rows go to the expansion list.
// ---------------------------------------------------------------------
template <int NT, int NC, int RPL>
__device__ __forceinline__ void recover_vertex_warp(const DevMesh& m, const double* __restrict__ ip,
                                                    double* __restrict__ rec, const ExpandList& xl, int v,
                                                    int lane) {
  const int beg = m.p_off[v];
  const int cnt = m.p_off[v + 1] - beg;
  if (cnt < NT || cnt > 32 * RPL) {
    if (lane == 0) {
      int slot = atomicAdd(xl.count, 1);
      if (slot < xl.cap) xl.items[slot] = v;
    }
    return;
  }
  double a[RPL][NT], b[RPL][NC];
#pragma unroll
  for (int r = 0; r < RPL; ++r) {
    int i = lane + 32 * r;
    if (i < cnt) {
      int el = m.p_el[beg + i];
      V3 p = elem_ip_point(m, el);
      a[r][0] = 1.0;
      a[r][1] = p.v[0];
      a[r][2] = p.v[1];
      if (NT == 4) a[r][NT - 1] = p.v[2];
#pragma unroll
      for (int c = 0; c < NC; ++c) b[r][c] = ip[(size_t)el * NC + c];
    } else {
#pragma unroll
      for (int j = 0; j < NT; ++j) a[r][j] = 0;
#pragma unroll
      for (int c = 0; c < NC; ++c) b[r][c] = 0;
    }
  }
  // Householder QR without pivoting; rank test as mth::get_reflector
  // (column residual norm below 1e-10 absolute = rank deficient).
#pragma unroll
  for (int k = 0; k < NT; ++k) {
    double s = 0;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      int i = lane + 32 * r;
      if (i >= k) s += a[r][k] * a[r][k];
    }
    double cn = sqrt(warp_sum(s));
    if (cn < 1e-10) {  // uniform across the warp
      if (lane == 0) {
        int slot = atomicAdd(xl.count, 1);
        if (slot < xl.cap) xl.items[slot] = v;
      }
      return;
    }
    double akk = __shfl_sync(0xffffffffu, a[0][k], k);
    double vv[RPL];
    double s2 = 0;
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      int i = lane + 32 * r;
      vv[r] = (i >= k) ? a[r][k] : 0.0;
      if (i == k) vv[r] += ((akk < 0) ? -1 : 1) * cn;
      s2 += vv[r] * vv[r];
    }
    double rinv = 1.0 / sqrt(warp_sum(s2));
#pragma unroll
    for (int r = 0; r < RPL; ++r) vv[r] *= rinv;
#pragma unroll
    for (int j = k; j < NT; ++j) {
      double d = 0;
#pragma unroll
      for (int r = 0; r < RPL; ++r) d += a[r][j] * vv[r];
      d = warp_sum(d);
#pragma unroll
      for (int r = 0; r < RPL; ++r) a[r][j] -= 2 * d * vv[r];
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double d = 0;
#pragma unroll
      for (int r = 0; r < RPL; ++r) d += b[r][c] * vv[r];
      d = warp_sum(d);
#pragma unroll
      for (int r = 0; r < RPL; ++r) b[r][c] -= 2 * d * vv[r];
    }
  }
  // R (NT x NT) sits in lanes 0..NT-1 of slot 0.
  double R[NT][NT], y[NT][NC];
#pragma unroll
  for (int i = 0; i < NT; ++i) {
#pragma unroll
    for (int j = 0; j < NT; ++j) R[i][j] = __shfl_sync(0xffffffffu, a[0][j], i);
#pragma unroll
    for (int c = 0; c < NC; ++c) y[i][c] = __shfl_sync(0xffffffffu, b[0][c], i);
  }
  V3 xv = load_xyz(m.xyz, v);
  double terms[4] = {1.0, xv.v[0], xv.v[1], xv.v[2]};
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    double x[NT];
#pragma unroll
    for (int ii = 0; ii < NT; ++ii) {
      int i = NT - ii - 1;
      double t = y[i][c];
#pragma unroll
      for (int j = i + 1; j < NT; ++j) t -= R[i][j] * x[j];
      x[i] = t / R[i][i];
    }
    double sres = 0;
#pragma unroll
    for (int j = 0; j < NT; ++j) sres += x[j] * terms[j];
    if (lane == c) rec[(size_t)v * NC + c] = sres;
  }
}

// the warp path over a vertex list (the triangle patches too large for the
// thread path); a fixed grid of warps strides over the device-side count
template <int NT, int NC, int RPL>
__global__ void __launch_bounds__(kBlock) k_recover_list(DevMesh m, const double* __restrict__ ip,
                                                         double* __restrict__ rec, ExpandList xl, ExpandList list) {
  const int lane = threadIdx.x & 31;
  int n = *list.count;
  n = n < list.cap ? n : list.cap;
  const int nw = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  for (int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); w < n; w += nw)
    recover_vertex_warp<NT, NC, RPL>(m, ip, rec, xl, list.items[w], lane);
}

// ---------------------------------------------------------------------
// spr::recoverField on triangles -- one thread per vertex for patches of
// NT..MAXM elements, in the reference's own operation order
// (mth/mthQR.cc:19-160, spr/sprRecoverField.cc:226-353):
//   get_reflector      column norm from row k down, the 1e-10 rank test,
//                      v = column + sgn * norm at k, v /= |v|;
//   reflect_columns    dot from row k down, a -= (2 dot) v_i;
//   reflect_rows       Q = I H_1 H_2 H_3: every row of Q evolves on its own,
//                      so the rows are built one at a time and only their
//                      first NT entries (the columns y = Q^T b reads) kept;
//   solveFromQR        y_i = sum over rows in ascending order, back
//                      substitution, then the fit evaluated at the vertex.
// Columns left of k, which reflect_columns also updates, are never read
// again and are skipped.  Compiled without FMA contraction, the results
// are bitwise those of that sequence.  Patches with fewer than NT elements
// or rank deficient go to the expansion list, larger ones to `big` (the
// warp path).
// ---------------------------------------------------------------------
template <int NC, int MAXM>
__global__ void __launch_bounds__(128) k_recover_tri(DevMesh m, const double* __restrict__ ip,
                                                     double* __restrict__ rec, ExpandList xl, ExpandList big) {
  constexpr int NT = 3;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  const int beg = m.p_off[v];
  const int cnt = m.p_off[v + 1] - beg;
  if (cnt < NT || cnt > MAXM) {
    const ExpandList& l = cnt < NT ? xl : big;
    const int slot = atomicAdd(l.count, 1);
    if (slot < l.cap) l.items[slot] = v;
    return;
  }
  int el[MAXM];
  double R[MAXM][NT];
#pragma unroll
  for (int i = 0; i < MAXM; ++i) {
    el[i] = 0;
    R[i][0] = R[i][1] = R[i][2] = 0;
    if (i < cnt) {
      el[i] = m.p_el[beg + i];
      const V3 p = elem_ip_point(m, el[i]);
      R[i][0] = 1.0;
      R[i][1] = p.v[0];
      R[i][2] = p.v[1];
    }
  }
  double H[NT][MAXM];  // the reflectors
#pragma unroll
  for (int k = 0; k < NT; ++k) {
    double cn = 0;
#pragma unroll
    for (int i = k; i < MAXM; ++i)
      if (i < cnt) cn += R[i][k] * R[i][k];
    cn = sqrt(cn);
    if (cn < 1e-10) {
      const int slot = atomicAdd(xl.count, 1);
      if (slot < xl.cap) xl.items[slot] = v;
      return;
    }
#pragma unroll
    for (int i = 0; i < MAXM; ++i) H[k][i] = (i >= k && i < cnt) ? R[i][k] : 0.0;
    H[k][k] += ((R[k][k] < 0) ? -1 : 1) * cn;
    double rn = 0;
#pragma unroll
    for (int i = k; i < MAXM; ++i)
      if (i < cnt) rn += H[k][i] * H[k][i];
    rn = sqrt(rn);
#pragma unroll
    for (int i = k; i < MAXM; ++i)
      if (i < cnt) H[k][i] /= rn;
#pragma unroll
    for (int j = k; j < NT; ++j) {
      double dot = 0;
#pragma unroll
      for (int i = k; i < MAXM; ++i)
        if (i < cnt) dot += R[i][j] * H[k][i];
#pragma unroll
      for (int i = k; i < MAXM; ++i)
        if (i < cnt) R[i][j] -= 2 * dot * H[k][i];
    }
  }
  // the first NT columns of Q, row by row
  double Qc[MAXM][NT];
#pragma unroll
  for (int r = 0; r < MAXM; ++r) {
    double q[MAXM];
#pragma unroll
    for (int j = 0; j < MAXM; ++j) q[j] = (j == r) ? 1.0 : 0.0;
#pragma unroll
    for (int k = 0; k < NT; ++k) {
      double dot = 0;
#pragma unroll
      for (int j = k; j < MAXM; ++j)
        if (j < cnt) dot += q[j] * H[k][j];
#pragma unroll
      for (int j = k; j < MAXM; ++j)
        if (j < cnt) q[j] -= 2 * dot * H[k][j];
    }
#pragma unroll
    for (int i = 0; i < NT; ++i) Qc[r][i] = q[i];
  }
  const V3 xv = load_xyz(m.xyz, v);
#pragma unroll 1
  for (int c = 0; c < NC; ++c) {
    double y[NT] = {0, 0, 0};
#pragma unroll
    for (int r = 0; r < MAXM; ++r)
      if (r < cnt) {
        const double b = ip[(size_t)el[r] * NC + c];
#pragma unroll
        for (int i = 0; i < NT; ++i) y[i] += Qc[r][i] * b;
      }
    double x[NT];
#pragma unroll
    for (int ii = 0; ii < NT; ++ii) {
      const int i = NT - ii - 1;
      x[i] = y[i];
#pragma unroll
      for (int j = i + 1; j < NT; ++j) x[i] -= R[i][j] * x[j];
      x[i] /= R[i][i];
    }
    double sres = 0;
    sres += x[0] * 1.0;
    sres += x[1] * xv.v[0];
    sres += x[2] * xv.v[1];
    rec[(size_t)v * NC + c] = sres;
  }
}

// ---------------------------------------------------------------------
// Patch growth (spr/sprRecoverField.cc:155-386) for listed vertices: one
// warp per vertex, element set in shared memory, rows in a global slab.
// ---------------------------------------------------------------------
__device__ bool hash_insert(int* hs, int key) {
  unsigned h = ((unsigned)key * 2654435761u) & (kExpandHash - 1);
  for (int probe = 0; probe < kExpandHash; ++probe) {
    int prev = atomicCAS(&hs[h], -1, key);
    if (prev == -1) return true;
    if (prev == key) return false;
    h = (h + 1) & (kExpandHash - 1);
  }
  return false;
}

__device__ void warp_sort_set(int* S, int n, int* tmp) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < n; i += 32) {
    int x = S[i], rank = 0;
    for (int j = 0; j < n; ++j) rank += (S[j] < x);
    tmp[rank] = x;
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) S[i] = tmp[i];
  __syncwarp();
}

// QR fit over the element set S (sorted).  Returns false if rank deficient.
// rows: n x (NT + nc + 1) doubles; the last column holds the reflector.
__device__ bool slab_fit(const DevMesh& m, const int* S, int n, const double* __restrict__ ip,
                         const double* __restrict__ u, int nc, double* rows, int v, double* rec) {
  const int lane = threadIdx.x & 31;
  const int NT = m.dim == 3 ? 4 : 3;
  const int W = NT + nc;
  const int LD = W + 1;
  if (n < NT) return false;
  for (int i = lane; i < n; i += 32) {
    int el = S[i];
    V3 p = elem_ip_point(m, el);
    double* rw = rows + (size_t)i * LD;
    rw[0] = 1.0; rw[1] = p.v[0]; rw[2] = p.v[1];
    if (NT == 4) rw[3] = p.v[2];
    if (ip) {
      for (int c = 0; c < nc; ++c) rw[NT + c] = ip[(size_t)el * nc + c];
    } else if (nc == 3) {  // no resident ip field: the gradient of the scalar field u
      V3 g = elem_grad_scalar(m, el, u);
      for (int c = 0; c < 3; ++c) rw[NT + c] = g.v[c];
    } else {  // ... or of the VECTOR field u (V x 3): MATRIX rows, row r = grad u_r
      for (int r = 0; r < 3; ++r) {
        V3 g = elem_grad_component(m, el, u, 3, r);
        for (int c = 0; c < 3; ++c) rw[NT + 3 * r + c] = g.v[c];
      }
    }
  }
  __syncwarp();
  for (int k = 0; k < NT; ++k) {
    double s = 0;
    for (int i = k + lane; i < n; i += 32) s += rows[(size_t)i * LD + k] * rows[(size_t)i * LD + k];
    double cn = sqrt(warp_sum(s));
    if (cn < 1e-10) return false;  // uniform across the warp
    double akk = rows[(size_t)k * LD + k];
    double s2 = 0;
    for (int i = k + lane; i < n; i += 32) {
      double vi = rows[(size_t)i * LD + k];
      if (i == k) vi += ((akk < 0) ? -1 : 1) * cn;
      rows[(size_t)i * LD + W] = vi;
      s2 += vi * vi;
    }
    double rn = sqrt(warp_sum(s2));
    for (int i = k + lane; i < n; i += 32) rows[(size_t)i * LD + W] /= rn;
    __syncwarp();
    for (int j = k; j < W; ++j) {
      double d = 0;
      for (int i = k + lane; i < n; i += 32) d += rows[(size_t)i * LD + j] * rows[(size_t)i * LD + W];
      d = warp_sum(d);
      for (int i = k + lane; i < n; i += 32) rows[(size_t)i * LD + j] -= 2 * d * rows[(size_t)i * LD + W];
      __syncwarp();
    }
  }
  V3 xv = load_xyz(m.xyz, v);
  double terms[4] = {1.0, xv.v[0], xv.v[1], xv.v[2]};
  for (int c = 0; c < nc; ++c) {
    double x[4];
    for (int ii = 0; ii < NT; ++ii) {
      int i = NT - ii - 1;
      double t = rows[(size_t)i * LD + NT + c];
      for (int j = i + 1; j < NT; ++j) t -= rows[(size_t)i * LD + j] * x[j];
      x[i] = t / rows[(size_t)i * LD + i];
    }
    double sres = 0;
    for (int j = 0; j < NT; ++j) sres += x[j] * terms[j];
    if (lane == 0) rec[(size_t)v * nc + c] = sres;
  }
  __syncwarp();
  return true;
}

__global__ void __launch_bounds__(32) k_expand(DevMesh m, const double* __restrict__ ip,
                                               const double* __restrict__ u, int nc,
                                               double* __restrict__ rec, const int* __restrict__ items,
                                               const int* __restrict__ n_items_ptr, int cap, double* slab,
                                               DevStatus* st, int* cache_v, int* cache_n, int* cache_el) {
  __shared__ int S[kExpandMaxElems];
  __shared__ int old[kExpandMaxElems];
  __shared__ int tmp[kExpandMaxElems];
  __shared__ int hs[kExpandHash];
  __shared__ int nS;
  __shared__ double srows[kExpandSmemRows * 8];
  const int lane = threadIdx.x;
  const int NT = m.dim == 3 ? 4 : 3;
  double* grows = slab + (size_t)blockIdx.x * kExpandMaxElems * (NT + nc + 1);
  int n_items = *n_items_ptr;
  if (n_items > cap) {
    if (lane == 0 && blockIdx.x == 0) set_status(st, SPRG_EPATCH, -1);
    n_items = cap;
  }
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int v = items[it];
    for (int i = lane; i < kExpandHash; i += 32) hs[i] = -1;
    if (lane == 0) nS = 0;
    __syncwarp();
    bool overflow = false;
    for (int k = m.p_off[v] + lane; k < m.p_off[v + 1]; k += 32) {
      int f = m.p_el[k];
      if (hash_insert(hs, f)) {
        int slot = atomicAdd(&nS, 1);
        if (slot < kExpandMaxElems) S[slot] = f; else overflow = true;
      }
    }
    __syncwarp();
    bool done = false, failed = false;
    for (int round = 0; round < 64 && !done && !failed; ++round) {
      overflow = __any_sync(0xffffffffu, overflow);
      if (overflow || nS > kExpandMaxElems) { failed = true; break; }
      int n0 = nS;
      warp_sort_set(S, n0, tmp);
      double* rows = (n0 * (NT + nc + 1) <= kExpandSmemRows * 8) ? srows : grows;
      if (slab_fit(m, S, n0, ip, u, nc, rows, v, rec)) { done = true; break; }
      for (int i = lane; i < n0; i += 32) old[i] = S[i];
      __syncwarp();
      for (int sd = m.dim - 1; sd >= 0 && !done; --sd) {
        for (int i = lane; i < n0; i += 32) {
          int e = old[i];
          const int* ev = m.ev + (size_t)e * m.nn;
          for (int a = 0; a < m.nn; ++a) {
            int w = ev[a];
            for (int k = m.p_off[w]; k < m.p_off[w + 1]; ++k) {
              int f = m.p_el[k];
              const int* fv = m.ev + (size_t)f * m.nn;
              int shared = 0;
              for (int p = 0; p < m.nn; ++p)
                for (int q = 0; q < m.nn; ++q) shared += (ev[p] == fv[q]);
              if (shared >= sd + 1 && hash_insert(hs, f)) {
                int slot = atomicAdd(&nS, 1);
                if (slot < kExpandMaxElems) S[slot] = f; else overflow = true;
              }
            }
          }
        }
        __syncwarp();
        overflow = __any_sync(0xffffffffu, overflow);
        if (overflow || nS > kExpandMaxElems) { failed = true; break; }
        int n1 = nS;
        warp_sort_set(S, n1, tmp);
        double* rows1 = (n1 * (NT + nc + 1) <= kExpandSmemRows * 8) ? srows : grows;
        if (slab_fit(m, S, n1, ip, u, nc, rows1, v, rec)) { done = true; break; }
      }
      if (!done && !failed && !(nS > n0)) failed = true;  // "all hope is lost"
    }
    if (!done && lane == 0) set_status(st, SPRG_EPATCH, v);
    if (cache_v) {  // the grown patch depends on geometry only: keep it for later passes
      int nfin = done ? nS : -1;
      if (lane == 0) {
        cache_v[it] = v;
        cache_n[it] = nfin;
      }
      for (int i = lane; i < nfin; i += 32) cache_el[(size_t)it * kExpandMaxElems + i] = S[i];
    }
    __syncwarp();
  }
}

// Later passes: the listed vertices' final patches come from the cache; one
// QR fit each, no growth rounds.
__global__ void __launch_bounds__(32) k_cached_fit(DevMesh m, const double* __restrict__ ip,
                                                   const double* __restrict__ u, int nc, double* __restrict__ rec,
                                                   int n_cached, const int* __restrict__ cache_v,
                                                   const int* __restrict__ cache_n, const int* __restrict__ cache_el,
                                                   double* slab, DevStatus* st) {
  __shared__ double srows[kExpandSmemRows * 8];
  const int NT = m.dim == 3 ? 4 : 3;
  double* grows = slab + (size_t)blockIdx.x * kExpandMaxElems * (NT + nc + 1);
  for (int it = blockIdx.x; it < n_cached; it += gridDim.x) {
    const int v = cache_v[it], n = cache_n[it];
    if (n < 0) {
      if (threadIdx.x == 0) set_status(st, SPRG_EPATCH, v);
      continue;
    }
    double* rows = (n * (NT + nc + 1) <= kExpandSmemRows * 8) ? srows : grows;
    if (!slab_fit(m, cache_el + (size_t)it * kExpandMaxElems, n, ip, u, nc, rows, v, rec) && threadIdx.x == 0)
      set_status(st, SPRG_EPATCH, v);
    __syncwarp();
  }
}

// Tets: the cached patches' fits are linear in the samples as well.  Per mesh,
// the fit's Householder QR (slab_fit's reflectors and 1e-10 rank test) of the
// rows [1, x_ip, y_ip, z_ip] gives w = Q1 R^-T t (t = [1, x_v, y_v, z_v]),
// and every pass recovers rec(v) = sum_i w_i b_i.  Warp per cached patch;
// rows (4 geometry columns, then the 4 reflectors) in shared memory up to
// kExpandSmemRows elements, else in the block's slab.  wn[it] = the patch
// size, or -1 where the rank test fails (the fit's SPRG_EPATCH).
__global__ void __launch_bounds__(32) k_cached_weights(DevMesh m, int n_cached, const int* __restrict__ cache_v,
                                                       const int* __restrict__ cache_n,
                                                       const int* __restrict__ cache_el,
                                                       const long long* __restrict__ woff, double* __restrict__ w,
                                                       int* __restrict__ wn, double* slab) {
  constexpr int NT = 4, LD = 2 * NT;
  __shared__ double srows[kExpandSmemRows * 8];
  const int lane = threadIdx.x & 31;
  double* grows = slab + (size_t)blockIdx.x * kExpandMaxElems * LD;
  for (int it = blockIdx.x; it < n_cached; it += gridDim.x) {
    const int v = cache_v[it], n = cache_n[it];
    if (n < NT) {  // a failed growth (-1) or too few elements
      if (lane == 0) wn[it] = -1;
      continue;
    }
    const int* S = cache_el + (size_t)it * kExpandMaxElems;
    double* rows = n <= kExpandSmemRows ? srows : grows;
    for (int i = lane; i < n; i += 32) {
      const V3 p = elem_ip_point(m, S[i]);
      double* rw = rows + (size_t)i * LD;
      rw[0] = 1.0; rw[1] = p.v[0]; rw[2] = p.v[1]; rw[3] = p.v[2];
    }
    __syncwarp();
    bool ok = true;
    for (int k = 0; k < NT && ok; ++k) {
      double sq = 0;
      for (int i = k + lane; i < n; i += 32) sq += rows[(size_t)i * LD + k] * rows[(size_t)i * LD + k];
      const double cn = sqrt(warp_sum(sq));
      if (cn < 1e-10) {  // uniform across the warp
        ok = false;
        break;
      }
      const double akk = rows[(size_t)k * LD + k];
      double s2 = 0;
      for (int i = lane; i < n; i += 32) {
        double vi = i < k ? 0.0 : rows[(size_t)i * LD + k];
        if (i == k) vi += ((akk < 0) ? -1 : 1) * cn;
        rows[(size_t)i * LD + NT + k] = vi;
        s2 += vi * vi;
      }
      const double rn = sqrt(warp_sum(s2));
      for (int i = lane; i < n; i += 32) rows[(size_t)i * LD + NT + k] /= rn;
      __syncwarp();
      for (int j = k; j < NT; ++j) {
        double d = 0;
        for (int i = k + lane; i < n; i += 32) d += rows[(size_t)i * LD + j] * rows[(size_t)i * LD + NT + k];
        d = warp_sum(d);
        for (int i = k + lane; i < n; i += 32) rows[(size_t)i * LD + j] -= 2 * d * rows[(size_t)i * LD + NT + k];
        __syncwarp();
      }
    }
    if (!ok) {
      if (lane == 0) wn[it] = -1;
      __syncwarp();
      continue;
    }
    // y = R^-T t (forward substitution), then z = H_0 ... H_{NT-1} [y; 0]
    const V3 xv = load_xyz(m.xyz, v);
    const double t[4] = {1.0, xv.v[0], xv.v[1], xv.v[2]};
    double y[4];
    for (int i = 0; i < NT; ++i) {
      double a = t[i];
      for (int j = 0; j < i; ++j) a -= rows[(size_t)j * LD + i] * y[j];
      y[i] = a / rows[(size_t)i * LD + i];
    }
    double* out = w + woff[it];
    for (int i = lane; i < n; i += 32) out[i] = i < NT ? y[i] : 0.0;
    __syncwarp();
    for (int k = NT - 1; k >= 0; --k) {
      double d = 0;
      for (int i = k + lane; i < n; i += 32) d += rows[(size_t)i * LD + NT + k] * out[i];
      d = warp_sum(d);
      for (int i = k + lane; i < n; i += 32) out[i] -= 2 * d * rows[(size_t)i * LD + NT + k];
      __syncwarp();
    }
    if (lane == 0) wn[it] = n;
    __syncwarp();
  }
}

// rec(v) = sum_i w_i b_i over a cached patch, warp per patch (lanes over the
// elements, fixed reduction tree); b_i = the element's IP value, or the
// gradient of the scalar field (nc = 3) / of the vector field (nc = 9)
__global__ void __launch_bounds__(kBlock) k_cached_wsum(DevMesh m, const double* __restrict__ ip,
                                                        const double* __restrict__ u, int nc,
                                                        double* __restrict__ rec, int n_cached,
                                                        const int* __restrict__ cache_v,
                                                        const int* __restrict__ cache_el,
                                                        const long long* __restrict__ woff,
                                                        const double* __restrict__ w, const int* __restrict__ wn,
                                                        DevStatus* st) {
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < n_cached; it += nwarps) {
    const int v = cache_v[it], n = wn[it];
    if (n < 0) {
      if (lane == 0) set_status(st, SPRG_EPATCH, v);
      continue;
    }
    const int* S = cache_el + (size_t)it * kExpandMaxElems;
    const double* wi = w + woff[it];
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = lane; i < n; i += 32) {
      const int el = S[i];
      const double wk = wi[i];
      if (ip) {
        for (int c = 0; c < nc; ++c) acc[c] += wk * ip[(size_t)el * nc + c];
      } else if (nc == 3) {
        const V3 g = elem_grad_scalar(m, el, u);
        for (int c = 0; c < 3; ++c) acc[c] += wk * g.v[c];
      } else {
        for (int r = 0; r < 3; ++r) {
          const V3 g = elem_grad_component(m, el, u, 3, r);
          for (int c = 0; c < 3; ++c) acc[3 * r + c] += wk * g.v[c];
        }
      }
    }
    for (int c = 0; c < nc; ++c) {
      const double a = warp_sum(acc[c]);
      if (lane == 0) rec[(size_t)v * nc + c] = a;
    }
  }
}

// ---------------------------------------------------------------------
// Element error terms (SelfProduct / ElementError, spr/sprEstimateError.cc:98-170)
// ---------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double x, double* sh) {
  x = warp_sum(x);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = x;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
  return t;
}

__global__ void __launch_bounds__(kBlock) k_error(DevMesh m, const double* __restrict__ ip, int nc,
                                                  const double* __restrict__ rec, double* __restrict__ err,
                                                  double* __restrict__ partials, double g_exponent) {
  __shared__ double sh[kBlock / 32];
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  double self_term = 0, g_term = 0;
  if (e < m.T) {
    const int* ev = m.ev + (size_t)e * m.nn;
    V3 x[4];
    for (int a = 0; a < m.nn; ++a) x[a] = load_xyz(m.xyz, ev[a]);
    M3 J = ref::jacobian(x, m.nn, m.dim);
    double dV = ref::jacobian_det(J, m.dim);
    double w = ref::ip_weight(m.dim);
    double N[4];
    ref::ip_shape_values(m.dim, N);
    double v2[9], v1[9];
    for (int k = 0; k < nc; ++k) v2[k] = 0;
    for (int a = 0; a < m.nn; ++a)
      for (int k = 0; k < nc; ++k) v2[k] += rec[(size_t)ev[a] * nc + k] * N[a];
    double vv = 0;
    for (int k = 0; k < nc; ++k) vv += v2[k] * v2[k];
    self_term = vv * w * dV;
    for (int k = 0; k < nc; ++k) v1[k] = ip[(size_t)e * nc + k];
    for (int k = 0; k < nc; ++k) v1[k] -= v2[k];
    double dd = 0;
    for (int k = 0; k < nc; ++k) dd += v1[k] * v1[k];
    double sum = 0;
    sum += dd * w * dV;
    err[e] = sum;
    g_term = pow(sqrt(sum), g_exponent);
  }
  double s1 = block_sum(self_term, sh);
  double s2 = block_sum(g_term, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = s1;
    partials[2 * blockIdx.x + 1] = s2;
  }
}

// one block: fixed-order reduction of the partials, then the size factor
// (the FP32 error kernel's last block runs the same function)
__global__ void __launch_bounds__(kBlock) k_size_factor(const double* __restrict__ partials, int nb, int mode,
                                                        double adapt_ratio, double target, int dim,
                                                        double* out3) {
  __shared__ double sh[kBlock / 32];
  rd_size_factor(partials, nb, mode, adapt_ratio, target, dim, out3, sh);
}

// one block per mesh of a batch: its segments' partials in a fixed order
__global__ void __launch_bounds__(kBlock) k_size_factor_batch(const double* __restrict__ partials, BatchView bv,
                                                              double* __restrict__ out4) {
  __shared__ double sh[kBlock / 32];
  const int k = blockIdx.x;
  double a = 0, g = 0;
  for (int i = bv.segoff[k] + threadIdx.x; i < bv.segoff[k + 1]; i += blockDim.x) {
    a += partials[2 * i];
    g += partials[2 * i + 1];
  }
  double snorm = block_sum(a, sh);
  double gsum = block_sum(g, sh);
  if (threadIdx.x == 0) {
    const double r = bv.ratios[k];
    const double esn = sqrt(snorm);
    out4[4 * k] = snorm;
    out4[4 * k + 1] = gsum;
    out4[4 * k + 2] = pow(r * r * esn * esn / gsum, 0.5);
    out4[4 * k + 3] = 0;
  }
}

// apf::measure of a linear edge (N1 rule, w = 2)
__device__ __forceinline__ double edge_measure(const V3& x0, const V3& x1) {
  V3 x[2] = {x0, x1};
  M3 J = ref::jacobian(x, 2, 1);
  double dV = ref::jacobian_det(J, 1);
  double r = 0;
  r += 2 * dV;
  return r;
}

__constant__ int c_tet_edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
__constant__ int c_tri_edges[3][2] = {{0, 1}, {1, 2}, {2, 0}};

__global__ void __launch_bounds__(kBlock) k_esize(DevMesh m, const double* __restrict__ err,
                                                  const double* __restrict__ out3, int mode, double alpha,
                                                  double beta, double* __restrict__ esize) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.T) return;
  const int* ev = m.ev + (size_t)e * m.nn;
  V3 x[4];
  for (int a = 0; a < m.nn; ++a) x[a] = load_xyz(m.xyz, ev[a]);
  double h = 0;
  for (int i = 0; i < m.ne_el; ++i) {
    int p = m.dim == 3 ? c_tet_edges[i][0] : c_tri_edges[i][0];
    int q = m.dim == 3 ? c_tet_edges[i][1] : c_tri_edges[i][1];
    double l = edge_measure(x[p], x[q]);
    h = (h < l) ? l : h;
  }
  double sf = out3[2];
  double pp = 1, d = m.dim;
  if (mode == 0) {
    double errorNorm = pow(sqrt(err[e]), -(2 / (2 * pp + d)));
    esize[e] = h * errorNorm * sf;
  } else {
    double theta_e = sqrt(err[e]);
    double r = pow(theta_e, ((-2.0) / (2.0 * 1 + m.dim)));
    double h_new = sf * r * h;
    if (h_new < alpha * h) h_new = alpha * h;
    if (h_new > beta * h) h_new = beta * h;
    esize[e] = h_new;
  }
}

__global__ void __launch_bounds__(kBlock) k_average(DevMesh m, const double* __restrict__ esize,
                                                    double* __restrict__ size) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  int b = m.a_off[v], e = m.a_off[v + 1];
  double s = 0;
  for (int k = b; k < e; ++k) s += esize[m.a_el[k]];
  s /= (double)(size_t)(e - b);
  size[v] = s;
}

// MetricSizeField::measure, 2-point Gauss (ma/maSize.cc:158-214)
__device__ __forceinline__ double metric_length(const V3& x0, const V3& x1, const double* hv, const double* Rv) {
  V3 x[2] = {x0, x1};
  M3 J = ref::jacobian(x, 2, 1);
  const double gp[2] = {0.577350269189626, -0.577350269189626};
  double measurement = 0;
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    double N[2];
    ref::edge_shape_values(gp[p], N);
    M3 Q = ref::get_transform(hv, Rv, N, 2);
    double dV2 = ref::jacobian_det(ref::mul(J, Q), 1);
    measurement += 1 * dV2;
  }
  return measurement;
}

__device__ __forceinline__ void identity9(double* R) {
  for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? 1.0 : 0.0;
}

__global__ void __launch_bounds__(kBlock) k_measure_iso(DevMesh m, const double* __restrict__ size,
                                                        double* __restrict__ L) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.E) return;
  int a = m.edv[2 * (size_t)e], b = m.edv[2 * (size_t)e + 1];
  double hv[6], Rv[18];
  double sa = size[a], sb = size[b];
  hv[0] = hv[1] = hv[2] = sa;
  hv[3] = hv[4] = hv[5] = sb;
  identity9(Rv);
  identity9(Rv + 9);
  L[e] = metric_length(load_xyz(m.xyz, a), load_xyz(m.xyz, b), hv, Rv);
}

__global__ void __launch_bounds__(kBlock) k_measure_aniso(DevMesh m, const double* __restrict__ sizes,
                                                          const double* __restrict__ frames,
                                                          double* __restrict__ L) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.E) return;
  int vv[2] = {m.edv[2 * (size_t)e], m.edv[2 * (size_t)e + 1]};
  double hv[6], Rv[18];
  for (int a = 0; a < 2; ++a) {
    for (int k = 0; k < 3; ++k) hv[3 * a + k] = sizes[3 * (size_t)vv[a] + k];
    for (int k = 0; k < 9; ++k) Rv[9 * a + k] = frames[9 * (size_t)vv[a] + k];
  }
  L[e] = metric_length(load_xyz(m.xyz, vv[0]), load_xyz(m.xyz, vv[1]), hv, Rv);
}

// Counting sweeps over entities stride over one wave of blocks and add their
// count with one atomic per block: a per-warp atomic on the one counter
// serialises (about a million same-address atomics per 28.9M-edge sweep).
constexpr int kCountGrid = 152 * 32;  // a wave deep enough for 4-byte accesses
__device__ __forceinline__ void block_count2(unsigned long long* dst0, unsigned a, unsigned long long* dst1,
                                             unsigned b) {
  __shared__ unsigned tot[2][kBlock / 32];
  a = __reduce_add_sync(0xffffffffu, a);
  b = __reduce_add_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0) {
    tot[0][threadIdx.x >> 5] = a;
    tot[1][threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long ta = 0, tb = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      ta += tot[0][w];
      tb += tot[1][w];
    }
    if (ta) atomicAdd(dst0, ta);
    if (dst1 && tb) atomicAdd(dst1, tb);
  }
}


// ma::markEntities (ma/maAdapt.cc:293-324)
__global__ void __launch_bounds__(kBlock) k_mark(int E, const double* __restrict__ L, int which,
                                                 int* __restrict__ flags, unsigned long long* count,
                                                 DevStatus* st) {
  int trueFlag = which == 0 ? SPRG_SPLIT : SPRG_COLLAPSE;
  int setFalse = which == 0 ? SPRG_NEED_NOT_SPLIT : SPRG_NEED_NOT_COLLAPSE;
  int allFalse = which == 0 ? (SPRG_DONT_SPLIT | SPRG_NEED_NOT_SPLIT) : (SPRG_DONT_COLLAPSE | SPRG_NEED_NOT_COLLAPSE);
  unsigned marked = 0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    int f = flags[e];
    if (f & trueFlag) {
      set_status(st, SPRG_EFLAGS, e);
    } else if (!(allFalse & f)) {
      double l = L[e];
      bool pred = which == 0 ? (l > 1.5) : (l < .5);
      if (pred) { f |= trueFlag; ++marked; }
      else f |= setFalse;
      flags[e] = f;
    }
  }
  block_count2(count, marked, nullptr, 0);
}

// ShouldSplit / ShouldCollapse predicates as the device edge-mark bitmap
__global__ void __launch_bounds__(kBlock) k_mark_bits(int E, const double* __restrict__ L, uint32_t* __restrict__ split,
                                                      uint32_t* __restrict__ collapse) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  bool s = false, c = false;
  if (e < E) {
    double l = L[e];
    s = l > 1.5;
    c = l < .5;
  }
  unsigned bs = __ballot_sync(0xffffffffu, s), bc = __ballot_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && e < E) {
    split[e >> 5] = bs;
    collapse[e >> 5] = bc;
  }
}

// markEntities semantics (ma/maAdapt.cc:293-324) applied from a predicate bitmap
__global__ void __launch_bounds__(kBlock) k_apply_bits(int E, const uint32_t* __restrict__ bits, int which,
                                                       int* __restrict__ flags, unsigned long long* count,
                                                       DevStatus* st) {
  int trueFlag = which == 0 ? SPRG_SPLIT : SPRG_COLLAPSE;
  int setFalse = which == 0 ? SPRG_NEED_NOT_SPLIT : SPRG_NEED_NOT_COLLAPSE;
  int allFalse = which == 0 ? (SPRG_DONT_SPLIT | SPRG_NEED_NOT_SPLIT) : (SPRG_DONT_COLLAPSE | SPRG_NEED_NOT_COLLAPSE);
  unsigned marked = 0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    int f = flags[e];
    if (f & trueFlag) {
      set_status(st, SPRG_EFLAGS, e);
    } else if (!(allFalse & f)) {
      if ((bits[e >> 5] >> (e & 31)) & 1u) { f |= trueFlag; ++marked; }
      else f |= setFalse;
      flags[e] = f;
    }
  }
  block_count2(count, marked, nullptr, 0);
}

// both marking passes over one read and one write of the flag words: per
// edge the collapse rule, then the split rule (they test and set disjoint
// bits, so the result equals the two passes in turn); counts[0] split,
// counts[1] collapse.  Four flag words per thread and step (one 16-byte
// access; their four bits sit in one bitmap word).
__device__ __forceinline__ int apply_marks_edge(int f, uint32_t split_bit, uint32_t collapse_bit, int e,
                                                unsigned& ms, unsigned& mc, DevStatus* st) {
  if (f & SPRG_COLLAPSE) {
    set_status(st, SPRG_EFLAGS, e);
  } else if (!((SPRG_DONT_COLLAPSE | SPRG_NEED_NOT_COLLAPSE) & f)) {
    if (collapse_bit) { f |= SPRG_COLLAPSE; ++mc; }
    else f |= SPRG_NEED_NOT_COLLAPSE;
  }
  if (f & SPRG_SPLIT) {
    set_status(st, SPRG_EFLAGS, e);
  } else if (!((SPRG_DONT_SPLIT | SPRG_NEED_NOT_SPLIT) & f)) {
    if (split_bit) { f |= SPRG_SPLIT; ++ms; }
    else f |= SPRG_NEED_NOT_SPLIT;
  }
  return f;
}

__global__ void __launch_bounds__(kBlock) k_apply_marks(int E, const uint32_t* __restrict__ split_bits,
                                                        const uint32_t* __restrict__ collapse_bits,
                                                        int* __restrict__ flags, unsigned long long* counts,
                                                        DevStatus* st, const int* __restrict__ skip) {
  if (skip && *skip) return;  // the caller runs the pass again in FP64
  unsigned ms = 0, mc = 0;
  const int n4 = E >> 2, step = gridDim.x * blockDim.x;
  int4* __restrict__ f4 = reinterpret_cast<int4*>(flags);
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n4; g += step) {
    const int4 v = f4[g];
    const int e0 = g << 2;
    const uint32_t sw = __ldg(split_bits + (e0 >> 5)) >> (e0 & 31);
    const uint32_t cw = __ldg(collapse_bits + (e0 >> 5)) >> (e0 & 31);
    int4 w;
    w.x = apply_marks_edge(v.x, sw & 1u, cw & 1u, e0, ms, mc, st);
    w.y = apply_marks_edge(v.y, (sw >> 1) & 1u, (cw >> 1) & 1u, e0 + 1, ms, mc, st);
    w.z = apply_marks_edge(v.z, (sw >> 2) & 1u, (cw >> 2) & 1u, e0 + 2, ms, mc, st);
    w.w = apply_marks_edge(v.w, (sw >> 3) & 1u, (cw >> 3) & 1u, e0 + 3, ms, mc, st);
    if (w.x != v.x || w.y != v.y || w.z != v.z || w.w != v.w) f4[g] = w;
  }
  for (int e = (n4 << 2) + blockIdx.x * blockDim.x + threadIdx.x; e < E; e += step) {
    const int f = flags[e];
    const int w = apply_marks_edge(f, (split_bits[e >> 5] >> (e & 31)) & 1u, (collapse_bits[e >> 5] >> (e & 31)) & 1u,
                                   e, ms, mc, st);
    if (w != f) flags[e] = w;
  }
  block_count2(counts, ms, counts + 1, mc);
}

// measureTetQuality / measureTriQuality, useMax = true (ma/maQuality.cc:83-167)
__device__ __forceinline__ double q_measure(const V3* x, int nn, int edim, const M3& Q) {
  M3 J = ref::jacobian(x, nn, edim);
  double w = edim == 3 ? 1.0 / 6.0 : (edim == 2 ? 1.0 / 2.0 : 2.0);
  double dV2 = ref::jacobian_det(ref::mul(J, Q), edim);
  double measurement = 0;
  measurement += w * dV2;
  return measurement;
}

template <bool LOG>
__global__ void __launch_bounds__(kBlock) k_quality(DevMesh m, const double* __restrict__ size,
                                                    const double* __restrict__ sizes,
                                                    const double* __restrict__ frames,
                                                    const double* __restrict__ logm, double* __restrict__ q,
                                                    DevStatus* st) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.T) return;
  const int* ev = m.ev + (size_t)e * m.nn;
  M3 Q;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Q.m[i][j] = 0;
  double maxJ = -1.0;
  for (int i = 0; i < m.nn; ++i) {
    int v = ev[i];
    double hv[3], Rv[9], N[1] = {1.0};
    M3 cQ;
    if (LOG) {  // LogAnisoSizeField: the vertex's own log-metric
      bool ok = true;
      cQ = ref::log_transform(logm + 9 * (size_t)v, N, 1, &ok);
      if (!ok) set_status(st, SPRG_EEIGEN, e);
    } else {
      if (size) { hv[0] = hv[1] = hv[2] = size[v]; identity9(Rv); }
      else {
        for (int k = 0; k < 3; ++k) hv[k] = sizes[3 * (size_t)v + k];
        for (int k = 0; k < 9; ++k) Rv[k] = frames[9 * (size_t)v + k];
      }
      cQ = ref::get_transform(hv, Rv, N, 1);
    }
    double cJ = ref::jacobian_det(cQ, m.dim);
    if (cJ > maxJ) { maxJ = cJ; Q = cQ; }
  }
  V3 x[4];
  for (int a = 0; a < m.nn; ++a) x[a] = load_xyz(m.xyz, ev[a]);
  double s = 0;
  for (int i = 0; i < m.ne_el; ++i) {
    int p = m.dim == 3 ? c_tet_edges[i][0] : c_tri_edges[i][0];
    int r = m.dim == 3 ? c_tet_edges[i][1] : c_tri_edges[i][1];
    V3 xe[2] = {x[p], x[r]};
    double l = q_measure(xe, 2, 1, Q);
    s += l * l;
  }
  double Vm = q_measure(x, m.nn, m.dim, Q);
  double res;
  if (m.dim == 3) {
    if (Vm < 0) res = -15552 * (Vm * Vm) / (s * s * s);
    else res = 15552 * (Vm * Vm) / (s * s * s);
  } else {
    res = 48 * (Vm * Vm) / (s * s);
  }
  q[e] = res;
}


// ---------------------------------------------------------------------
// FP64 guard band of the FP32 path: for each listed edge, recompute the
// sizes of both end vertices in FP64 (patch fits of every vertex of their
// elements, element errors and sizes, the vertex averages) and re-decide the
// edge's split/collapse bits.
// ---------------------------------------------------------------------
constexpr int kGuardMaxTets = 96;  // elements around one end vertex

// FP64 gradient of the scalar field on tet t (cofactor inverse; FP64
// accuracy, not the reference's rounding).  Every guard kernel that needs an
// element's gradient evaluates it with this function, so all of them see the
// same bits.
// (explicit fused multiply-adds: the guard wants FP64 accuracy, not the
// reference's rounding, and the FP64 pipe bounds these kernels)
__device__ __forceinline__ void tet_grad_f64(const DevMesh& m, int t, const double* __restrict__ u, double* g) {
  const int4 tv = __ldg(reinterpret_cast<const int4*>(m.ev) + t);
  const V3 x0 = load_xyz(m.xyz, tv.x), x1 = load_xyz(m.xyz, tv.y), x2 = load_xyz(m.xyz, tv.z),
           x3 = load_xyz(m.xyz, tv.w);
  const double u0 = u[tv.x];
  const V3 e1 = ref::sub(x1, x0), e2 = ref::sub(x2, x0), e3 = ref::sub(x3, x0);
  const double d1 = u[tv.y] - u0, d2 = u[tv.z] - u0, d3 = u[tv.w] - u0;
  auto crs = [](const V3& a, const V3& b) {
    return V3{{fma(a.v[1], b.v[2], -a.v[2] * b.v[1]), fma(a.v[2], b.v[0], -a.v[0] * b.v[2]),
               fma(a.v[0], b.v[1], -a.v[1] * b.v[0])}};
  };
  const V3 c1 = crs(e2, e3), c2 = crs(e3, e1), c3 = crs(e1, e2);
  const double inv = 1.0 / fma(e1.v[0], c1.v[0], fma(e1.v[1], c1.v[1], e1.v[2] * c1.v[2]));
  for (int k = 0; k < 3; ++k) g[k] = fma(c1.v[k], d1, fma(c2.v[k], d2, c3.v[k] * d3)) * inv;
}

// Guard pipeline, three kernels over all listed edges at once:
//   collect  thread per (edge, end, element around the end): the distinct
//            vertices of those elements (a per-vertex stamp de-duplicates
//            across edges)
//   fit      warp per collected vertex, lanes over its patch: the FP64
//            element gradients, weighted with the per-mesh FP64 SPR weights
//            (fixed reduction tree), the recovered value
//   decide   warp per edge: FP64 element errors and sizes around both ends,
//            the vertex averages in adjacency order, the metric length, the
//            edge's split/collapse bits
// An element shared by several collected patches has its gradient evaluated
// once per patch: a few thousand extra FP64 gradients per pass cost less
// than a de-duplication stage and its per-element scratch (at 160^3 a stage
// listing the distinct elements and one evaluating them took 12 + 14 us and
// saved 19 us in the fit and decide stages: these small kernels wait on
// their chains of dependent loads, not on the FP64 rate).
// a slot for every winning lane of the warp from one atomic on the shared
// counter (all 32 lanes call it)
__device__ __forceinline__ int warp_slot(bool win, int* counter) {
  const unsigned mask = __ballot_sync(0xffffffffu, win);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (mask) {
    const int leader = __ffs(mask) - 1;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
  }
  return base + __popc(mask & ((1u << lane) - 1));
}

__global__ void k_guard_collect(DevMesh m, const int* __restrict__ items, const int* __restrict__ count, int cap,
                                const int* __restrict__ stamp_id_ptr, int* __restrict__ stamp,
                                int* __restrict__ fit_items,
                                int* __restrict__ fit_count, int fit_cap, int* __restrict__ unresolved) {
  // warp per (edge, end): lanes over the end's elements in rounds of 32
  const int n = min(*count, cap);
  const int stamp_id = *stamp_id_ptr;
  const long total = (long)n * 2 * 32;
  const int lane = threadIdx.x & 31;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int it = (int)(i >> 6);
    const int s = (int)((i >> 5) & 1);
    const int v = m.edv[2 * (size_t)items[it] + s];
    const int b = m.a_off[v], cnt = min(m.a_off[v + 1] - b, kGuardMaxTets);
    for (int r = 0; r < cnt; r += 32) {
      const int j = r + lane;
      const bool valid = j < cnt;
      const int* ev = valid ? m.ev + 4 * (size_t)m.a_el[b + j] : nullptr;
      for (int a = 0; a < 4; ++a) {
        const int w = valid ? ev[a] : 0;
        const bool win = valid && atomicExch(&stamp[w], stamp_id) != stamp_id;
        const int slot = warp_slot(win, fit_count);
        if (win) {
          if (slot < fit_cap) fit_items[slot] = w;
          else atomicAdd(unresolved, 1);
        }
      }
    }
  }
}

// eps*(w) = sum_t w_wt eps_t with the per-mesh FP64 SPR weights, warp per
// collected vertex (lanes over the patch, fixed reduction tree); listed
// patches take their FP64 reference (QR, grown patch) result
__global__ void k_guard_fit(DevMesh m, const double* __restrict__ u, const int* __restrict__ fit_items,
                            const int* __restrict__ fit_count, int fit_cap, GuardScratch g) {
  const int n = min(*fit_count, fit_cap);
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nwarps) {
    const int w = fit_items[i];
    if (g.listed[w]) {
      if (lane < 3) g.rec64[3 * (size_t)w + lane] = g.rec_ref[3 * (size_t)w + lane];
      continue;
    }
    const int beg = m.p_off[w], cnt = m.p_off[w + 1] - beg;
    double r0 = 0, r1 = 0, r2 = 0;
    for (int k = lane; k < cnt; k += 32) {
      double gt[3];
      tet_grad_f64(m, m.p_el[beg + k], u, gt);
      const double wk = g.w64[beg + k];
      r0 += wk * gt[0];
      r1 += wk * gt[1];
      r2 += wk * gt[2];
    }
    for (int o = 16; o > 0; o >>= 1) {
      r0 += __shfl_xor_sync(0xffffffffu, r0, o);
      r1 += __shfl_xor_sync(0xffffffffu, r1, o);
      r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    }
    if (lane == 0) {
      g.rec64[3 * (size_t)w] = r0;
      g.rec64[3 * (size_t)w + 1] = r1;
      g.rec64[3 * (size_t)w + 2] = r2;
    }
  }
}

// 64 threads per edge (two edges per block): thread j takes element j of
// the two ends' lists, so each computes one element size
__global__ void __launch_bounds__(128) k_guard_decide(DevMesh m, const double* __restrict__ u,
                                                      const double* __restrict__ out3, GuardScratch g,
                                                      const int* __restrict__ items, const int* __restrict__ count,
                                                      int cap, uint32_t* split, uint32_t* collapse,
                                                      int* __restrict__ unresolved, BatchView bv) {
  // the stamp id of the next guard pass (the collect stage of this one is
  // done): a device counter, so a pass replayed from a CUDA graph still
  // de-duplicates with a fresh id; 0, the stamps' initial value, is skipped
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int next = *g.stamp_id + 1;
    *g.stamp_id = next > 0 ? next : 1;
  }
  __shared__ double esz[2][2 * kGuardMaxTets];
  const int half = threadIdx.x >> 6, j0 = threadIdx.x & 63;
  const int n = min(*count, cap);
  // every thread of the block runs the same number of rounds (the barriers)
  for (int base = blockIdx.x * 2; base < n; base += gridDim.x * 2) {
    const int it = base + half;
    const bool live = it < n;
    int e = 0, ab[2] = {0, 0}, cnt[2] = {0, 0}, off[2] = {0, 0};
    bool bad = false;
    double sf = 0;
    if (live) {
      e = items[it];
      ab[0] = m.edv[2 * (size_t)e];
      ab[1] = m.edv[2 * (size_t)e + 1];
      sf = batch_sf(bv, out3, ab[0]);
      for (int s = 0; s < 2; ++s) {
        off[s] = m.a_off[ab[s]];
        cnt[s] = m.a_off[ab[s] + 1] - off[s];
      }
      bad = cnt[0] > kGuardMaxTets || cnt[1] > kGuardMaxTets;
      if (!bad)
        for (int j = j0; j < cnt[0] + cnt[1]; j += 64) {
          const int s = j < cnt[0] ? 0 : 1;
          const int t = m.a_el[off[s] + j - (s ? cnt[0] : 0)];
          const int* ev = m.ev + 4 * (size_t)t;
          double gt[3];
          tet_grad_f64(m, t, u, gt);
          double v2[3] = {0, 0, 0};
          for (int k = 0; k < 4; ++k)
            for (int c = 0; c < 3; ++c) v2[c] += g.rec64[3 * (size_t)ev[k] + c] * 0.25;
          const double2 dh = g.geo64[t];  // det J, h_max
          double dd = 0;
          for (int c = 0; c < 3; ++c) dd += (gt[c] - v2[c]) * (gt[c] - v2[c]);
          esz[half][j] = dh.y * pow(dd * (1.0 / 6.0) * dh.x, -0.2) * sf;
        }
    }
    __syncthreads();
    if (live && j0 == 0) {
      double sz[2] = {0, 0};
      for (int s = 0; s < 2 && !bad; ++s) {
        for (int i = 0; i < cnt[s]; ++i) sz[s] += esz[half][(s ? cnt[0] : 0) + i];
        sz[s] /= (double)cnt[s];
      }
      if (bad || !(sz[0] == sz[0]) || !(sz[1] == sz[1])) {  // too many elements, or a NaN size
        atomicAdd(unresolved, 1);
      } else {
        double hv[6] = {sz[0], sz[0], sz[0], sz[1], sz[1], sz[1]}, Rv[18];
        identity9(Rv);
        identity9(Rv + 9);
        double L = metric_length(load_xyz(m.xyz, ab[0]), load_xyz(m.xyz, ab[1]), hv, Rv);
        uint32_t bit = 1u << (e & 31);
        if (L > 1.5) atomicOr(&split[e >> 5], bit); else atomicAnd(&split[e >> 5], ~bit);
        if (L < .5) atomicOr(&collapse[e >> 5], bit); else atomicAnd(&collapse[e >> 5], ~bit);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------
// anisotropic metric from a nodal Hessian (the 2D anisotropic workload's
// size and frame fields): eigen-decompose the symmetric part, order the
// principal directions by |lambda| descending, sign each direction so its
// largest component is positive (2D: first direction's x >= 0, second its
// +90 degree rotation), h_i = clamp(sqrt(eps / |lambda_i|), h_min, h_max);
// frames row-major with the directions as columns (AnisoSizeField's R).
// ---------------------------------------------------------------------
__device__ void sym_eigen3(double A[3][3], double lam[3], double Vm[3][3]) {
  // cyclic Jacobi, fixed sweep count (deterministic)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Vm[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 8; ++sweep) {
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const double apq = A[p][q];
        if (apq == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 3; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = Vm[k][p], vkq = Vm[k][q];
          Vm[k][p] = c * vkp - sn * vkq;
          Vm[k][q] = sn * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) lam[i] = A[i][i];
}

__device__ __forceinline__ double metric_size(double lam, double eps, double hmin, double hmax) {
  const double a = fabs(lam);
  if (!(a > 0)) return hmax;
  return fmin(fmax(sqrt(eps / a), hmin), hmax);
}

// one vertex's metric from its Hessian row h (9 doubles): sizes hs, frame R
// (directions as columns)
// Power-of-two prescaling of a Hessian before its eigen-decomposition, from
// the largest biased exponent E of its entries (integer operations): none
// while the largest entry lies in [2^-400, 2^401) or an entry is not finite,
// else by 2^-e with e = E - 1022 (the largest entry then in [1/2, 1); e =
// -1022 when every entry is zero or subnormal).  Eigenvectors are scale-free
// and eigenvalues scale exactly (they are scaled back by 2^e), so this only
// changes Hessians whose products underflow or overflow: a field flat to
// 1e-160, where hd^2 + b^2 underflowed and the direction came out 0 / 0, now
// gets the direction the exact arithmetic would.
__device__ __forceinline__ int dbexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }
__device__ __forceinline__ int hessian_scale_exp(int E) {
  if (E == 2047 || (E >= 623 && E <= 1423)) return 0;
  return E == 0 ? -1022 : E - 1022;
}
// x 2^k, exact unless the result under- or overflows (two factors where 2^k
// itself is outside the normal range)
__device__ __forceinline__ double times_pow2(double x, int k) {
  auto p2 = [](int j) { return __longlong_as_double((long long)(1023 + j) << 52); };  // -1022 <= j <= 1023
  if (k >= -1022 && k <= 1023) return x * p2(k);
  return x * p2(k / 2) * p2(k - k / 2);
}

__device__ void hessian_metric_vertex(int dim, const double* __restrict__ h, double eps, double hmin, double hmax,
                                      double hs[3], double R[3][3]) {
  if (dim == 2) {
    const double b0 = 0.5 * (h[1] + h[3]);
    const int es = hessian_scale_exp(max(max(dbexp(h[0]), dbexp(h[4])), dbexp(b0)));
    double a = h[0], b = b0, c = h[4];
    if (es) {
      a = times_pow2(a, -es);
      b = times_pow2(b, -es);
      c = times_pow2(c, -es);
    }
    const double mid = 0.5 * (a + c), hd = 0.5 * (a - c);
    const double d = sqrt(hd * hd + b * b);
    double l1 = mid + d, l2 = mid - d;
    double x, y;
    if (b == 0.0) {
      x = a >= c ? 1.0 : 0.0;
      y = a >= c ? 0.0 : 1.0;
    } else if (a >= c) {
      x = l1 - c;
      y = b;
    } else {
      x = b;
      y = l1 - a;
    }
    const double n = sqrt(x * x + y * y);
    x /= n;
    y /= n;
    if (fabs(l2) > fabs(l1)) {  // the second direction is (-y, x)
      const double tl = l1;
      l1 = l2;
      l2 = tl;
      const double tx = x;
      x = -y;
      y = tx;
    }
    if (x < 0 || (x == 0 && y < 0)) {
      x = -x;
      y = -y;
    }
    R[0][0] = x; R[0][1] = -y; R[0][2] = 0;
    R[1][0] = y; R[1][1] = x;  R[1][2] = 0;
    R[2][0] = 0; R[2][1] = 0;  R[2][2] = 1;
    hs[0] = metric_size(es ? times_pow2(l1, es) : l1, eps, hmin, hmax);
    hs[1] = metric_size(es ? times_pow2(l2, es) : l2, eps, hmin, hmax);
    hs[2] = hmax;
  } else {
    double A[3][3], lam[3], Vm[3][3];
    int E = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        A[i][j] = 0.5 * (h[3 * i + j] + h[3 * j + i]);
        E = max(E, dbexp(A[i][j]));
      }
    const int es = hessian_scale_exp(E);
    if (es)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = times_pow2(A[i][j], -es);
    sym_eigen3(A, lam, Vm);
    if (es)
      for (int i = 0; i < 3; ++i) lam[i] = times_pow2(lam[i], es);
    int o[3] = {0, 1, 2};
    for (int i = 0; i < 3; ++i)
      for (int j = i + 1; j < 3; ++j)
        if (fabs(lam[o[j]]) > fabs(lam[o[i]])) {
          const int t = o[i];
          o[i] = o[j];
          o[j] = t;
        }
    for (int k = 0; k < 2; ++k) {
      double col[3] = {Vm[0][o[k]], Vm[1][o[k]], Vm[2][o[k]]};
      int im = 0;
      for (int i = 1; i < 3; ++i)
        if (fabs(col[i]) > fabs(col[im])) im = i;
      const double sg = col[im] < 0 ? -1.0 : 1.0;
      for (int i = 0; i < 3; ++i) R[i][k] = sg * col[i];
      hs[k] = metric_size(lam[o[k]], eps, hmin, hmax);
    }
    // third direction: right-handed completion
    R[0][2] = R[1][0] * R[2][1] - R[2][0] * R[1][1];
    R[1][2] = R[2][0] * R[0][1] - R[0][0] * R[2][1];
    R[2][2] = R[0][0] * R[1][1] - R[1][0] * R[0][1];
    hs[2] = metric_size(lam[o[2]], eps, hmin, hmax);
  }
}

__global__ void k_hessian_metric(int V, int dim, const double* __restrict__ H, double eps, double hmin, double hmax,
                                 double* __restrict__ sizes, double* __restrict__ frames) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  double R[3][3], hs[3];
  hessian_metric_vertex(dim, H + 9 * (size_t)v, eps, hmin, hmax, hs, R);
  for (int k = 0; k < 3; ++k) sizes[3 * (size_t)v + k] = hs[k];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) frames[9 * (size_t)v + 3 * i + j] = R[i][j];
}

// The FP64 metric of a vertex for the guard and the quality's tie-breaks:
// read from the materialised arrays, or (mixed pass on triangles, where they
// are not stored) rebuilt from the Hessian by hessian_metric_vertex, the
// same function as the FP64 pass's, so the values are that pass's bits.
struct MetricSrc {
  const double* sizes;   // V x 3, or null: rebuild from H
  const double* frames;  // V x 9
  const double* H;       // V x 9
  int dim;
  double eps, hmin, hmax;
};
__device__ __forceinline__ void metric_at(const MetricSrc& src, int v, double* hs, double* R) {
  if (src.sizes) {
    for (int k = 0; k < 3; ++k) hs[k] = src.sizes[3 * (size_t)v + k];
    for (int k = 0; k < 9; ++k) R[k] = src.frames[9 * (size_t)v + k];
    return;
  }
  double Rm[3][3];
  hessian_metric_vertex(src.dim, src.H + 9 * (size_t)v, src.eps, src.hmin, src.hmax, hs, Rm);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = Rm[i][j];
}

// ---------------------------------------------------------------------
// adjacency construction
// ---------------------------------------------------------------------
__global__ void k_count_v2e(DevMesh m, int* cnt) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.T) return;
  for (int a = 0; a < m.nn; ++a) atomicAdd(&cnt[m.ev[(size_t)e * m.nn + a]], 1);
}
__global__ void k_fill_v2e(DevMesh m, const int* off, int* cursor, int* el) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.T) return;
  for (int a = 0; a < m.nn; ++a) {
    int v = m.ev[(size_t)e * m.nn + a];
    int pos = off[v] + atomicAdd(&cursor[v], 1);
    el[pos] = e;
  }
}
// short segments: insertion sort by one thread per segment
__global__ void k_sort_segments(int V, const int* off, int* el) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  int b = off[v], e = off[v + 1];
  for (int i = b + 1; i < e; ++i) {
    int x = el[i], j = i - 1;
    while (j >= b && el[j] > x) { el[j + 1] = el[j]; --j; }
    el[j + 1] = x;
  }
}
__global__ void k_xyz_fixed(DevMesh m, double cx, double cy, double cz, double s, int* xyzq) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  const double q = s * 0x1p30;  // (x - c) s in [0, 1]
  reinterpret_cast<int4*>(xyzq)[v] =
      make_int4(__double2int_rn((m.xyz[3 * (size_t)v] - cx) * q), __double2int_rn((m.xyz[3 * (size_t)v + 1] - cy) * q),
                __double2int_rn((m.xyz[3 * (size_t)v + 2] - cz) * q), 0);
}

inline int nblk(long n, int b = kBlock) { return (int)((n + b - 1) / b); }
inline int count_grid(long n) { return (int)std::min<long>((n + kBlock - 1) / kBlock, kCountGrid); }

// ---------------------------------------------------------------------
// MA sweeps around the marks (ma/maSize.cc:652-690, ma/maShape.cc:132-169,
// ma/maCoarsen.cc:36-60)
// ---------------------------------------------------------------------
// MetricSizeField::measure under LogAnisoSizeField (ma/maSize.cc:158-216,
// 508-523): two Gauss points, log-metrics of both ends interpolated
__device__ __forceinline__ double log_metric_length(const V3& x0, const V3& x1, const double* __restrict__ la,
                                                    const double* __restrict__ lb, bool* ok) {
  V3 x[2] = {x0, x1};
  M3 J = ref::jacobian(x, 2, 1);
  double Mv[18];
  for (int k = 0; k < 9; ++k) {
    Mv[k] = la[k];
    Mv[9 + k] = lb[k];
  }
  const double gp[2] = {0.577350269189626, -0.577350269189626};
  double measurement = 0;
  for (int p = 0; p < 2; ++p) {
    double N[2];
    ref::edge_shape_values(gp[p], N);
    M3 Q = ref::log_transform(Mv, N, 2, ok);
    double dV2 = ref::jacobian_det(ref::mul(J, Q), 1);
    measurement += 1 * dV2;
  }
  return measurement;
}

// length of the vertex pair (a, b) under a size field: kind 0 the identity
// field (apf::measure of the edge, ma/maSize.cc:54-60), 1 the isotropic
// user field, 2 the anisotropic one, 3 LogAnisoSizeField (per-vertex
// log-metrics) -- the same evaluation as the edge measure kernels, for
// edges that may not exist yet
__device__ __forceinline__ double pair_length(const DevMesh& m, int kind, int a, int b,
                                              const double* __restrict__ size, const double* __restrict__ sizes,
                                              const double* __restrict__ frames, const double* __restrict__ logm,
                                              bool* ok) {
  const V3 xa = load_xyz(m.xyz, a), xb = load_xyz(m.xyz, b);
  if (kind == 0) return edge_measure(xa, xb);
  if (kind == 3) return log_metric_length(xa, xb, logm + 9 * (size_t)a, logm + 9 * (size_t)b, ok);
  double hv[6], Rv[18];
  if (kind == 1) {
    const double sa = size[a], sb = size[b];
    hv[0] = hv[1] = hv[2] = sa;
    hv[3] = hv[4] = hv[5] = sb;
    identity9(Rv);
    identity9(Rv + 9);
  } else {
    const int vv[2] = {a, b};
    for (int i = 0; i < 2; ++i) {
      for (int k = 0; k < 3; ++k) hv[3 * i + k] = sizes[3 * (size_t)vv[i] + k];
      for (int k = 0; k < 9; ++k) Rv[9 * i + k] = frames[9 * (size_t)vv[i] + k];
    }
  }
  return metric_length(xa, xb, hv, Rv);
}

// pairs == nullptr: the mesh's own edges
__global__ void __launch_bounds__(kBlock) k_measure_pairs(DevMesh m, int kind, long long n,
                                                          const int* __restrict__ pairs,
                                                          const double* __restrict__ size,
                                                          const double* __restrict__ sizes,
                                                          const double* __restrict__ frames,
                                                          const double* __restrict__ logm, double* __restrict__ L,
                                                          DevStatus* st) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int* ab = pairs ? pairs + 2 * i : m.edv + 2 * i;
  bool ok = true;
  L[i] = pair_length(m, kind, ab[0], ab[1], size, sizes, frames, logm, &ok);
  if (!ok) set_status(st, SPRG_EEIGEN, (int)i);
}

// LogAnisoSizeField::init: per-vertex log-metric from sizes and frames
__global__ void __launch_bounds__(kBlock) k_log_metric(int V, const double* __restrict__ sizes,
                                                       const double* __restrict__ frames,
                                                       double* __restrict__ logm) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  ref::vertex_logm(sizes + 3 * (size_t)v, frames + 9 * (size_t)v, logm + 9 * (size_t)v);
}

// getMaximumEdgeLength: the reference keeps `length > maxLength` from 0, so
// NaN and non-positive lengths never win; positive doubles order like their
// bit patterns, so the block maxima meet in one 64-bit atomicMax
__global__ void __launch_bounds__(kBlock) k_max_positive(long long n, const double* __restrict__ x,
                                                         unsigned long long* __restrict__ out) {
  double best = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    if (v > best) best = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

// fixed-grid partial sums in a fixed order, then one thread sums the
// partials: the same bits on every run
constexpr int kSumBlocks = 1024;
__global__ void __launch_bounds__(kBlock) k_sum_partials(long long n, const double* __restrict__ x,
                                                         double* __restrict__ partials) {
  __shared__ double sh[kBlock / 32];
  double s = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    s += x[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < kBlock / 32; ++w) t += sh[w];
    partials[blockIdx.x] = t;
  }
}
__global__ void k_sum_final(int nb, const double* __restrict__ partials, double* __restrict__ out) {
  double t = 0;
  for (int b = 0; b < nb; ++b) t += partials[b];
  *out = t;
}

// getMinQuality: the reference scans the elements in order and keeps
// `qual < minqual` from 1, i.e. the first element attaining the minimum
// below 1 (NaN never wins).  Pass 1 finds the minimum value (-0 and +0
// alike) through an order-preserving 64-bit key, pass 2 the first index
// holding it; the result is that element's value.
__device__ __forceinline__ unsigned long long order_key(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v == 0.0 ? 0.0 : v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__global__ void __launch_bounds__(kBlock) k_min_below(long long n, const double* __restrict__ x, double start,
                                                      unsigned long long* __restrict__ key) {
  double best = start;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    if (v < best) best = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best < start) atomicMin(key, order_key(best));
}
__global__ void __launch_bounds__(kBlock) k_first_equal(long long n, const double* __restrict__ x,
                                                        const unsigned long long* __restrict__ key,
                                                        unsigned long long* __restrict__ first) {
  const unsigned long long k = *key;
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  const double target = __longlong_as_double((long long)b);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (x[i] == target) {
      atomicMin(first, (unsigned long long)i);
      break;
    }
}

// markBadQuality: ma::markEntities over the elements with predicate
// quality < goodQuality, BAD_QUALITY / OK_QUALITY (ma/maShape.cc:132-136)
__global__ void __launch_bounds__(kBlock) k_mark_quality(int T, const double* __restrict__ q, double good,
                                                         int* __restrict__ flags, unsigned long long* count,
                                                         DevStatus* st) {
  unsigned marked = 0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < T; e += gridDim.x * blockDim.x) {
    int f = flags[e];
    if (f & SPRG_BAD_QUALITY) {
      set_status(st, SPRG_EFLAGS, e);
    } else if (!(f & SPRG_OK_QUALITY)) {
      if (q[e] < good) {
        f |= SPRG_BAD_QUALITY;
        ++marked;
      } else {
        f |= SPRG_OK_QUALITY;
      }
      flags[e] = f;
    }
  }
  block_count2(count, marked, nullptr, 0);
}


// ---------------------------------------------------------------------
// Mixed-precision anisotropic pass (SPRG_FP32 on the Hessian-metric
// workload).  The recoveries use per-mesh FP64 patch weights, the metric
// stays FP64, the edge measure and the qualities run in FP32: every edge
// whose FP32 length is within its error bound of 0.5 or 1.5 is re-measured
// by the FP64 kernel, so the marks equal the FP64 pass's.
// ---------------------------------------------------------------------
// SPR weights of a triangle patch: the fitted value at the vertex is a
// fixed combination of the patch samples, eps*(v) = sum_j w_j b_j with
// w = Q_c R^-T t (Q_c the first NT columns of Q, t = [1, x_v, y_v]).  The QR
// is the reference's (as in k_recover_tri); listed: patches the weights do
// not cover (fewer than NT or more than MAXM elements, rank deficient),
// which take the FP64 fit paths every pass.
template <int MAXM>
__global__ void __launch_bounds__(128) k_tri_weights(DevMesh m, double* __restrict__ w,
                                                     unsigned char* __restrict__ listed, ExpandList lst) {
  constexpr int NT = 3;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  const int beg = m.p_off[v];
  const int cnt = m.p_off[v + 1] - beg;
  auto give_up = [&]() {
    listed[v] = 1;
    const int slot = atomicAdd(lst.count, 1);
    if (slot < lst.cap) lst.items[slot] = v;
  };
  if (cnt < NT || cnt > MAXM) {
    give_up();
    return;
  }
  double R[MAXM][NT];
#pragma unroll
  for (int i = 0; i < MAXM; ++i) {
    R[i][0] = R[i][1] = R[i][2] = 0;
    if (i < cnt) {
      const V3 p = elem_ip_point(m, m.p_el[beg + i]);
      R[i][0] = 1.0;
      R[i][1] = p.v[0];
      R[i][2] = p.v[1];
    }
  }
  double H[NT][MAXM];
#pragma unroll
  for (int k = 0; k < NT; ++k) {
    double cn = 0;
#pragma unroll
    for (int i = k; i < MAXM; ++i)
      if (i < cnt) cn += R[i][k] * R[i][k];
    cn = sqrt(cn);
    if (cn < 1e-10) {
      give_up();
      return;
    }
#pragma unroll
    for (int i = 0; i < MAXM; ++i) H[k][i] = (i >= k && i < cnt) ? R[i][k] : 0.0;
    H[k][k] += ((R[k][k] < 0) ? -1 : 1) * cn;
    double rn = 0;
#pragma unroll
    for (int i = k; i < MAXM; ++i)
      if (i < cnt) rn += H[k][i] * H[k][i];
    rn = sqrt(rn);
#pragma unroll
    for (int i = k; i < MAXM; ++i)
      if (i < cnt) H[k][i] /= rn;
#pragma unroll
    for (int j = k; j < NT; ++j) {
      double dot = 0;
#pragma unroll
      for (int i = k; i < MAXM; ++i)
        if (i < cnt) dot += R[i][j] * H[k][i];
#pragma unroll
      for (int i = k; i < MAXM; ++i)
        if (i < cnt) R[i][j] -= 2 * dot * H[k][i];
    }
  }
  // z = R^-T t
  const V3 xv = load_xyz(m.xyz, v);
  double z[NT];
  z[0] = 1.0 / R[0][0];
  z[1] = (xv.v[0] - R[0][1] * z[0]) / R[1][1];
  z[2] = (xv.v[1] - R[0][2] * z[0] - R[1][2] * z[1]) / R[2][2];
#pragma unroll
  for (int r = 0; r < MAXM; ++r) {
    if (r >= cnt) break;
    double q[MAXM];
#pragma unroll
    for (int j = 0; j < MAXM; ++j) q[j] = (j == r) ? 1.0 : 0.0;
#pragma unroll
    for (int k = 0; k < NT; ++k) {
      double dot = 0;
#pragma unroll
      for (int j = k; j < MAXM; ++j)
        if (j < cnt) dot += q[j] * H[k][j];
#pragma unroll
      for (int j = k; j < MAXM; ++j)
        if (j < cnt) q[j] -= 2 * dot * H[k][j];
    }
    w[beg + r] = q[0] * z[0] + q[1] * z[1] + q[2] * z[2];
  }
  listed[v] = 0;
}

// Per vertex: the FP32 metric record h (3), frame (9, row-major) for the
// edge measure, and the quality record: the vertex transform Q =
// orth(R) diag(1/h) and its Jacobian determinant in FP32.  The quality
// kernel picks the vertex with the largest determinant as the reference
// does; where the FP32 determinants cannot separate the candidates and the
// candidates give different qualities, it decides with the FP64
// determinants of the FP64 quality kernel's arithmetic.
// 48 bytes (three 16-byte words) so the records move with vector accesses
struct __align__(16) QualityRec {
  float q[9];
  float cj;
  float pad[2];
};
__device__ __forceinline__ void store_qrec(QualityRec* dst, const float Q[3][3], float cj) {
  float4* d = reinterpret_cast<float4*>(dst);
  d[0] = make_float4(Q[0][0], Q[0][1], Q[0][2], Q[1][0]);
  d[1] = make_float4(Q[1][1], Q[1][2], Q[2][0], Q[2][1]);
  d[2] = make_float4(Q[2][2], cj, 0.f, 0.f);
}
// a metric record (12 floats: h, frame) as three 16-byte stores / loads
__device__ __forceinline__ void store_met(float* dst, const float* o) {
  float4* d = reinterpret_cast<float4*>(dst);
  d[0] = make_float4(o[0], o[1], o[2], o[3]);
  d[1] = make_float4(o[4], o[5], o[6], o[7]);
  d[2] = make_float4(o[8], o[9], o[10], o[11]);
}
__device__ __forceinline__ void load_met(const float* src, float* o) {
  const float4* p = reinterpret_cast<const float4*>(src);
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
  o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
  o[8] = c.x; o[9] = c.y; o[10] = c.z; o[11] = c.w;
}
__device__ __forceinline__ void transform_f32(const float* h, const float* R, float Q[3][3]) {
  // orthogonalised frame columns, then Q = R diag(1 / h)
  float c0x = R[0], c0y = R[3], c0z = R[6], c1x = R[1], c1y = R[4], c1z = R[7];
  const float l0 = sqrtf(c0x * c0x + c0y * c0y + c0z * c0z);
  c0x /= l0; c0y /= l0; c0z /= l0;
  const float d = c0x * c1x + c0y * c1y + c0z * c1z;
  c1x -= c0x * d; c1y -= c0y * d; c1z -= c0z * d;
  const float l1 = sqrtf(c1x * c1x + c1y * c1y + c1z * c1z);
  c1x /= l1; c1y /= l1; c1z /= l1;
  const float c2x = c0y * c1z - c0z * c1y, c2y = c0z * c1x - c0x * c1z, c2z = c0x * c1y - c0y * c1x;
  Q[0][0] = c0x / h[0]; Q[0][1] = c1x / h[1]; Q[0][2] = c2x / h[2];
  Q[1][0] = c0y / h[0]; Q[1][1] = c1y / h[1]; Q[1][2] = c2y / h[2];
  Q[2][0] = c0z / h[0]; Q[2][1] = c1z / h[1]; Q[2][2] = c2z / h[2];
}
__device__ __forceinline__ float det_f32(const float Q[3][3], int dim) {
  if (dim == 3)
    return Q[0][0] * (Q[1][1] * Q[2][2] - Q[1][2] * Q[2][1]) - Q[0][1] * (Q[1][0] * Q[2][2] - Q[1][2] * Q[2][0]) +
           Q[0][2] * (Q[1][0] * Q[2][1] - Q[1][1] * Q[2][0]);
  const float x = Q[0][1] * Q[1][2] - Q[0][2] * Q[1][1], y = Q[0][2] * Q[1][0] - Q[0][0] * Q[1][2],
              z = Q[0][0] * Q[1][1] - Q[0][1] * Q[1][0];
  return sqrtf(x * x + y * y + z * z);  // |row0 x row1|
}

__global__ void __launch_bounds__(kBlock) k_metric_f32(int V, int dim, const double* __restrict__ sizes,
                                                       const double* __restrict__ frames, float* __restrict__ out,
                                                       QualityRec* __restrict__ qrec) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  float o[12];
  for (int k = 0; k < 3; ++k) o[k] = (float)sizes[3 * (size_t)v + k];
  for (int k = 0; k < 9; ++k) o[3 + k] = (float)frames[9 * (size_t)v + k];
  store_met(out + 12 * (size_t)v, o);
  float Q[3][3];
  transform_f32(o, o + 3, Q);
  store_qrec(qrec + v, Q, det_f32(Q, dim));
}

// Integer forms of the FP64 tests and conversions the mixed metric needs
// (on this GPU the FP64 pipe is the scarce one: the comparisons, min / max
// and conversions would each take an FP64 issue slot).  Non-NaN operands.
__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ bool d_is_zero(double x) { return (dbits(x) << 1) == 0; }
__device__ __forceinline__ bool d_is_neg(double x) { return (dbits(x) >> 63) && !d_is_zero(x); }  // x < 0
__device__ __forceinline__ bool d_abs_gt(double x, double y) { return (dbits(x) << 1) > (dbits(y) << 1); }
// x >= y: doubles ordered as signed integers after flipping the magnitude
// bits of negatives (-0 taken as +0)
__device__ __forceinline__ long long d_key(double x) {
  const long long b = __double_as_longlong(x);
  return d_is_zero(x) ? 0 : (b ^ ((b >> 63) & 0x7fffffffffffffffLL));
}
// x 2^-e rounded toward zero to FP32; below FP32's normal range 0, above it
// infinity
__device__ __forceinline__ float d_to_f32_scaled(double x, int e) {
  const unsigned long long b = dbits(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int ef = (int)((b >> 52) & 0x7ff) - 1023 - e + 127;
  if (ef <= 0 || d_is_zero(x)) return __uint_as_float(sign);
  if (ef >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((unsigned)ef << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

// Mixed pass on triangles: the FP32 metric records and quality records
// straight from the FP64 Hessian.  Every decision of hessian_metric_vertex
// (the b == 0 and a >= c branches, the |lambda| order, the sign convention)
// is taken on the same FP64 values as there, with the FP64 arithmetic those
// values need (one square root); the tests themselves and the conversions
// run as integer operations on the bit patterns.  The magnitudes that
// follow (the direction's normalisation, sqrt(eps / |lambda|)) are FP32
// operations on those values rounded toward zero, a few ulps from the FP64
// results, inside the FP32 measure's bound.  The sign test runs on the
// unnormalised FP64 direction (the normalisation by a positive length keeps
// signs and zeros).
__global__ void __launch_bounds__(kBlock) k_metric_mixed2d(int V, const double* __restrict__ H, double eps,
                                                           double hmin, double hmax, float* __restrict__ out,
                                                           QualityRec* __restrict__ qrec) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  const double* h = H + 9 * (size_t)v;
  // the same power-of-two prescaling as hessian_metric_vertex, so every
  // decision below sees that function's values
  const double b0 = 0.5 * (h[1] + h[3]);
  const int es = hessian_scale_exp(max(max(dbexp(h[0]), dbexp(h[4])), dbexp(b0)));
  double a = h[0], b = b0, c = h[4];
  if (es) {
    a = times_pow2(a, -es);
    b = times_pow2(b, -es);
    c = times_pow2(c, -es);
  }
  const double mid = 0.5 * (a + c), hd = 0.5 * (a - c);
  const double d = sqrt(hd * hd + b * b);
  double l1 = mid + d, l2 = mid - d;
  double x, y;
  const bool ageqc = d_key(a) >= d_key(c);
  if (d_is_zero(b)) {
    x = ageqc ? 1.0 : 0.0;
    y = ageqc ? 0.0 : 1.0;
  } else if (ageqc) {
    x = l1 - c;
    y = b;
  } else {
    x = b;
    y = l1 - a;
  }
  if (d_abs_gt(l2, l1)) {
    const double tl = l1;
    l1 = l2;
    l2 = tl;
    const double tx = x;
    x = -y;
    y = tx;
  }
  const bool flip = d_is_neg(x) || (d_is_zero(x) && d_is_neg(y));
  // FP32 direction scaled by 2^-e, e the exponent of max(|x|, |y|) (> 0: one
  // of them is b != 0 or l1 - c > 0), then normalised in FP32
  const unsigned long long mx = (dbits(x) << 1) > (dbits(y) << 1) ? dbits(x) : dbits(y);
  const int ex = (int)((mx >> 52) & 0x7ff) - 1023;
  float xf = d_to_f32_scaled(x, ex), yf = d_to_f32_scaled(y, ex);
  if (flip) {
    xf = -xf;
    yf = -yf;
  }
  const float nf = sqrtf(xf * xf + yf * yf);
  xf /= nf;
  yf /= nf;
  const float epsf = (float)eps, hminf = (float)hmin, hmaxf = (float)hmax;
  auto size_f32 = [&](double l) {
    if (d_is_zero(l) || (((dbits(l) >> 52) & 0x7ff) == 0x7ff && (dbits(l) << 12) != 0)) return hmaxf;  // 0, NaN
    return fminf(fmaxf(sqrtf(epsf / fabsf(d_to_f32_scaled(l, 0))), hminf), hmaxf);
  };
  if (es) {
    l1 = times_pow2(l1, es);
    l2 = times_pow2(l2, es);
  }
  const float o[12] = {size_f32(l1), size_f32(l2), hmaxf, xf, -yf, 0.f, yf, xf, 0.f, 0.f, 0.f, 1.f};
  store_met(out + 12 * (size_t)v, o);
  float Q[3][3];
  transform_f32(o, o + 3, Q);
  store_qrec(qrec + v, Q, det_f32(Q, 2));
}

// AnisoSizeField measure in FP32 with a relative error bound.  Per Gauss
// point: R(xi) interpolated and orthogonalised, dV = |(J.r_j / h_j)_j|.  Each
// term J.r_j / h_j carries an absolute error of a few units of |J| / h_j
// times 2^-24, amplified by the orthogonalisation's conditioning (the first
// column divided by its length |c0|, the second, after the projection, by
// |r1|); relative to dV that is at most
// kAnisoUlps 2^-24 (1 + 1/|c0|)(1 + 1/|r1|) sum_j (|J| / h_j) / dV,
// where the last factor is >= 1 and kAnisoUlps covers the few roundings of
// each step (inputs, interpolation, normalisations, dot products, sqrt).
constexpr float kAnisoUlps = 64.f;
__device__ __forceinline__ float aniso_dv_f32(float Jx, float Jy, float Jz, const float* ma, const float* mb,
                                              float n0, float n1, float* bound) {
  float h[3], R[9];
#pragma unroll
  for (int k = 0; k < 3; ++k) h[k] = n0 * ma[k] + n1 * mb[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = n0 * ma[3 + k] + n1 * mb[3 + k];
  // columns of R, normalised by hardware reciprocal square roots, and the
  // sizes' hardware reciprocals (each within 2 ulps: a few ulps per term on
  // top of the roundings kAnisoUlps already covers, against the dozen or so
  // the terms carry)
  float c0x = R[0], c0y = R[3], c0z = R[6];
  float c1x = R[1], c1y = R[4], c1z = R[7];
  const float il0 = rsqrtf(c0x * c0x + c0y * c0y + c0z * c0z);
  const float r0x = c0x * il0, r0y = c0y * il0, r0z = c0z * il0;
  const float d01 = r0x * c1x + r0y * c1y + r0z * c1z;
  c1x -= r0x * d01; c1y -= r0y * d01; c1z -= r0z * d01;
  const float il1 = rsqrtf(c1x * c1x + c1y * c1y + c1z * c1z);
  const float r1x = c1x * il1, r1y = c1y * il1, r1z = c1z * il1;
  const float r2x = r0y * r1z - r0z * r1y, r2y = r0z * r1x - r0x * r1z, r2z = r0x * r1y - r0y * r1x;
  const float ih0 = __fdividef(1.f, h[0]), ih1 = __fdividef(1.f, h[1]), ih2 = __fdividef(1.f, h[2]);
  const float t0 = (Jx * r0x + Jy * r0y + Jz * r0z) * ih0;
  const float t1 = (Jx * r1x + Jy * r1y + Jz * r1z) * ih1;
  const float t2 = (Jx * r2x + Jy * r2y + Jz * r2z) * ih2;
  const float dv = sqrtf(t0 * t0 + t1 * t1 + t2 * t2);
  const float jn = sqrtf(Jx * Jx + Jy * Jy + Jz * Jz);
  const float sum = jn * (fabsf(ih0) + fabsf(ih1) + fabsf(ih2));
  const float cond = (1.f + il0) * (1.f + il1);
  *bound = fmaxf(*bound, kAnisoUlps * 5.9604645e-8f * cond * sum / dv);
  return dv;
}

// crec: the FP32 path's coordinate records (per vertex {x,y,z}_hi then
// {x,y,z}_lo, coordinates mapped into [1, 2] by x' = (x - c) s + 1), so the
// edge Jacobian J = (x_b - x_a) / 2 = ((hi_b - hi_a) + (lo_b - lo_a)) 0.5 / s
// comes out of exact high-word differences with one rounding, without FP64
// arithmetic; jscale = 0.5 / s (a power of two)
__global__ void __launch_bounds__(kBlock) k_measure_aniso_f32(DevMesh m, const float* __restrict__ met,
                                                              const float4* __restrict__ crec, float jscale,
                                                              uint32_t* __restrict__ split,
                                                              uint32_t* __restrict__ collapse,
                                                              int* __restrict__ guard, int* __restrict__ gcount,
                                                              int gcap) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  bool sp = false, co = false, g = false;
  if (e < m.E) {
    const int a = m.edv[2 * (size_t)e], b = m.edv[2 * (size_t)e + 1];
    // J = x_b / 2 - x_a / 2 (the reference's edge Jacobian) to half an ulp
    const float4 ha = __ldg(crec + 2 * (size_t)a), la = __ldg(crec + 2 * (size_t)a + 1);
    const float4 hb = __ldg(crec + 2 * (size_t)b), lb = __ldg(crec + 2 * (size_t)b + 1);
    const float Jx = ((hb.x - ha.x) + (lb.x - la.x)) * jscale;
    const float Jy = ((hb.y - ha.y) + (lb.y - la.y)) * jscale;
    const float Jz = ((hb.z - ha.z) + (lb.z - la.z)) * jscale;
    float ma[12], mb[12];
    load_met(met + 12 * (size_t)a, ma);
    load_met(met + 12 * (size_t)b, mb);
    float bound = 0.f;
    const float g0 = 0.577350269189626f;
    const float L = aniso_dv_f32(Jx, Jy, Jz, ma, mb, (1.f - g0) * 0.5f, (1.f + g0) * 0.5f, &bound) +
                    aniso_dv_f32(Jx, Jy, Jz, ma, mb, (1.f + g0) * 0.5f, (1.f - g0) * 0.5f, &bound);
    const float lo = L * (1.f - bound), hi = L * (1.f + bound);
    if (!(bound < 0.25f) || !isfinite(L)) {
      g = true;
    } else {
      if (lo > 1.5f) sp = true;
      else if (hi > 1.5f) g = true;
      if (hi < 0.5f) co = true;
      else if (lo < 0.5f) g = true;
    }
  }
  const unsigned bs = __ballot_sync(0xffffffffu, sp), bc = __ballot_sync(0xffffffffu, co);
  if ((threadIdx.x & 31) == 0 && e < m.E) {
    split[e >> 5] = bs;
    collapse[e >> 5] = bc;
  }
  const unsigned bg = __ballot_sync(0xffffffffu, g);
  if (bg) {
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(bg) - 1) base = atomicAdd(gcount, __popc(bg));
    base = __shfl_sync(0xffffffffu, base, __ffs(bg) - 1);
    const int slot = base + __popc(bg & ((1u << lane) - 1));
    if (g && slot < gcap) guard[slot] = e;
  }
}

// the guarded edges re-measured by the FP64 kernel's arithmetic
__global__ void __launch_bounds__(kBlock) k_measure_guard_f64(DevMesh m, MetricSrc src,
                                                              const int* __restrict__ guard,
                                                              const int* __restrict__ gcount, int gcap,
                                                              uint32_t* __restrict__ split,
                                                              uint32_t* __restrict__ collapse) {
  int n = *gcount;
  n = n < gcap ? n : gcap;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int e = guard[i];
    const int vv[2] = {m.edv[2 * (size_t)e], m.edv[2 * (size_t)e + 1]};
    double hv[6], Rv[18];
    for (int a = 0; a < 2; ++a) metric_at(src, vv[a], hv + 3 * a, Rv + 9 * a);
    const double L = metric_length(load_xyz(m.xyz, vv[0]), load_xyz(m.xyz, vv[1]), hv, Rv);
    const uint32_t bit = 1u << (e & 31);
    if (L > 1.5) atomicOr(split + (e >> 5), bit);
    else atomicAnd(split + (e >> 5), ~bit);
    if (L < .5) atomicOr(collapse + (e >> 5), bit);
    else atomicAnd(collapse + (e >> 5), ~bit);
  }
}

// mean-ratio quality under the anisotropic metric in FP32 (the vertex
// transform with the largest determinant, ma/maQuality.cc:83-167)
// FP32 mean-ratio quality of an element under transform Q, from its edge
// vectors E[k] = x_{k+1} - x_0 (FP64 differences rounded to FP32 once per
// element): t_k = Q^T E_k, the element's edges map to t_1, t_2 - t_1, -t_2
// (and t_3, t_3 - t_1, t_3 - t_2 on tets), the volume to det(t_1, t_2, t_3)
__device__ __forceinline__ float quality_with_f32(const DevMesh& m, const float (*E)[3], const float Q[3][3]) {
  float t[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) t[k][c] = E[k][0] * Q[0][c] + E[k][1] * Q[1][c] + E[k][2] * Q[2][c];
  auto n2 = [](float x, float y, float z) { return x * x + y * y + z * z; };
  float s = n2(t[0][0], t[0][1], t[0][2]) + n2(t[1][0] - t[0][0], t[1][1] - t[0][1], t[1][2] - t[0][2]) +
            n2(t[1][0], t[1][1], t[1][2]);
  const float cx = t[0][1] * t[1][2] - t[0][2] * t[1][1], cy = t[0][2] * t[1][0] - t[0][0] * t[1][2],
              cz = t[0][0] * t[1][1] - t[0][1] * t[1][0];
  if (m.dim == 3) {
    s += n2(t[2][0], t[2][1], t[2][2]) + n2(t[2][0] - t[0][0], t[2][1] - t[0][1], t[2][2] - t[0][2]) +
         n2(t[2][0] - t[1][0], t[2][1] - t[1][1], t[2][2] - t[1][2]);
    const float Vm = (cx * t[2][0] + cy * t[2][1] + cz * t[2][2]) / 6.f;  // det(J Q) / 6
    const float res = 15552.f * (Vm * Vm) / (s * s * s);
    return Vm < 0 ? -res : res;
  }
  const float A = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
  return 48.f * (A * A) / (s * s);
}

// the element's edge vectors from vertex 0 out of the coordinate records
// (exact high-word differences plus the low words' difference, one
// rounding; escale = 1 / s)
__device__ __forceinline__ void elem_edges_f32(const DevMesh& m, const float4* __restrict__ crec, float escale,
                                               const int* ev, float (*E)[3]) {
  const float4 h0 = __ldg(crec + 2 * (size_t)ev[0]), l0 = __ldg(crec + 2 * (size_t)ev[0] + 1);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const bool in = k < m.nn - 1;  // triangles: E[2] = 0
    const float4 hk = in ? __ldg(crec + 2 * (size_t)ev[k + 1]) : h0;
    const float4 lk = in ? __ldg(crec + 2 * (size_t)ev[k + 1] + 1) : l0;
    E[k][0] = ((hk.x - h0.x) + (lk.x - l0.x)) * escale;
    E[k][1] = ((hk.y - h0.y) + (lk.y - l0.y)) * escale;
    E[k][2] = ((hk.z - h0.z) + (lk.z - l0.z)) * escale;
  }
}

// relative separation of FP32 determinants taken as certain (their error
// is a few ulps for the orthonormal frames of the metric), and the
// relative agreement of the candidates' qualities within which any of them
// is the reference's value to the FP32 accuracy
constexpr float kDetTie = 1e-5f, kQualTie = 4e-6f;

// element e's vertex coordinates and FP32 determinant pick: best (the first
// largest, as the reference picks) and the candidates the FP32 determinants
// cannot rule out
__device__ __forceinline__ int quality_pick_f32(const DevMesh& m, const QualityRec* __restrict__ qrec, const int* ev,
                                                unsigned* cand) {
  float cj[4];
  int best = 0;
  float cb = 0.f;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    cj[i] = i < m.nn ? qrec[ev[i]].cj : 0.f;
    if (i < m.nn && (i == 0 || cj[i] > cb)) {
      best = i;
      cb = cj[i];
    }
  }
  unsigned c = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (i < m.nn && cj[i] * (1.f + kDetTie) >= cb) c |= 1u << i;
  *cand = c;
  return best;
}

__device__ __forceinline__ void load_qrec(const QualityRec& r, float (*T)[3]) {
  const float4* p = reinterpret_cast<const float4*>(&r);
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  T[0][0] = a.x; T[0][1] = a.y; T[0][2] = a.z; T[1][0] = a.w;
  T[1][1] = b.x; T[1][2] = b.y; T[2][0] = b.z; T[2][1] = b.w;
  T[2][2] = c.x;
}

// FP32 qualities.  Elements whose candidate vertices give qualities that
// differ by more than kQualTie are listed for k_quality_ties (FP64
// determinants decide there); their entry here is the FP32 pick's quality.
__global__ void __launch_bounds__(kBlock) k_quality_aniso_f32(DevMesh m, const QualityRec* __restrict__ qrec,
                                                              const float4* __restrict__ crec, float escale,
                                                              int* __restrict__ tie_items, int* __restrict__ tie_count,
                                                              double* __restrict__ q) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.T) return;
  const int* ev = m.ev + (size_t)e * m.nn;
  float E[3][3];
  elem_edges_f32(m, crec, escale, ev, E);
  // getMetricWithMaxJacobean (ma/maQuality.cc:83-108): the first vertex with
  // the largest determinant
  unsigned cand;
  const int best = quality_pick_f32(m, qrec, ev, &cand);
  float Q[3][3];
  load_qrec(qrec[ev[best]], Q);
  const float res = quality_with_f32(m, E, Q);
  bool tie = false;
  if (cand != (1u << best)) {
    for (int i = 0; i < m.nn; ++i) {
      if (!(cand >> i & 1) || i == best) continue;
      float T[3][3];
      load_qrec(qrec[ev[i]], T);
      const float qi = quality_with_f32(m, E, T);
      if (!(fabsf(qi - res) <= kQualTie * fabsf(res))) tie = true;
    }
  }
  q[e] = res;
  // list the ties, one counter atomic per warp
  const unsigned act = __activemask();
  const unsigned bal = __ballot_sync(act, tie);
  if (bal) {
    const int lane = threadIdx.x & 31, leader = __ffs(bal) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(tie_count, __popc(bal));
    base = __shfl_sync(act, base, leader);
    if (tie) tie_items[base + __popc(bal & ((1u << lane) - 1))] = e;
  }
}

// The listed ties: the FP64 determinants of the FP64 quality kernel's
// arithmetic pick the vertex, in the reference's order.  cj64: per-vertex
// FP64 determinants of this pass, NaN until first needed (concurrent
// writers store the same bits).
__global__ void __launch_bounds__(kBlock) k_quality_ties(DevMesh m, const QualityRec* __restrict__ qrec, MetricSrc src,
                                                         const float4* __restrict__ crec, float escale,
                                                         double* __restrict__ cj64, const int* __restrict__ tie_items,
                                                         const int* __restrict__ tie_count, double* __restrict__ q) {
  const int n = *tie_count;
  for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    const int e = tie_items[i0];
    const int* ev = m.ev + (size_t)e * m.nn;
    unsigned cand;
    const int best = quality_pick_f32(m, qrec, ev, &cand);
    double maxJ = -1.0;
    int pick = best;
    for (int i = 0; i < m.nn; ++i) {
      double cJ = cj64[ev[i]];
      if (cJ != cJ) {
        double hv[3], Rv[9];
        metric_at(src, ev[i], hv, Rv);
        const double N[1] = {1.0};
        cJ = ref::jacobian_det(ref::get_transform(hv, Rv, N, 1), m.dim);
        cj64[ev[i]] = cJ;
      }
      if (cJ > maxJ) {
        maxJ = cJ;
        pick = i;
      }
    }
    if (pick != best) {
      float E[3][3];
      elem_edges_f32(m, crec, escale, ev, E);
      float Q[3][3];
      load_qrec(qrec[ev[pick]], Q);
      q[e] = quality_with_f32(m, E, Q);
    }
  }
}


// Recovery composed with the element gradient: on a P1 field f the
// recovered gradient at a covered vertex is
//   eps*(v) = sum_t w_vt grad_t f = sum_a K_va f_a,
// K_va = sum over the patch elements t holding a of w_vt (J_t^-1 grad N_a),
// a linear operator over the patch's vertices that depends on the geometry
// only.  It is built once per mesh (FP64) and the two recoveries of the
// Hessian workload become two sparse products with it.  kOpSlots slots per
// vertex (a fan of up to kTriThreadRows triangles touches at most
// kTriThreadRows + 2 vertices); a patch touching more is listed for the
// FP64 slab fit instead.
constexpr int kOpSlots = kTriThreadRows + 2;
// KC: components stored per slot, 3, or 2 on a mesh in the z = 0 plane
// (there the z component of every element gradient is exactly zero)
template <int KC>
__global__ void __launch_bounds__(kBlock) k_tri_operator(DevMesh m, const double* __restrict__ w,
                                                         unsigned char* __restrict__ listed, ExpandList lst,
                                                         int* __restrict__ kidx, double* __restrict__ kval,
                                                         int* __restrict__ klen) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  if (listed[v]) {
    klen[v] = 0;
    return;
  }
  int ids[kOpSlots];
  double acc[kOpSlots][3];
  int n = 0;
  for (int k = m.p_off[v]; k < m.p_off[v + 1]; ++k) {
    const int t = m.p_el[k];
    const double wk = w[k];
    const int* ev = m.ev + (size_t)t * 3;
    V3 x[3];
    for (int a = 0; a < 3; ++a) x[a] = load_xyz(m.xyz, ev[a]);
    const M3 J = ref::jacobian(x, 3, 2);
    const M3 jinv = ref::jacobian_inverse(J, 2);
    V3 lg[4];
    ref::shape_grads(2, lg);
    for (int a = 0; a < 3; ++a) {
      const V3 g = ref::mulv(jinv, lg[a]);
      int s = 0;
      while (s < n && ids[s] != ev[a]) ++s;
      if (s == n) {
        if (n == kOpSlots) {  // not a fan: the slab fit takes it
          listed[v] = 1;
          klen[v] = 0;
          const int slot = atomicAdd(lst.count, 1);
          if (slot < lst.cap) lst.items[slot] = v;
          return;
        }
        ids[n] = ev[a];
        acc[n][0] = acc[n][1] = acc[n][2] = 0;
        ++n;
      }
      for (int c = 0; c < 3; ++c) acc[s][c] += wk * g.v[c];
    }
  }
  klen[v] = n;
  for (int s = 0; s < n; ++s) {
    kidx[(size_t)v * kOpSlots + s] = ids[s];
    for (int c = 0; c < KC; ++c) kval[((size_t)v * kOpSlots + s) * KC + c] = acc[s][c];
  }
}

// out (V x 3 NCIN) = K f (f: V x NCIN) at the covered vertices; row r of a
// MATRIX value is the recovered gradient of component r.  KC = 2 (mesh in
// the z = 0 plane): K's z components, and the z components of a gradient
// input, are zero, so only the x / y products are formed and the z entries
// of the output are zero.
template <int NCIN, int KC>
__global__ void __launch_bounds__(kBlock) k_apply_operator(int V, const unsigned char* __restrict__ listed,
                                                           const int* __restrict__ kidx,
                                                           const double* __restrict__ kval,
                                                           const int* __restrict__ klen, const double* __restrict__ f,
                                                           double* __restrict__ out) {
  constexpr int NR = (KC == 2 && NCIN == 3) ? 2 : NCIN;  // input components that can be nonzero
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V || listed[v]) return;
  const int n = klen[v];
  double acc[NCIN][3];
#pragma unroll
  for (int r = 0; r < NCIN; ++r) acc[r][0] = acc[r][1] = acc[r][2] = 0;
  for (int s = 0; s < n; ++s) {
    const size_t slot = (size_t)v * kOpSlots + s;
    const int a = kidx[slot];
    double k[KC];
    if (KC == 2) {  // one 16-byte load per slot
      const double2 kk = __ldg(reinterpret_cast<const double2*>(kval) + slot);
      k[0] = kk.x;
      k[KC - 1] = kk.y;
    } else {
#pragma unroll
      for (int c = 0; c < KC; ++c) k[c] = kval[KC * slot + c];
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const double fa = f[(size_t)a * NCIN + r];
#pragma unroll
      for (int c = 0; c < KC; ++c) acc[r][c] = fma(k[c], fa, acc[r][c]);
    }
  }
#pragma unroll
  for (int r = 0; r < NCIN; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) out[(size_t)v * 3 * NCIN + 3 * r + c] = acc[r][c];
}

// ---------------------------------------------------------------------
// incremental mesh update: row scatter and the bounding box
// ---------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kBlock) k_scatter_rows(long long n, int width, const int* __restrict__ ids,
                                                         const T* __restrict__ vals, T* __restrict__ dst) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n * width) return;
  const long long r = i / width;
  dst[(size_t)ids[r] * width + (i - r * width)] = vals[i];
}

// per axis min and max of the coordinates as order-preserving 64-bit keys
// (keys[0..2] minima, keys[3..5] maxima)
__global__ void __launch_bounds__(kBlock) k_bbox(int V, const double* __restrict__ xyz,
                                                 unsigned long long* __restrict__ keys) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const unsigned long long key = order_key(xyz[3 * (size_t)v + k]);
      lo[k] = key < lo[k] ? key : lo[k];
      hi[k] = key > hi[k] ? key : hi[k];
    }
  for (int k = 0; k < 3; ++k) {
    atomicMin(keys + k, lo[k]);
    atomicMax(keys + 3 + k, hi[k]);
  }
}

__global__ void __launch_bounds__(kBlock) k_count_out_of_range(long long n, const int* __restrict__ a, int limit,
                                                               unsigned long long* __restrict__ bad) {
  unsigned long long c = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    c += (a[i] < 0 || a[i] >= limit);
  if (c) atomicAdd(bad, c);
}

// ---------------------------------------------------------------------
// FP64 SPR weights of tet patches (once per mesh): the patch fit evaluated
// at the vertex is linear in the samples, eps*(v) = sum_j w_j b_j, with
// w = Q [R^-T t; 0] (t = [1, x_v, y_v, z_v]).  One warp per vertex, a row
// per lane: the reference's Householder QR and 1e-10 rank test
// (mth/mthQR.cc:19-126) as in recover_vertex_warp, then R^T z = t solved
// from R and [z; 0] taken through the reflectors in reverse order.  Every
// later FP64 recovery of the mesh is a weighted sum per vertex.  Patches
// with fewer than 4 or more than 32 elements or rank deficient are listed
// (lst) for the FP64 slab fits.
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_qr_weights(DevMesh m, double* __restrict__ w,
                                                       unsigned char* __restrict__ listed, ExpandList lst) {
  constexpr int NT = 4;
  const int lane = threadIdx.x & 31;
  const int v = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (v >= m.V) return;
  const int beg = m.p_off[v];
  const int cnt = m.p_off[v + 1] - beg;
  auto give_up = [&]() {
    if (lane == 0) {
      listed[v] = 1;
      const int slot = atomicAdd(lst.count, 1);
      if (slot < lst.cap) lst.items[slot] = v;
    }
  };
  if (cnt < NT || cnt > 32) {
    give_up();
    return;
  }
  double a[NT];
  if (lane < cnt) {
    const V3 p = elem_ip_point(m, m.p_el[beg + lane]);
    a[0] = 1.0;
    a[1] = p.v[0];
    a[2] = p.v[1];
    a[3] = p.v[2];
  } else {
    a[0] = a[1] = a[2] = a[3] = 0;
  }
  double vk[NT];  // this lane's entry of each reflector
#pragma unroll
  for (int k = 0; k < NT; ++k) {
    const double cn = sqrt(warp_sum(lane >= k ? a[k] * a[k] : 0.0));
    if (cn < 1e-10) {  // uniform across the warp
      give_up();
      return;
    }
    const double akk = __shfl_sync(0xffffffffu, a[k], k);
    double vv = lane >= k ? a[k] : 0.0;
    if (lane == k) vv += ((akk < 0) ? -1 : 1) * cn;
    const double rn = sqrt(warp_sum(vv * vv));
    vv /= rn;
    vk[k] = vv;
#pragma unroll
    for (int j = k; j < NT; ++j) {
      const double d = warp_sum(a[j] * vv);
      a[j] -= 2 * d * vv;
    }
  }
  // R in lanes 0..3; z = R^-T t by forward substitution
  double R[NT][NT];
#pragma unroll
  for (int i = 0; i < NT; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j) R[i][j] = __shfl_sync(0xffffffffu, a[j], i);
  const V3 xv = load_xyz(m.xyz, v);
  const double t[NT] = {1.0, xv.v[0], xv.v[1], xv.v[2]};
  double z[NT];
#pragma unroll
  for (int i = 0; i < NT; ++i) {
    double acc = t[i];
#pragma unroll
    for (int j = 0; j < i; ++j) acc -= R[j][i] * z[j];
    z[i] = acc / R[i][i];
  }
  // y = H_1 H_2 H_3 H_4 [z; 0]: the reflectors from the last to the first
  double y = 0;
#pragma unroll
  for (int i = 0; i < NT; ++i)
    if (lane == i) y = z[i];
#pragma unroll
  for (int k = NT - 1; k >= 0; --k) {
    const double d = warp_sum(vk[k] * y);
    y -= 2 * d * vk[k];
  }
  if (lane < cnt) w[beg + lane] = y;
  if (lane == 0) listed[v] = 0;
}

// FP64 recovery from the weights: thread per vertex, NC components
template <int NC>
__global__ void __launch_bounds__(kBlock) k_recover_w64(DevMesh m, const double* __restrict__ ip,
                                                        const double* __restrict__ w,
                                                        const unsigned char* __restrict__ listed,
                                                        double* __restrict__ rec) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V || listed[v]) return;
  const int beg = m.p_off[v], end = m.p_off[v + 1];
  double acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = 0;
  for (int k = beg; k < end; ++k) {
    const double wk = w[k];
    const double* b = ip + (size_t)m.p_el[k] * NC;
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] += wk * b[c];
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) rec[(size_t)v * NC + c] = acc[c];
}

}  // namespace

// ----------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------
void launch_grad_ip_f64(const DevMesh& m, const double* f, int ncin, double* ip, cudaStream_t s) {
  if (m.T) k_grad_ip<<<nblk(m.T), kBlock, 0, s>>>(m, f, ncin, ip);
}

void launch_recover_f64(const DevMesh& m, const double* ip, int nc, double* rec, ExpandList xl, ExpandList big,
                        DevStatus* st, cudaStream_t s) {
  (void)st;
  if (!m.V || m.dim != 2) return;  // tets recover through the per-mesh QR weights
  // triangles: a thread per vertex up to kTriThreadRows patch elements, then
  // the warp path over the vertices it listed
  const int grid = (m.V + 127) / 128;
  const int lgrid = 152 * 8;
  if (nc == 3) {
    k_recover_tri<3, kTriThreadRows><<<grid, 128, 0, s>>>(m, ip, rec, xl, big);
    k_recover_list<3, 3, 1><<<lgrid, kBlock, 0, s>>>(m, ip, rec, xl, big);
  } else {
    k_recover_tri<9, kTriThreadRows><<<grid, 128, 0, s>>>(m, ip, rec, xl, big);
    k_recover_list<3, 9, 1><<<lgrid, kBlock, 0, s>>>(m, ip, rec, xl, big);
  }
}

int expand_max_elems() { return kExpandMaxElems; }

int expand_grid() { return kExpandGrid; }

void launch_expand_f64(const DevMesh& m, const double* ip, const double* u, int nc, double* rec, ExpandList xl,
                       double* slab, DevStatus* st, cudaStream_t s, int* cache_v, int* cache_n, int* cache_el) {
  k_expand<<<kExpandGrid, 32, 0, s>>>(m, ip, u, nc, rec, xl.items, xl.count, xl.cap, slab, st, cache_v, cache_n,
                                      cache_el);
}

void launch_cached_fit_f64(const DevMesh& m, const double* ip, const double* u, int nc, double* rec, int n_cached,
                           const int* cache_v, const int* cache_n, const int* cache_el, double* slab, DevStatus* st,
                           cudaStream_t s) {
  if (n_cached > 0)
    k_cached_fit<<<n_cached < kExpandGrid ? n_cached : kExpandGrid, 32, 0, s>>>(m, ip, u, nc, rec, n_cached, cache_v,
                                                                                cache_n, cache_el, slab, st);
}

void launch_cached_weights_f64(const DevMesh& m, int n_cached, const int* cache_v, const int* cache_n,
                               const int* cache_el, const long long* woff, double* w, int* wn, double* slab,
                               cudaStream_t s) {
  if (n_cached > 0)
    k_cached_weights<<<n_cached < kExpandGrid ? n_cached : kExpandGrid, 32, 0, s>>>(m, n_cached, cache_v, cache_n,
                                                                                   cache_el, woff, w, wn, slab);
}

void launch_cached_wsum_f64(const DevMesh& m, const double* ip, const double* u, int nc, double* rec, int n_cached,
                            const int* cache_v, const int* cache_el, const long long* woff, const double* w,
                            const int* wn, DevStatus* st, cudaStream_t s) {
  if (n_cached > 0)
    k_cached_wsum<<<std::min(nblk((long)n_cached * 32), 152 * 8), kBlock, 0, s>>>(m, ip, u, nc, rec, n_cached, cache_v,
                                                                                cache_el, woff, w, wn, st);
}

int error_blocks(int T) { return nblk(T); }

void launch_error_f64(const DevMesh& m, const double* ip, int nc, const double* rec, double* err,
                      double* partials, int n_blocks, double g_exponent, cudaStream_t s) {
  if (n_blocks) k_error<<<n_blocks, kBlock, 0, s>>>(m, ip, nc, rec, err, partials, g_exponent);
}

void launch_size_factor(const double* partials, int n_blocks, int mode, double adapt_ratio, double target, int dim,
                        double* out3, cudaStream_t s) {
  k_size_factor<<<1, kBlock, 0, s>>>(partials, n_blocks, mode, adapt_ratio, target, dim, out3);
}

void launch_size_factor_batch(const double* partials, BatchView bv, int dim, double* out4, cudaStream_t s) {
  (void)dim;  // p = 1: size_factor = (ratio^2 |eps*|^2 / G)^(1/2) in 2D and 3D
  if (bv.n) k_size_factor_batch<<<bv.n, kBlock, 0, s>>>(partials, bv, out4);
}

void launch_esize_f64(const DevMesh& m, const double* err, const double* out3, int mode, double alpha, double beta,
                      double* esize, cudaStream_t s) {
  if (m.T) k_esize<<<nblk(m.T), kBlock, 0, s>>>(m, err, out3, mode, alpha, beta, esize);
}

void launch_average(const DevMesh& m, const double* esize, double* size, cudaStream_t s) {
  if (m.V) k_average<<<nblk(m.V), kBlock, 0, s>>>(m, esize, size);
}

void launch_measure_iso_f64(const DevMesh& m, const double* size, double* L, cudaStream_t s) {
  if (m.E) k_measure_iso<<<nblk(m.E), kBlock, 0, s>>>(m, size, L);
}

void launch_measure_aniso_f64(const DevMesh& m, const double* sizes, const double* frames, double* L,
                              cudaStream_t s) {
  if (m.E) k_measure_aniso<<<nblk(m.E), kBlock, 0, s>>>(m, sizes, frames, L);
}

void launch_mark(int E, const double* L, int which, int* flags, unsigned long long* count, DevStatus* st,
                 cudaStream_t s) {
  if (E) k_mark<<<count_grid(E), kBlock, 0, s>>>(E, L, which, flags, count, st);
}

void launch_mark_bits(int E, const double* L, uint32_t* split, uint32_t* collapse, cudaStream_t s) {
  if (E) k_mark_bits<<<nblk(E), kBlock, 0, s>>>(E, L, split, collapse);
}

void launch_apply_bits(int E, const uint32_t* bits, int which, int* flags, unsigned long long* count, DevStatus* st,
                       cudaStream_t s) {
  if (E) k_apply_bits<<<count_grid(E), kBlock, 0, s>>>(E, bits, which, flags, count, st);
}

void launch_apply_marks(int E, const uint32_t* split_bits, const uint32_t* collapse_bits, int* flags,
                        unsigned long long* counts, DevStatus* st, const int* skip, cudaStream_t s) {
  if (E)
    k_apply_marks<<<count_grid((E + 3) / 4), kBlock, 0, s>>>(E, split_bits, collapse_bits, flags, counts, st, skip);
}

void launch_quality_f64(const DevMesh& m, const double* size, const double* sizes, const double* frames, double* q,
                        cudaStream_t s, const double* logm, DevStatus* st) {
  if (!m.T) return;
  if (logm) k_quality<true><<<nblk(m.T), kBlock, 0, s>>>(m, size, sizes, frames, logm, q, st);
  else k_quality<false><<<nblk(m.T), kBlock, 0, s>>>(m, size, sizes, frames, logm, q, st);
}

void launch_guard_stage(int stage, const DevMesh& m, const double* u, const double* out3, const int* items,
                        const int* count, int cap, uint32_t* split, uint32_t* collapse, int* unresolved,
                        GuardScratch g, BatchView bv, cudaStream_t s) {
  switch (stage) {
    case 0:
      cudaMemsetAsync(g.fit_count, 0, sizeof(int), s);
      k_guard_collect<<<152 * 4, 256, 0, s>>>(m, items, count, cap, g.stamp_id, g.stamp, g.fit_items, g.fit_count,
                                          g.fit_cap, unresolved);
      break;
    case 1:
      k_guard_fit<<<152 * 8, 256, 0, s>>>(m, u, g.fit_items, g.fit_count, g.fit_cap, g);
      break;
    default:
      k_guard_decide<<<152 * 4, 128, 0, s>>>(m, u, out3, g, items, count, cap, split, collapse, unresolved, bv);
  }
}

void launch_hessian_metric(const DevMesh& m, const double* H, double eps, double hmin, double hmax, double* sizes,
                           double* frames, cudaStream_t s) {
  if (m.V) k_hessian_metric<<<nblk(m.V), kBlock, 0, s>>>(m.V, m.dim, H, eps, hmin, hmax, sizes, frames);
}

void launch_build_v2e(const DevMesh& m, int* off, int* el, int* tmp, cudaStream_t s) {
  cudaMemsetAsync(tmp, 0, sizeof(int) * (size_t)m.V, s);
  cudaMemsetAsync(off, 0, sizeof(int) * ((size_t)m.V + 1), s);
  if (m.T) k_count_v2e<<<nblk(m.T), kBlock, 0, s>>>(m, off);
  // exclusive scan of the V+1 counts (last is 0) -> offsets
  size_t bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, bytes, off, off, m.V + 1, s);
  void* scratch = nullptr;
  cudaMallocAsync(&scratch, bytes, s);
  cub::DeviceScan::ExclusiveSum(scratch, bytes, off, off, m.V + 1, s);
  cudaFreeAsync(scratch, s);
  if (m.T) k_fill_v2e<<<nblk(m.T), kBlock, 0, s>>>(m, off, tmp, el);
}

void launch_sort_segments(int V, const int* off, int* el, cudaStream_t s) {
  if (V) k_sort_segments<<<nblk(V), kBlock, 0, s>>>(V, off, el);
}

void launch_xyz_to_fixed(const DevMesh& m, const double* frame, int* xyzq, cudaStream_t s) {
  if (m.V) k_xyz_fixed<<<nblk(m.V), kBlock, 0, s>>>(m, frame[0], frame[1], frame[2], frame[3], xyzq);
}


void launch_measure_pairs(const DevMesh& m, int kind, long long n, const int* pairs, const double* size,
                          const double* sizes, const double* frames, const double* logm, double* L, DevStatus* st,
                          cudaStream_t s) {
  if (n > 0)
    k_measure_pairs<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, kind, n, pairs, size, sizes, frames,
                                                                            logm, L, st);
}

void launch_log_metric(int V, const double* sizes, const double* frames, double* logm, cudaStream_t s) {
  if (V) k_log_metric<<<nblk(V), kBlock, 0, s>>>(V, sizes, frames, logm);
}

void launch_max_positive(long long n, const double* x, unsigned long long* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
  if (n > 0) k_max_positive<<<kSumBlocks, kBlock, 0, s>>>(n, x, out);
}

int sum_partials_count() { return kSumBlocks; }

void launch_sum(long long n, const double* x, double* partials, double* out, cudaStream_t s) {
  k_sum_partials<<<kSumBlocks, kBlock, 0, s>>>(n, x, partials);
  k_sum_final<<<1, 1, 0, s>>>(kSumBlocks, partials, out);
}

void launch_first_min_below(long long n, const double* x, double start, unsigned long long* key,
                            unsigned long long* first, cudaStream_t s) {
  cudaMemsetAsync(key, 0xff, sizeof(unsigned long long), s);
  cudaMemsetAsync(first, 0xff, sizeof(unsigned long long), s);
  if (n > 0) {
    k_min_below<<<kSumBlocks, kBlock, 0, s>>>(n, x, start, key);
    k_first_equal<<<kSumBlocks, kBlock, 0, s>>>(n, x, key, first);
  }
}

void launch_mark_quality(int T, const double* q, double good, int* flags, unsigned long long* count, DevStatus* st,
                         cudaStream_t s) {
  if (T) k_mark_quality<<<count_grid(T), kBlock, 0, s>>>(T, q, good, flags, count, st);
}
void launch_tri_weights(const DevMesh& m, double* w, unsigned char* listed, ExpandList lst, cudaStream_t s) {
  if (m.V) k_tri_weights<kTriThreadRows><<<(m.V + 127) / 128, 128, 0, s>>>(m, w, listed, lst);
}

void launch_metric_f32(int V, int dim, const double* sizes, const double* frames, float* out, void* qrec,
                       cudaStream_t s) {
  if (V) k_metric_f32<<<nblk(V), kBlock, 0, s>>>(V, dim, sizes, frames, out, static_cast<QualityRec*>(qrec));
}

void launch_measure_aniso_f32(const DevMesh& m, const float* met, const float4* crec, double frame_scale,
                              uint32_t* split, uint32_t* collapse, int* guard, int* gcount, int gcap, cudaStream_t s) {
  const float jscale = (float)(0.5 / frame_scale);
  if (m.E)
    k_measure_aniso_f32<<<nblk(m.E), kBlock, 0, s>>>(m, met, crec, jscale, split, collapse, guard, gcount, gcap);
}

void launch_measure_guard_f64(const DevMesh& m, const double* sizes, const double* frames, const double* H,
                              double eps, double hmin, double hmax, const int* guard, const int* gcount, int gcap,
                              uint32_t* split, uint32_t* collapse, cudaStream_t s) {
  const MetricSrc src{sizes, frames, H, m.dim, eps, hmin, hmax};
  k_measure_guard_f64<<<152 * 4, kBlock, 0, s>>>(m, src, guard, gcount, gcap, split, collapse);
}

void launch_metric_mixed2d(int V, const double* H, double eps, double hmin, double hmax, float* out, void* qrec,
                           cudaStream_t s) {
  if (V) k_metric_mixed2d<<<nblk(V), kBlock, 0, s>>>(V, H, eps, hmin, hmax, out, static_cast<QualityRec*>(qrec));
}

int quality_rec_bytes() { return (int)sizeof(QualityRec); }

void launch_quality_aniso_f32(const DevMesh& m, const void* qrec, const float4* crec, double frame_scale,
                              const double* sizes, const double* frames, const double* H, double eps, double hmin,
                              double hmax, double* cj64, int* tie_items, int* tie_count, double* q, cudaStream_t s) {
  const MetricSrc src{sizes, frames, H, m.dim, eps, hmin, hmax};
  if (!m.T) return;
  const QualityRec* r = static_cast<const QualityRec*>(qrec);
  const float escale = (float)(1.0 / frame_scale);
  cudaMemsetAsync(cj64, 0xff, sizeof(double) * (size_t)m.V, s);  // all NaN
  cudaMemsetAsync(tie_count, 0, sizeof(int), s);
  k_quality_aniso_f32<<<nblk(m.T), kBlock, 0, s>>>(m, r, crec, escale, tie_items, tie_count, q);
  k_quality_ties<<<152 * 8, kBlock, 0, s>>>(m, r, src, crec, escale, cj64, tie_items, tie_count, q);
}

int tri_operator_slots() { return kOpSlots; }

void launch_tri_operator(const DevMesh& m, int kc, const double* w, unsigned char* listed, ExpandList lst, int* kidx,
                         double* kval, int* klen, cudaStream_t s) {
  if (!m.V) return;
  if (kc == 2) k_tri_operator<2><<<nblk(m.V), kBlock, 0, s>>>(m, w, listed, lst, kidx, kval, klen);
  else k_tri_operator<3><<<nblk(m.V), kBlock, 0, s>>>(m, w, listed, lst, kidx, kval, klen);
}

void launch_apply_operator(int V, int ncin, int kc, const unsigned char* listed, const int* kidx, const double* kval,
                           const int* klen, const double* f, double* out, cudaStream_t s) {
  if (!V) return;
  const int g = nblk(V);
  if (kc == 2) {
    if (ncin == 1) k_apply_operator<1, 2><<<g, kBlock, 0, s>>>(V, listed, kidx, kval, klen, f, out);
    else k_apply_operator<3, 2><<<g, kBlock, 0, s>>>(V, listed, kidx, kval, klen, f, out);
  } else {
    if (ncin == 1) k_apply_operator<1, 3><<<g, kBlock, 0, s>>>(V, listed, kidx, kval, klen, f, out);
    else k_apply_operator<3, 3><<<g, kBlock, 0, s>>>(V, listed, kidx, kval, klen, f, out);
  }
}

void launch_scatter_rows_f64(long long n, int width, const int* ids, const double* vals, double* dst, cudaStream_t s) {
  if (n > 0) k_scatter_rows<double><<<(unsigned)((n * width + kBlock - 1) / kBlock), kBlock, 0, s>>>(n, width, ids,
                                                                                                   vals, dst);
}

void launch_scatter_rows_i32(long long n, int width, const int* ids, const int* vals, int* dst, cudaStream_t s) {
  if (n > 0) k_scatter_rows<int><<<(unsigned)((n * width + kBlock - 1) / kBlock), kBlock, 0, s>>>(n, width, ids,
                                                                                                vals, dst);
}

void launch_bbox(int V, const double* xyz, unsigned long long* keys, cudaStream_t s) {
  cudaMemsetAsync(keys, 0xff, 3 * sizeof(unsigned long long), s);
  cudaMemsetAsync(keys + 3, 0, 3 * sizeof(unsigned long long), s);
  if (V) k_bbox<<<152 * 4, kBlock, 0, s>>>(V, xyz, keys);
}

double key_to_double(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
}

void launch_count_out_of_range(long long n, const int* a, int limit, unsigned long long* bad, cudaStream_t s) {
  if (n > 0) k_count_out_of_range<<<152 * 4, kBlock, 0, s>>>(n, a, limit, bad);
}

void launch_qr_weights(const DevMesh& m, double* w, unsigned char* listed, ExpandList lst, cudaStream_t s) {
  if (m.V) k_qr_weights<<<nblk((long)m.V * 32), kBlock, 0, s>>>(m, w, listed, lst);
}

void launch_recover_w64(const DevMesh& m, const double* ip, int nc, const double* w, const unsigned char* listed,
                        double* rec, cudaStream_t s) {
  if (!m.V) return;
  if (nc == 3) k_recover_w64<3><<<nblk(m.V), kBlock, 0, s>>>(m, ip, w, listed, rec);
  else k_recover_w64<9><<<nblk(m.V), kBlock, 0, s>>>(m, ip, w, listed, rec);
}

}  // namespace sprg
