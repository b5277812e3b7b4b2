// FP32 fast path of the estimate-and-mark pass (3D tets, scalar field).
//
// Every FP64 input value is carried as an unevaluated float pair (hi, lo):
// one 32-byte record per vertex {x,y,z,u}_hi, {x,y,z,u}_lo, so a vertex gather
// is one DRAM sector.  All arithmetic is FP32; the places where the SPR
// estimator cancels are done with error-free transformations (TwoSum,
// TwoProd via fmaf) instead of wider types:
//
//  * differences of nearby coordinates / field values keep the pair
//    (a_hi - b_hi exactly, a_lo - b_lo);
//  * a tet gradient is formed relative to a reference gradient g as
//    J^{-1} (du - J g), with the residual du - J g evaluated by compensated
//    dot products, so only the small deviation carries FP32 rounding;
//  * the recovered field is stored as (g_ref, deviation) per vertex, and the
//    element error |eps - eps*|^2 is taken from those deviations.
//
// That keeps the element errors (and so the sizes) at ~1e-7 relative even
// where |eps - eps*| is 1e-3 |eps|.  FP64 appears only in the per-warp
// combination of the two global integrals and in the reference (FP64) path
// for listed patches.
//
// Phases:
//   prep      thread per vertex: pack the records
//   tet       thread per tet: its gradient as (g_t, d_t) with g_t the plain
//             FP32 value and d_t = J^{-1}(du - J g_t) the compensated
//             correction, its volume weight, h_max and its integration point
//             as a pair (64 bytes per tet), so the gradient is evaluated once
//             instead of once per use and the recover kernel gathers no
//             vertex records
//   recover   4 lanes per vertex: patch tets split over the lanes, FP32 normal
//             equations on centred, scaled coordinates; condition estimate
//             > 1e6, fewer than 4 points or a non-positive pivot send the
//             vertex to the FP64 reference path (growth + Householder QR)
//   error     thread per tet: element error, SelfProduct and Error terms
//             (compensated), q_t = h_max * err^(-1/5)
//   average   thread per vertex: size = size_factor * mean(q_t) (compensated)
//   measure   thread per edge: metric length, split/collapse bitmaps, and the
//             list of edges within the guard band of 0.5 / 1.5
#include "sprg_fast.h"

namespace sprg {
namespace {

constexpr int kBlock = 256;
constexpr int kGroup = 4;  // lanes per vertex in the recover kernel

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// pair difference a - b of two records: (dh + dl) = a - b to ~2^-48 relative
__device__ __forceinline__ void pdiff(const float4& ah, const float4& al, const float4& bh, const float4& bl,
                                      float4& dh, float4& dl) {
  float e;
  two_sum(ah.x, -bh.x, dh.x, e); dl.x = (al.x - bl.x) + e;
  two_sum(ah.y, -bh.y, dh.y, e); dl.y = (al.y - bl.y) + e;
  two_sum(ah.z, -bh.z, dh.z, e); dl.z = (al.z - bl.z) + e;
  two_sum(ah.w, -bh.w, dh.w, e); dl.w = (al.w - bl.w) + e;
}

// du - e.g with du = (dh.w + dl.w), e = (dh.xyz + dl.xyz), compensated
__device__ __forceinline__ float comp_residual(const float4& dh, const float4& dl, float g0, float g1, float g2) {
  float s = dh.w, err = dl.w, p, pe, se;
  p = dh.x * g0; pe = fmaf(dh.x, g0, -p); two_sum(s, -p, s, se); err += se - pe;
  p = dh.y * g1; pe = fmaf(dh.y, g1, -p); two_sum(s, -p, s, se); err += se - pe;
  p = dh.z * g2; pe = fmaf(dh.z, g2, -p); two_sum(s, -p, s, se); err += se - pe;
  err -= dl.x * g0 + dl.y * g1 + dl.z * g2;
  return s + err;
}

struct Cof {
  float c[3][3];  // cofactors of J (rows e1, e2, e3)
  float det;
};

__device__ __forceinline__ Cof cofactors(const float4& e1, const float4& e2, const float4& e3) {
  Cof k;
  k.c[0][0] = e2.y * e3.z - e2.z * e3.y;
  k.c[0][1] = e2.z * e3.x - e2.x * e3.z;
  k.c[0][2] = e2.x * e3.y - e2.y * e3.x;
  k.c[1][0] = e3.y * e1.z - e3.z * e1.y;
  k.c[1][1] = e3.z * e1.x - e3.x * e1.z;
  k.c[1][2] = e3.x * e1.y - e3.y * e1.x;
  k.c[2][0] = e1.y * e2.z - e1.z * e2.y;
  k.c[2][1] = e1.z * e2.x - e1.x * e2.z;
  k.c[2][2] = e1.x * e2.y - e1.y * e2.x;
  k.det = e1.x * k.c[0][0] + e1.y * k.c[0][1] + e1.z * k.c[0][2];
  return k;
}

// J^{-1} r = C^T r / det
__device__ __forceinline__ void apply_inv(const Cof& k, float r1, float r2, float r3, float* g) {
  float inv = 1.0f / k.det;
#pragma unroll
  for (int j = 0; j < 3; ++j) g[j] = (k.c[0][j] * r1 + k.c[1][j] * r2 + k.c[2][j] * r3) * inv;
}

__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }

// x^(-1/5) for the element error x: powf's estimate refined by one Newton
// step on x r^5 = 1 whose residual is taken with a single rounding (fmaf).
// powf alone is biased by several ulp for these exponents, which would shift
// the global error sum and with it every size.
__device__ __forceinline__ float inv_fifth_root(float x) {
  float r = powf(x, -0.2f);
  if (!(x > 1e-30f) || !(x < 1e30f)) return r;
  float r2 = r * r;
  float r5 = r2 * r2 * r;
  float e = fmaf(-x, r5, 1.0f);
  return fmaf(r * 0.2f, e, r);
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_prep(int V, const double* __restrict__ xyz, const double* __restrict__ u,
                                                 float4* __restrict__ rec) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  double x = xyz[3 * (size_t)v], y = xyz[3 * (size_t)v + 1], z = xyz[3 * (size_t)v + 2], w = u[v];
  float xh = (float)x, yh = (float)y, zh = (float)z, wh = (float)w;
  rec[2 * (size_t)v] = make_float4(xh, yh, zh, wh);
  rec[2 * (size_t)v + 1] = make_float4((float)(x - xh), (float)(y - yh), (float)(z - zh), (float)(w - wh));
}

// tet t's edge pairs (x_i - x_0, u_i - u_0), i = 1..3, their rounded sums
// e (geometry: Jacobian, volume, lengths) and vertex 0's record
struct TetData {
  float4 eh[3], el[3];
  float4 e[3];
  float4 h0, l0;
};

__device__ __forceinline__ TetData load_tet(const float4* __restrict__ vr, int4 tv) {
  TetData d;
  d.h0 = ld4(vr + 2 * (size_t)tv.x);
  d.l0 = ld4(vr + 2 * (size_t)tv.x + 1);
  float4 h1 = ld4(vr + 2 * (size_t)tv.y), l1 = ld4(vr + 2 * (size_t)tv.y + 1);
  float4 h2 = ld4(vr + 2 * (size_t)tv.z), l2 = ld4(vr + 2 * (size_t)tv.z + 1);
  float4 h3 = ld4(vr + 2 * (size_t)tv.w), l3 = ld4(vr + 2 * (size_t)tv.w + 1);
  pdiff(h1, l1, d.h0, d.l0, d.eh[0], d.el[0]);
  pdiff(h2, l2, d.h0, d.l0, d.eh[1], d.el[1]);
  pdiff(h3, l3, d.h0, d.l0, d.eh[2], d.el[2]);
#pragma unroll
  for (int i = 0; i < 3; ++i)
    d.e[i] = make_float4(d.eh[i].x + d.el[i].x, d.eh[i].y + d.el[i].y, d.eh[i].z + d.el[i].z,
                         d.eh[i].w + d.el[i].w);
  return d;
}

// ---------------------------------------------------------------------------
// tet: gradient pair, volume weight, h_max
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_tet(DevMesh m, const float4* __restrict__ vr,
                                                     float4* __restrict__ td) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m.T) return;
  int4 tv = __ldg(reinterpret_cast<const int4*>(m.ev) + t);
  TetData d = load_tet(vr, tv);
  Cof cf = cofactors(d.e[0], d.e[1], d.e[2]);
  float g[3], c[3];
  apply_inv(cf, d.e[0].w, d.e[1].w, d.e[2].w, g);
  apply_inv(cf, comp_residual(d.eh[0], d.el[0], g[0], g[1], g[2]), comp_residual(d.eh[1], d.el[1], g[0], g[1], g[2]),
            comp_residual(d.eh[2], d.el[2], g[0], g[1], g[2]), c);
  float4 a1 = d.e[0], a2 = d.e[1], a3 = d.e[2];
  float hm = fmaxf(fmaxf(len3(a1.x, a1.y, a1.z), len3(a2.x, a2.y, a2.z)), len3(a3.x, a3.y, a3.z));
  hm = fmaxf(hm, len3(a2.x - a1.x, a2.y - a1.y, a2.z - a1.z));
  hm = fmaxf(hm, len3(a3.x - a1.x, a3.y - a1.y, a3.z - a1.z));
  hm = fmaxf(hm, len3(a3.x - a2.x, a3.y - a2.y, a3.z - a2.z));
  // integration point (centroid) as a pair: x_0 + (e1 + e2 + e3) / 4
  float px = 0.25f * ((d.eh[0].x + d.eh[1].x) + d.eh[2].x), pxl = 0.25f * ((d.el[0].x + d.el[1].x) + d.el[2].x);
  float py = 0.25f * ((d.eh[0].y + d.eh[1].y) + d.eh[2].y), pyl = 0.25f * ((d.el[0].y + d.el[1].y) + d.el[2].y);
  float pz = 0.25f * ((d.eh[0].z + d.eh[1].z) + d.eh[2].z), pzl = 0.25f * ((d.el[0].z + d.el[1].z) + d.el[2].z);
  float cxh, cxl, cyh, cyl, czh, czl;
  two_sum(d.h0.x, px, cxh, cxl);
  two_sum(d.h0.y, py, cyh, cyl);
  two_sum(d.h0.z, pz, czh, czl);
  cxl += d.l0.x + pxl;
  cyl += d.l0.y + pyl;
  czl += d.l0.z + pzl;
  float4* o = td + 4 * (size_t)t;
  o[0] = make_float4(g[0], g[1], g[2], cf.det * (1.0f / 6.0f));
  o[1] = make_float4(c[0], c[1], c[2], hm);
  o[2] = make_float4(cxh, cyh, czh, 0.f);
  o[3] = make_float4(cxl, cyl, czl, 0.f);
}

// ---------------------------------------------------------------------------
// recover: kGroup lanes per vertex
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_recover(DevMesh m, const float4* __restrict__ vr,
                                                         const float4* __restrict__ td, float4* __restrict__ rec,
                                                         ExpandList xl, int* __restrict__ n_refit) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = gid / kGroup;
  const int gl = gid % kGroup;
  const int lane = threadIdx.x & 31;
  const int leader = lane & ~(kGroup - 1);
  const bool valid = v < m.V;
  int beg = 0, cnt = 0;
  if (valid) {
    beg = m.p_off[v];
    cnt = m.p_off[v + 1] - beg;
  }
  const bool active = valid && cnt >= 4;
  // reference gradient (the plain value of the first patch tet) and scale
  float gr0 = 0.f, gr1 = 0.f, gr2 = 0.f, inv_h = 0.f;
  if (active && gl == 0) {
    int t0 = m.p_el[beg];
    float4 a = ld4(td + 4 * (size_t)t0), b = ld4(td + 4 * (size_t)t0 + 1);
    gr0 = a.x; gr1 = a.y; gr2 = a.z;
    inv_h = 1.0f / b.w;
  }
  gr0 = __shfl_sync(0xffffffffu, gr0, leader);
  gr1 = __shfl_sync(0xffffffffu, gr1, leader);
  gr2 = __shfl_sync(0xffffffffu, gr2, leader);
  inv_h = __shfl_sync(0xffffffffu, inv_h, leader);
  // normal equations of [1, sx, sy, sz] against the deviations eps_t - g_ref
  float a[10];
  float r[4][3];
#pragma unroll
  for (int i = 0; i < 10; ++i) a[i] = 0.f;
#pragma unroll
  for (int i = 0; i < 4; ++i) r[i][0] = r[i][1] = r[i][2] = 0.f;
  if (active) {
    float4 vh = ld4(vr + 2 * (size_t)v), vl = ld4(vr + 2 * (size_t)v + 1);
#pragma unroll 2
    for (int k = gl; k < cnt; k += kGroup) {
      int t = m.p_el[beg + k];
      const float4* tp = td + 4 * (size_t)t;
      float4 ga = ld4(tp), gb = ld4(tp + 1), ch = ld4(tp + 2), cl = ld4(tp + 3);
      // integration point relative to v
      float sx = ((ch.x - vh.x) + (cl.x - vl.x)) * inv_h;
      float sy = ((ch.y - vh.y) + (cl.y - vl.y)) * inv_h;
      float sz = ((ch.z - vh.z) + (cl.z - vl.z)) * inv_h;
      float dev[3] = {(ga.x - gr0) + gb.x, (ga.y - gr1) + gb.y, (ga.z - gr2) + gb.z};
      a[0] += 1.f; a[1] += sx; a[2] += sy; a[3] += sz;
      a[4] += sx * sx; a[5] += sx * sy; a[6] += sx * sz;
      a[7] += sy * sy; a[8] += sy * sz; a[9] += sz * sz;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        r[0][c] += dev[c]; r[1][c] += sx * dev[c]; r[2][c] += sy * dev[c]; r[3][c] += sz * dev[c];
      }
    }
  }
#pragma unroll
  for (int o = 1; o < kGroup; o <<= 1) {
#pragma unroll
    for (int i = 0; i < 10; ++i) a[i] += __shfl_xor_sync(0xffffffffu, a[i], o);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c) r[i][c] += __shfl_xor_sync(0xffffffffu, r[i][c], o);
  }
  if (!valid || gl != 0) return;
  bool to_ref = !active;
  if (!to_ref) {
    // Cholesky of the normal matrix; the pivot spread estimates its condition
    float l00 = sqrtf(a[0]);
    float l10 = a[1] / l00, l20 = a[2] / l00, l30 = a[3] / l00;
    float d1 = a[4] - l10 * l10;
    float l11 = sqrtf(fmaxf(d1, 0.f));
    float l21 = (a[5] - l20 * l10) / l11, l31 = (a[6] - l30 * l10) / l11;
    float d2 = a[7] - l20 * l20 - l21 * l21;
    float l22 = sqrtf(fmaxf(d2, 0.f));
    float l32 = (a[8] - l30 * l20 - l31 * l21) / l22;
    float d3 = a[9] - l30 * l30 - l31 * l31 - l32 * l32;
    float l33 = sqrtf(fmaxf(d3, 0.f));
    float pmin = fminf(fminf(d1, d2), fminf(d3, a[0]));
    float pmax = fmaxf(fmaxf(d1, d2), fmaxf(d3, a[0]));
    to_ref = !(pmin > 0.f) || !(pmax <= 1e6f * pmin);
    if (!to_ref) {
      float x0[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float y0 = r[0][c] / l00;
        float y1 = (r[1][c] - l10 * y0) / l11;
        float y2 = (r[2][c] - l20 * y0 - l21 * y1) / l22;
        float y3 = (r[3][c] - l30 * y0 - l31 * y1 - l32 * y2) / l33;
        float z3 = y3 / l33;
        float z2 = (y2 - l32 * z3) / l22;
        float z1 = (y1 - l21 * z2 - l31 * z3) / l11;
        x0[c] = (y0 - l10 * z1 - l20 * z2 - l30 * z3) / l00;
      }
      rec[2 * (size_t)v] = make_float4(gr0, gr1, gr2, 0.f);
      rec[2 * (size_t)v + 1] = make_float4(x0[0], x0[1], x0[2], 0.f);
      return;
    }
  }
  int slot = atomicAdd(xl.count, 1);
  if (slot < xl.cap) xl.items[slot] = v;
  if (cnt >= 4) atomicAdd(n_refit, 1);
}

// listed vertices take the FP64 reference result, split into (hi, lo)
__global__ void k_merge_ref(const int* __restrict__ items, const int* __restrict__ count, int cap,
                            const double* __restrict__ rec64, float4* __restrict__ rec) {
  int n = min(*count, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int v = items[i];
    double a = rec64[3 * (size_t)v], b = rec64[3 * (size_t)v + 1], c = rec64[3 * (size_t)v + 2];
    float ah = (float)a, bh = (float)b, ch = (float)c;
    rec[2 * (size_t)v] = make_float4(ah, bh, ch, 0.f);
    rec[2 * (size_t)v + 1] = make_float4((float)(a - ah), (float)(b - bh), (float)(c - ch), 0.f);
  }
}

// ---------------------------------------------------------------------------
// error: thread per tet, grid-stride over a fixed grid
// ---------------------------------------------------------------------------
struct PairSum {
  float h, l;
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum(h, x, s, e);
    h = s;
    l += e;
  }
};

__device__ __forceinline__ double warp_pair_total(PairSum p) {
  // per-warp combination: pairs summed with TwoSum, one FP64 value per warp
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float oh = __shfl_xor_sync(0xffffffffu, p.h, o);
    float ol = __shfl_xor_sync(0xffffffffu, p.l, o);
    float s, e;
    two_sum(p.h, oh, s, e);
    p.h = s;
    p.l = p.l + ol + e;
  }
  return (double)p.h + (double)p.l;
}

__global__ void __launch_bounds__(kBlock) k_fast_error(DevMesh m, const float4* __restrict__ td,
                                                       const float4* __restrict__ rec, float* __restrict__ q,
                                                       double* __restrict__ partials) {
  __shared__ double sh[2][kBlock / 32];
  PairSum self{0.f, 0.f}, gsum{0.f, 0.f};
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m.T; t += gridDim.x * blockDim.x) {
    int4 tv = __ldg(reinterpret_cast<const int4*>(m.ev) + t);
    float4 ga = ld4(td + 4 * (size_t)t), gb = ld4(td + 4 * (size_t)t + 1);
    float4 G0 = ld4(rec + 2 * (size_t)tv.x), X0 = ld4(rec + 2 * (size_t)tv.x + 1);
    float4 G1 = ld4(rec + 2 * (size_t)tv.y), X1 = ld4(rec + 2 * (size_t)tv.y + 1);
    float4 G2 = ld4(rec + 2 * (size_t)tv.z), X2 = ld4(rec + 2 * (size_t)tv.z + 1);
    float4 G3 = ld4(rec + 2 * (size_t)tv.w), X3 = ld4(rec + 2 * (size_t)tv.w + 1);
    // eps*(IP) = g + D with g = G0, D = (sum (G_i - g) + X_i) / 4
    float g0 = G0.x, g1 = G0.y, g2 = G0.z;
    float D0 = 0.25f * ((X0.x + ((G1.x - g0) + X1.x)) + (((G2.x - g0) + X2.x) + ((G3.x - g0) + X3.x)));
    float D1 = 0.25f * ((X0.y + ((G1.y - g1) + X1.y)) + (((G2.y - g1) + X2.y) + ((G3.y - g1) + X3.y)));
    float D2 = 0.25f * ((X0.z + ((G1.z - g2) + X1.z)) + (((G2.z - g2) + X2.z) + ((G3.z - g2) + X3.z)));
    // eps_t - eps*(IP) = (g_t - g) + d_t - D
    float dx = ((ga.x - g0) + gb.x) - D0, dy = ((ga.y - g1) + gb.y) - D1, dz = ((ga.z - g2) + gb.z) - D2;
    float wdv = ga.w;
    float err = (dx * dx + dy * dy + dz * dz) * wdv;
    float ex = g0 + D0, ey = g1 + D1, ez = g2 + D2;
    self.add((ex * ex + ey * ey + ez * ez) * wdv);
    // (sqrt err)^(6/5) = err^(3/5) = err r^2 and h_max (sqrt err)^(-2/5) =
    // h_max r, with r = err^(-1/5)
    float rr = inv_fifth_root(err);
    gsum.add(err * (rr * rr));
    q[t] = gb.w * rr;
  }
  double s1 = warp_pair_total(self), s2 = warp_pair_total(gsum);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][w] = s1;
    sh[1][w] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < kBlock / 32; ++i) {
      a += sh[0][i];
      b += sh[1][i];
    }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

// ---------------------------------------------------------------------------
// average: size = size_factor * mean(q_t) over the vertex's elements
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_average(DevMesh m, const float* __restrict__ q,
                                                         const double* __restrict__ out3, float* __restrict__ size32) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  int b = m.a_off[v], e = m.a_off[v + 1];
  PairSum s{0.f, 0.f};
  // batches of 8 independent gathers, summed in order
  for (int k0 = b; k0 < e; k0 += 8) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = (k0 + j < e) ? __ldg(q + __ldg(m.a_el + k0 + j)) : 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (k0 + j < e) s.add(x[j]);
  }
  size32[v] = (float)out3[2] * ((s.h + s.l) / (float)(e - b));
}

// ---------------------------------------------------------------------------
// measure: metric length with 2-point Gauss, h linearly interpolated
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_measure(DevMesh m, const float4* __restrict__ vr,
                                                         const float* __restrict__ size32, uint32_t* __restrict__ split,
                                                         uint32_t* __restrict__ collapse, int* __restrict__ guard_items,
                                                         int* __restrict__ guard_count, int guard_cap,
                                                         float guard_rel) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  bool s = false, c = false;
  if (e < m.E) {
    int2 ab = __ldg(reinterpret_cast<const int2*>(m.edv) + e);
    float4 ha = ld4(vr + 2 * (size_t)ab.x), la = ld4(vr + 2 * (size_t)ab.x + 1);
    float4 hb = ld4(vr + 2 * (size_t)ab.y), lb = ld4(vr + 2 * (size_t)ab.y + 1);
    float4 dh, dl;
    pdiff(hb, lb, ha, la, dh, dl);
    float half = 0.5f * len3(dh.x + dl.x, dh.y + dl.y, dh.z + dl.z);
    float s0 = __ldg(size32 + ab.x), s1 = __ldg(size32 + ab.y);
    const float gp = 0.577350269189626f;
    const float n0 = 0.5f * (1.f - gp), n1 = 0.5f * (1.f + gp);
    float L = half * (1.f / (n0 * s0 + n1 * s1) + 1.f / (n1 * s0 + n0 * s1));
    s = L > 1.5f;
    c = L < 0.5f;
    if (fabsf(L - 1.5f) < guard_rel * 1.5f || fabsf(L - 0.5f) < guard_rel * 0.5f) {
      int slot = atomicAdd(guard_count, 1);
      if (slot < guard_cap) guard_items[slot] = e;
    }
  }
  unsigned bs = __ballot_sync(0xffffffffu, s), bc = __ballot_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && e < m.E) {
    split[e >> 5] = bs;
    collapse[e >> 5] = bc;
  }
}

__global__ void k_size_to_f64(int V, const float* __restrict__ s32, double* __restrict__ s64) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < V) s64[v] = (double)s32[v];
}

inline int nblk(long n, int b = kBlock) { return (int)((n + b - 1) / b); }

constexpr int kErrorGrid = 152 * 8;  // 8 resident 256-thread blocks per SM

}  // namespace

int fast_error_blocks(int T) {
  int nb = nblk(T);
  return nb < kErrorGrid ? nb : kErrorGrid;
}

void fast_prep(const DevMesh& m, const double* u, float4* vrec, cudaStream_t s) {
  if (m.V) k_prep<<<nblk(m.V), kBlock, 0, s>>>(m.V, m.xyz, u, vrec);
}

void fast_tet(const DevMesh& m, const float4* vrec, float4* td, cudaStream_t s) {
  if (m.T) k_fast_tet<<<nblk(m.T), kBlock, 0, s>>>(m, vrec, td);
}

void fast_recover(const DevMesh& m, const float4* vrec, const float4* td, float4* rec, ExpandList xl, int* n_refit,
                  cudaStream_t s) {
  if (m.V) k_fast_recover<<<nblk((long)m.V * kGroup), kBlock, 0, s>>>(m, vrec, td, rec, xl, n_refit);
}

void fast_merge_ref(ExpandList xl, const double* rec64, float4* rec, cudaStream_t s) {
  k_merge_ref<<<152, 256, 0, s>>>(xl.items, xl.count, xl.cap, rec64, rec);
}

void fast_error(const DevMesh& m, const float4* td, const float4* rec, float* q, double* partials, int nb,
                cudaStream_t s) {
  if (nb) k_fast_error<<<nb, kBlock, 0, s>>>(m, td, rec, q, partials);
}

void fast_average(const DevMesh& m, const float* q, const double* out3, float* size32, cudaStream_t s) {
  if (m.V) k_fast_average<<<nblk(m.V), kBlock, 0, s>>>(m, q, out3, size32);
}

void fast_measure(const DevMesh& m, const float4* vrec, const float* size32, uint32_t* split, uint32_t* collapse,
                  float* L32, int* guard_items, int* guard_count, int guard_cap, float guard_rel, cudaStream_t s) {
  (void)L32;
  if (m.E)
    k_fast_measure<<<nblk(m.E), kBlock, 0, s>>>(m, vrec, size32, split, collapse, guard_items, guard_count,
                                                guard_cap, guard_rel);
}

void fast_size_to_f64(int V, const float* s32, double* s64, cudaStream_t s) {
  if (V) k_size_to_f64<<<nblk(V), kBlock, 0, s>>>(V, s32, s64);
}

}  // namespace sprg
