// FP32 fast path of the estimate-and-mark pass (3D tets, scalar field).
//
// Every FP64 input value is carried as an unevaluated float pair (hi, lo):
// one 32-byte coordinate record per vertex {x,y,z,-}_hi, {x,y,z,-}_lo (built
// once per mesh, a vertex gather is one DRAM sector) and one 8-byte field
// pair per vertex (rebuilt each pass).  All arithmetic is FP32; the places where the SPR
// estimator cancels are done with error-free transformations (TwoSum,
// TwoProd via fmaf) instead of wider types:
//
//  * differences of nearby coordinates / field values keep the pair
//    (a_hi - b_hi exactly, a_lo - b_lo);
//  * a tet gradient is formed relative to a reference gradient g as
//    J^{-1} (du - J g), with the residual du - J g evaluated by compensated
//    dot products, so only the small deviation carries FP32 rounding;
//  * the recovered value is stored as a value + packed remainder pair, and the
//    element error |eps - eps*|^2 is taken from those deviations.
//
// That keeps the element errors (and so the sizes) at ~1e-7 relative even
// where |eps - eps*| is 1e-3 |eps|.  FP64 appears only in the per-warp
// combination of the two global integrals and in the reference (FP64) path
// for listed patches.
//
// Per-mesh setup (geometry only): the coordinate records, the SPR weights
// w_vt of every patch (FP64, rounded), and per tet {w dV, h_max} and per edge
// half its length (FP64, rounded).
//
// Phases of a pass:
//   prep      four vertices per thread: the field pairs
//   tet       thread per tet: its gradient as 16 bytes, the FP32 value s
//             and the packed correction r (exact = s + r, see pack_corr)
//   recover   1, 2 or 4 lanes per vertex (tuned per patch-size bin):
//             eps*(v) = g_ref + sum w_vt (eps_t - g_ref)
//   error     thread per tet: element error, SelfProduct and Error terms
//             (compensated), q_t = h_max * err^(-1/5) and a relative error
//             bound of q_t
//   average   2 lanes per vertex: size = size_factor * mean(q_t)
//             (compensated) and the size's error bound, packed as a pair
//   measure   thread per edge: metric length, split/collapse bitmaps, and the
//             list of edges whose distance to 0.5 / 1.5 is within the error
//             bound (re-decided in FP64 by the guard kernels)
#include "sprg_fast.h"
#include "sprg_ld.cuh"
#include "sprg_reduce.cuh"

namespace sprg {
namespace {

constexpr int kBlock = 256;
// lanes per vertex in the average kernel (2: 166 -> 129 us at 160^3 against
// 4; 1 or 8, or more entries unrolled per lane, were slower)
constexpr int kGroup = 2;
// relative accuracy assumed for each quantity entering an element-error
// deviation (about 4 FP32 ulps), scaled into the error bound of q_t; on the
// 160^3 workload the largest observed error is 0.43 of the resulting bound
constexpr float kBoundUlps = 2.5e-7f;
// error of the packed corrections: at most 2^-31 of the largest gradient
// component per tet, times about 4 through the recovered values (sum |w_vt|
// of an SPR patch), plus the recovered values' own packing, times 0.4 into
// q = h err^(-1/5)
constexpr float kQuantRel = 1e-9f;

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

// J^{-1} r = C^T r / det (approximate reciprocal: both uses are corrected or
// are corrections)
__device__ __forceinline__ void apply_inv(const Cof& k, float r1, float r2, float r3, float* g) {
  float inv = __fdividef(1.0f, k.det);
#pragma unroll
  for (int j = 0; j < 3; ++j) g[j] = (k.c[0][j] * r1 + k.c[1][j] * r2 + k.c[2][j] * r3) * inv;
}

// x^(-1/5) for the element error x: a hardware log2 / exp2 estimate
// (relative error below 1e-5 for x in (1e-30, 1e30)) refined by one Newton
// step on x r^5 = 1 whose residual is taken with a single rounding (fmaf);
// the step squares the estimate's error, leaving the FP32 rounding of the
// last operations.  Outside that range powf handles zero, inf and NaN.
__device__ __forceinline__ float inv_fifth_root(float x) {
  if (!(x > 1e-30f) || !(x < 1e30f)) return powf(x, -0.2f);
  float r = exp2f(-0.2f * __log2f(x));
  float r2 = r * r;
  float r5 = r2 * r2 * r;
  float e = fmaf(-x, r5, 1.0f);
  return fmaf(r * 0.2f, e, r);
}

// A tet gradient is kept as 16 bytes: the FP32 value s (3 floats) and its
// correction r = exact - s with |r_j| <= ulp(s_j)/2, packed into one word on
// the grid of the largest component: with E_s the exponent of max |s_j|,
//   r_j ~ m_j 2^(E_s - 31),  m_j = rint(r_j 2^(31 - E_s)) in [-128, 128]
// (|r_j| <= 2^(E_s - 24)), stored as m_j + 256 in bits 18..26, 9..17, 0..8.
// The stored correction is exact to 2^(E_s - 32) <= 2^-32 max |s_j|.  The
// grid follows from s alone, so scaling s by a power of two scales the
// decoded r with it.  Values with max |s_j| below 2^-95, infinite or NaN
// carry no correction (kNoCorr, m_j = 0).  Rounding and the int <-> float
// steps use the 1.5 * 2^23 constant (integer and FMA pipes) instead of
// conversion instructions, which run at a quarter rate.
constexpr uint32_t kNoCorr = (256u << 18) | (256u << 9) | 256u;
__device__ __forceinline__ int fexp(float a) { return ((__float_as_int(a) >> 23) & 0xff) - 127; }
// 2^k as a float, -126 <= k <= 127
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

__device__ __forceinline__ uint32_t pack_corr(float s0, float s1, float s2, float r0, float r1, float r2) {
  const float smax = fmaxf(fabsf(s0), fmaxf(fabsf(s1), fabsf(s2)));
  if (!(smax >= 0x1p-95f) || !(smax < 3.0e38f)) return kNoCorr;
  // 2^(31 - E_s) as a float: exponent field 158 - E_s in [31, 253]
  const float sc = __int_as_float((158 - fexp(smax)) << 23);
  auto q9 = [&](float r) {  // rint(r 2^(31 - E_s)) + 256, clamped to [1, 511]
    const int mj = __float_as_int(fmaf(r, sc, 12582912.f)) - 0x4B400000;
    return (uint32_t)(max(-255, min(255, mj)) + 256);
  };
  return (q9(r0) << 18) | (q9(r1) << 9) | q9(r2);
}

struct Grad {
  float s[3], r[3];
  float gmax;  // max |s_j|
};

__device__ __forceinline__ Grad unpack_grad(uint4 a) {
  Grad g;
  g.s[0] = __uint_as_float(a.x);
  g.s[1] = __uint_as_float(a.y);
  g.s[2] = __uint_as_float(a.z);
  g.gmax = fmaxf(fabsf(g.s[0]), fmaxf(fabsf(g.s[1]), fabsf(g.s[2])));
  // 2^(E_s - 31); below 2^-126 (max |s_j| < 2^-95) the correction is zero
  const int ex = fexp(g.gmax) - 31;
  const float sc = ex > -127 ? __int_as_float((ex + 127) << 23) : 0.f;
  // m_j as a float: 1.5 * 2^23 + (m_j + 256) read as a float, minus the offset
  const float off = 12582912.f + 256.f;
  g.r[0] = (__int_as_float(0x4B400000 + ((a.w >> 18) & 0x1ffu)) - off) * sc;
  g.r[1] = (__int_as_float(0x4B400000 + ((a.w >> 9) & 0x1ffu)) - off) * sc;
  g.r[2] = (__int_as_float(0x4B400000 + (a.w & 0x1ffu)) - off) * sc;
  return g;
}

// a recovered value's 32-byte record {s0, s1, s2, r0}, {r1, r2, -, -}: the
// value and its exact FP32 remainder (gmax unused for these)
__device__ __forceinline__ Grad rec_grad(const float4& h, const float4& l) {
  Grad g;
  g.s[0] = h.x; g.s[1] = h.y; g.s[2] = h.z;
  g.r[0] = h.w; g.r[1] = l.x; g.r[2] = l.y;
  g.gmax = 0.f;
  return g;
}

// ---------------------------------------------------------------------------
// coordinate records (once per mesh) and the field pair (once per pass).
// The coordinates are mapped into [1, 2] (x' = (x - c) s + 1, s a power of
// two): differences of the high words of two records are then exact (Sterbenz)
// and gradients scale back exactly (du/dx = s du/dx').
__global__ void __launch_bounds__(kBlock) k_prep_coords(int V, const double* __restrict__ xyz, double cx, double cy,
                                                        double cz, double cs, float4* __restrict__ rec) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  double x = (xyz[3 * (size_t)v] - cx) * cs + 1.0, y = (xyz[3 * (size_t)v + 1] - cy) * cs + 1.0,
         z = (xyz[3 * (size_t)v + 2] - cz) * cs + 1.0;
  float xh = (float)x, yh = (float)y, zh = (float)z;
  rec[2 * (size_t)v] = make_float4(xh, yh, zh, 0.f);
  rec[2 * (size_t)v + 1] = make_float4((float)(x - xh), (float)(y - yh), (float)(z - zh), 0.f);
}

// w = hi + lo with hi = w truncated to 24 significant bits and lo the rest
// rounded to 24 bits (w to 2^-48 relative), by integer operations: a split
// with FP64 arithmetic would run on the FP64 pipe, which bounds this kernel.
// Magnitudes outside [2^-74, 2^128) (zero, tiny, huge, inf, NaN) take the
// FP64 conversion.
__device__ __forceinline__ float2 split_pair(double w) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(w);
  const int e = (int)((b >> 52) & 0x7ff);  // biased exponent
  if (e >= 949 && e <= 1150) {
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const unsigned hb = sign | ((unsigned)(e - 896) << 23) | (unsigned)((b >> 29) & 0x7fffffu);
    const float lo = (float)(unsigned)(b & 0x1fffffffu) * __uint_as_float((unsigned)(e - 948) << 23);
    return make_float2(__uint_as_float(hb), sign ? -lo : lo);
  }
  const float h = (float)w;
  return make_float2(h, (float)(w - h));
}

// the pass's vertex records: the per-mesh coordinate records with the field
// pair in the fourth slots, {x,y,z,u}_hi, {x,y,z,u}_lo (one sector per vertex)
// (also the field's largest |u| in FP32, for the rounding-dominance test:
// one atomic per block)
__global__ void __launch_bounds__(kBlock) k_prep(int V, const double* __restrict__ u, const float4* __restrict__ crec,
                                                 float4* __restrict__ vrec, int* __restrict__ umax_bits) {
  // |u_hi| as float bits: non-negative floats order as their bit patterns,
  // a NaN (sign cleared) above +inf, so an integer max keeps it
  int um = 0;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < V) {
    const float2 p = split_pair(__ldg(u + v));
    float4 h = ld4(crec + 2 * (size_t)v), l = ld4(crec + 2 * (size_t)v + 1);
    h.w = p.x;
    l.w = p.y;
    vrec[2 * (size_t)v] = h;
    vrec[2 * (size_t)v + 1] = l;
    um = __float_as_int(p.x) & 0x7fffffff;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) um = max(um, __shfl_xor_sync(0xffffffffu, um, o));
  __shared__ int sw[kBlock / 32];
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = um;
  __syncthreads();
  if (threadIdx.x == 0) {
    int b = sw[0];
    for (int i = 1; i < kBlock / 32; ++i) b = max(b, sw[i]);
    if (b != 0) atomicMax(umax_bits, b);
  }
}

// per tet {w dV, h_max} (FP32 for the pass, {det J, h_max} in FP64 for the
// guard) and per edge half its length, FP64 then rounded (once per mesh)
__global__ void __launch_bounds__(kBlock) k_fast_geo(DevMesh m, float2* __restrict__ geo, double2* __restrict__ geo64,
                                                     double* __restrict__ cent, unsigned long long* __restrict__ qmax) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double qv = 0;
  if (t < m.T) {
    const int* ev = m.ev + 4 * (size_t)t;
    double x[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) x[i][k] = m.xyz[3 * (size_t)ev[i] + k];
    double e[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) e[i][k] = x[i + 1][k] - x[0][k];
    double det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) + e[0][1] * (e[1][2] * e[2][0] - e[1][0] * e[2][2]) +
                 e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
    double h2 = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = i + 1; j < 4; ++j) {
        double dx = x[j][0] - x[i][0], dy = x[j][1] - x[i][1], dz = x[j][2] - x[i][2];
        h2 = fmax(h2, dx * dx + dy * dy + dz * dz);
      }
    const double h = sqrt(h2);
    geo[t] = make_float2((float)(det * (1.0 / 6.0)), (float)h);
    geo64[t] = make_double2(det, h);
    // the integration point, summed in vertex order as the weights use it
#pragma unroll
    for (int k = 0; k < 3; ++k) cent[3 * (size_t)t + k] = 0.25 * (((x[0][k] + x[1][k]) + x[2][k]) + x[3][k]);
    // |cof(J)|_F^2 / |det J| (= |J^-1|_F^2 |det J|): the element's share of the
    // reference's gradient rounding in the error integral scales with it; the
    // largest over the mesh, for the rounding-dominance test
    double c2 = 0;
    for (int i = 0; i < 3; ++i) {
      const double* a = e[(i + 1) % 3];
      const double* b = e[(i + 2) % 3];
      const double c0 = a[1] * b[2] - a[2] * b[1], c1 = a[2] * b[0] - a[0] * b[2], cc = a[0] * b[1] - a[1] * b[0];
      c2 += c0 * c0 + c1 * c1 + cc * cc;
    }
    qv = c2 / fabs(det);  // inf for a flat element
    if (!(qv == qv)) qv = INFINITY;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) qv = fmax(qv, __shfl_xor_sync(0xffffffffu, qv, o));
  // non-negative doubles order as their bit patterns (one atomic per warp)
  if ((threadIdx.x & 31) == 0 && qv > 0) atomicMax(qmax, (unsigned long long)__double_as_longlong(qv));
}

__global__ void __launch_bounds__(kBlock) k_fast_elen(DevMesh m, float* __restrict__ half_len) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.E) return;
  const int a = m.edv[2 * (size_t)e], b = m.edv[2 * (size_t)e + 1];
  double dx = m.xyz[3 * (size_t)b] - m.xyz[3 * (size_t)a], dy = m.xyz[3 * (size_t)b + 1] - m.xyz[3 * (size_t)a + 1],
         dz = m.xyz[3 * (size_t)b + 2] - m.xyz[3 * (size_t)a + 2];
  half_len[e] = (float)(0.5 * sqrt(dx * dx + dy * dy + dz * dz));
}

// tet t's edge pairs (x_i - x_0, u_i - u_0), i = 1..3, as (hi, lo)
struct TetData {
  float4 eh[3], el[3];
};

// record difference a - b: coordinates in [1, 2], so the high words
// subtract exactly; the field pair takes a TwoSum
__device__ __forceinline__ void rdiff(const float4& ah, const float4& al, const float4& bh, const float4& bl,
                                      float4& dh, float4& dl) {
  dh.x = ah.x - bh.x; dl.x = al.x - bl.x;
  dh.y = ah.y - bh.y; dl.y = al.y - bl.y;
  dh.z = ah.z - bh.z; dl.z = al.z - bl.z;
  float e;
  two_sum(ah.w, -bh.w, dh.w, e);
  dl.w = (al.w - bl.w) + e;
}

__device__ __forceinline__ TetData load_tet(const float4* __restrict__ vr, int4 tv) {
  TetData d;
  float4 h0, l0, h1, l1, h2, l2, h3, l3;
  ld_record(vr + 2 * (size_t)tv.x, h0, l0);
  ld_record(vr + 2 * (size_t)tv.y, h1, l1);
  ld_record(vr + 2 * (size_t)tv.z, h2, l2);
  ld_record(vr + 2 * (size_t)tv.w, h3, l3);
  rdiff(h1, l1, h0, l0, d.eh[0], d.el[0]);
  rdiff(h2, l2, h0, l0, d.eh[1], d.el[1]);
  rdiff(h3, l3, h0, l0, d.eh[2], d.el[2]);
  return d;
}

// ---------------------------------------------------------------------------
// tet: gradient value and packed correction
// ---------------------------------------------------------------------------
// Blocks take chunks of kTetChunk x blockDim elements from a counter (so a
// kernel running beside this one, such as the listed patches' FP64 fits on
// the side stream, only delays the chunks of the blocks it displaces); in a
// chunk each thread loads the next element's vertex ids before working on
// the current one, so only the record gathers (mostly L2 hits) stay on the
// dependent chain.
constexpr int kTetChunk = 8;

// The gradient of an ill-conditioned tet from the mesh's FP64 coordinates and
// field: J g = du solved with FP64 cofactors (the FP64 path's arithmetic,
// accurate to about cond(J) 2^-53), as FP32 value + packed remainder in the
// mesh's units
__device__ __noinline__ uint4 tet_grad_f64(const double* __restrict__ xyz, const double* __restrict__ u, int4 tv) {
  const int id[4] = {tv.x, tv.y, tv.z, tv.w};
  double e[3][3], du[3];
  const double u0 = u[id[0]];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int k = 0; k < 3; ++k) e[i][k] = xyz[3 * (size_t)id[i + 1] + k] - xyz[3 * (size_t)id[0] + k];
    du[i] = u[id[i + 1]] - u0;
  }
  double cf[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double* a = e[(i + 1) % 3];
    const double* b = e[(i + 2) % 3];
    cf[i][0] = a[1] * b[2] - a[2] * b[1];
    cf[i][1] = a[2] * b[0] - a[0] * b[2];
    cf[i][2] = a[0] * b[1] - a[1] * b[0];
  }
  const double det = e[0][0] * cf[0][0] + e[0][1] * cf[0][1] + e[0][2] * cf[0][2];
  float s[3], r[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double g = (cf[0][j] * du[0] + cf[1][j] * du[1] + cf[2][j] * du[2]) / det;
    s[j] = (float)g;
    r[j] = (float)(g - (double)s[j]);
  }
  return make_uint4(__float_as_uint(s[0]), __float_as_uint(s[1]), __float_as_uint(s[2]),
                    pack_corr(s[0], s[1], s[2], r[0], r[1], r[2]));
}

__global__ void __launch_bounds__(kBlock, 4) k_fast_tet(DevMesh m, const float4* __restrict__ vr, const double* __restrict__ u,
                                                        float gscale, uint4* __restrict__ td, int* __restrict__ next_chunk) {
  const int4* __restrict__ ev4 = reinterpret_cast<const int4*>(m.ev);
  __shared__ int chunk;
  for (;;) {
    if (threadIdx.x == 0) chunk = atomicAdd(next_chunk, 1);
    __syncthreads();
    const long t0 = (long)chunk * (kTetChunk * kBlock);
    __syncthreads();
    if (t0 >= m.T) break;  // every thread of the block leaves here together
    const int t_end = (int)min((long)m.T, t0 + kTetChunk * kBlock);
    int t = (int)t0 + threadIdx.x;
    int4 next = t < t_end ? __ldg(ev4 + t) : make_int4(0, 0, 0, 0);
    for (; t < t_end; t += kBlock) {
      const int4 tv = next;
      if (t + kBlock < t_end) next = __ldg(ev4 + t + kBlock);
      TetData d = load_tet(vr, tv);
      // first estimate with an approximate inverse of the rounded edge matrix
      // (hi + lo: the high words alone, exact differences of [1, 2] values, are
      // off by up to 2^-23 absolute, which squared through the correction would
      // exceed the accuracy the error bound assumes); the correction
      // J^{-1}(du - J g) with the compensated residual makes the result accurate
      // to second order in both approximations
      Cof cf;
      {
        float4 er[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
          er[i] = make_float4(d.eh[i].x + d.el[i].x, d.eh[i].y + d.el[i].y, d.eh[i].z + d.el[i].z, 0.f);
        cf = cofactors(er[0], er[1], er[2]);
      }
      float g[3], c[3], s[3], r[3];
      apply_inv(cf, d.eh[0].w + d.el[0].w, d.eh[1].w + d.el[1].w, d.eh[2].w + d.el[2].w, g);
      apply_inv(cf, comp_residual(d.eh[0], d.el[0], g[0], g[1], g[2]), comp_residual(d.eh[1], d.el[1], g[0], g[1], g[2]),
                comp_residual(d.eh[2], d.el[2], g[0], g[1], g[2]), c);
      // (the first estimate takes du rounded to FP32, so) |c| is about
      // cond(J) 2^-23 |g|, and what the correction leaves about
      // |c|^2 / |g|; past |c| = 2^-17 |g| (cond(J) around 64 and up: a few
      // elements per million of a jittered box) that and the records' own
      // 2^-48 rounding, amplified by cond(J), pass the accuracy the error
      // bound assumes, so the gradient is solved in FP64 instead
      if (c[0] * c[0] + c[1] * c[1] + c[2] * c[2] > 0x1p-34f * (g[0] * g[0] + g[1] * g[1] + g[2] * g[2])) {
        td[t] = tet_grad_f64(m.xyz, u, tv);
        continue;
      }
      // s + r = g + c exactly (|c| << |g|: Fast2Sum)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        s[j] = g[j] + c[j];
        r[j] = c[j] - (s[j] - g[j]);
      }
      // back to the mesh's coordinates: the correction word is relative to the
      // largest |s_j|, so scaling s by a power of two scales r with it
      const uint32_t corr = pack_corr(s[0], s[1], s[2], r[0], r[1], r[2]);
      td[t] = make_uint4(__float_as_uint(s[0] * gscale), __float_as_uint(s[1] * gscale),
                         __float_as_uint(s[2] * gscale), corr);
    }
  }
}

// ---------------------------------------------------------------------------
// SPR weights (once per mesh).  The constant term of the patch fit, which is
// the recovered value at the patch vertex when the fit is centred there, is
// a fixed linear combination of the patch samples:
//     eps*(v) = sum_t w_vt eps_t,   w_vt = e_0^T (A^T A)^{-1} [1, s_t],
// with s_t the integration point of t relative to v, scaled.  The weights
// depend on the geometry only, so they are computed once per mesh in FP64
// (normal equations, Cholesky) and stored in patch-CSR order.  Patches with
// fewer than four elements or a condition estimate above 1e6 are listed for
// the FP64 reference path (growth + Householder QR) instead.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_weights(DevMesh m, const double* __restrict__ cent,
                                                         float* __restrict__ w, double* __restrict__ w64, ExpandList xl,
                                                         int* __restrict__ n_refit, unsigned char* __restrict__ listed) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  const int beg = m.p_off[v], cnt = m.p_off[v + 1] - beg;
  const double xv = m.xyz[3 * (size_t)v], yv = m.xyz[3 * (size_t)v + 1], zv = m.xyz[3 * (size_t)v + 2];
  double a[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  double inv_h = 0;
  bool ok = cnt >= 4;
  for (int k = 0; ok && k < cnt; ++k) {
    const double* ce = cent + 3 * (size_t)m.p_el[beg + k];
    double sx = ce[0] - xv, sy = ce[1] - yv, sz = ce[2] - zv;
    if (k == 0) inv_h = 1.0 / sqrt(sx * sx + sy * sy + sz * sz);
    sx *= inv_h; sy *= inv_h; sz *= inv_h;
    a[0] += 1; a[1] += sx; a[2] += sy; a[3] += sz;
    a[4] += sx * sx; a[5] += sx * sy; a[6] += sx * sz; a[7] += sy * sy; a[8] += sy * sz; a[9] += sz * sz;
  }
  double l00 = 0, l10 = 0, l20 = 0, l30 = 0, l11 = 0, l21 = 0, l31 = 0, l22 = 0, l32 = 0, l33 = 0;
  if (ok) {
    l00 = sqrt(a[0]);
    l10 = a[1] / l00; l20 = a[2] / l00; l30 = a[3] / l00;
    double d1 = a[4] - l10 * l10;
    l11 = sqrt(fmax(d1, 0.0));
    l21 = (a[5] - l20 * l10) / l11; l31 = (a[6] - l30 * l10) / l11;
    double d2 = a[7] - l20 * l20 - l21 * l21;
    l22 = sqrt(fmax(d2, 0.0));
    l32 = (a[8] - l30 * l20 - l31 * l21) / l22;
    double d3 = a[9] - l30 * l30 - l31 * l31 - l32 * l32;
    l33 = sqrt(fmax(d3, 0.0));
    double pmin = fmin(fmin(d1, d2), fmin(d3, a[0])), pmax = fmax(fmax(d1, d2), fmax(d3, a[0]));
    ok = (pmin > 0) && (pmax <= 1e6 * pmin);
  }
  listed[v] = ok ? 0 : 1;
  if (!ok) {
    int slot = atomicAdd(xl.count, 1);
    if (slot < xl.cap) xl.items[slot] = v;
    if (cnt >= 4) atomicAdd(n_refit, 1);
    return;
  }
  // row q = e_0^T (L L^T)^{-1}: solve L y = e_0, then L^T q = y
  double y0 = 1.0 / l00;
  double y1 = (-l10 * y0) / l11;
  double y2 = (-l20 * y0 - l21 * y1) / l22;
  double y3 = (-l30 * y0 - l31 * y1 - l32 * y2) / l33;
  double q3 = y3 / l33;
  double q2 = (y2 - l32 * q3) / l22;
  double q1 = (y1 - l21 * q2 - l31 * q3) / l11;
  double q0 = (y0 - l10 * q1 - l20 * q2 - l30 * q3) / l00;
  for (int k = 0; k < cnt; ++k) {
    const double* ce = cent + 3 * (size_t)m.p_el[beg + k];
    double sx = (ce[0] - xv) * inv_h, sy = (ce[1] - yv) * inv_h, sz = (ce[2] - zv) * inv_h;
    const double wk = q0 + q1 * sx + q2 * sy + q3 * sz;
    w[beg + k] = (float)wk;
    w64[beg + k] = wk;
  }
}

// ---------------------------------------------------------------------------
// recover: eps*(v) = g_ref + sum_t w_vt ((s_t - g_ref) + r_t), stored as the
// value + FP32 remainder in a 32-byte record (the error kernel reads it with
// one 256-bit load and no decoding).  Vertices are binned by patch size; one
// persistent grid takes tiles (first, count, lanes, bin) from a counter and
// gives a tile's vertices `lanes` lanes each.  Lane l sums the elements
// k = l, l + L, ... of the patch into the class sums x_{k mod 4} (each in
// increasing k) and the classes are combined as (x0 + x1) + (x2 + x3): the
// same operations for every lane count, so every tiling gives bitwise the
// same result.
// ---------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ void recover_tile(const DevMesh& m, const float* __restrict__ w,
                                             const uint4* __restrict__ td, float4* __restrict__ rec,
                                             const int* __restrict__ verts, int first, int count) {
  constexpr int NX = 4 / L;
  const int gl = threadIdx.x % L, slot = threadIdx.x / L;
  const int lane = threadIdx.x & 31, leader = lane & ~(L - 1);
  for (int i0 = 0; i0 < count; i0 += blockDim.x / L) {
    const int i = i0 + slot;
    const bool active = i < count;
    const int v = active ? __ldg(verts + first + i) : 0;
    int beg = 0, cnt = 0;
    float gr0 = 0.f, gr1 = 0.f, gr2 = 0.f;
    if (active) {
      beg = m.p_off[v];
      cnt = m.p_off[v + 1] - beg;
      if (gl == 0) {
        const uint4 a = __ldg(td + m.p_el[beg]);
        gr0 = __uint_as_float(a.x); gr1 = __uint_as_float(a.y); gr2 = __uint_as_float(a.z);
      }
    }
    if (L > 1) {
      gr0 = __shfl_sync(0xffffffffu, gr0, leader);
      gr1 = __shfl_sync(0xffffffffu, gr1, leader);
      gr2 = __shfl_sync(0xffffffffu, gr2, leader);
    }
    float x[NX][3];
#pragma unroll
    for (int c = 0; c < NX; ++c) x[c][0] = x[c][1] = x[c][2] = 0.f;
    for (int k = gl; k < cnt; k += L) {
      const int t = __ldg(m.p_el + beg + k);
      const float wk = __ldg(w + beg + k);
      const Grad g = unpack_grad(__ldg(td + t));
      const int c = (k & 3) / L;
#pragma unroll
      for (int cc = 0; cc < NX; ++cc)
        if (cc == c) {
          x[cc][0] = fmaf(wk, (g.s[0] - gr0) + g.r[0], x[cc][0]);
          x[cc][1] = fmaf(wk, (g.s[1] - gr1) + g.r[1], x[cc][1]);
          x[cc][2] = fmaf(wk, (g.s[2] - gr2) + g.r[2], x[cc][2]);
        }
    }
    float tot[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (L == 4) {
        float a = x[0][d];
        a += __shfl_xor_sync(0xffffffffu, a, 1);
        a += __shfl_xor_sync(0xffffffffu, a, 2);
        tot[d] = a;
      } else if (L == 2) {
        const float a = x[0][d] + __shfl_xor_sync(0xffffffffu, x[0][d], 1);
        const float b = x[NX - 1][d] + __shfl_xor_sync(0xffffffffu, x[NX - 1][d], 1);
        tot[d] = a + b;
      } else {
        tot[d] = (x[0][d] + x[NX > 1 ? 1 : 0][d]) + (x[NX > 2 ? 2 : 0][d] + x[NX > 3 ? 3 : 0][d]);
      }
    }
    if (active && gl == 0) {
      float s0, s1, s2, r0, r1, r2;
      two_sum(gr0, tot[0], s0, r0);
      two_sum(gr1, tot[1], s1, r1);
      two_sum(gr2, tot[2], s2, r2);
      rec[2 * (size_t)v] = make_float4(s0, s1, s2, r0);
      rec[2 * (size_t)v + 1] = make_float4(r1, r2, 0.f, 0.f);
    }
  }
}

// One lane per vertex over the sliced copy of the patch lists (lanes = 0):
// warp j of the tile takes slice `slice0 + j`, whose entry k of lane i sits
// at off + 32 k + i, so each step reads the 32 patches' element ids and
// weights as two 128-byte lines.  Same operations as recover_tile<1>
// (classes x_{k mod 4}, then (x0 + x1) + (x2 + x3)): the same bits.
__device__ __forceinline__ void recover_tile_sliced(const DevMesh& m, SlicedPatches sp,
                                                    const uint4* __restrict__ td, float4* __restrict__ rec,
                                                    const int* __restrict__ verts, int first, int count,
                                                    int slice0) {
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j = threadIdx.x >> 5; 32 * j < count; j += nw) {
    const int i = 32 * j + lane;
    const bool active = i < count;
    const int v = active ? __ldg(verts + first + i) : 0;
    const int cnt = active ? m.p_off[v + 1] - m.p_off[v] : 0;
    const int* __restrict__ el = sp.el + __ldg(sp.off + slice0 + j) + lane;
    const float* __restrict__ wt = sp.w + (el - sp.el);
    float gr0 = 0.f, gr1 = 0.f, gr2 = 0.f;
    if (cnt > 0) {
      const uint4 a = __ldg(td + __ldg(el));
      gr0 = __uint_as_float(a.x); gr1 = __uint_as_float(a.y); gr2 = __uint_as_float(a.z);
    }
    float x[4][3];
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c][0] = x[c][1] = x[c][2] = 0.f;
    // groups of four entries (entry k + c in class c); the next group's ids
    // and weights load while this group's gradients are gathered
    int tn[4];
    float wn[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      tn[c] = c < cnt ? __ldg(el + 32 * c) : 0;
      wn[c] = c < cnt ? __ldg(wt + 32 * c) : 0.f;
    }
    for (int k = 0; k < cnt; k += 4) {
      int t[4];
      float wk[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        t[c] = tn[c];
        wk[c] = wn[c];
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const bool more = k + 4 + c < cnt;
        tn[c] = more ? __ldg(el + 32 * (k + 4 + c)) : 0;
        wn[c] = more ? __ldg(wt + 32 * (k + 4 + c)) : 0.f;
      }
      uint4 a[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) a[c] = k + c < cnt ? __ldg(td + t[c]) : make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (k + c < cnt) {
          const Grad g = unpack_grad(a[c]);
          x[c][0] = fmaf(wk[c], (g.s[0] - gr0) + g.r[0], x[c][0]);
          x[c][1] = fmaf(wk[c], (g.s[1] - gr1) + g.r[1], x[c][1]);
          x[c][2] = fmaf(wk[c], (g.s[2] - gr2) + g.r[2], x[c][2]);
        }
    }
    if (active) {
      float tot[3], s3[3], r3[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) tot[d] = (x[0][d] + x[1][d]) + (x[2][d] + x[3][d]);
      two_sum(gr0, tot[0], s3[0], r3[0]);
      two_sum(gr1, tot[1], s3[1], r3[1]);
      two_sum(gr2, tot[2], s3[2], r3[2]);
      rec[2 * (size_t)v] = make_float4(s3[0], s3[1], s3[2], r3[0]);
      rec[2 * (size_t)v + 1] = make_float4(r3[1], r3[2], 0.f, 0.f);
    }
  }
}

// MODE: the lane mode of every tile (0 sliced, 1, 2, 4), or -1 for tiles of
// mixed modes (a kernel per mode keeps each mode's own register count).  The
// gathers want loads in flight more than resident warps: capping 2 lanes at
// 32 registers for eight blocks per SM made it a third slower.
template <int MODE>
__global__ void __launch_bounds__(kBlock, MODE <= 0 ? 4 : 5)
    k_fast_recover_tiles(DevMesh m, const float* __restrict__ w, SlicedPatches sp, const uint4* __restrict__ td,
                         float4* __restrict__ rec, const int* __restrict__ verts, const int4* __restrict__ tiles,
                         int n_tiles, int* __restrict__ next) {
  __shared__ int cur;
  for (;;) {
    if (threadIdx.x == 0) cur = atomicAdd(next, 1);
    __syncthreads();
    const int t = cur;
    __syncthreads();
    if (t >= n_tiles) return;
    const int4 tile = tiles[t];  // (first, count, lanes, slice of `first`)
    const int mode = MODE >= 0 ? MODE : tile.z;
    if (mode == 0) recover_tile_sliced(m, sp, td, rec, verts, tile.x, tile.y, tile.w);
    else if (mode == 1) recover_tile<1>(m, w, td, rec, verts, tile.x, tile.y);
    else if (mode == 2) recover_tile<2>(m, w, td, rec, verts, tile.x, tile.y);
    else recover_tile<4>(m, w, td, rec, verts, tile.x, tile.y);
  }
}

// sliced copy of the patch lists: slice widths (thread per slice), then,
// with the slices' offsets, the fill (thread per binned vertex)
__device__ __forceinline__ int slice_bin(const BinSlices& bs, int s) {
  int b = 0;
  while (b < 3 && s >= bs.slice0[b + 1]) ++b;
  return b;
}

__global__ void k_slice_width(DevMesh m, BinSlices bs, const int* __restrict__ verts, int* __restrict__ width) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= bs.slice0[4]) return;
  const int b = slice_bin(bs, s);
  const int i0 = bs.start[b] + 32 * (s - bs.slice0[b]), i1 = min(i0 + 32, bs.start[b + 1]);
  int wmax = 0;
  for (int i = i0; i < i1; ++i) {
    const int v = verts[i];
    wmax = max(wmax, m.p_off[v + 1] - m.p_off[v]);
  }
  width[s] = wmax;
}

__global__ void k_slice_fill(DevMesh m, BinSlices bs, const int* __restrict__ verts, const float* __restrict__ w,
                             const int* __restrict__ off, int* __restrict__ sel, float* __restrict__ sw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= bs.start[4]) return;
  int b = 0;
  while (b < 3 && i >= bs.start[b + 1]) ++b;
  const int r = i - bs.start[b];
  const int s = bs.slice0[b] + r / 32, lane = r % 32;
  const int v = verts[i], beg = m.p_off[v], cnt = m.p_off[v + 1] - beg;
  int* el = sel + off[s] + lane;
  float* wt = sw + off[s] + lane;
  for (int k = 0; k < cnt; ++k) {
    el[32 * k] = m.p_el[beg + k];
    wt[32 * k] = w[beg + k];
  }
}

// patch-size class of a vertex: <= 8, <= 16, <= 32, more elements
__device__ __forceinline__ int patch_class(int cnt) { return cnt <= 8 ? 0 : cnt <= 16 ? 1 : cnt <= 32 ? 2 : 3; }

__global__ void k_patch_class(DevMesh m, const unsigned char* __restrict__ listed, unsigned char* __restrict__ cls) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  cls[v] = listed[v] ? 4 : (unsigned char)patch_class(m.p_off[v + 1] - m.p_off[v]);
}

constexpr int kBinBlock = 1024;

// Stable partition of the vertices by patch class (bins 0..3; class 4, the
// listed patches, stays out): per-block class counts, then a scatter over
// the same blocks, each class in ascending vertex order.  Counts are sums of
// ballots, the ranks prefix sums over warps: the order is fixed.
__global__ void __launch_bounds__(kBinBlock) k_bin_count(int V, const unsigned char* __restrict__ cls,
                                                         int* __restrict__ counts) {
  __shared__ int sc[4];
  if (threadIdx.x < 4) sc[threadIdx.x] = 0;
  __syncthreads();
  const int v = blockIdx.x * kBinBlock + threadIdx.x;
  const int b = v < V ? cls[v] : 4;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const unsigned mask = __ballot_sync(0xffffffffu, b == k);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&sc[k], __popc(mask));
  }
  __syncthreads();
  if (threadIdx.x < 4) counts[4 * blockIdx.x + threadIdx.x] = sc[threadIdx.x];
}

__global__ void __launch_bounds__(kBinBlock) k_bin_scatter(int V, const unsigned char* __restrict__ cls,
                                                           const int* __restrict__ offs, int* __restrict__ order) {
  __shared__ int wc[kBinBlock / 32][4];
  const int v = blockIdx.x * kBinBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int b = v < V ? cls[v] : 4;
  unsigned mine = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const unsigned mask = __ballot_sync(0xffffffffu, b == k);
    if (lane == 0) wc[w][k] = __popc(mask);
    if (b == k) mine = mask;
  }
  __syncthreads();
  if (b < 4) {
    int before = 0;
    for (int j = 0; j < w; ++j) before += wc[j][b];
    order[offs[4 * blockIdx.x + b] + before + __popc(mine & ((1u << lane) - 1))] = v;
  }
}

// listed vertices take the FP64 reference result, as value + remainder
__global__ void k_merge_ref(const int* __restrict__ items, const int* __restrict__ count, int cap,
                            const double* __restrict__ rec64, float4* __restrict__ rec) {
  int n = min(*count, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int v = items[i];
    double a = rec64[3 * (size_t)v], b = rec64[3 * (size_t)v + 1], c = rec64[3 * (size_t)v + 2];
    float ah = (float)a, bh = (float)b, ch = (float)c;
    rec[2 * (size_t)v] = make_float4(ah, bh, ch, (float)(a - ah));
    rec[2 * (size_t)v + 1] = make_float4((float)(b - bh), (float)(c - ch), 0.f, 0.f);
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

// grid-stride over all elements, or (batch) block b over the element range
// seg[b] of one mesh, so each block's partials belong to one mesh
// done != null (one mesh): the last block to finish reduces the partials
// and writes the size factor to out3 (the work of the FP64 size-factor
// kernel, the same function), then clears the counter for the next pass
__global__ void __launch_bounds__(kBlock) k_fast_error(DevMesh m, const uint4* __restrict__ td,
                                                       const float2* __restrict__ geo,
                                                       const float4* __restrict__ rec, float2* __restrict__ q,
                                                       double* __restrict__ partials, const int2* __restrict__ seg,
                                                       unsigned* __restrict__ done, double adapt_ratio, int dim,
                                                       double* __restrict__ out3, int* __restrict__ n_round,
                                                       const unsigned long long* __restrict__ qmax) {
  __shared__ double sh[2][kBlock / 32];
  PairSum self{0.f, 0.f}, gsum{0.f, 0.f};
  int t_beg = blockIdx.x * blockDim.x + threadIdx.x, t_end = m.T, t_step = gridDim.x * blockDim.x;
  if (seg) {
    const int2 r = seg[blockIdx.x];
    t_beg = r.x + threadIdx.x;
    t_end = r.y;
    t_step = blockDim.x;
  }
  // the next element's ids, gradient and geometry are loaded one iteration
  // ahead: only the recovered-value gathers stay on the dependent chain
  int4 ntv = make_int4(0, 0, 0, 0);
  uint4 nta = make_uint4(0, 0, 0, 0);
  float2 ngm = make_float2(0.f, 0.f);
  if (t_beg < t_end) {
    ntv = __ldg(reinterpret_cast<const int4*>(m.ev) + t_beg);
    nta = __ldg(td + t_beg);
    ngm = __ldg(geo + t_beg);
  }
  for (int t = t_beg; t < t_end; t += t_step) {
    {
      const int4 tv = ntv;
      const uint4 ta = nta;
      const float2 gm = ngm;
      if (t + t_step < t_end) {
        ntv = __ldg(reinterpret_cast<const int4*>(m.ev) + t + t_step);
        nta = __ldg(td + t + t_step);
        ngm = __ldg(geo + t + t_step);
      }
      float4 H0, L0, H1, L1, H2, L2, H3, L3;
      ld_record(rec + 2 * (size_t)tv.x, H0, L0);
      ld_record(rec + 2 * (size_t)tv.y, H1, L1);
      ld_record(rec + 2 * (size_t)tv.z, H2, L2);
      ld_record(rec + 2 * (size_t)tv.w, H3, L3);
      Grad ga = unpack_grad(ta);
      const Grad E0 = rec_grad(H0, L0), E1 = rec_grad(H1, L1), E2 = rec_grad(H2, L2), E3 = rec_grad(H3, L3);
      // eps*(IP) = g + D with g = s of vertex 0, D = sum ((s_i - g) + r_i) / 4
      const float g0 = E0.s[0], g1 = E0.s[1], g2 = E0.s[2];
      float D0 = 0.25f * ((E0.r[0] + ((E1.s[0] - g0) + E1.r[0])) + (((E2.s[0] - g0) + E2.r[0]) + ((E3.s[0] - g0) + E3.r[0])));
      float D1 = 0.25f * ((E0.r[1] + ((E1.s[1] - g1) + E1.r[1])) + (((E2.s[1] - g1) + E2.r[1]) + ((E3.s[1] - g1) + E3.r[1])));
      float D2 = 0.25f * ((E0.r[2] + ((E1.s[2] - g2) + E1.r[2])) + (((E2.s[2] - g2) + E2.r[2]) + ((E3.s[2] - g2) + E3.r[2])));
      // eps_t - eps*(IP) = (s_t - g) + r_t - D
      float dx = ((ga.s[0] - g0) + ga.r[0]) - D0, dy = ((ga.s[1] - g1) + ga.r[1]) - D1,
            dz = ((ga.s[2] - g2) + ga.r[2]) - D2;
      float wdv = gm.x;
      float ex = g0 + D0, ey = g1 + D1, ez = g2 + D2;
      self.add((ex * ex + ey * ey + ez * ez) * wdv);
      // error bound of q: the deviation (dx, dy, dz) is a difference of
      // quantities of size `scale`, each good to a few FP32 ulps, plus the
      // packed corrections; delta is 0.4 x that absolute deviation error
      float scale = fmaxf(fmaxf(fabsf(ga.s[0] - g0), fabsf(ga.s[1] - g1)), fabsf(ga.s[2] - g2)) +
                    fmaxf(fmaxf(fabsf(D0), fabsf(D1)), fabsf(D2));
      // (plus a floor for field values below FP32's range, which read as 0)
      const float delta = kBoundUlps * scale + kQuantRel * ga.gmax + 1e-30f;
      const float amax = fmaxf(fmaxf(fabsf(dx), fabsf(dy)), fabsf(dz));
      float qv, b;
      if (!(amax < 0x1p-40f)) {
        float err = (dx * dx + dy * dy + dz * dz) * wdv;
        // (sqrt err)^(6/5) = err^(3/5) = err r^2 and h_max (sqrt err)^(-2/5) =
        // h_max r, with r = err^(-1/5)
        float rr = inv_fifth_root(err);
        gsum.add(err > 0.f ? err * (rr * rr) : 0.f);  // (sqrt 0)^(6/5) = 0; q = +inf as in FP64
        qv = gm.y * rr;
        b = delta / sqrtf(dx * dx + dy * dy + dz * dz);
      } else if (amax > 0.f) {
        // a deviation this small (the field almost linear over the patch,
        // against the largest gradient) would underflow when squared: it is
        // scaled by 2^(5j) into [2^-5, 2) first, and err^(-1/5) = rs 2^(2j),
        // err^(3/5) = es rs^2 2^(-6j) with es, rs the scaled values
        const int j = (-fexp(amax)) / 5;  // 8 <= j <= 25
        const float up = pow2f(5 * j), dn3 = pow2f(-3 * j);
        const float sx = dx * up, sy = dy * up, sz = dz * up;
        const float es = (sx * sx + sy * sy + sz * sz) * wdv;
        const float rs = inv_fifth_root(es);
        gsum.add(es > 0.f ? ((es * (rs * rs)) * dn3) * dn3 : 0.f);
        qv = (gm.y * rs) * pow2f(2 * j);
        b = (delta * up) / sqrtf(sx * sx + sy * sy + sz * sz);
      } else {
        // a zero deviation (q = +inf) keeps a lower bound of q instead: the FP64
        // deviation is at most delta / 0.4, so q >= h_max (w dV (delta / 0.4)^2)^(-1/5)
        // (stored negated; delta scaled like a small deviation)
        const int j = delta < 0x1p-40f ? (-fexp(delta)) / 5 : 0;
        const float ds = (2.5f * delta) * pow2f(5 * j);
        qv = gm.y * __int_as_float(0x7f800000);
        b = -((gm.y * inv_fifth_root(wdv * ds * ds)) * pow2f(2 * j));
      }
      q[t] = make_float2(qv, b);
    }
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
  if (!done) return;
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();  // this block's partials before its arrival
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();  // every block's partials are visible to the last one
  __shared__ double shr[kBlock / 32];
  rd_size_factor(partials, gridDim.x, 0, adapt_ratio, 0.0, dim, out3, shr);
  __syncthreads();
  if (threadIdx.x == 0) {
    *done = 0;
    // The reference forms an IP gradient as sum u_i grad N_i in FP64, whose
    // rounding is about 2^-50 max|u| |J^-1|_F; 256 times that would give an
    // element error (2^-42 max|u| |J^-1|_F)^2 |det J| / 6 = 2^-84 / 6 max|u|^2
    // |cof|_F^2 / |det J|.  Over T elements the reference's rounding could
    // move its error integral G by up to T times the largest share
    // err^(3/5); at 1e-7 of G (the size factor's stated error), or for a G
    // that is zero or not finite, the pass is rounding-dominated (a constant
    // field, one offset far above its variation): 1 here, else 0.  (max|u|
    // from the prep kernel, the largest |cof|^2 / |det| once per mesh.)
    const double G = out3[1];
    const double um = (double)__int_as_float(*n_round);
    const double en = 0x1p-84 / 6.0 * um * um * __longlong_as_double((long long)*qmax);
    const double worst = (double)m.T * pow(en, 0.6);
    *n_round = (!(worst <= 1e-7 * G) || !(G > 0.0)) ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// average: size = size_factor * mean(q_t) over the vertex's elements
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_average(DevMesh m, const float2* __restrict__ q,
                                                         const double* __restrict__ out3, float2* __restrict__ sz2,
                                                         BatchView bv) {
  // kGroup lanes per vertex; each lane sums every kGroup-th entry with a
  // compensated sum, the lane sums are combined in a fixed order.  The
  // size's relative error bound is the q-weighted mean of the element
  // bounds (|d size| <= sf/n sum q_t b_t).
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = gid / kGroup, gl = gid % kGroup;
  int b = 0, e = 0;
  if (v < m.V) {
    b = m.a_off[v];
    e = m.a_off[v + 1];
  }
  PairSum s{0.f, 0.f};
  float qb = 0.f, bmax = 0.f, lo = 0.f;
  float2 x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    int k = b + gl + j * kGroup;
    x[j] = (k < e) ? __ldg(q + __ldg(m.a_el + k)) : make_float2(0.f, 0.f);
  }
  // element (q, b): b >= 0 a relative bound; b < 0 for q = +inf, -b a lower
  // bound of the FP64 q
  auto take = [&](float2 y) {
    s.add(y.x);
    if (y.y >= 0.f) {
      qb = fmaf(y.x, y.y, qb);
      bmax = fmaxf(bmax, y.y);
      lo += y.x * fmaxf(1.f - y.y, 0.f);
    } else {
      lo += -y.y;
    }
  };
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (b + gl + j * kGroup < e) take(x[j]);
  for (int k = b + gl + 8 * kGroup; k < e; k += kGroup) take(__ldg(q + __ldg(m.a_el + k)));  // > 16 elements
#pragma unroll
  for (int o = 1; o < kGroup; o <<= 1) {
    float oh = __shfl_xor_sync(0xffffffffu, s.h, o), ol = __shfl_xor_sync(0xffffffffu, s.l, o);
    float oq = __shfl_xor_sync(0xffffffffu, qb, o), ob = __shfl_xor_sync(0xffffffffu, bmax, o);
    const float olo = __shfl_xor_sync(0xffffffffu, lo, o);
    // combine the lower lane's pair first so every lane gets the same sum
    bool low = (gl & o) == 0;
    float ah = low ? s.h : oh, al = low ? s.l : ol, bh = low ? oh : s.h, bl = low ? ol : s.l;
    float t, err;
    two_sum(ah, bh, t, err);
    s.h = t;
    s.l = (al + bl) + err;
    qb = low ? qb + oq : oq + qb;
    lo = low ? lo + olo : olo + lo;
    bmax = fmaxf(bmax, ob);
  }
  if (v < m.V && gl == 0) {
    // an infinite q (zero element error) leaves +inf in the high part and NaN
    // in the compensation
    float tot = isfinite(s.h) ? s.h + s.l : s.h;
    const float sf = (float)batch_sf(bv, out3, v), inv_n = 1.f / (float)(e - b);
    float bound = qb / tot;
    if (!(bmax < 1e30f) || !(bound <= 1e30f)) bound = 3.0e38f;
    // an element with a zero deviation makes the size +inf (as FP64 does for
    // a zero error); its record then carries the negated lower bound of the
    // FP64 size
    if (!isfinite(tot)) bound = -(sf * (lo * inv_n) * (1.f - 1e-6f));
    sz2[v] = make_float2(sf * (tot * inv_n), bound);
  }
}

// ---------------------------------------------------------------------------
// measure: metric length with 2-point Gauss, h linearly interpolated
// ---------------------------------------------------------------------------
// four edges per thread (e, e + 32, e + 64, e + 96 within the warp's 128-edge chunk), all
// loads issued before use; the edge's half length is per-mesh data
__global__ void __launch_bounds__(kBlock) k_fast_measure(DevMesh m, const float* __restrict__ half_len,
                                                         const float2* __restrict__ sz2, uint32_t* __restrict__ split,
                                                         uint32_t* __restrict__ collapse, int* __restrict__ guard_items,
                                                         int* __restrict__ guard_count, int guard_cap,
                                                         float guard_rel) {
  const int lane = threadIdx.x & 31;
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int e0 = (int)(warp * 128) + lane;
  const int eids[4] = {e0, e0 + 32, e0 + 64, e0 + 96};
  int2 ab[4];
  float hl[4];
  float2 A[4], B[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    bool in = eids[i] < m.E;
    ab[i] = in ? __ldg(reinterpret_cast<const int2*>(m.edv) + eids[i]) : make_int2(0, 0);
    hl[i] = in ? __ldg(half_len + eids[i]) : 0.f;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    A[i] = __ldg(sz2 + ab[i].x);
    B[i] = __ldg(sz2 + ab[i].y);
  }
  const float gp = 0.577350269189626f;
  const float n0 = 0.5f * (1.f - gp), n1 = 0.5f * (1.f + gp);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    bool s = false, c = false;
    const int e = eids[i];
    if (e < m.E) {
      // 2-point Gauss: h(xi) interpolated linearly between the end sizes
      float L = hl[i] * (1.f / (n0 * A[i].x + n1 * B[i].x) + 1.f / (n1 * A[i].x + n0 * B[i].x));
      s = L > 1.5f;
      c = L < 0.5f;
      // guard band: the interval of the FP64 length from the ends' size
      // intervals (relative bounds, or a lower bound for an infinite size),
      // widened by guard_rel for the FP32 length itself
      bool near;
      if (A[i].y >= 0.f && B[i].y >= 0.f) {
        // finite ends: L moves by at most guard_rel + b_a + b_b relative
        const float band = guard_rel + A[i].y + B[i].y;
        near = fabsf(L - 1.5f) <= band * 1.5f || fabsf(L - 0.5f) <= band * 0.5f;
        if (near && L < 0.5f) {
          // a short edge stays a collapse unless the upper end of its length,
          // from the ends' size lower bounds, reaches 0.5.  An element's
          // bound b is 0.4 times its deviation's relative error, so q is at
          // least q (1 + 2.5 b)^(-2/5), and by convexity (Jensen) a vertex
          // size at least size (1 + 2.5 b_v)^(-2/5) with b_v its q-weighted
          // mean bound: far tighter than the linear band where flat fields
          // make b large (margin 1e-6 for this arithmetic and the size factor)
          const float alo = A[i].x * (powf(1.f + 2.5f * A[i].y, -0.4f) * (1.f - 1e-6f));
          const float blo = B[i].x * (powf(1.f + 2.5f * B[i].y, -0.4f) * (1.f - 1e-6f));
          const float Lhi = hl[i] * (1.f / (n0 * alo + n1 * blo) + 1.f / (n1 * alo + n0 * blo)) * (1.f + guard_rel);
          near = !(Lhi < 0.5f);
        }
      } else {
        // an infinite end: the upper end of L from the sizes' lower bounds
        const float alo = A[i].y >= 0.f ? A[i].x * fmaxf(1.f - A[i].y, 0.f) : -A[i].y;
        const float blo = B[i].y >= 0.f ? B[i].x * fmaxf(1.f - B[i].y, 0.f) : -B[i].y;
        const float Lhi = hl[i] * (1.f / (n0 * alo + n1 * blo) + 1.f / (n1 * alo + n0 * blo)) * (1.f + guard_rel);
        near = !(Lhi < 0.5f);  // the FP32 length is 0 here: only a collapse can be in doubt
      }
      if (near || !(L == L)) {
        int slot = atomicAdd(guard_count, 1);
        if (slot < guard_cap) guard_items[slot] = e;
      }
    }
    unsigned bs = __ballot_sync(0xffffffffu, s), bc = __ballot_sync(0xffffffffu, c);
    if (lane == 0 && e < m.E) {
      split[e >> 5] = bs;
      collapse[e >> 5] = bc;
    }
  }
}

__global__ void k_size_to_f64(int V, const float2* __restrict__ s32, double* __restrict__ s64) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < V) s64[v] = (double)s32[v].x;
}

inline int nblk(long n, int b = kBlock) { return (int)((n + b - 1) / b); }

// the error kernel runs one full wave: resident blocks per SM x SMs
int error_grid() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fast_error, kBlock, 0);
    grid = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 4);
  }
  return grid;
}

// the tet kernel runs one full wave of resident blocks as well
int tet_grid(int T) {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fast_tet, kBlock, 0);
    grid = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 5);
  }
  const int nb = (int)((T + (long)kTetChunk * kBlock - 1) / ((long)kTetChunk * kBlock));
  return nb < grid ? nb : grid;
}

}  // namespace

int fast_error_blocks(int T) {
  int nb = nblk(T), g = error_grid();
  return nb < g ? nb : g;
}

void fast_prep_coords(const DevMesh& m, const double* frame, float4* vrec, cudaStream_t s) {
  if (m.V) k_prep_coords<<<nblk(m.V), kBlock, 0, s>>>(m.V, m.xyz, frame[0], frame[1], frame[2], frame[3], vrec);
}

void fast_geometry(const DevMesh& m, float2* geo, double2* geo64, double* cent, unsigned long long* qmax,
                   float* half_len, cudaStream_t s) {
  cudaMemsetAsync(qmax, 0, sizeof(unsigned long long), s);
  if (m.T) k_fast_geo<<<nblk(m.T), kBlock, 0, s>>>(m, geo, geo64, cent, qmax);
  if (m.E) k_fast_elen<<<nblk(m.E), kBlock, 0, s>>>(m, half_len);
}

void fast_prep(const DevMesh& m, const double* u, const float4* crec, float4* vrec, int* umax_bits, cudaStream_t s) {
  if (m.V) k_prep<<<nblk(m.V), kBlock, 0, s>>>(m.V, u, crec, vrec, umax_bits);
}

void fast_tet(const DevMesh& m, const float4* vrec, const double* u, float gscale, uint4* td, int* next_chunk,
              cudaStream_t s) {
  if (!m.T) return;
  cudaMemsetAsync(next_chunk, 0, sizeof(int), s);
  k_fast_tet<<<tet_grid(m.T), kBlock, 0, s>>>(m, vrec, u, gscale, td, next_chunk);
}

void fast_weights(const DevMesh& m, const double* cent, float* w, double* w64, ExpandList xl, int* n_refit,
                  unsigned char* listed, cudaStream_t s) {
  if (m.V) k_fast_weights<<<nblk(m.V), kBlock, 0, s>>>(m, cent, w, w64, xl, n_refit, listed);
}


void fast_patch_class(const DevMesh& m, const unsigned char* listed, unsigned char* cls, cudaStream_t s) {
  if (m.V) k_patch_class<<<nblk(m.V), kBlock, 0, s>>>(m, listed, cls);
}

int fast_bin_blocks(int V) { return (V + kBinBlock - 1) / kBinBlock; }

void fast_bin_count(int V, const unsigned char* cls, int* counts, cudaStream_t s) {
  if (V) k_bin_count<<<fast_bin_blocks(V), kBinBlock, 0, s>>>(V, cls, counts);
}

void fast_bin_scatter(int V, const unsigned char* cls, const int* offs, int* order, cudaStream_t s) {
  if (V) k_bin_scatter<<<fast_bin_blocks(V), kBinBlock, 0, s>>>(V, cls, offs, order);
}

void fast_recover_tiles(const DevMesh& m, const float* w, SlicedPatches sp, const uint4* td, float4* rec,
                        const int* verts, const int4* tiles, int n_tiles, int mode, int* next, int grid,
                        cudaStream_t s) {
  cudaMemsetAsync(next, 0, sizeof(int), s);
  if (!n_tiles) return;
  switch (mode) {
    case 0: k_fast_recover_tiles<0><<<grid, kBlock, 0, s>>>(m, w, sp, td, rec, verts, tiles, n_tiles, next); break;
    case 1: k_fast_recover_tiles<1><<<grid, kBlock, 0, s>>>(m, w, sp, td, rec, verts, tiles, n_tiles, next); break;
    case 2: k_fast_recover_tiles<2><<<grid, kBlock, 0, s>>>(m, w, sp, td, rec, verts, tiles, n_tiles, next); break;
    case 4: k_fast_recover_tiles<4><<<grid, kBlock, 0, s>>>(m, w, sp, td, rec, verts, tiles, n_tiles, next); break;
    default: k_fast_recover_tiles<-1><<<grid, kBlock, 0, s>>>(m, w, sp, td, rec, verts, tiles, n_tiles, next);
  }
}

void fast_slice_width(const DevMesh& m, const BinSlices& bs, const int* verts, int* width, cudaStream_t s) {
  if (bs.slice0[4]) k_slice_width<<<nblk(bs.slice0[4]), kBlock, 0, s>>>(m, bs, verts, width);
}

void fast_slice_fill(const DevMesh& m, const BinSlices& bs, const int* verts, const float* w, const int* off,
                     int* sel, float* sw, cudaStream_t s) {
  if (bs.start[4]) k_slice_fill<<<nblk(bs.start[4]), kBlock, 0, s>>>(m, bs, verts, w, off, sel, sw);
}

void fast_merge_ref(ExpandList xl, const double* rec64, float4* rec, cudaStream_t s) {
  k_merge_ref<<<152, 256, 0, s>>>(xl.items, xl.count, xl.cap, rec64, rec);
}

void fast_error(const DevMesh& m, const uint4* td, const float2* geo, const float4* rec, float2* q, double* partials,
                int nb, const int2* seg, unsigned* done, double adapt_ratio, double* out3, int* n_round,
                const unsigned long long* qmax, cudaStream_t s) {
  if (nb)
    k_fast_error<<<nb, kBlock, 0, s>>>(m, td, geo, rec, q, partials, seg, done, adapt_ratio, m.dim, out3, n_round,
                                       qmax);
}

void fast_average(const DevMesh& m, const float2* q, const double* out3, float2* sz2, BatchView bv, cudaStream_t s) {
  if (m.V) k_fast_average<<<nblk((long)m.V * kGroup), kBlock, 0, s>>>(m, q, out3, sz2, bv);
}

void fast_measure(const DevMesh& m, const float* half_len, const float2* sz2, uint32_t* split, uint32_t* collapse,
                  int* guard_items, int* guard_count, int guard_cap, float guard_rel, cudaStream_t s) {
  if (m.E)
    k_fast_measure<<<nblk((m.E + 3) / 4), kBlock, 0, s>>>(m, half_len, sz2, split, collapse, guard_items, guard_count,
                                                          guard_cap, guard_rel);
}

void fast_size_to_f64(int V, const float2* sz2, double* s64, cudaStream_t s) {
  if (V) k_size_to_f64<<<nblk(V), kBlock, 0, s>>>(V, sz2, s64);
}

}  // namespace sprg
