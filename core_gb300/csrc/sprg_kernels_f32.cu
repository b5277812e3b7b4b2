// FP32 fast path of the estimate-and-mark pass (3D tets, scalar field).
//
// Data: every vertex is one 32-byte record {x_hi, y_hi, z_hi, u_hi, x_lo,
// y_lo, z_lo, u_lo} (an unevaluated float pair per FP64 value), so a vertex
// gather is one DRAM sector and differences of nearby coordinates or field
// values, (a_hi - b_hi) + (a_lo - b_lo), keep ~FP32 relative accuracy of the
// difference itself.  All arithmetic is FP32 except the two global integrals
// (FP64 block partials).
//
// Phases (one kernel each):
//   A  fast_recover   thread per vertex: gradient of each patch tet, FP32
//                     normal equations on centred, scaled coordinates with the
//                     data shifted by the first sample; 4x4 Cholesky; patches
//                     with a condition estimate > 1e6, too few points or a
//                     zero pivot go to the FP64 reference path (growth + QR).
//   B  fast_error     thread per tet: element error, SelfProduct and Error
//                     terms (FP64 partials), and q_t = h_max * err^(-1/5).
//   C  fast_average   thread per vertex: size = size_factor * mean(q_t).
//   D  fast_measure   thread per edge: metric length, split/collapse bitmap.
#include "sprg_fast.h"

namespace sprg {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

// double-float difference a - b of the packed records (xyz and u)
__device__ __forceinline__ float4 diff(const float4& ah, const float4& al, const float4& bh, const float4& bl) {
  return make_float4((ah.x - bh.x) + (al.x - bl.x), (ah.y - bh.y) + (al.y - bl.y), (ah.z - bh.z) + (al.z - bl.z),
                     (ah.w - bh.w) + (al.w - bl.w));
}

struct TetGeom {
  float g[3];   // gradient of u (the integration-point value)
  float det;    // det J = 6 * volume
};

// Gradient of the linear interpolant from the three edge vectors e1..e3
// (x_i - x_0) and field differences du_i: solve J g = du with J rows e_i.
__device__ __forceinline__ TetGeom tet_grad(const float4& e1, const float4& e2, const float4& e3) {
  // cofactors of J (rows e1, e2, e3)
  float c00 = e2.y * e3.z - e2.z * e3.y;
  float c01 = e2.z * e3.x - e2.x * e3.z;
  float c02 = e2.x * e3.y - e2.y * e3.x;
  float c10 = e3.y * e1.z - e3.z * e1.y;
  float c11 = e3.z * e1.x - e3.x * e1.z;
  float c12 = e3.x * e1.y - e3.y * e1.x;
  float c20 = e1.y * e2.z - e1.z * e2.y;
  float c21 = e1.z * e2.x - e1.x * e2.z;
  float c22 = e1.x * e2.y - e1.y * e2.x;
  float det = e1.x * c00 + e1.y * c01 + e1.z * c02;
  float inv = 1.0f / det;
  TetGeom t;
  // g = J^{-1} du, J^{-1} = C^T / det with C the cofactor matrix
  t.g[0] = (c00 * e1.w + c10 * e2.w + c20 * e3.w) * inv;
  t.g[1] = (c01 * e1.w + c11 * e2.w + c21 * e3.w) * inv;
  t.g[2] = (c02 * e1.w + c12 * e2.w + c22 * e3.w) * inv;
  t.det = det;
  return t;
}

__device__ __forceinline__ float len3(const float4& a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }

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

// ---------------------------------------------------------------------------
// Phase A
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_recover(DevMesh m, const float4* __restrict__ vr,
                                                         float4* __restrict__ rec32, ExpandList xl,
                                                         int* __restrict__ n_refit) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  const int beg = m.p_off[v], end = m.p_off[v + 1];
  const int cnt = end - beg;
  bool to_ref = cnt < 4;
  float4 vh = ld4(vr + 2 * (size_t)v), vl = ld4(vr + 2 * (size_t)v + 1);
  // normal equations of [1, sx, sy, sz] with data b - b0
  float a00 = 0, a01 = 0, a02 = 0, a03 = 0, a11 = 0, a12 = 0, a13 = 0, a22 = 0, a23 = 0, a33 = 0;
  float r0[3] = {0, 0, 0}, r1[3] = {0, 0, 0}, r2[3] = {0, 0, 0}, r3[3] = {0, 0, 0};
  float b0[3] = {0, 0, 0};
  float inv_h = 0.f;
  if (!to_ref) {
    for (int k = beg; k < end; ++k) {
      int t = m.p_el[k];
      int4 tv = __ldg(reinterpret_cast<const int4*>(m.ev) + t);
      float4 d[4];
      int vid[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        if (vid[a] == v) {
          d[a] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
          float4 h = ld4(vr + 2 * (size_t)vid[a]), l = ld4(vr + 2 * (size_t)vid[a] + 1);
          d[a] = diff(h, l, vh, vl);
        }
      }
      float4 e1 = make_float4(d[1].x - d[0].x, d[1].y - d[0].y, d[1].z - d[0].z, d[1].w - d[0].w);
      float4 e2 = make_float4(d[2].x - d[0].x, d[2].y - d[0].y, d[2].z - d[0].z, d[2].w - d[0].w);
      float4 e3 = make_float4(d[3].x - d[0].x, d[3].y - d[0].y, d[3].z - d[0].z, d[3].w - d[0].w);
      TetGeom tg = tet_grad(e1, e2, e3);
      // integration point relative to v
      float cx = 0.25f * (d[0].x + d[1].x + d[2].x + d[3].x);
      float cy = 0.25f * (d[0].y + d[1].y + d[2].y + d[3].y);
      float cz = 0.25f * (d[0].z + d[1].z + d[2].z + d[3].z);
      if (k == beg) {
        inv_h = 1.0f / fmaxf(fmaxf(len3(e1), len3(e2)), len3(e3));
        b0[0] = tg.g[0]; b0[1] = tg.g[1]; b0[2] = tg.g[2];
      }
      float sx = cx * inv_h, sy = cy * inv_h, sz = cz * inv_h;
      a00 += 1.f; a01 += sx; a02 += sy; a03 += sz;
      a11 += sx * sx; a12 += sx * sy; a13 += sx * sz;
      a22 += sy * sy; a23 += sy * sz; a33 += sz * sz;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float b = tg.g[c] - b0[c];
        r0[c] += b; r1[c] += sx * b; r2[c] += sy * b; r3[c] += sz * b;
      }
    }
    // Cholesky of the 4x4 normal matrix
    float l00 = sqrtf(a00);
    float l10 = a01 / l00, l20 = a02 / l00, l30 = a03 / l00;
    float d1 = a11 - l10 * l10;
    float d1min = d1;
    float l11 = sqrtf(fmaxf(d1, 0.f));
    float l21 = (a12 - l20 * l10) / l11, l31 = (a13 - l30 * l10) / l11;
    float d2 = a22 - l20 * l20 - l21 * l21;
    float l22 = sqrtf(fmaxf(d2, 0.f));
    float l32 = (a23 - l30 * l20 - l31 * l21) / l22;
    float d3 = a33 - l30 * l30 - l31 * l31 - l32 * l32;
    float l33 = sqrtf(fmaxf(d3, 0.f));
    float pmin = fminf(fminf(d1min, d2), fminf(d3, a00));
    float pmax = fmaxf(fmaxf(d1, d2), fmaxf(d3, a00));
    // condition estimate of the normal matrix from the pivots
    to_ref = !(pmin > 0.f) || !(pmax <= 1e6f * pmin);
    if (!to_ref) {
      float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
      float o[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        // forward then backward substitution; only the constant term is needed
        float y0 = r0[c] / l00;
        float y1 = (r1[c] - l10 * y0) / l11;
        float y2 = (r2[c] - l20 * y0 - l21 * y1) / l22;
        float y3 = (r3[c] - l30 * y0 - l31 * y1 - l32 * y2) / l33;
        float x3 = y3 / l33;
        float x2 = (y2 - l32 * x3) / l22;
        float x1 = (y1 - l21 * x2 - l31 * x3) / l11;
        float x0 = (y0 - l10 * x1 - l20 * x2 - l30 * x3) / l00;
        o[c] = b0[c] + x0;
      }
      out.x = o[0]; out.y = o[1]; out.z = o[2];
      rec32[v] = out;
      return;
    }
  }
  // FP64 reference path for this vertex (growth if needed)
  int slot = atomicAdd(xl.count, 1);
  if (slot < xl.cap) xl.items[slot] = v;
  if (cnt >= 4) atomicAdd(n_refit, 1);
}

// ---------------------------------------------------------------------------
// Phase B
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_sum_d(double x, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = x;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
  return t;
}

__global__ void __launch_bounds__(kBlock) k_fast_error(DevMesh m, const float4* __restrict__ vr,
                                                       const float4* __restrict__ rec32, float* __restrict__ q,
                                                       double* __restrict__ partials) {
  __shared__ double sh[kBlock / 32];
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  double self_term = 0, g_term = 0;
  if (t < m.T) {
    int4 tv = __ldg(reinterpret_cast<const int4*>(m.ev) + t);
    float4 h0 = ld4(vr + 2 * (size_t)tv.x), l0 = ld4(vr + 2 * (size_t)tv.x + 1);
    float4 h1 = ld4(vr + 2 * (size_t)tv.y), l1 = ld4(vr + 2 * (size_t)tv.y + 1);
    float4 h2 = ld4(vr + 2 * (size_t)tv.z), l2 = ld4(vr + 2 * (size_t)tv.z + 1);
    float4 h3 = ld4(vr + 2 * (size_t)tv.w), l3 = ld4(vr + 2 * (size_t)tv.w + 1);
    float4 e1 = diff(h1, l1, h0, l0), e2 = diff(h2, l2, h0, l0), e3 = diff(h3, l3, h0, l0);
    TetGeom tg = tet_grad(e1, e2, e3);
    float4 s0 = ld4(rec32 + tv.x), s1 = ld4(rec32 + tv.y), s2 = ld4(rec32 + tv.z), s3 = ld4(rec32 + tv.w);
    float ex = 0.25f * ((s0.x + s1.x) + (s2.x + s3.x));
    float ey = 0.25f * ((s0.y + s1.y) + (s2.y + s3.y));
    float ez = 0.25f * ((s0.z + s1.z) + (s2.z + s3.z));
    float wdv = tg.det * (1.0f / 6.0f);
    float dx = tg.g[0] - ex, dy = tg.g[1] - ey, dz = tg.g[2] - ez;
    float err = (dx * dx + dy * dy + dz * dz) * wdv;
    self_term = (double)((ex * ex + ey * ey + ez * ez) * wdv);
    // (sqrt err)^(6/5) = err^(3/5); h_max * (sqrt err)^(-2/5) = h_max * err^(-1/5)
    g_term = (double)powf(err, 0.6f);
    float4 e4 = diff(h2, l2, h1, l1), e5 = diff(h3, l3, h1, l1), e6 = diff(h3, l3, h2, l2);
    float hm = fmaxf(fmaxf(fmaxf(len3(e1), len3(e2)), fmaxf(len3(e3), len3(e4))), fmaxf(len3(e5), len3(e6)));
    q[t] = hm * powf(err, -0.2f);
  }
  double s1 = block_sum_d(self_term, sh);
  double s2 = block_sum_d(g_term, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = s1;
    partials[2 * blockIdx.x + 1] = s2;
  }
}

// elements of the FP64-refit patches use the FP64 recovered values
__global__ void k_merge_ref(const int* __restrict__ items, const int* __restrict__ count, int cap,
                            const double* __restrict__ rec64, float4* __restrict__ rec32) {
  int n = min(*count, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int v = items[i];
    rec32[v] = make_float4((float)rec64[3 * (size_t)v], (float)rec64[3 * (size_t)v + 1],
                           (float)rec64[3 * (size_t)v + 2], 0.f);
  }
}

// ---------------------------------------------------------------------------
// Phase C
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_average(DevMesh m, const float* __restrict__ q,
                                                         const double* __restrict__ out3, float* __restrict__ size32) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.V) return;
  int b = m.a_off[v], e = m.a_off[v + 1];
  float s = 0.f;
  for (int k = b; k < e; ++k) s += __ldg(q + m.a_el[k]);
  size32[v] = (float)out3[2] * (s / (float)(e - b));
}

// ---------------------------------------------------------------------------
// Phase D: metric length with 2-point Gauss, h linearly interpolated
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_fast_measure(DevMesh m, const float4* __restrict__ vr,
                                                         const float* __restrict__ size32, uint32_t* __restrict__ split,
                                                         uint32_t* __restrict__ collapse, float* __restrict__ L32,
                                                         int* __restrict__ guard_items, int* __restrict__ guard_count,
                                                         int guard_cap, float guard_rel) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  bool s = false, c = false;
  if (e < m.E) {
    int2 ab = __ldg(reinterpret_cast<const int2*>(m.edv) + e);
    float4 ha = ld4(vr + 2 * (size_t)ab.x), la = ld4(vr + 2 * (size_t)ab.x + 1);
    float4 hb = ld4(vr + 2 * (size_t)ab.y), lb = ld4(vr + 2 * (size_t)ab.y + 1);
    float4 d = diff(hb, lb, ha, la);
    float half = 0.5f * len3(d);
    float s0 = __ldg(size32 + ab.x), s1 = __ldg(size32 + ab.y);
    const float gp = 0.577350269189626f;
    float n0 = 0.5f * (1.f - gp), n1 = 0.5f * (1.f + gp);
    float L = half * (1.f / (n0 * s0 + n1 * s1) + 1.f / (n1 * s0 + n0 * s1));
    s = L > 1.5f;
    c = L < 0.5f;
    if (L32) L32[e] = L;
    if (guard_items && (fabsf(L - 1.5f) < guard_rel * 1.5f || fabsf(L - 0.5f) < guard_rel * 0.5f)) {
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

}  // namespace

int fast_error_blocks(int T) { return nblk(T); }

void fast_prep(const DevMesh& m, const double* u, float4* vrec, cudaStream_t s) {
  if (m.V) k_prep<<<nblk(m.V), kBlock, 0, s>>>(m.V, m.xyz, u, vrec);
}

void fast_recover(const DevMesh& m, const float4* vrec, float4* rec32, ExpandList xl, int* n_refit, cudaStream_t s) {
  if (m.V) k_fast_recover<<<nblk(m.V), kBlock, 0, s>>>(m, vrec, rec32, xl, n_refit);
}

void fast_merge_ref(ExpandList xl, const double* rec64, float4* rec32, cudaStream_t s) {
  k_merge_ref<<<152, 256, 0, s>>>(xl.items, xl.count, xl.cap, rec64, rec32);
}

void fast_error(const DevMesh& m, const float4* vrec, const float4* rec32, float* q, double* partials, int nb,
                cudaStream_t s) {
  if (nb) k_fast_error<<<nb, kBlock, 0, s>>>(m, vrec, rec32, q, partials);
}

void fast_average(const DevMesh& m, const float* q, const double* out3, float* size32, cudaStream_t s) {
  if (m.V) k_fast_average<<<nblk(m.V), kBlock, 0, s>>>(m, q, out3, size32);
}

void fast_measure(const DevMesh& m, const float4* vrec, const float* size32, uint32_t* split, uint32_t* collapse,
                  float* L32, int* guard_items, int* guard_count, int guard_cap, float guard_rel, cudaStream_t s) {
  if (m.E)
    k_fast_measure<<<nblk(m.E), kBlock, 0, s>>>(m, vrec, size32, split, collapse, L32, guard_items, guard_count,
                                                guard_cap, guard_rel);
}

void fast_size_to_f64(int V, const float* s32, double* s64, cudaStream_t s) {
  if (V) k_size_to_f64<<<nblk(V), kBlock, 0, s>>>(V, s32, s64);
}

}  // namespace sprg
