// Internal declarations shared by the CUDA translation units of the
// estimate-and-mark library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "spr_gb300.h"

namespace sprg {

// Device view of the flattened mesh.  All index arrays are int32.
struct DevMesh {
  int dim;             // 2 or 3
  int nn;              // vertices per element (dim + 1)
  int ne_el;           // edges per element (3 or 6)
  int V, T, E;
  const double* xyz;   // V x 3 (FP64 master copy)
  const int* xyzq;     // V x 4 (X, Y, Z, 0): 32-bit fixed point on the frame, the learned form's records
  const int* ev;       // T x nn  (getDownward(e,0) order)
  const int* edv;      // E x 2
  const int* p_off;    // V + 1, patch CSR: elements of each vertex, ascending
  const int* p_el;
  const int* a_off;    // V + 1, averaging CSR (reference getAdjacent order)
  const int* a_el;
};

// A batch of independent meshes flattened into one context (disjoint union,
// entity ids offset per mesh).  n = 0: a single mesh.  Per mesh k:
// vertices [voff[k], voff[k+1]); error-kernel segments [segoff[k],
// segoff[k+1]) of seg (element ranges that never cross a mesh); the size
// factor of mesh k at out3[4 k + 2].
struct BatchView {
  int n;
  const int* voff;
  const int2* seg;
  const int* segoff;
  const double* ratios;
};

// mesh of vertex v (binary search over the vertex offsets)
__device__ __forceinline__ int batch_mesh(const BatchView& b, int v) {
  int lo = 0, hi = b.n;  // voff[lo] <= v < voff[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(b.voff + mid) <= v) lo = mid;
    else hi = mid;
  }
  return lo;
}

// the size factor that applies at vertex v
__device__ __forceinline__ double batch_sf(const BatchView& b, const double* out3, int v) {
  return b.n ? out3[4 * batch_mesh(b, v) + 2] : out3[2];
}

// Device status word written by kernels (first error wins).
struct DevStatus {
  int code;        // SPRG_OK or SPRG_E*
  int where;       // entity index that raised it
};

// Expansion work list for patches that need growth or are too large for the
// register path.
struct ExpandList {
  int* items;   // vertex ids
  int* count;   // device counter
  int cap;
};

// ---- kernel launchers (sprg_kernels_f64.cu) ---------------------------
void launch_grad_ip_f64(const DevMesh& m, const double* f, int ncin, double* ip, cudaStream_t s);
// Triangles (tets recover through launch_qr_weights / launch_recover_w64):
// xl: patches that need growth; big: patches above the thread-per-vertex
// size (fitted by the warp path inside this call; its counter must be zero
// on entry)
void launch_recover_f64(const DevMesh& m, const double* ip, int nc, double* rec, ExpandList xl, ExpandList big,
                        DevStatus* st, cudaStream_t s);
// Patches on the expansion list: grow as the reference does, then fit.
// The list length is read on the device (no host round trip).
// slab: expand_grid() * expand_max_elems() * (4 + nc + 1) doubles.
// ip may be NULL: the element gradients of u are computed in place (nc 3:
// u scalar; nc 9: u a VECTOR field, V x 3) -- for the forms that keep no ip
// field.
// cache_* (optional): record each listed vertex's final element set
// (expand_max_elems() ints per list slot) for launch_cached_fit_f64.
void launch_expand_f64(const DevMesh& m, const double* ip, const double* u, int nc, double* rec, ExpandList xl,
                       double* slab, DevStatus* st, cudaStream_t s, int* cache_v = nullptr, int* cache_n = nullptr,
                       int* cache_el = nullptr);
// One QR fit per cached listed vertex (patch growth depends on geometry only).
void launch_cached_fit_f64(const DevMesh& m, const double* ip, const double* u, int nc, double* rec, int n_cached,
                           const int* cache_v, const int* cache_n, const int* cache_el, double* slab, DevStatus* st,
                           cudaStream_t s);
// Tets: per-mesh weights of the cached patches (w = Q1 R^-T t from the fit's
// QR; woff: each patch's offset into w, wn: its size or -1 where the rank
// test fails) and the per-pass weighted sums that replace the fits
void launch_cached_weights_f64(const DevMesh& m, int n_cached, const int* cache_v, const int* cache_n,
                               const int* cache_el, const long long* woff, double* w, int* wn, double* slab,
                               cudaStream_t s);
void launch_cached_wsum_f64(const DevMesh& m, const double* ip, const double* u, int nc, double* rec, int n_cached,
                            const int* cache_v, const int* cache_el, const long long* woff, const double* w,
                            const int* wn, DevStatus* st, cudaStream_t s);
int expand_max_elems();
int expand_grid();
// Per-element error terms + deterministic block partials (2 per block).
void launch_error_f64(const DevMesh& m, const double* ip, int nc, const double* rec, double* err,
                      double* partials, int n_blocks, double g_exponent, cudaStream_t s);
int error_blocks(int T);
// Sum partials in fixed order, compute size factor.  mode 0: SPR; 1: target.
void launch_size_factor(const double* partials, int n_blocks, int mode, double adapt_ratio, double target,
                        int dim, double* out3, cudaStream_t s);
void launch_esize_f64(const DevMesh& m, const double* err, const double* out3, int mode, double alpha,
                      double beta, double* esize, cudaStream_t s);
void launch_average(const DevMesh& m, const double* esize, double* size, cudaStream_t s);
void launch_measure_iso_f64(const DevMesh& m, const double* size, double* L, cudaStream_t s);
void launch_measure_aniso_f64(const DevMesh& m, const double* sizes, const double* frames, double* L,
                              cudaStream_t s);
void launch_mark(int E, const double* L, int which, int* flags, unsigned long long* count, DevStatus* st,
                 cudaStream_t s);
// predicate bitmaps: bit e of split = L[e] > 1.5, of collapse = L[e] < 0.5
void launch_mark_bits(int E, const double* L, uint32_t* split, uint32_t* collapse, cudaStream_t s);
// markEntities semantics from a predicate bitmap
void launch_apply_bits(int E, const uint32_t* bits, int which, int* flags, unsigned long long* count,
                       DevStatus* st, cudaStream_t s);
// the collapse and split passes in one sweep (counts[0] split, counts[1] collapse)
// skip (device int, or null): when nonzero the flags stay unchanged
void launch_apply_marks(int E, const uint32_t* split_bits, const uint32_t* collapse_bits, int* flags,
                        unsigned long long* counts, DevStatus* st, const int* skip, cudaStream_t s);
// MA sweeps around the marks.  kind: 0 identity size field, 1 isotropic
// (size), 2 anisotropic (sizes, frames), 3 log-interpolated anisotropic
// (logm); pairs: n x 2 vertex ids, or NULL for the mesh's edges (n = E);
// st records SPRG_EEIGEN when an eigen iteration fails
void launch_measure_pairs(const DevMesh& m, int kind, long long n, const int* pairs, const double* size,
                          const double* sizes, const double* frames, const double* logm, double* L, DevStatus* st,
                          cudaStream_t s);
// LogAnisoSizeField: per-vertex log-metric (V x 9) of sizes and frames; kind
// 3 of launch_measure_pairs and the logm argument of launch_quality_f64 read it
void launch_log_metric(int V, const double* sizes, const double* frames, double* logm, cudaStream_t s);
// *out = bits of max(0, the positive values of x) (NaN ignored)
void launch_max_positive(long long n, const double* x, unsigned long long* out, cudaStream_t s);
// deterministic sum: partials holds sum_partials_count() doubles
int sum_partials_count();
void launch_sum(long long n, const double* x, double* partials, double* out, cudaStream_t s);
// first index (in *first, all ones if none) holding the minimum of the
// values below `start`; *key is scratch
void launch_first_min_below(long long n, const double* x, double start, unsigned long long* key,
                            unsigned long long* first, cudaStream_t s);
void launch_mark_quality(int T, const double* q, double good, int* flags, unsigned long long* count, DevStatus* st,
                         cudaStream_t s);
// Mixed-precision anisotropic pass.  Triangle patch weights (FP64, patch
// CSR layout) with the listed vertices (weights not covering them) in lst;
// FP32 metric records (12 floats per
// vertex: h, frame) and quality records (FP32 vertex transforms and
// determinants; ambiguous choices that matter are decided in FP64);
// FP32 edge measure writing the mark bitmaps and the
// edges within their error bound of 0.5 / 1.5 (guard); the guard's FP64
// re-measure fixing those bits; FP32 qualities.
void launch_tri_weights(const DevMesh& m, double* w, unsigned char* listed, ExpandList lst, cudaStream_t s);
// qrec: quality_rec_bytes() per vertex
void launch_metric_f32(int V, int dim, const double* sizes, const double* frames, float* out, void* qrec,
                       cudaStream_t s);
int quality_rec_bytes();
// crec: the FP32 path's coordinate records in the frame x' = (x - c) s + 1
// (frame_scale = s)
void launch_measure_aniso_f32(const DevMesh& m, const float* met, const float4* crec, double frame_scale,
                              uint32_t* split, uint32_t* collapse, int* guard, int* gcount, int gcap, cudaStream_t s);
// sizes / frames: the FP64 metric, or null to rebuild the guarded edges'
// ends from the Hessian H (hessian_metric_vertex, the FP64 pass's bits)
void launch_measure_guard_f64(const DevMesh& m, const double* sizes, const double* frames, const double* H,
                              double eps, double hmin, double hmax, const int* guard, const int* gcount, int gcap,
                              uint32_t* split, uint32_t* collapse, cudaStream_t s);
// sizes / frames as for the guard (the FP64 determinants of tie-breaks)
// two launches: FP32 qualities (listing the elements whose vertex pick the
// FP32 determinants leave open), then the FP64 tie-breaks; cj64: V doubles,
// tie_items: T ints, tie_count: one int (scratch, cleared here)
void launch_quality_aniso_f32(const DevMesh& m, const void* qrec, const float4* crec, double frame_scale,
                              const double* sizes, const double* frames, const double* H, double eps, double hmin,
                              double hmax, double* cj64, int* tie_items, int* tie_count, double* q, cudaStream_t s);
// triangles: FP32 metric records (12 floats) and quality records straight
// from the Hessian (FP64 decisions, FP32 magnitudes)
void launch_metric_mixed2d(int V, const double* H, double eps, double hmin, double hmax, float* out, void* qrec,
                           cudaStream_t s);
// Triangle recovery-of-gradient operator (per mesh, FP64): K_va over the
// patch vertices, tri_operator_slots() slots per vertex (kidx ints, kval 3
// doubles each, klen counts; patches that are not fans are added to the
// listed set); applied to a scalar (ncin 1 -> V x 3) or a
// VECTOR field (ncin 3 -> V x 9) at the covered (not listed) vertices
int tri_operator_slots();
// kc: components per operator slot, 3, or 2 for a mesh in the z = 0 plane
void launch_tri_operator(const DevMesh& m, int kc, const double* w, unsigned char* listed, ExpandList lst, int* kidx,
                         double* kval, int* klen, cudaStream_t s);
void launch_apply_operator(int V, int ncin, int kc, const unsigned char* listed, const int* kidx, const double* kval,
                           const int* klen, const double* f, double* out, cudaStream_t s);
// incremental mesh update: dst[ids[r] * width + j] = vals[r * width + j];
// the coordinates' bounding box as order keys (3 minima, 3 maxima)
void launch_scatter_rows_f64(long long n, int width, const int* ids, const double* vals, double* dst, cudaStream_t s);
void launch_scatter_rows_i32(long long n, int width, const int* ids, const int* vals, int* dst, cudaStream_t s);
void launch_bbox(int V, const double* xyz, unsigned long long* keys, cudaStream_t s);
// *bad += the number of entries of a outside [0, limit)
void launch_count_out_of_range(long long n, const int* a, int limit, unsigned long long* bad, cudaStream_t s);
double key_to_double(unsigned long long k);
// FP64 SPR weights of tet patches (per mesh, the reference's QR; listed
// patches in lst) and the FP64 recovery from them (listed vertices skipped)
void launch_qr_weights(const DevMesh& m, double* w, unsigned char* listed, ExpandList lst, cudaStream_t s);
void launch_recover_w64(const DevMesh& m, const double* ip, int nc, const double* w, const unsigned char* listed,
                        double* rec, cudaStream_t s);
// FP64 guard band of the FP32 path: re-decide the listed edges' bits.
struct GuardScratch {
  int* stamp;      // V ints, persistent (de-duplication stamps)
  int* stamp_id;   // device counter: this pass's stamp id (starts at 1; the decide stage bumps it)
  int* fit_items;  // fit_cap ints
  int* fit_count;
  int fit_cap;
  double* rec64;   // V x 3 doubles (FP64 recovered values of collected vertices)
  const double* w64;            // FP64 SPR weights in patch-CSR order
  const unsigned char* listed;  // patches on the FP64 reference path
  const double* rec_ref;        // their FP64 reference results (V x 3)
  const double2* geo64;         // per element {det J, h_max} in FP64
};
// unresolved[0]: edges left to the FP32 decision.  Three stages in order:
// 0 collect vertices, 1 fits, 2 decide.
constexpr int kGuardStages = 3;
void launch_guard_stage(int stage, const DevMesh& m, const double* u, const double* out3, const int* items,
                        const int* count, int cap, uint32_t* split, uint32_t* collapse, int* unresolved,
                        GuardScratch g, BatchView bv, cudaStream_t s);
// per-mesh size factors of a batch (SPR mode) from segment partials
void launch_size_factor_batch(const double* partials, BatchView bv, int dim, double* out4, cudaStream_t s);
void launch_quality_f64(const DevMesh& m, const double* size, const double* sizes, const double* frames,
                        double* q, cudaStream_t s, const double* logm = nullptr, DevStatus* st = nullptr);
// anisotropic metric (sizes V x 3, frames V x 9) from a nodal Hessian (V x 9)
void launch_hessian_metric(const DevMesh& m, const double* H, double eps, double hmin, double hmax, double* sizes,
                           double* frames, cudaStream_t s);

// ---- adjacency builders (sprg_kernels_f64.cu) ---------------------------
// Ascending vertex->element CSR via counting sort on the device.
// off must hold V + 1 ints, el T * nn ints, tmp V ints.
void launch_build_v2e(const DevMesh& m, int* off, int* el, int* tmp, cudaStream_t s);
// Sort each CSR segment ascending (segments are short).
void launch_sort_segments(int V, const int* off, int* el, cudaStream_t s);
// X = rint((x - c) s 2^30) per coordinate (c the frame's corner, s its scale)
void launch_xyz_to_fixed(const DevMesh& m, const double* frame, int* xyzq, cudaStream_t s);

}  // namespace sprg
