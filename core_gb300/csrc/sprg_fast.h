// FP32 fast path (sprg_kernels_f32.cu): 3D tets, scalar field, isotropic size.
#pragma once
#include "sprg_internal.h"

namespace sprg {

int fast_error_blocks(int T);
// packed double-float coordinate records {x,y,z,0}_hi, {x,y,z,0}_lo (2 float4 per
// vertex) of the coordinates mapped into [1, 2]: x' = (x - c) s + 1 with
// frame = {c_x, c_y, c_z, s}, s a power of two
void fast_prep_coords(const DevMesh& m, const double* frame, float4* vrec, cudaStream_t s);
// once per mesh: per tet {w dV, h_max} (FP32) and {det J, h_max} (FP64), per
// edge half its length
// cent: 3 doubles per element, the integration point (once per mesh, read by
// fast_weights); qmax: one double (as its bits, set here), the largest
// |cof J|_F^2 / |det J| over the elements
void fast_geometry(const DevMesh& m, float2* geo, double2* geo64, double* cent, unsigned long long* qmax,
                   float* half_len, cudaStream_t s);
// the pass's vertex records: coordinate records with the field pair (u_hi,
// u_lo); umax_bits (zeroed by the caller): max |u_hi| as float bits
void fast_prep(const DevMesh& m, const double* u, const float4* crec, float4* vrec, int* umax_bits, cudaStream_t s);
// per tet: gradient value (3 floats) and packed correction (1 word)
// gscale = the frame's s (gradients in the mesh's coordinates); u: the FP64
// field, read for the ill-conditioned tets solved in FP64
// next_chunk: one device int (the kernel's work counter, cleared here)
void fast_tet(const DevMesh& m, const float4* vrec, const double* u, float gscale, uint4* td, int* next_chunk,
              cudaStream_t s);
// once per mesh: SPR weights in patch-CSR order (FP32 for the pass, FP64 for
// the guard), listed patches
void fast_weights(const DevMesh& m, const double* cent, float* w, double* w64, ExpandList xl, int* n_refit,
                  unsigned char* listed, cudaStream_t s);
// recovered value per vertex as a 32-byte record {s0, s1, s2, r0}, {r1, r2,
// 0, 0}: the FP32 value and its FP32 remainder (listed vertices: from rec64)
void fast_merge_ref(ExpandList xl, const double* rec64, float4* rec32, cudaStream_t s);
// patch-size class per vertex: 0 (<= 8 elements), 1 (<= 16), 2 (<= 32), 3, 4 = listed
void fast_patch_class(const DevMesh& m, const unsigned char* listed, unsigned char* cls, cudaStream_t s);
// the bins' vertex order on the device: per-block class counts (4 ints per
// block of fast_bin_blocks(V)), then, with the blocks' exclusive offsets per
// class (4 ints per block), the scatter: each bin in ascending vertex order
int fast_bin_blocks(int V);
void fast_bin_count(int V, const unsigned char* cls, int* counts, cudaStream_t s);
void fast_bin_scatter(int V, const unsigned char* cls, const int* offs, int* order, cudaStream_t s);
// sliced copy of the patch lists (element ids and FP32 weights): the binned
// vertex order cut into slices of 32 aligned to each bin's start (bin b:
// entries [start[b], start[b + 1]) of the order, slices [slice0[b],
// slice0[b + 1])); entry k of the slice's lane i at off[s] + 32 k + i
struct BinSlices {
  int start[5], slice0[5];
};
struct SlicedPatches {
  const int* off;
  const int* el;
  const float* w;
};
// per slice its width (the largest patch of its vertices)
void fast_slice_width(const DevMesh& m, const BinSlices& bs, const int* verts, int* width, cudaStream_t s);
// with off set (exclusive sums of 32 x width): the element ids and weights
void fast_slice_fill(const DevMesh& m, const BinSlices& bs, const int* verts, const float* w, const int* off,
                     int* sel, float* sw, cudaStream_t s);
// binned recover: tiles (first, count, lanes, slice of first) over verts,
// taken from a counter by a persistent grid; lanes 1, 2, 4 per vertex over
// the patch-CSR lists, or 0: one per vertex over the sliced copy (tiles then
// start on a slice); every tiling gives the same bits.  mode: the lane count
// of every tile (a kernel for that mode alone), or -1 for mixed tiles
void fast_recover_tiles(const DevMesh& m, const float* w, SlicedPatches sp, const uint4* td, float4* rec,
                        const int* verts, const int4* tiles, int n_tiles, int mode, int* next, int grid,
                        cudaStream_t s);
// q: (h_max err^(-1/5), its relative error bound) per tet
// seg (batch): one element range per block, nb = number of segments
// done (one unsigned, zero between passes) and out3: the last block also
// computes the size factor (one mesh; pass null for a batch); n_round (max
// |u| from fast_prep) is replaced by the last block with 1 when the
// reference's FP64 rounding of its IP gradients (bounded with qmax from
// fast_geometry) could move the error integral by 1e-7 of it, else 0
void fast_error(const DevMesh& m, const uint4* td, const float2* geo, const float4* rec, float2* q, double* partials,
                int nb, const int2* seg, unsigned* done, double adapt_ratio, double* out3, int* n_round,
                const unsigned long long* qmax, cudaStream_t s);
// sz2: (size, its relative error bound) per vertex
void fast_average(const DevMesh& m, const float2* q, const double* out3, float2* sz2, BatchView bv, cudaStream_t s);
void fast_measure(const DevMesh& m, const float* half_len, const float2* sz2, uint32_t* split, uint32_t* collapse,
                  int* guard_items, int* guard_count, int guard_cap, float guard_rel, cudaStream_t s);
void fast_size_to_f64(int V, const float2* sz2, double* s64, cudaStream_t s);

}  // namespace sprg
