// FP32 fast path (sprg_kernels_f32.cu): 3D tets, scalar field, isotropic size.
#pragma once
#include "sprg_internal.h"

namespace sprg {

int fast_error_blocks(int T);
// packed double-float vertex records {x,y,z,u}_hi, {x,y,z,u}_lo (2 float4 per vertex)
void fast_prep(const DevMesh& m, const double* u, float4* vrec, cudaStream_t s);
// per tet: {g_t, wdv}, {d_t, h_max}, {ip_hi, 0}, {ip_lo, 0} (4 float4)
void fast_tet(const DevMesh& m, const float4* vrec, float4* td, cudaStream_t s);
void fast_recover(const DevMesh& m, const float4* vrec, const float4* td, float4* rec, ExpandList xl, int* n_refit,
                  cudaStream_t s);
void fast_merge_ref(ExpandList xl, const double* rec64, float4* rec32, cudaStream_t s);
void fast_error(const DevMesh& m, const float4* td, const float4* rec, float* q, double* partials, int nb,
                cudaStream_t s);
void fast_average(const DevMesh& m, const float* q, const double* out3, float* size32, cudaStream_t s);
void fast_measure(const DevMesh& m, const float4* vrec, const float* size32, uint32_t* split, uint32_t* collapse,
                  float* L32, int* guard_items, int* guard_count, int guard_cap, float guard_rel, cudaStream_t s);
void fast_size_to_f64(int V, const float* s32, double* s64, cudaStream_t s);

}  // namespace sprg
