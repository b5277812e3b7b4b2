// Learned form of the estimate-and-mark pass (sprg_learned.cu): 3D tets,
// scalar field.  An MLP (2 x 64 GELU, BF16 weights and activations, FP32
// accumulation) predicts the correction from a cheap least-squares vertex
// gradient to the SPR recovered gradient; plain SPR is its fallback.
#pragma once
#include "sprg_internal.h"

namespace sprg {

constexpr int kMlpSlots = 32;                  // neighbour slots per vertex
constexpr int kMlpIn = 4 * kMlpSlots;          // (dx, dy, dz, residual) per slot
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 3;
// FP32 master parameter vector: W1 [64][128], b1 [64], W2 [64][64], b2 [64],
// W3 [3][64], b3 [3] (weights row-major, [output][input])
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpHidden * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpOut * kMlpHidden;
constexpr int kMlpParams = kMlpB3 + kMlpOut;   // 12611
// device-packed inference parameters (bytes): BF16 weight tiles in the
// tensor-core operand layout plus FP32 biases
constexpr int kMlpPackedBytes = 2 * (kMlpHidden * kMlpIn + kMlpHidden * kMlpHidden + 16 * kMlpHidden) +
                                4 * (kMlpHidden + kMlpHidden + 16);
// per-vertex auxiliary record of the features: g_c (3), output scale, flag
constexpr int kMlpAux = 5;

struct LearnMesh {
  const int* vv_off;                // V + 1: vertex -> neighbour vertices (edge CSR, ascending)
  const int* vv;
  const unsigned char* listed;      // patches on the FP64 reference path
  const unsigned char* tile_half;   // per 128-vertex tile: all degrees <= 16
};

// vertex -> vertex CSR from the edge list (off: V + 1, nb: 2E, tmp: V ints),
// the per-tile degree flags (ceil(V / 128) bytes) and the largest degree
void learned_build_v2v(const DevMesh& m, int* off, int* nb, int* tmp, unsigned char* tile_half, int* max_deg,
                       cudaStream_t s);
// fixed-point vertex records {X, Y, Z, U} (16 bytes): the coordinates from
// m.xyzq, the field on the pass's range.  range: learned_range_bytes() of
// scratch, done: one device counter (zero before the first call, left zero),
// lsc: the two difference scales {cs, cu} (cs = 2^-30 / the frame's s)
size_t learned_range_bytes();
void learned_prep(const DevMesh& m, const double* u, float cs, double* range, unsigned* done, float* lsc,
                  float4* vr16, cudaStream_t s);
// features for training: x [V][128] BF16 (row-major), aux [V][5]
void learned_features(const DevMesh& m, const LearnMesh& lm, const float4* vr16, const float* lsc, uint16_t* x,
                      float* aux, cudaStream_t s);
// pack FP32 master parameters into the inference layout
void learned_pack(const float* params, void* packed, cudaStream_t s);
// MLP inference over all vertices (tensor cores): rec16 (32-byte records
// {X, Y, Z, U}, {eps*, 0}) for the vertices the
// network answers, the rest appended to fb_items (fb_count); use_mlp = 0
// gives the cheap gradient alone.  err: set when a wait timed out.
// max_degree <= 16 selects the K = 64 kernel (two blocks per SM)
// stall_polls > 0 (test hook): the first layer-1 completion wait of each
// block waits that many polls on a barrier nothing completes and runs out
void learned_infer(const DevMesh& m, const LearnMesh& lm, const float4* vr16, const float* lsc, const void* packed,
                   float4* rec16, int* fb_items, int* fb_count, float z_max, int use_mlp, int max_degree,
                   int stall_polls, int* err, cudaStream_t s);
// plain SPR for the fallback vertices (FP32 weights, FP32 element gradients;
// listed patches take rec64, their FP64 reference result)
void learned_fallback(const DevMesh& m, const LearnMesh& lm, const float4* vr16, const float* lsc, const float* w,
                      const double* rec64, const int* fb_items, const int* fb_count, int fb_cap, float4* rec16,
                      cudaStream_t s);
int learned_error_blocks(int T);
// rec: one 32-byte record per vertex {X, Y, Z, U}, {eps*, 0} (written by the
// network and fallback kernels); w dV and h_max from the per-mesh element
// geometry (geo)
void learned_error(const DevMesh& m, const float4* rec, const float* lsc, const float2* geo, float* q, double* partials,
                   int nb, cudaStream_t s);
void learned_average(const DevMesh& m, const float* q, const double* out3, float* size, cudaStream_t s);
void learned_measure(const DevMesh& m, const float* half_len, const float* size, uint32_t* split, uint32_t* collapse,
                     cudaStream_t s);
void learned_size_to_f64(int V, const float* s32, double* s64, cudaStream_t s);

// training (SIMT kernels; BF16 weights and activations, FP32 accumulation)
size_t mlp_scratch_bytes(int n);
// mode 0: forward, out [n][3]; mode 1: gradient of the mean squared error
// against y [n][3] into grad [kMlpParams], sum of squared errors into loss
void mlp_run(int mode, const float* params, const uint16_t* x, const float* y, int n, float* out, float* grad,
             float* loss, void* scratch, cudaStream_t s);
void mlp_adam(float* params, float* m1, float* m2, const float* grad, float lr, float beta1, float beta2, float eps,
              int step, cudaStream_t s);

}  // namespace sprg
