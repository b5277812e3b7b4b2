// Fixed-order block reductions and the SPR size factor, shared by the FP64
// size-factor kernel and the FP32 error kernel's last block, so both give
// the same bits (additions and products only: no fused operations arise
// under either unit's contraction setting).
#pragma once

namespace sprg {

__device__ __forceinline__ double rd_warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// block total, in warp order, valid in thread 0 (every thread calls it)
__device__ __forceinline__ double rd_block_sum(double x, double* sh) {
  x = rd_warp_sum(x);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = x;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
  return t;
}

// the two integrals from per-block partials (thread i sums blocks i, i +
// blockDim.x, ...), then getSPRSizeField's factor (adapt ratio, p = 1) or the
// target-error factor; out3 = {||eps*||^2, sum of err^(2d/(2p+d)), factor},
// written by thread 0
__device__ __forceinline__ void rd_size_factor(const double* partials, int nb, int mode, double adapt_ratio,
                                               double target, int dim, double* out3, double* sh) {
  double a = 0, g = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {  // L2 reads: other blocks wrote them
    a += __ldcg(partials + 2 * i);
    g += __ldcg(partials + 2 * i + 1);
  }
  const double snorm = rd_block_sum(a, sh);
  const double gsum = rd_block_sum(g, sh);
  if (threadIdx.x == 0) {
    const double p = 1;
    double sf;
    if (mode == 0) {
      const double esn = sqrt(snorm);
      const double aa = adapt_ratio * adapt_ratio * esn * esn;
      const double b = aa / gsum;
      sf = pow(b, 1.0 / (2.0 * p));
    } else {
      sf = pow((gsum / target), (1.0 / dim));
    }
    out3[0] = snorm;
    out3[1] = gsum;
    out3[2] = sf;
  }
}

}  // namespace sprg
