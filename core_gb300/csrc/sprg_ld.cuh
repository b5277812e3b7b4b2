// 256-bit read-only gather of one 32-byte record, shared by the FP32 and
// learned kernels.
#pragma once

namespace sprg {

// one 32-byte record (two float4 halves) with a single 256-bit load: a
// warp's gather then asks L1 for one sector per lane instead of two.  The
// records start at a cudaMalloc base (256-byte aligned), 32 bytes each.
__device__ __forceinline__ void ld_record(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

}  // namespace sprg
