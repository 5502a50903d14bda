// Reading the wavefield registers in any storage kind from the small kernels (receivers,
// snapshots, checks); the stage kernel has its own compile-time typed path.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "kernels.h"

namespace fw {

// Component f (storage order: Vx Vy Vz Tzz Txz Tyz Txx Tyy Txy) at element offset p of a
// register set, converted to the physical FP32 value.
__device__ __forceinline__ float load_component(const void* w, int storage, long long fstride, int f, long long p,
                                                float isv, float ist) {
  const long long o = (long long)f * fstride + p;
  if (storage == ST_F32) return static_cast<const float*>(w)[o];
  const float inv = f < 3 ? isv : ist;
  if (storage == ST_BF16) return __bfloat162float(static_cast<const __nv_bfloat16*>(w)[o]) * inv;
  return __half2float(static_cast<const __half*>(w)[o]) * inv;
}

}  // namespace fw
