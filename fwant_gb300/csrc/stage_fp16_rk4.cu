// Instantiation unit of the stage kernel (stage_impl.cuh): fast arithmetic, FP16 storage (FP32 arithmetic);
// RK kind 4 (RK_inn without t).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_fp16_rk4(const BatchArgs& b, int variant, int lean, int ctas, cudaStream_t st) {
  return launch_batch_rk_variant<__half, false, 4>(b, variant, lean, ctas, st);
}
int configure_stage_fp16_rk4() { return configure_rk<__half, false, 4>(); }
}  // namespace fw
