// Instantiation unit of the stage kernel (stage_impl.cuh): fast arithmetic, BF16 storage (FP32 arithmetic);
// RK kind 5 (RK_inn forming t from the stage values).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_bf16_rk5(const BatchArgs& b, int variant, int lean, int ctas, cudaStream_t st) {
  return launch_batch_rk_variant<__nv_bfloat16, false, 5>(b, variant, lean, ctas, st);
}
int configure_stage_bf16_rk5() { return configure_rk<__nv_bfloat16, false, 5>(); }
}  // namespace fw
