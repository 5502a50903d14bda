// Instantiation unit of the stage kernel (stage_impl.cuh): fast arithmetic, FP32 storage, compiled with FMA contraction;
// the tall tile (32 x 16 columns); RK kind 3 (RK_beg without t).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_fast16_rk3(const BatchArgs& b, int variant, int lean, int ctas, cudaStream_t st) {
  return launch_batch_rk_variant<float, false, 3, STAGE_TY_TALL>(b, variant, lean, ctas, st);
}
int configure_stage_fast16_rk3() { return configure_rk<float, false, 3, STAGE_TY_TALL>(); }
}  // namespace fw
