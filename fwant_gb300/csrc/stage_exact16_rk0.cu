// Instantiation unit of the stage kernel (stage_impl.cuh): reference-order (exact) arithmetic, FP32 storage, compiled with -fmad=false;
// the tall tile (32 x 16 columns); RK kind 0 (0 RK_beg, 1 RK_inn, 2 RK_fin).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_exact16_rk0(const BatchArgs& b, int variant, int lean, int ctas, cudaStream_t st) {
  return launch_batch_rk_variant<float, true, 0, STAGE_TY_TALL>(b, variant, lean, ctas, st);
}
int configure_stage_exact16_rk0() { return configure_rk<float, true, 0, STAGE_TY_TALL>(); }
}  // namespace fw
