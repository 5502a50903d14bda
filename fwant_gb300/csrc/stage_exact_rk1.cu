// Instantiation unit: reference-order (exact) arithmetic, RK kind 1 (RK_inn).
// Compiled with -fmad=false; the kernel itself is in stage_impl.cuh.
#include "stage_impl.cuh"

namespace fw {
void launch_stage_exact_rk1(const StageArgs<float>& a, int variant, cudaStream_t st) {
  launch_rk_variant<true, 1>(a, variant, st);
}
}  // namespace fw
