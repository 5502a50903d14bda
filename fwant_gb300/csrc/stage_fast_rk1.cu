// Instantiation unit: fast arithmetic, RK kind 1 (RK_inn).
// Compiled with FMA contraction; the kernel itself is in stage_impl.cuh.
#include "stage_impl.cuh"

namespace fw {
void launch_stage_fast_rk1(const StageArgs<float>& a, int variant, cudaStream_t st) {
  launch_rk_variant<false, 1>(a, variant, st);
}
}  // namespace fw
