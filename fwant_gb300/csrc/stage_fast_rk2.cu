// Instantiation unit: fast arithmetic, RK kind 2 (RK_fin).
// Compiled with FMA contraction; the kernel itself is in stage_impl.cuh.
#include "stage_impl.cuh"

namespace fw {
void launch_stage_fast_rk2(const StageArgs<float>& a, int variant, cudaStream_t st) {
  launch_rk_variant<false, 2>(a, variant, st);
}
}  // namespace fw
