// Instantiation unit: fast arithmetic, RK kind 0 (RK_beg).
// Compiled with FMA contraction; the kernel itself is in stage_impl.cuh.
#include "stage_impl.cuh"

namespace fw {
void launch_stage_fast_rk0(const StageArgs<float>& a, int variant, cudaStream_t st) {
  launch_rk_variant<false, 0>(a, variant, st);
}
}  // namespace fw
