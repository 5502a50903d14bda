// Instantiation unit of the stage kernel (stage_impl.cuh): the terrain-following form (FP32
// storage, full form, reference operand order, compiled without FMA contraction); RK kind 0 (0 RK_beg, 1 RK_inn, 2 RK_fin).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_topo_exact_rk0(const BatchArgs& b, int variant, int ctas, cudaStream_t st) {
  return launch_batch_topo_variant<true, 0>(b, variant, ctas, st);
}
int configure_stage_topo_exact_rk0() { return configure_topo_rk<true, 0>(); }
}  // namespace fw
