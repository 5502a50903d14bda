// Instantiation unit of the stage kernel (stage_impl.cuh): the terrain-following form (FP32
// storage, full form, fast arithmetic); RK kind 4 (RK_inn without t).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_topo_rk4(const BatchArgs& b, int variant, int ctas, cudaStream_t st) {
  return launch_batch_topo_variant<false, 4>(b, variant, ctas, st);
}
int configure_stage_topo_rk4() { return configure_topo_rk<false, 4>(); }
}  // namespace fw
