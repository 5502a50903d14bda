// Instantiation unit of the stage kernel (stage_impl.cuh): the terrain-following form (FP32
// storage, full form, fast arithmetic); RK kind 5 (RK_inn forming t from the stage values).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_topo_rk5(const BatchArgs& b, int variant, int ctas, cudaStream_t st) {
  return launch_batch_topo_variant<false, 5>(b, variant, ctas, st);
}
int configure_stage_topo_rk5() { return configure_topo_rk<false, 5>(); }
}  // namespace fw
