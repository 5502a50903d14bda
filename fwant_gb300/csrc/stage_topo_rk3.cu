// Instantiation unit of the stage kernel (stage_impl.cuh): the terrain-following form (FP32
// storage, full form, fast arithmetic); RK kind 3 (RK_beg without t).
#include "stage_impl.cuh"

namespace fw {
int launch_stage_batch_topo_rk3(const BatchArgs& b, int variant, int ctas, cudaStream_t st) {
  return launch_batch_topo_variant<false, 3>(b, variant, ctas, st);
}
int configure_stage_topo_rk3() { return configure_topo_rk<false, 3>(); }
}  // namespace fw
