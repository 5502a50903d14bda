// Selection of the stage-kernel instantiation and of the k-chunk length.
#include <cuda_runtime.h>

#include "kernels.h"

namespace fw {

void launch_stage_fast_rk0(const StageArgs<float>&, int, cudaStream_t);
void launch_stage_fast_rk1(const StageArgs<float>&, int, cudaStream_t);
void launch_stage_fast_rk2(const StageArgs<float>&, int, cudaStream_t);
void launch_stage_exact_rk0(const StageArgs<float>&, int, cudaStream_t);
void launch_stage_exact_rk1(const StageArgs<float>&, int, cudaStream_t);
void launch_stage_exact_rk2(const StageArgs<float>&, int, cudaStream_t);

void launch_stage_f32(const StageArgs<float>& a, int variant, int rk, int exact, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (exact) {
    if (rk == 0) launch_stage_exact_rk0(a, variant, st);
    else if (rk == 1) launch_stage_exact_rk1(a, variant, st);
    else launch_stage_exact_rk2(a, variant, st);
  } else {
    if (rk == 0) launch_stage_fast_rk0(a, variant, st);
    else if (rk == 1) launch_stage_fast_rk1(a, variant, st);
    else launch_stage_fast_rk2(a, variant, st);
  }
}

// Planes per CTA: long enough that the z-halo re-load (4 planes per chunk) stays small,
// short enough to give at least ~4 CTAs per SM.
int stage_planes_per_cta(const Geom& g, int sm_count) {
  const long long tiles = (long long)((g.ni + STAGE_TX - 1) / STAGE_TX) * ((g.nj + STAGE_TY - 1) / STAGE_TY);
  const long long want = 4LL * sm_count;
  long long chunks = (want + tiles - 1) / tiles;
  if (chunks < 1) chunks = 1;
  int kc = int((g.nk + chunks - 1) / chunks);
  if (kc < 8) kc = 8;
  if (kc > 32) kc = 32;
  return kc;
}

}  // namespace fw
