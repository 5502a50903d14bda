// Selection of the stage-kernel instantiation and of the k-chunk length.
#include <cuda_runtime.h>

#include "kernels.h"
#include "stage_impl.cuh"

namespace fw {

int launch_stage_fast_rk0(const StageArgs&, int, cudaStream_t);
int launch_stage_fast_rk1(const StageArgs&, int, cudaStream_t);
int launch_stage_fast_rk2(const StageArgs&, int, cudaStream_t);
int launch_stage_exact_rk0(const StageArgs&, int, cudaStream_t);
int launch_stage_exact_rk1(const StageArgs&, int, cudaStream_t);
int launch_stage_exact_rk2(const StageArgs&, int, cudaStream_t);

int launch_stage_f32(const StageArgs& a, int variant, int rk, int exact, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (exact) {
    if (rk == 0) return launch_stage_exact_rk0(a, variant, st);
    if (rk == 1) return launch_stage_exact_rk1(a, variant, st);
    return launch_stage_exact_rk2(a, variant, st);
  }
  if (rk == 0) return launch_stage_fast_rk0(a, variant, st);
  if (rk == 1) return launch_stage_fast_rk1(a, variant, st);
  return launch_stage_fast_rk2(a, variant, st);
}

size_t stage_smem_bytes() { return SMEM_BYTES; }

int configure_stage_fast_rk0();
int configure_stage_fast_rk1();
int configure_stage_fast_rk2();
int configure_stage_exact_rk0();
int configure_stage_exact_rk1();
int configure_stage_exact_rk2();

int stage_configure() {
  int e = configure_stage_fast_rk0();
  if (!e) e = configure_stage_fast_rk1();
  if (!e) e = configure_stage_fast_rk2();
  if (!e) e = configure_stage_exact_rk0();
  if (!e) e = configure_stage_exact_rk1();
  if (!e) e = configure_stage_exact_rk2();
  return e;
}

// Planes per CTA.  Short chunks keep the CTAs that share halo rows marching through the
// same planes at the same time, which is what lets L2 serve the halo and z-queue
// re-reads; measured on 400x400x200: 16 planes 1.68 ms per RK_inn stage, 32 planes 1.78,
// 64 planes 2.01, the whole column 3.04.  Small grids get shorter chunks so that there
// are at least ~4 CTAs per SM.
int stage_planes_per_cta(const Geom& g, int sm_count) {
  const long long tiles = (long long)((g.ni + STAGE_TX - 1) / STAGE_TX) * ((g.nj + STAGE_TY - 1) / STAGE_TY);
  const long long want = 4LL * sm_count;
  long long chunks = (want + tiles - 1) / tiles;
  if (chunks < 1) chunks = 1;
  int kc = int((g.nk + chunks - 1) / chunks);
  if (kc < 8) kc = 8;
  if (kc > 16) kc = 16;
  return kc;
}

}  // namespace fw
