// Selection of the stage-kernel instantiation and of the k-chunk length.
#include <cuda_runtime.h>

#include "kernels.h"

namespace fw {

#define FW_DECL(mode)                                                            \
  int launch_stage_##mode##_rk0(const StageArgs&, int, cudaStream_t);            \
  int launch_stage_##mode##_rk1(const StageArgs&, int, cudaStream_t);            \
  int launch_stage_##mode##_rk2(const StageArgs&, int, cudaStream_t);            \
  int launch_stage_batch_##mode##_rk0(const BatchArgs&, int, int, cudaStream_t); \
  int launch_stage_batch_##mode##_rk1(const BatchArgs&, int, int, cudaStream_t); \
  int launch_stage_batch_##mode##_rk2(const BatchArgs&, int, int, cudaStream_t); \
  int configure_stage_##mode##_rk0();                                            \
  int configure_stage_##mode##_rk1();                                            \
  int configure_stage_##mode##_rk2();
FW_DECL(fast)
FW_DECL(exact)
FW_DECL(bf16)
FW_DECL(fp16)
#undef FW_DECL

int launch_stage(const StageArgs& a, int variant, int rk, int exact, int storage, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
#define FW_RK(mode)                                                    \
  return rk == 0 ? launch_stage_##mode##_rk0(a, variant, st)           \
                 : (rk == 1 ? launch_stage_##mode##_rk1(a, variant, st) \
                            : launch_stage_##mode##_rk2(a, variant, st));
  if (storage == ST_BF16) { FW_RK(bf16) }
  if (storage == ST_F16) { FW_RK(fp16) }
  if (exact) { FW_RK(exact) }
  FW_RK(fast)
#undef FW_RK
}

int launch_stage_batch(const BatchArgs& b, int variant, int rk, int exact, int storage, int ctas, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
#define FW_RK(mode)                                                                  \
  return rk == 0 ? launch_stage_batch_##mode##_rk0(b, variant, ctas, st)             \
                 : (rk == 1 ? launch_stage_batch_##mode##_rk1(b, variant, ctas, st)  \
                            : launch_stage_batch_##mode##_rk2(b, variant, ctas, st));
  if (storage == ST_BF16) { FW_RK(bf16) }
  if (storage == ST_F16) { FW_RK(fp16) }
  if (exact) { FW_RK(exact) }
  FW_RK(fast)
#undef FW_RK
}

int stage_configure() {
  int (*const fns[])() = {configure_stage_fast_rk0, configure_stage_fast_rk1, configure_stage_fast_rk2,
                          configure_stage_exact_rk0, configure_stage_exact_rk1, configure_stage_exact_rk2,
                          configure_stage_bf16_rk0, configure_stage_bf16_rk1, configure_stage_bf16_rk2,
                          configure_stage_fp16_rk0, configure_stage_fp16_rk1, configure_stage_fp16_rk2};
  for (auto fn : fns)
    if (int e = fn()) return e;
  return 0;
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
