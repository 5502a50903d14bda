// Selection of the stage-kernel instantiation and of the k-chunk length.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "kernels.h"

namespace fw {

#define FW_DECL(mode)                                                                       \
  int launch_stage_batch_##mode##_rk0(const BatchArgs&, int, int, int, cudaStream_t);       \
  int launch_stage_batch_##mode##_rk1(const BatchArgs&, int, int, int, cudaStream_t);       \
  int launch_stage_batch_##mode##_rk2(const BatchArgs&, int, int, int, cudaStream_t);       \
  int configure_stage_##mode##_rk0();                                                       \
  int configure_stage_##mode##_rk1();                                                       \
  int configure_stage_##mode##_rk2();
FW_DECL(fast)
FW_DECL(exact)
// the stages of the fast FP32 form without t (RK kinds 3-5)
#define FW_DECL_NOT(mode)                                                                   \
  int launch_stage_batch_##mode##_rk3(const BatchArgs&, int, int, int, cudaStream_t);       \
  int launch_stage_batch_##mode##_rk4(const BatchArgs&, int, int, int, cudaStream_t);       \
  int launch_stage_batch_##mode##_rk5(const BatchArgs&, int, int, int, cudaStream_t);       \
  int configure_stage_##mode##_rk3();                                                       \
  int configure_stage_##mode##_rk4();                                                       \
  int configure_stage_##mode##_rk5();
FW_DECL_NOT(fast)
FW_DECL_NOT(fast16)
FW_DECL_NOT(bf16)
FW_DECL_NOT(fp16)
#undef FW_DECL_NOT
FW_DECL(fast16)
FW_DECL(exact16)
FW_DECL(bf16)
FW_DECL(fp16)
#undef FW_DECL
#define FW_DECL_TOPO(mode)                                                  \
  int launch_stage_batch_##mode##_rk0(const BatchArgs&, int, int, cudaStream_t); \
  int launch_stage_batch_##mode##_rk1(const BatchArgs&, int, int, cudaStream_t); \
  int launch_stage_batch_##mode##_rk2(const BatchArgs&, int, int, cudaStream_t); \
  int configure_stage_##mode##_rk0();                                           \
  int configure_stage_##mode##_rk1();                                           \
  int configure_stage_##mode##_rk2();
FW_DECL_TOPO(topo)
FW_DECL_TOPO(topo_exact)
#undef FW_DECL_TOPO
int launch_stage_batch_topo_rk3(const BatchArgs&, int, int, cudaStream_t);
int launch_stage_batch_topo_rk4(const BatchArgs&, int, int, cudaStream_t);
int launch_stage_batch_topo_rk5(const BatchArgs&, int, int, cudaStream_t);
int configure_stage_topo_rk3();
int configure_stage_topo_rk4();
int configure_stage_topo_rk5();

int launch_stage_batch_topo(const BatchArgs& b, int variant, int rk, int exact, int ctas, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (rk >= 3) {  // fast form only
    if (rk > 5 || exact) return int(cudaErrorInvalidValue);
    return rk == 3 ? launch_stage_batch_topo_rk3(b, variant, ctas, st)
                   : (rk == 4 ? launch_stage_batch_topo_rk4(b, variant, ctas, st)
                              : launch_stage_batch_topo_rk5(b, variant, ctas, st));
  }
  if (exact)
    return rk == 0 ? launch_stage_batch_topo_exact_rk0(b, variant, ctas, st)
                   : (rk == 1 ? launch_stage_batch_topo_exact_rk1(b, variant, ctas, st)
                              : launch_stage_batch_topo_exact_rk2(b, variant, ctas, st));
  return rk == 0 ? launch_stage_batch_topo_rk0(b, variant, ctas, st)
                 : (rk == 1 ? launch_stage_batch_topo_rk1(b, variant, ctas, st)
                            : launch_stage_batch_topo_rk2(b, variant, ctas, st));
}

int launch_stage_batch(const BatchArgs& b, int variant, int rk, int exact, int storage, int lean, int ctas,
                       void* stream, int ty) {
  cudaStream_t st = (cudaStream_t)stream;
  if (rk >= 3) {  // fast forms only
    if (rk > 5 || exact || (ty != STAGE_TY && ty != STAGE_TY_TALL) || (storage != ST_F32 && ty != STAGE_TY))
      return int(cudaErrorInvalidValue);
#define FW_RKN(mode)                                                                        \
  return rk == 3 ? launch_stage_batch_##mode##_rk3(b, variant, lean, ctas, st)              \
                 : (rk == 4 ? launch_stage_batch_##mode##_rk4(b, variant, lean, ctas, st)   \
                            : launch_stage_batch_##mode##_rk5(b, variant, lean, ctas, st));
    if (ty == STAGE_TY_TALL) { FW_RKN(fast16) }
    if (storage == ST_BF16) { FW_RKN(bf16) }
    if (storage == ST_F16) { FW_RKN(fp16) }
    FW_RKN(fast)
#undef FW_RKN
  }
#define FW_RK(mode)                                                                         \
  return rk == 0 ? launch_stage_batch_##mode##_rk0(b, variant, lean, ctas, st)              \
                 : (rk == 1 ? launch_stage_batch_##mode##_rk1(b, variant, lean, ctas, st)   \
                            : launch_stage_batch_##mode##_rk2(b, variant, lean, ctas, st));
  if (ty == STAGE_TY_TALL) {
    if (storage != ST_F32) return int(cudaErrorInvalidValue);
    if (exact) { FW_RK(exact16) }
    FW_RK(fast16)
  }
  if (ty != STAGE_TY) return int(cudaErrorInvalidValue);
  if (storage == ST_BF16) { FW_RK(bf16) }
  if (storage == ST_F16) { FW_RK(fp16) }
  if (exact) { FW_RK(exact) }
  FW_RK(fast)
#undef FW_RK
}

int stage_configure() {
  int (*const fns[])() = {configure_stage_fast_rk0, configure_stage_fast_rk1, configure_stage_fast_rk2,
                          configure_stage_exact_rk0, configure_stage_exact_rk1, configure_stage_exact_rk2,
                          configure_stage_fast16_rk0, configure_stage_fast16_rk1, configure_stage_fast16_rk2,
                          configure_stage_exact16_rk0, configure_stage_exact16_rk1, configure_stage_exact16_rk2,
                          configure_stage_bf16_rk0, configure_stage_bf16_rk1, configure_stage_bf16_rk2,
                          configure_stage_fp16_rk0, configure_stage_fp16_rk1, configure_stage_fp16_rk2,
                          configure_stage_topo_rk0, configure_stage_topo_rk1, configure_stage_topo_rk2,
                          configure_stage_topo_exact_rk0, configure_stage_topo_exact_rk1,
                          configure_stage_topo_exact_rk2,
                          configure_stage_fast_rk3,   configure_stage_fast_rk4,   configure_stage_fast_rk5,
                          configure_stage_fast16_rk3, configure_stage_fast16_rk4, configure_stage_fast16_rk5,
                          configure_stage_topo_rk3,   configure_stage_topo_rk4,   configure_stage_topo_rk5,
                          configure_stage_bf16_rk3,   configure_stage_bf16_rk4,   configure_stage_bf16_rk5,
                          configure_stage_fp16_rk3,   configure_stage_fp16_rk4,   configure_stage_fp16_rk5};
  for (auto fn : fns)
    if (int e = fn()) return e;
  return 0;
}

long long stage_item_count(const Geom& g, int kc, int ty, int kz_lo, int kz_hi) {
  return (long long)((g.ni + STAGE_TX - 1) / STAGE_TX) * ((g.nj + ty - 1) / ty) *
         stage_chunk_count(g, kc, kz_lo, kz_hi);
}

void stage_z_bands(const Geom& g, const Slab slab[6], int* kz_lo, int* kz_hi) {
  static const bool bands = [] {  // measurement override: FWANT_Z_BANDS=0 cuts the planes as one band
    const char* env = std::getenv("FWANT_Z_BANDS");
    return !(env && std::atoi(env) == 0);
  }();
  int lo = g.k1, hi = g.k2 + 1;
  if (!bands) {
    *kz_lo = lo;
    *kz_hi = hi;
    return;
  }
  if (slab[4].on) lo = std::min(std::max(slab[4].k2 + 1, g.k1), g.k2 + 1);
  if (g.freesurf) hi = g.k2 - 3;
  else if (slab[5].on) hi = slab[5].k1;
  *kz_lo = lo;
  *kz_hi = std::min(std::max(hi, lo), g.k2 + 1);
}

// An item is lean when none of its points lies in a PML slab, within reach (3 points) of
// a smoothed source box, or within four planes of a free surface (images, VLOW rows,
// T*Src): exactly the code the lean form compiles out.
void stage_items(const Geom& g, int kc, int ty, int kz_lo, int kz_hi, const Slab slab[6], const int* force_c,
                 int nforce, const int* mom_c, int nmom, int* lean, int* nlean, int* full, int* nfull) {
  const int nbx = (g.ni + STAGE_TX - 1) / STAGE_TX, nby = (g.nj + ty - 1) / ty;
  const int nbz = stage_chunk_count(g, kc, kz_lo, kz_hi);
  auto overlap = [](int a0, int a1, int b0, int b1) { return a0 <= b1 && b0 <= a1; };
  int nl = 0, nf = 0;
  for (int bz = 0; bz < nbz; ++bz)
    for (int by = 0; by < nby; ++by)
      for (int bx = 0; bx < nbx; ++bx) {
        const int i0 = g.i1 + bx * STAGE_TX, i1 = std::min(i0 + STAGE_TX - 1, g.i2);
        const int j0 = g.j1 + by * ty, j1 = std::min(j0 + ty - 1, g.j2);
        int k0, k1;
        stage_chunk(g, kc, kz_lo, kz_hi, bz, &k0, &k1);
        bool is_lean = !(g.freesurf && k1 > g.k2 - 4);
        for (int f = 0; f < 6 && is_lean; ++f) {
          const Slab& s = slab[f];
          if (s.on && overlap(i0, i1, s.i1, s.i2) && overlap(j0, j1, s.j1, s.j2) && overlap(k0, k1, s.k1, s.k2))
            is_lean = false;
        }
        for (int n = 0; n < nforce && is_lean; ++n)
          if (overlap(i0, i1, force_c[3 * n] - 3, force_c[3 * n] + 3) &&
              overlap(j0, j1, force_c[3 * n + 1] - 3, force_c[3 * n + 1] + 3) &&
              overlap(k0, k1, force_c[3 * n + 2] - 3, force_c[3 * n + 2] + 3))
            is_lean = false;
        for (int n = 0; n < nmom && is_lean; ++n)
          if (overlap(i0, i1, mom_c[3 * n] - 3, mom_c[3 * n] + 3) &&
              overlap(j0, j1, mom_c[3 * n + 1] - 3, mom_c[3 * n + 1] + 3) &&
              overlap(k0, k1, mom_c[3 * n + 2] - 3, mom_c[3 * n + 2] + 3))
            is_lean = false;
        const int packed = int(unsigned(bx) | unsigned(by) << 10 | unsigned(bz) << 20);
        if (is_lean) lean[nl++] = packed;
        else full[nf++] = packed;
      }
  *nlean = nl;
  *nfull = nf;
}

}  // namespace fw
