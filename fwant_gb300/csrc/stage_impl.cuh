// Fused LDDRK4 stage kernel for sm_103a (included by the stage_*.cu instantiation units).
//
// One launch performs, for every interior point, what the reference does in five
// separate sweeps of one Runge-Kutta stage:
//   free_timg        traction image above the free surface   mod_macdrp.F90:3414-3436
//   L<X>             18 one-sided derivatives, spherical RHS  mod_macdrp.F90:790-962
//   abs_L<X>         CFS-PML memory-variable corrections      mod_abs_npml.F90:1149-2123
//   src_stress/force source injection with 7^3 smoothing      mod_src.F90:207-345
//   RK_beg/inn/fin   register update of W, t (and PML aux)    mod_macdrp.F90:291-393
// The right-hand side h never goes to memory.  Image values above the free surface are
// substituted while loading instead of being written: the stored stress on k = nk2 keeps
// its RK value, as in the reference where the RK update overwrites the imaged value.
//
// Data movement (2.5-D, TMA pipeline): a CTA owns a 32 x 8 (i, j) tile and marches along
// k over kc planes.  For every plane one elected thread issues TMA tensor loads
// (cp.async.bulk.tensor) of
//   * the stage input W around the tile (40 x 12 columns: the halo rows on the side the
//     one-sided y operator reads; all nine components),
//   * the six k-differentiated components of plane k+LEAD (the z-queue feed),
//   * lambda, mu, rho and the RK registers m and t of the tile,
// into one of two shared-memory buffers, one plane ahead of the compute; completion is
// tracked by an mbarrier per buffer.  Each thread keeps its column of the
// k-differentiated components in a five-plane register queue.  Every wait on an
// mbarrier is bounded: on expiry the kernel records DEVERR_TMA_TIMEOUT, waits (bounded)
// for the copy still in flight and returns.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "kernels.h"

namespace fw {

constexpr int TX = STAGE_TX;  // tile columns (one warp per tile row); the rows TY are a template parameter
constexpr int WAIT_SPINS = 1 << 22;

// Shared-memory layout of one pipeline buffer for storage type S (byte offsets,
// 128-byte aligned).  The tile box starts HX columns left of the CTA's first column so
// that its x origin stays 16-byte aligned (4 columns of 4 bytes, 8 columns of 2 bytes).
// TOPO (terrain-following grid): the z queue holds all nine components, and the plane's
// terrain metric (r, zeta_r, zeta_theta/r, zeta_phi/(r sin theta)) follows the medium.
template <class S, bool TOPO = false, int TY = STAGE_TY>
struct Lay {
  static constexpr int TBY = tile_by(TY);
  static constexpr int ES = sizeof(S);
  static constexpr int HX = tile_halo_x(ES);
  static constexpr int TBX = tile_box_x(ES);
  static constexpr int SZ_TILE = NF * TBY * TBX * ES;
  static constexpr int OFF_Q = ((SZ_TILE + 127) / 128) * 128;
  static constexpr int NQ = TOPO ? NF : 6;  // components of the z queue
  static constexpr int SZ_Q = NQ * TY * TX * ES;
  static constexpr int OFF_MED = OFF_Q + SZ_Q;
  static constexpr int SZ_MED = 3 * TY * TX * 4;  // the medium stays FP32
  static constexpr int OFF_TOPO = OFF_MED + SZ_MED;
  static constexpr int SZ_TOPO = TOPO ? 4 * TY * TX * 4 : 0;
  static constexpr int OFF_M = OFF_TOPO + SZ_TOPO;
  static constexpr int SZ_PT = NF * TY * TX * ES;
  static constexpr int OFF_T = OFF_M + SZ_PT;
  static constexpr int BUF_BYTES = ((OFF_T + SZ_PT + 1023) / 1024) * 1024;
  static constexpr int SMEM_BYTES = 2 * BUF_BYTES + 64;  // + the mbarriers (up to 5 x 8 bytes)
  // Interior-only (lean) form: the tile holds the eight x/y-differentiated components
  // (Tzz comes from the z queue) as two boxes, components 0-2 and 4-8, each starting on a
  // 128-byte boundary; the RK registers m and t of the current plane are staged in one
  // buffer after the two pipeline buffers.
  static constexpr int SZ_PLANE = TBY * TBX * ES;
  static constexpr int OFF_HI_L = ((3 * SZ_PLANE + 127) / 128) * 128;
  static constexpr int SZ_TILE_L = OFF_HI_L + 5 * SZ_PLANE;
  static constexpr int OFF_Q_L = ((SZ_TILE_L + 127) / 128) * 128;
  static constexpr int OFF_MED_L = OFF_Q_L + SZ_Q;
  static constexpr int BUF_BYTES_LEAN = ((OFF_MED_L + SZ_MED + 127) / 128) * 128;
  static constexpr int OFF_MT_L = 2 * BUF_BYTES_LEAN;
  template <int RK>
  static constexpr int SZ_MT_L = RK == 1 ? 2 * SZ_PT : (RK == 2 ? SZ_PT : 0);
  // Full form: the PML memory variables of staged slab faces (up to pml_slots per item; the
  // terrain form stages none).  The stage input's six variables of a face (TX x TY x 6 FP32)
  // ride in the pipeline buffer with the tile, one plane ahead: RK_beg and RK_fin put them
  // in the buffer's m / t space that they do not use (when it is large enough), RK_inn after
  // t.  RK_fin's t variables follow in the buffer (at off_pb); RK_inn's m and t variables,
  // for which two CTAs per SM leave no room in the buffers, go to one area after the two
  // buffers, loaded at the start of their plane on a barrier of their own and waited for at
  // the final update.
  static constexpr int SZ_PML_PLANE = 6 * TY * TX * 4;
  __host__ __device__ static constexpr int pml_slots(int rk) { return TOPO ? 0 : (rk == 0 ? 3 : 1); }
  __host__ __device__ static constexpr int pml_single_roles(int rk) { return rk == 1 ? 2 : 0; }
  __host__ __device__ static constexpr int pml_buf_roles(int rk) { return rk == 2 ? 1 : 0; }  // t in the buffer
  __host__ __device__ static constexpr bool pml_in_mt(int rk) {  // the input slots reuse the m / t space
    return rk != 1 && pml_slots(rk) * SZ_PML_PLANE <= (rk == 0 ? 2 : 1) * SZ_PT;
  }
  __host__ __device__ static constexpr int off_pa(int rk) { return pml_in_mt(rk) ? OFF_M : OFF_T + SZ_PT; }
  __host__ __device__ static constexpr int off_pb(int rk) {
    return pml_in_mt(rk) ? OFF_T + SZ_PT : OFF_T + SZ_PT + pml_slots(rk) * SZ_PML_PLANE;
  }
  __host__ __device__ static constexpr int buf_full(int rk) {
    return (pml_in_mt(rk) && pml_buf_roles(rk) == 0)
               ? BUF_BYTES
               : ((off_pb(rk) + pml_slots(rk) * pml_buf_roles(rk) * SZ_PML_PLANE + 1023) / 1024) * 1024;
  }
  __host__ __device__ static constexpr int pml_single_bytes(int rk) {
    return pml_slots(rk) * pml_single_roles(rk) * SZ_PML_PLANE;
  }
  static int smem_bytes(bool lean, int rk_kind) {
    const int rk = rk_base(rk_kind);  // the layout of the reference kind it follows
    return lean ? OFF_MT_L + (rk == 1 ? 2 * SZ_PT : (rk == 2 ? SZ_PT : 0)) + 64
                : 2 * buf_full(rk) + pml_single_bytes(rk) + 64;
  }
};

// Storage conversions.  BF16/FP16 registers hold value * scale (a power of two per
// component group, so scaling is exact); arithmetic is FP32.
template <class S> __device__ __forceinline__ float to_f(S v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float to_f<__half>(__half v) { return __half2float(v); }
template <class S> __device__ __forceinline__ S from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <class S>
constexpr bool is_f32_v = std::is_same<S, float>::value;

#define MCA_1 (-0.30874f)
#define MCA0 (-0.6326f)
#define MCA1 (1.233f)
#define MCA2 (-0.3334f)
#define MCA3 (0.04168f)

// ---- PTX helpers: mbarrier and TMA --------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false after WAIT_SPINS unsuccessful polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int spins = WAIT_SPINS) {
  for (int n = 0; n < spins; ++n)
    if (mbar_try(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void mbar_inval(uint32_t bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// 5-D tiled load (the PML faces: x, y, z, variable, register set); the descriptor may sit
// in device memory.
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int v, int r,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(v), "r"(r), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int w,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}
// Same with an L2 cache policy (createpolicy) attached.
__device__ __forceinline__ void tma_load_4d_hint(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int w,
                                                 uint32_t bar, uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, %3, "
      "%4, %5}], [%6], %7;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar), "l"(policy)
      : "memory");
}
// L2 policies: streams with no reuse inside the launch are marked evict-first so that the
// stage input planes, which neighbouring tiles and later planes re-read, stay in L2.
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_stream(float* p, float v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(policy) : "memory");
}
__device__ __forceinline__ float ld_stream(const float* p, uint64_t policy) {
  float v;
  asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(policy));
  return v;
}
// read of a location this thread writes back afterwards (not the non-coherent path)
__device__ __forceinline__ float ld_rw_stream(const float* p, uint64_t policy) {
  float v;
  asm volatile("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(policy) : "memory");
  return v;
}

// streaming store of one register element in its storage type
template <class S>
__device__ __forceinline__ void st_stream_s(S* p, S v, uint64_t policy);
template <>
__device__ __forceinline__ void st_stream_s<float>(float* p, float v, uint64_t policy) {
  st_stream(p, v, policy);
}
template <>
__device__ __forceinline__ void st_stream_s<__nv_bfloat16>(__nv_bfloat16* p, __nv_bfloat16 v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.b16 [%0], %1, %2;" ::"l"(p), "h"(__bfloat16_as_ushort(v)), "l"(policy)
               : "memory");
}
template <>
__device__ __forceinline__ void st_stream_s<__half>(__half* p, __half v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.b16 [%0], %1, %2;" ::"l"(p), "h"(__half_as_ushort(v)), "l"(policy)
               : "memory");
}

// ---- one-sided operators ------------------------------------------------------------
// DRP/opt MacCormack operators (mod_macdrp.h:69-103) on values at offsets -3..+3 of c.
template <int F>
__device__ __forceinline__ float dop(const float* c, int s) {
  if (F)
    return MCA_1 * c[-s] + MCA0 * c[0] + MCA1 * c[s] + MCA2 * c[2 * s] + MCA3 * c[3 * s];
  else
    return -MCA3 * c[-3 * s] - MCA2 * c[-2 * s] - MCA1 * c[-s] - MCA0 * c[0] - MCA_1 * c[s];
}
// Same operator on stored values (converted to FP32 element by element).
template <int F, class S>
__device__ __forceinline__ float dopS(const S* c, int s) {
  if constexpr (is_f32_v<S>) {
    return dop<F>(c, s);
  } else if (F) {
    return MCA_1 * to_f(c[-s]) + MCA0 * to_f(c[0]) + MCA1 * to_f(c[s]) + MCA2 * to_f(c[2 * s]) +
           MCA3 * to_f(c[3 * s]);
  } else {
    return -MCA3 * to_f(c[-3 * s]) - MCA2 * to_f(c[-2 * s]) - MCA1 * to_f(c[-s]) - MCA0 * to_f(c[0]) -
           MCA_1 * to_f(c[s]);
  }
}
// Same operator on a five-entry z queue (F: planes -1..+3, B: planes -3..+1).
template <int F>
__device__ __forceinline__ float dopq(const float* q) {
  if (F)
    return MCA_1 * q[0] + MCA0 * q[1] + MCA1 * q[2] + MCA2 * q[3] + MCA3 * q[4];
  else
    return -MCA3 * q[0] - MCA2 * q[1] - MCA1 * q[2] - MCA0 * q[3] - MCA_1 * q[4];
}
// 2-2 and 2-4 MacCormack operators of CondFreeVLOW (mod_macdrp.h:230-268) on the queue.
template <int F>
__device__ __forceinline__ float dop22q(const float* q) {
  if (F) return -1.0f * q[1] + 1.0f * q[2];  // centre at q[1]
  else return -1.0f * q[2] - -1.0f * q[3];   // centre at q[3]
}
template <int F>
__device__ __forceinline__ float dop24q(const float* q) {
  const float A0 = -7.0f / 6.0f, A1 = 8.0f / 6.0f, A2 = -1.0f / 6.0f;
  if (F) return A0 * q[1] + A1 * q[2] + A2 * q[3];
  else return -A2 * q[1] - A1 * q[2] - A0 * q[3];
}

// T*Src / V*Src (comp 0 x, 1 y, 2 z) at an interior column for global stage gst:
// src_surface (mod_src.F90:373-414), the last window of the last force wins.
__device__ __forceinline__ float surf_val(const Sources& S, const float* tab, int gst, int comp, int i, int j) {
  float v = 0.0f;
  for (int e = 0; e < S.nsurf; ++e)
    if (S.surf_ij[2 * e] == i && S.surf_ij[2 * e + 1] == j)
      v = S.surf_q[3 * e + comp] * tab[(long long)gst * S.nw_f + S.surf_w[e]];
  return v;
}

// One CTA's work: columns [bx*TX, +TX) x [by*TY, +TY) of the interior, planes
// [bz*kc, +kc).  Returns false when a bounded wait gave up (error word set).  The
// mbarriers are initialised on entry and invalidated on a normal exit, so a persistent
// CTA can run several work items in turn.
// LEAN: the item holds no PML slab point, no source box and no plane within 4 of a free
// surface (the host classifies the items); that code is compiled out, and the RK
// registers m and t are read from global memory instead of being staged, so that the
// lean form fits three CTAs per SM (registers and shared memory).
template <class S, bool EXACT, int FX, int FY, int FZ, int RKV, bool LEAN, bool TOPO, int TY>
__device__ __forceinline__ bool stage_body(const StageArgs& A, int bx, int by, int bz, unsigned char* smem) {
  static_assert(!EXACT || is_f32_v<S>, "the reference-order form exists for FP32 storage only");
  static_assert(!TOPO || (is_f32_v<S> && !LEAN), "the terrain form is FP32, full form");
  static_assert(RKV <= 2 || !EXACT, "the stages without t are fast forms");
  // RK: the reference kind whose data movement this stage follows (kinds in kernels.h);
  // NO_T: the stage neither reads nor writes t; RECON: stage 3 forming t from W2, W3, W4, m
  // (A.tm_t / PML set pml_set[2] then hold W2, which the stage overwrites with W4, and
  // A.wt / A.at receive t)
  constexpr int RK = rk_base(RKV);
  constexpr bool NO_T = RKV == 3 || RKV == 4;
  constexpr bool RECON = RKV == 5;
  using L = Lay<S, TOPO, TY>;
  constexpr int TBY = L::TBY;
  constexpr int NQ = L::NQ;
  constexpr int TBX = L::TBX, HX = L::HX;
  constexpr int BUF_BYTES = LEAN ? L::BUF_BYTES_LEAN : L::buf_full(RK), OFF_Q = LEAN ? L::OFF_Q_L : L::OFF_Q,
                OFF_MED = LEAN ? L::OFF_MED_L : L::OFF_MED, OFF_M = L::OFF_M, OFF_T = L::OFF_T;
  // PML staging (full form): faces staged per item; the input variables at OFF_PA of each
  // pipeline buffer, the m / t variables (NROLE_S roles) in the area at OFF_PS
  constexpr int NSLOT = LEAN ? 0 : L::pml_slots(RK);
  constexpr int NROLE_S = L::pml_single_roles(RK);
  constexpr int NROLE_B = L::pml_buf_roles(RK);
  constexpr int OFF_PA = L::off_pa(RK), OFF_PB = L::off_pb(RK);
  constexpr int OFF_PS = 2 * BUF_BYTES;
  constexpr int OFF_BAR = LEAN ? L::OFF_MT_L + L::template SZ_MT_L<RK> : OFF_PS + L::pml_single_bytes(RK);
  constexpr int HY = FY ? 1 : 3;  // row of the CTA's first row inside the tile box (tile_halo_y)
  const Geom& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = g.i1 + bx * TX, j0 = g.j1 + by * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool act = i <= g.i2 && j <= g.j2;  // interior point owned by this thread
  int kb, ke;
  stage_chunk(g, A.kc, A.kz_lo, A.kz_hi, bz, &kb, &ke);
  if (kb > ke) return true;
  const int px = g.px, plane = int(g.plane);
  const long long fs = g.fstride;
  const int col = (i + PADL) + px * j;
  const S* __restrict__ W = static_cast<const S*>(A.win);
  S* __restrict__ Wout = static_cast<S*>(A.wout);
  S* __restrict__ Wt = static_cast<S*>(A.wt);
  // stored -> physical value of component f, and back (BF16/FP16 registers are scaled)
  auto dec = [&](S v, int f) -> float {
    if constexpr (is_f32_v<S>) return to_f(v);
    else return to_f(v) * (f < 3 ? A.isv : A.ist);
  };
  auto enc = [&](float v, int f) -> S {
    if constexpr (is_f32_v<S>) return from_f<S>(v);
    else return from_f<S>(v * (f < 3 ? A.sv : A.st));
  };
  auto unscale = [&](float v, int f) -> float {
    if constexpr (is_f32_v<S>) return v;
    else return v * (f < 3 ? A.isv : A.ist);
  };
  const int gst = __ldg(A.ntime) * 4 + A.stage;
  const bool fsurf = !LEAN && g.freesurf != 0;
  const Sources& Src = A.src;

  constexpr int LEAD = FZ ? 3 : 1;   // planes ahead of k in the z operator
  constexpr int TRAIL = FZ ? 1 : 3;  // planes behind k
  // Full form, RK inn/fin: the RK registers of a plane complete on a barrier of their own
  // (one per buffer), so the stencil starts as soon as the tile, the z-queue plane and the
  // medium are in, while m and t are still arriving; they are waited for at the RK update.
  constexpr bool SPLIT = !LEAN && RK >= 1;
  constexpr uint32_t TX_BYTES = (LEAN ? 8 * L::SZ_PLANE : L::SZ_TILE) + L::SZ_Q + L::SZ_MED + L::SZ_TOPO;
  constexpr uint32_t RKR_BYTES = SPLIT ? (RK == 1 && !NO_T ? 2 : 1) * L::SZ_PT : 0;
  constexpr uint32_t MT_BYTES = NO_T ? (RK == 1 ? L::SZ_PT : 0) : L::template SZ_MT_L<RK>;  // lean: m and t of one plane

  const uint32_t bar0 = smem_u32(smem + OFF_BAR);
  const uint32_t bar_mt = bar0 + 16;
  auto bar_rk = [&](int b) -> uint32_t { return bar0 + 24 + 8 * b; };
  const uint32_t bar_pml = bar0 + 40;
  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    if (LEAN && RK >= 1) mbar_init(bar_mt, 1);
    if (NSLOT > 0 && NROLE_S > 0) mbar_init(bar_pml, 1);
    if (SPLIT) {
      mbar_init(bar_rk(0), 1);
      mbar_init(bar_rk(1), 1);
    }
    fence_barrier_init();
  }
  __syncthreads();

  // PML faces whose memory variables this item stages through shared memory (the first
  // NSLOT faces, in face order, that overlap the item): slot per face in 4-bit fields, 15
  // for a face read from global memory.
  unsigned slots = 0xFFFFFFu, staged = 0u;
  if (NSLOT > 0) {
    const int ie = min(i0 + TX - 1, g.i2), je = min(j0 + TY - 1, g.j2);
    int nq = 0;
#pragma unroll 1
    for (int sidx = 0; sidx < 6 && nq < NSLOT; ++sidx) {
      const Slab& sl = A.slab[sidx];
      if (sl.on && sl.i1 <= ie && sl.i2 >= i0 && sl.j1 <= je && sl.j2 >= j0 && sl.k1 <= ke && sl.k2 >= kb) {
        slots = (slots & ~(15u << (4 * sidx))) | (unsigned(nq) << (4 * sidx));
        staged |= 1u << sidx;
        ++nq;
      }
    }
  }
  // Staged faces holding plane kp (the same count in every thread).
  auto n_staged = [&](int kp) -> uint32_t {
    uint32_t n = 0;
#pragma unroll 1
    for (unsigned mk = staged; mk; mk &= mk - 1) {
      const Slab& sl = A.slab[__ffs(mk) - 1];
      n += (kp >= sl.k1 && kp <= sl.k2) ? 1u : 0u;
    }
    return n;
  };
  // One TMA box (TX x TY x 1 plane x 6 variables) of register set `set` of every staged face
  // holding plane kp, face slot q at dst + q * SZ_PML_PLANE * per_slot.  The box origin
  // (i0 - ox) is 16-byte aligned by the padded slab layout; parts outside the face read 0
  // and are never used.
  auto load_faces = [&](uint32_t dst, int per_slot, int kp, int set, uint32_t bar) {
#pragma unroll 1
    for (unsigned mk = staged; mk; mk &= mk - 1) {
      const int sidx = __ffs(mk) - 1;
      const Slab& sl = A.slab[sidx];
      if (kp < sl.k1 || kp > sl.k2) continue;
      const int q = int((slots >> (4 * sidx)) & 15u);
      tma_load_5d(dst + uint32_t(q * per_slot * L::SZ_PML_PLANE), A.pml_map + sidx, i0 - sl.ox, j0 - sl.j1,
                  kp - sl.k1, 0, set, bar);
    }
  };
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  auto issue = [&](int kp, int b) {
    const uint32_t base = smem_u32(smem + b * BUF_BYTES);
    const uint32_t bar = bar0 + 8 * b;
    fence_proxy_async();
    // the staged faces' input variables of plane kp ride with the tile
    const uint32_t npa = NSLOT > 0 ? n_staged(kp) : 0u;
    mbar_expect_tx(bar, TX_BYTES + npa * uint32_t((1 + NROLE_B) * L::SZ_PML_PLANE));
    if (npa) {
      load_faces(base + OFF_PA, 1, kp, A.pml_set[0], bar);
      if (NROLE_B > 0) load_faces(base + OFF_PB, 1, kp, A.pml_set[2], bar);
    }
    if (LEAN) {
      tma_load_4d(base, &A.tm_tile_lo, i0 - HX + PADL, j0 - HY, kp, 0, bar);
      tma_load_4d(base + L::OFF_HI_L, &A.tm_tile_hi, i0 - HX + PADL, j0 - HY, kp, 4, bar);
    } else {
      tma_load_4d(base, &A.tm_tile, i0 - HX + PADL, j0 - HY, kp, 0, bar);
    }
    // plane kp+LEAD comes back as the tile of a later iteration: keep it in L2
    tma_load_4d_hint(base + OFF_Q, &A.tm_q, i0 + PADL, j0, kp + LEAD, 0, bar, pol_keep);
    tma_load_4d_hint(base + OFF_MED, &A.tm_med, i0 + PADL, j0, kp, 0, bar, pol_stream);
    if (TOPO) tma_load_4d_hint(base + L::OFF_TOPO, &A.tm_topo, i0 + PADL, j0, kp, 0, bar, pol_stream);
    if (SPLIT) {
      const uint32_t brk = bar_rk(b);
      mbar_expect_tx(brk, RKR_BYTES);
      if (RK == 1) tma_load_4d_hint(base + OFF_M, &A.tm_m, i0 + PADL, j0, kp, 0, brk, pol_stream);
      if (!NO_T) tma_load_4d_hint(base + OFF_T, &A.tm_t, i0 + PADL, j0, kp, 0, brk, pol_stream);
    }
  };
  if (tid == 0) issue(kb, 0);
  // lean form: m and t of plane kp into the single RK buffer
  auto issue_mt = [&](int kp) {
    const uint32_t base = smem_u32(smem + L::OFF_MT_L);
    fence_proxy_async();
    mbar_expect_tx(bar_mt, MT_BYTES);
    if (RK == 1) tma_load_4d_hint(base, &A.tm_m, i0 + PADL, j0, kp, 0, bar_mt, pol_stream);
    if (!NO_T) tma_load_4d_hint(base + (RK == 1 ? L::SZ_PT : 0), &A.tm_t, i0 + PADL, j0, kp, 0, bar_mt, pol_stream);
  };

  // T*Src of this column (read on the top planes only)
  float tsx = 0.0f, tsy = 0.0f, tsz = 0.0f;
  if (fsurf && act && ke >= g.k2 - 3) {
    tsx = surf_val(Src, Src.disp, gst, 0, i, j);
    tsy = surf_val(Src, Src.disp, gst, 1, i, j);
    tsz = surf_val(Src, Src.disp, gst, 2, i, j);
  }
  // value pushed into the z queue for component qf (0..5 = storage index) at plane kk
  auto qval = [&](int qf, float raw, int kk) -> float {
    if (qf >= TZZ && qf <= TYZ && fsurf && kk >= g.k2) {  // free_timg image (mod_macdrp.F90:3414-3436)
      const float ts = qf == TZZ ? tsz : (qf == TXZ ? tsx : tsy);
      if (kk == g.k2) return ts;
      return 2.0f * ts - dec(W[qf * fs + col + (2 * g.k2 - kk) * plane], qf);
    }
    return raw;
  };
  // Terrain form: the column's surface normal m = (m1, m2, 1) scaled to a unit radial
  // part; a column slopes when m1 or m2 is non-zero (flat columns run the flat path).
  float m1s = 0.0f, m2s = 0.0f;
  if (TOPO && act) {
    m1s = __ldg(A.topo_sf + col);
    m2s = __ldg(A.topo_sf + plane + col);
  }
  const bool slope = TOPO && (m1s != 0.0f || m2s != 0.0f);
  // Terrain form, one plane's nine values as the queue holds them.  In a sloping column
  // the planes above the free surface carry the traction image G = sigma . m (slots Txz,
  // Tyz, Tzz: G_x, G_y, G_z, antisymmetric about the surface around T*Src; slots Txx,
  // Tyy, Txy: zero), and the surface plane's Txz, Tyz, Tzz are set so that sigma . m =
  // T*Src there.  Flat columns take free_timg's images.
  auto topo_img = [&](float* v, int kk) {
    if (!(fsurf && kk >= g.k2)) return;
    if (!slope) {
#pragma unroll
      for (int f = TZZ; f <= TYZ; ++f) v[f] = qval(f, v[f], kk);
      return;
    }
    if (kk == g.k2) {
      const float sxz = tsx - m1s * v[TXX] - m2s * v[TXY];
      const float syz = tsy - m1s * v[TXY] - m2s * v[TYY];
      v[TXZ] = sxz;
      v[TYZ] = syz;
      v[TZZ] = tsz - m1s * sxz - m2s * syz;
      return;
    }
    const long long pm = col + (long long)(2 * g.k2 - kk) * plane;
    const float xx = dec(W[TXX * fs + pm], TXX), yy = dec(W[TYY * fs + pm], TYY), xy = dec(W[TXY * fs + pm], TXY);
    const float xz = dec(W[TXZ * fs + pm], TXZ), yz = dec(W[TYZ * fs + pm], TYZ), zz = dec(W[TZZ * fs + pm], TZZ);
    v[TXZ] = 2.0f * tsx - (xz + m1s * xx + m2s * xy);
    v[TYZ] = 2.0f * tsy - (yz + m1s * xy + m2s * yy);
    v[TZZ] = 2.0f * tsz - (zz + m1s * xz + m2s * yz);
    v[TXX] = 0.0f;
    v[TYY] = 0.0f;
    v[TXY] = 0.0f;
  };

  float q[NQ][5];
  if constexpr (TOPO) {
#pragma unroll
    for (int f = 0; f < NQ; ++f) q[f][0] = 0.0f;
#pragma unroll
    for (int d = 1; d < 5; ++d) {
      const int kk = kb - TRAIL + d - 1;
      float v[NF];
#pragma unroll
      for (int f = 0; f < NF; ++f) v[f] = act ? dec(W[f * fs + col + kk * plane], f) : 0.0f;
      if (act) topo_img(v, kk);
#pragma unroll
      for (int f = 0; f < NF; ++f) q[f][d] = v[f];
    }
  } else {
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      q[f][0] = 0.0f;
#pragma unroll
      for (int d = 1; d < 5; ++d) {
        const int kk = kb - TRAIL + d - 1;
        q[f][d] = act ? qval(f, dec(W[f * fs + col + kk * plane], f), kk) : 0.0f;
      }
    }
  }

  const float xi = act ? __ldg(A.xi_x + i) : 0.0f;
  const float et = act ? __ldg(A.eta_y + j) : 0.0f;
  const float xs = act ? __ldg(A.xsin + i) : 1.0f;
  const float c = act ? __ldg(A.xcot + i) : 0.0f;
  const float rs = act ? __ldg(A.rsinv + i) : 0.0f;

  // Does this CTA's block of points touch any smoothed source box?  (tested once here
  // instead of per point and plane)
  bool cta_src = false;
  for (int n = 0; !LEAN && n < Src.nforce && !cta_src; ++n)
    cta_src = Src.force_c[3 * n] + 3 >= i0 && Src.force_c[3 * n] - 3 <= i0 + TX - 1 && Src.force_c[3 * n + 1] + 3 >= j0 &&
              Src.force_c[3 * n + 1] - 3 <= j0 + TY - 1 && Src.force_c[3 * n + 2] + 3 >= kb && Src.force_c[3 * n + 2] - 3 <= ke;
  for (int n = 0; !LEAN && n < Src.nmom && !cta_src; ++n)
    cta_src = Src.mom_c[3 * n] + 3 >= i0 && Src.mom_c[3 * n] - 3 <= i0 + TX - 1 && Src.mom_c[3 * n + 1] + 3 >= j0 &&
              Src.mom_c[3 * n + 1] - 3 <= j0 + TY - 1 && Src.mom_c[3 * n + 2] + 3 >= kb && Src.mom_c[3 * n + 2] - 3 <= ke;

  // PML slabs holding this column: the x and y slabs span every plane, so their
  // membership is fixed per thread (bits 0-3: x1 x2 y1 y2); the z slabs (bits 4, 5) are
  // tested per plane, uniformly across the CTA.
  unsigned xymask = 0;
  if (!LEAN && act)
#pragma unroll
    for (int sidx = 0; sidx < 4; ++sidx) {
      const Slab& sl = A.slab[sidx];
      if (sl.on && i >= sl.i1 && i <= sl.i2 && j >= sl.j1 && j <= sl.j2) xymask |= 1u << sidx;
    }
  auto slab_mask = [&](int kp) -> unsigned {
    if (LEAN) return 0u;
    unsigned m = act ? xymask : 0u;
    if (act && A.slab[4].on && kp >= A.slab[4].k1 && kp <= A.slab[4].k2) m |= 16u;
    if (act && A.slab[5].on && kp >= A.slab[5].k1 && kp <= A.slab[5].k2) m |= 32u;
    return m;
  };

  // Prefetch into L1 the PML memory variables of this point on plane kp (their global
  // loads then hit L1 instead of exposing DRAM latency inside the compute).
  auto prefetch_pml = [&](int kp) {
#pragma unroll 1
    for (unsigned mk = slab_mask(kp) & ~staged; mk; mk &= mk - 1) {
      const int sidx = __ffs(mk) - 1;
      const Slab& sl = A.slab[sidx];
      const int qa = (i - sl.ox) + sl.sx * ((j - sl.j1) + sl.sy * (kp - sl.k1));
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        asm volatile("prefetch.global.L1 [%0];" ::"l"(A.ain[sidx] + qa + v * sl.vstride));
        if (RK >= 1 && !NO_T)
          asm volatile("prefetch.global.L1 [%0];" ::"l"((RECON ? A.aout[sidx] : A.at[sidx]) + qa + v * sl.vstride));
        if (RK == 1) asm volatile("prefetch.global.L1 [%0];" ::"l"(A.am[sidx] + qa + v * sl.vstride));
      }
    }
  };
  if (!LEAN) prefetch_pml(kb);

  // m / t variables of plane kp into the single area (thread 0); bytes (all threads)
  auto issue_pml_mt = [&](int kp) -> uint32_t {
    constexpr int NLOAD = NO_T ? (NROLE_S > 0 ? 1 : 0) : NROLE_S;  // roles loaded (no t: m only)
    const uint32_t bytes = NLOAD > 0 ? n_staged(kp) * uint32_t(NLOAD * L::SZ_PML_PLANE) : 0u;
    if (bytes == 0 || tid != 0) return bytes;
    fence_proxy_async();
    mbar_expect_tx(bar_pml, bytes);
    const uint32_t base = smem_u32(smem + OFF_PS);
    load_faces(base, NROLE_S, kp, A.pml_set[1], bar_pml);  // m
    if (!NO_T) load_faces(base + uint32_t(L::SZ_PML_PLANE), NROLE_S, kp, A.pml_set[2], bar_pml);  // t
    return bytes;
  };
  int pml_ph = 0;  // completed PML staging phases

  int it = 0;
  for (int k = kb; k <= ke; ++k, ++it) {
    const int cur = it & 1;
    // (every thread finished the previous plane, so the RK buffer is free)
    if (LEAN && RK >= 1 && tid == 0) issue_mt(k);
    if (tid == 0 && k < ke) issue(k + 1, cur ^ 1);
    // this plane's staged PML m / t variables (the previous plane's readers are done)
    const uint32_t pml_k = NSLOT > 0 ? issue_pml_mt(k) : 0u;
    if (!LEAN && k < ke) prefetch_pml(k + 1);
    const bool ok = mbar_wait(bar0 + 8 * cur, (it >> 1) & 1);
    unsigned char* buf = smem + cur * BUF_BYTES;
    // component f of the halo'd tile (the lean tile has no Tzz)
    auto tl = [&](int f) -> S(*)[TBX] {
      if constexpr (LEAN)
        return reinterpret_cast<S(*)[TBX]>(buf + (f < 3 ? f * L::SZ_PLANE : L::OFF_HI_L + (f - 4) * L::SZ_PLANE));
      else
        return reinterpret_cast<S(*)[TBX]>(buf + f * L::SZ_PLANE);
    };
    const S(*qs)[TY][TX] = reinterpret_cast<const S(*)[TY][TX]>(buf + OFF_Q);
    const float(*med)[TY][TX] = reinterpret_cast<const float(*)[TY][TX]>(buf + OFF_MED);
    const S(*mbuf)[TY][TX] = reinterpret_cast<const S(*)[TY][TX]>(LEAN ? smem + L::OFF_MT_L : buf + OFF_M);
    const S(*tbuf)[TY][TX] = reinterpret_cast<const S(*)[TY][TX]>(
        LEAN ? smem + L::OFF_MT_L + (RK == 1 ? L::SZ_PT : 0) : buf + OFF_T);
    const bool top = fsurf && k == g.k2;
    if (top) {
      // the imaged stress components read T*Src on the free surface (interior columns)
      if (ok)
        for (int e = tid; e < TBX * TBY; e += TX * TY) {
          const int r = e / TBX, cc = e % TBX;
          const int ii = i0 - HX + cc, jj = j0 - HY + r;
          if (ii >= g.i1 && ii <= g.i2 && jj >= g.j1 && jj <= g.j2) {
            const float ux = surf_val(Src, Src.disp, gst, 0, ii, jj);
            const float uy = surf_val(Src, Src.disp, gst, 1, ii, jj);
            const float uz = surf_val(Src, Src.disp, gst, 2, ii, jj);
            float e1 = 0.0f, e2 = 0.0f;
            if (TOPO) {
              const int cq = (ii + PADL) + px * jj;
              e1 = __ldg(A.topo_sf + cq);
              e2 = __ldg(A.topo_sf + plane + cq);
            }
            if (TOPO && (e1 != 0.0f || e2 != 0.0f)) {  // sloping column: sigma . m = T*Src
              const float xx = dec(tl(TXX)[r][cc], TXX), yy = dec(tl(TYY)[r][cc], TYY);
              const float xy = dec(tl(TXY)[r][cc], TXY);
              const float sxz = ux - e1 * xx - e2 * xy, syz = uy - e1 * xy - e2 * yy;
              tl(TXZ)[r][cc] = enc(sxz, TXZ);
              tl(TYZ)[r][cc] = enc(syz, TYZ);
              tl(TZZ)[r][cc] = enc(uz - e1 * sxz - e2 * syz, TZZ);
            } else {
              tl(TXZ)[r][cc] = enc(ux, TXZ);
              tl(TYZ)[r][cc] = enc(uy, TYZ);
              tl(TZZ)[r][cc] = enc(uz, TZZ);
            }
          }
        }
      __syncthreads();
    }

    bool ok_mt = true, ok_p = true;
    if (ok && act) {
      // advance the z queue with plane k+LEAD (the image applies on and above the surface)
      const bool img = fsurf && k + LEAD >= g.k2;
      if constexpr (TOPO) {
        float v[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] = dec(qs[f][ty][tx], f);
        if (img) topo_img(v, k + LEAD);
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          q[f][0] = q[f][1]; q[f][1] = q[f][2]; q[f][2] = q[f][3]; q[f][3] = q[f][4];
          q[f][4] = v[f];
        }
      } else {
#pragma unroll
        for (int f = 0; f < 6; ++f) {
          q[f][0] = q[f][1]; q[f][1] = q[f][2]; q[f][2] = q[f][3]; q[f][3] = q[f][4];
          q[f][4] = img ? qval(f, dec(qs[f][ty][tx], f), k + LEAD) : dec(qs[f][ty][tx], f);
        }
      }
      const unsigned pmask = slab_mask(k);
      const int p = col + k * plane;
      const float lam = med[0][ty][tx], miu = med[1][ty][tx], rhov = med[2][ty][tx];
      // terrain form: r, zeta_r, zeta_theta / r, zeta_phi / (r sin theta) of the point
      const float(*tpo)[TY][TX] = reinterpret_cast<const float(*)[TY][TX]>(buf + L::OFF_TOPO);
      const float ze = TOPO ? tpo[1][ty][tx] : __ldg(A.zeta_z + k);
      const int r0 = ty + HY, c0 = tx + HX;
      // stencil sums along x (tile rows), y (tile columns), z (queue)
      const float sxTxx = unscale(dopS<FX>(&tl(TXX)[r0][c0], 1), TXX);
      const float sxTxy = unscale(dopS<FX>(&tl(TXY)[r0][c0], 1), TXY);
      const float sxTxz = unscale(dopS<FX>(&tl(TXZ)[r0][c0], 1), TXZ);
      const float sxVx = unscale(dopS<FX>(&tl(VX)[r0][c0], 1), VX);
      const float sxVy = unscale(dopS<FX>(&tl(VY)[r0][c0], 1), VY);
      const float sxVz = unscale(dopS<FX>(&tl(VZ)[r0][c0], 1), VZ);
      const float syTyy = unscale(dopS<FY>(&tl(TYY)[r0][c0], TBX), TYY);
      const float syTxy = unscale(dopS<FY>(&tl(TXY)[r0][c0], TBX), TXY);
      const float syTyz = unscale(dopS<FY>(&tl(TYZ)[r0][c0], TBX), TYZ);
      const float syVx = unscale(dopS<FY>(&tl(VX)[r0][c0], TBX), VX);
      const float syVy = unscale(dopS<FY>(&tl(VY)[r0][c0], TBX), VY);
      const float syVz = unscale(dopS<FY>(&tl(VZ)[r0][c0], TBX), VZ);
      const float szTzz = dopq<FZ>(q[TZZ]);
      const float szTxz = dopq<FZ>(q[TXZ]);
      const float szTyz = dopq<FZ>(q[TYZ]);
      float szVx, szVy, szVz;
      if (fsurf && k == g.k2 - 1) {
        szVx = dop22q<FZ>(q[VX]); szVy = dop22q<FZ>(q[VY]); szVz = dop22q<FZ>(q[VZ]);
      } else if (fsurf && k == g.k2 - 2) {
        szVx = dop24q<FZ>(q[VX]); szVy = dop24q<FZ>(q[VY]); szVz = dop24q<FZ>(q[VZ]);
      } else {
        szVx = dopq<FZ>(q[VX]); szVy = dopq<FZ>(q[VY]); szVz = dopq<FZ>(q[VZ]);
      }
      const float Vx = q[VX][TRAIL], Vy = q[VY][TRAIL], Vz = q[VZ][TRAIL];
      const float Tzz = q[TZZ][TRAIL], Txz = q[TXZ][TRAIL], Tyz = q[TYZ][TRAIL];
      const float Txx = dec(tl(TXX)[r0][c0], TXX), Tyy = dec(tl(TYY)[r0][c0], TYY);
      const float Txy = dec(tl(TXY)[r0][c0], TXY);
      const bool water = miu <= 1.0e-20f;

      float hVx, hVy, hVz, hTxx, hTyy, hTzz, hTxy, hTxz, hTyz;
      // PML derivative terms per axis: [0..2] stress terms of hVx,hVy,hVz; [3..5] Vx,Vy,Vz
      float dx_[6], dy_[6], dz_[6];
      const float lam2mu = lam + 2.0f * miu;
      float rrho;
      // Terrain form, sloping column: the zeta parts of the theta and phi derivatives (in
      // the top three planes the stress terms use the column's surface normal, so that
      // with the traction images they form d(sigma . m)/dzeta), and on the free surface the
      // traction condition sigma . m = T*Src: the velocity's zeta-derivatives u solve
      // M u = dT*Src/dt - S0 . m (M^-1 precomputed), S0 the stress of the strain without
      // its zeta parts (e13z, e23z: E13, E23 without them; E11, E12, E22 have none).
      auto topo_slope = [&](auto& hVx_, auto& hVy_, auto& hVz_, auto& E11_, auto& E22_, auto& E12_, auto& E33_,
                            auto& E13_, auto& E23_, float e13z, float e23z, float rrho_) {
        const float bxv = tpo[2][ty][tx], byv = tpo[3][ty][tx];
        const bool top3 = fsurf && k >= g.k2 - 2;
        const float bxm = top3 ? ze * m1s : bxv, bym = top3 ? ze * m2s : byv;
        const float szTxx = dopq<FZ>(q[TXX]), szTyy = dopq<FZ>(q[TYY]), szTxy = dopq<FZ>(q[TXY]);
        hVx_ = hVx_ + rrho_ * (szTxx * bxm + (water ? 0.0f : szTxy * bym));
        hVy_ = hVy_ + rrho_ * ((water ? 0.0f : szTxy * bxm) + szTyy * bym);
        hVz_ = hVz_ + rrho_ * ((water ? 0.0f : szTxz * bxm) + (water ? 0.0f : szTyz * bym));
        if (top) {
          const float S11 = lam2mu * E11_ + lam * E22_, S22 = lam2mu * E22_ + lam * E11_, S33 = lam * (E11_ + E22_);
          const float S12 = 2.0f * miu * E12_, S13 = 2.0f * miu * e13z, S23 = 2.0f * miu * e23z;
          const float r0 = surf_val(Src, Src.rate, gst, 0, i, j) - (S11 * m1s + S12 * m2s + S13);
          const float r1 = surf_val(Src, Src.rate, gst, 1, i, j) - (S12 * m1s + S22 * m2s + S23);
          const float r2 = surf_val(Src, Src.rate, gst, 2, i, j) - (S13 * m1s + S23 * m2s + S33);
          const float* mi = A.topo_sf + 2 * plane + col;
          const float ux = __ldg(mi) * r0 + __ldg(mi + plane) * r1 + __ldg(mi + 2 * plane) * r2;
          const float uy = __ldg(mi + 3 * plane) * r0 + __ldg(mi + 4 * plane) * r1 + __ldg(mi + 5 * plane) * r2;
          const float uz = __ldg(mi + 6 * plane) * r0 + __ldg(mi + 7 * plane) * r1 + __ldg(mi + 8 * plane) * r2;
          E11_ = E11_ + bxv * ux;
          E22_ = E22_ + byv * uy;
          E12_ = E12_ + 0.5f * (bxv * uy + byv * ux);
          E33_ = ze * uz;
          E13_ = e13z + 0.5f * (bxv * uz + ze * ux);
          E23_ = e23z + 0.5f * (byv * uz + ze * uy);
        } else {
          E11_ = E11_ + bxv * szVx;
          E22_ = E22_ + byv * szVy;
          E12_ = E12_ + 0.5f * (bxv * szVy + byv * szVx);
          E13_ = E13_ + 0.5f * bxv * szVz;
          E23_ = E23_ + 0.5f * byv * szVz;
        }
      };
      if constexpr (EXACT) {
        // reference operand order, IEEE division (mod_macdrp.F90:928-957)
        const float r = TOPO ? tpo[0][ty][tx] : __ldg(A.zc + k);
        rrho = 1.0f / rhov;
        const float DxTxx = sxTxx * xi, DxTxy = sxTxy * xi, DxTxz = sxTxz * xi;
        const float DxVx = sxVx * xi, DxVy = sxVy * xi, DxVz = sxVz * xi;
        const float DyTyy = syTyy * et, DyTxy = syTxy * et, DyTyz = syTyz * et;
        const float DyVx = syVx * et, DyVy = syVy * et, DyVz = syVz * et;
        const float DzTzz = szTzz * ze, DzTxz = szTxz * ze, DzTyz = szTyz * ze;
        const float DzVx = szVx * ze, DzVy = szVy * ze, DzVz = szVz * ze;
        const float wDxTxy = water ? 0.0f : DxTxy, wDxTxz = water ? 0.0f : DxTxz;
        const float wDyTxy = water ? 0.0f : DyTxy, wDyTyz = water ? 0.0f : DyTyz;
        const float wDzTxz = water ? 0.0f : DzTxz, wDzTyz = water ? 0.0f : DzTyz;
        hVx = rrho * (DxTxx / r + wDyTxy / r / xs + wDzTxz + (3.0f * Txz + Txx * c - Tyy * c) / r);
        hVy = rrho * (wDxTxy / r + DyTyy / r / xs + wDzTyz + (2.0f * Txy * c + 3.0f * Tyz) / r);
        hVz = rrho * (wDxTxz / r + wDyTyz / r / xs + DzTzz + (2.0f * Tzz - Txx - Tyy + Txz * c) / r);
        float E11 = (DxVx + Vz) / r;
        float E22 = (Vx * c + DyVy / xs + Vz) / r;
        float E12 = (DxVy + DyVx / xs - Vy * c) / r / 2.0f;
        float E33 = DzVz;
        float E13 = (DxVz / r + DzVx - Vx / r) / 2.0f;
        float E23 = (DyVz / r / xs + DzVy - Vy / r) / 2.0f;
        if constexpr (TOPO)
          if (slope)
            topo_slope(hVx, hVy, hVz, E11, E22, E12, E33, E13, E23, (DxVz / r - Vx / r) / 2.0f,
                       (DyVz / r / xs - Vy / r) / 2.0f, rrho);
        if (top && !(TOPO && slope)) {
          E33 = -(lam / lam2mu * (E11 + E22)) + surf_val(Src, Src.rate, gst, 2, i, j) / lam2mu;
          E13 = surf_val(Src, Src.rate, gst, 0, i, j) / miu / 2.0f;
          E23 = surf_val(Src, Src.rate, gst, 1, i, j) / miu / 2.0f;
        }
        hTxx = lam2mu * E11 + lam * (E22 + E33);
        hTyy = lam2mu * E22 + lam * (E11 + E33);
        hTzz = lam2mu * E33 + lam * (E11 + E22);
        hTxy = 2.0f * miu * E12;
        hTxz = 2.0f * miu * E13;
        hTyz = 2.0f * miu * E23;
        // PML terms (mod_abs_npml.F90:1179-1301, 1523-1645, 1867-1983)
        if (pmask) {
          dx_[0] = (DxTxx + 2.0f * Txz) / r; dx_[1] = (DxTxy + Tyz) / r; dx_[2] = (DxTxz - Txx + Tzz) / r;
          dx_[3] = (DxVx + Vz) / r; dx_[4] = DxVy / r; dx_[5] = (DxVz - Vx) / r;
          dy_[0] = (DyTxy / xs + (Txx - Tyy) * c + Txz) / r;
          dy_[1] = (DyTyy / xs + 2.0f * Txy * c + 2.0f * Tyz) / r;
          dy_[2] = (DyTyz / xs + Txz * c + (Tzz - Tyy)) / r;
          dy_[3] = (DyVx / xs - Vy * c) / r; dy_[4] = (DyVy / xs + Vx * c + Vz) / r; dy_[5] = (DyVz / xs - Vy) / r;
          dz_[0] = DzTxz; dz_[1] = DzTyz; dz_[2] = DzTzz; dz_[3] = DzVx; dz_[4] = DzVy; dz_[5] = DzVz;
        }
      } else {
        // same equations with the metric folded into one factor per axis
        const float rr = TOPO ? __frcp_rn(tpo[0][ty][tx]) : __ldg(A.rzinv + k);
        rrho = __frcp_rn(rhov);
        const float ax = xi * rr, ay = et * rr * rs;
        const float gxTxx = sxTxx * ax, gxTxy = sxTxy * ax, gxTxz = sxTxz * ax;
        const float gxVx = sxVx * ax, gxVy = sxVy * ax, gxVz = sxVz * ax;
        const float gyTyy = syTyy * ay, gyTxy = syTxy * ay, gyTyz = syTyz * ay;
        const float gyVx = syVx * ay, gyVy = syVy * ay, gyVz = syVz * ay;
        const float gzTzz = szTzz * ze, gzTxz = szTxz * ze, gzTyz = szTyz * ze;
        const float gzVx = szVx * ze, gzVy = szVy * ze, gzVz = szVz * ze;
        const float wxTxy = water ? 0.0f : gxTxy, wxTxz = water ? 0.0f : gxTxz;
        const float wyTxy = water ? 0.0f : gyTxy, wyTyz = water ? 0.0f : gyTyz;
        const float wzTxz = water ? 0.0f : gzTxz, wzTyz = water ? 0.0f : gzTyz;
        hVx = rrho * (gxTxx + wyTxy + wzTxz + (3.0f * Txz + (Txx - Tyy) * c) * rr);
        hVy = rrho * (wxTxy + gyTyy + wzTyz + (2.0f * Txy * c + 3.0f * Tyz) * rr);
        hVz = rrho * (wxTxz + wyTyz + gzTzz + (2.0f * Tzz - Txx - Tyy + Txz * c) * rr);
        float E11 = gxVx + Vz * rr;
        float E22 = (Vx * c + Vz) * rr + gyVy;
        float E12 = 0.5f * (gxVy + gyVx - Vy * c * rr);
        float E33 = gzVz;
        float E13 = 0.5f * (gxVz + gzVx - Vx * rr);
        float E23 = 0.5f * (gyVz + gzVy - Vy * rr);
        if constexpr (TOPO)
          if (slope)
            topo_slope(hVx, hVy, hVz, E11, E22, E12, E33, E13, E23, 0.5f * (gxVz - Vx * rr), 0.5f * (gyVz - Vy * rr),
                       rrho);
        if (top && !(TOPO && slope)) {
          E33 = (surf_val(Src, Src.rate, gst, 2, i, j) - lam * (E11 + E22)) / lam2mu;
          E13 = 0.5f * surf_val(Src, Src.rate, gst, 0, i, j) / miu;
          E23 = 0.5f * surf_val(Src, Src.rate, gst, 1, i, j) / miu;
        }
        hTxx = lam2mu * E11 + lam * (E22 + E33);
        hTyy = lam2mu * E22 + lam * (E11 + E33);
        hTzz = lam2mu * E33 + lam * (E11 + E22);
        hTxy = 2.0f * miu * E12;
        hTxz = 2.0f * miu * E13;
        hTyz = 2.0f * miu * E23;
        if (pmask) {
          dx_[0] = gxTxx + 2.0f * Txz * rr; dx_[1] = gxTxy + Tyz * rr; dx_[2] = gxTxz + (Tzz - Txx) * rr;
          dx_[3] = gxVx + Vz * rr; dx_[4] = gxVy; dx_[5] = gxVz - Vx * rr;
          dy_[0] = gyTxy + ((Txx - Tyy) * c + Txz) * rr;
          dy_[1] = gyTyy + (2.0f * Txy * c + 2.0f * Tyz) * rr;
          dy_[2] = gyTyz + (Txz * c + (Tzz - Tyy)) * rr;
          dy_[3] = gyVx - Vy * c * rr; dy_[4] = gyVy + (Vx * c + Vz) * rr; dy_[5] = gyVz - Vy * rr;
          dz_[0] = gzTxz; dz_[1] = gzTyz; dz_[2] = gzTzz; dz_[3] = gzVx; dz_[4] = gzVy; dz_[5] = gzVz;
        }
      }

      // ---- CFS-PML slabs in the reference's order x1 x2 y1 y2 z1 z2 (additive at corners)
      // staged faces: the input variables in this plane's buffer, m / t in the single area
      // (waited for at their first use)
      const float* pml_a = reinterpret_cast<const float*>(buf + OFF_PA) + ty * TX + tx;
      const float* pml_b = reinterpret_cast<const float*>(buf + OFF_PB) + ty * TX + tx;
      const float* pml_s = reinterpret_cast<const float*>(smem + OFF_PS) + ty * TX + tx;
      bool waited_s = false;
      const float tc13 = lam, tc66 = miu;
      const float tc11 = tc13 + 2.0f * tc66;
      const float tc12 = tc13, tc22 = tc11, tc23 = tc13, tc33 = tc11, tc44 = tc66, tc55 = tc66;
#pragma unroll 1
      for (unsigned mk = pmask; mk; mk &= mk - 1) {
        const int sidx = __ffs(mk) - 1;
        const Slab& sl = A.slab[sidx];
        const int axis = sidx >> 1;
        // staged face: slot q in shared memory, variable v (role r of the m / t area)
        const int q = int((slots >> (4 * sidx)) & 15u);
        const bool stg = NSLOT > 0 && q != 15;
        auto PA = [&](int v) -> float { return pml_a[(q * 6 + v) * TY * TX]; };
        auto PB = [&](int v) -> float { return pml_b[(q * 6 + v) * TY * TX]; };
        auto PS = [&](int r, int v) -> float { return pml_s[((q * NROLE_S + r) * 6 + v) * TY * TX]; };
        const int ia = axis == 0 ? i : (axis == 1 ? j : k);
        const float b1 = __ldg(A.pb1[axis] + ia), b1_1 = __ldg(A.pb11[axis] + ia);
        const float ad = __ldg(A.pad[axis] + ia), Dv = __ldg(A.pD[axis] + ia);
        float d[6];
#pragma unroll
        for (int v = 0; v < 6; ++v) d[v] = axis == 0 ? dx_[v] : (axis == 1 ? dy_[v] : dz_[v]);
        const int qa = (i - sl.ox) + sl.sx * ((j - sl.j1) + sl.sy * (k - sl.k1));
        const long long vs = sl.vstride;
        const float* __restrict__ ai = A.ain[sidx] + qa;
        float av[6], h[6];
#pragma unroll
        for (int v = 0; v < 6; ++v) av[v] = stg ? PA(v) : ld_stream(ai + v * vs, pol_stream);
        hVx = hVx + (b1_1 * d[0] - b1 * av[0]) * rrho; h[0] = Dv * d[0] - ad * av[0];
        hVy = hVy + (b1_1 * d[1] - b1 * av[1]) * rrho; h[1] = Dv * d[1] - ad * av[1];
        hVz = hVz + (b1_1 * d[2] - b1 * av[2]) * rrho; h[2] = Dv * d[2] - ad * av[2];
        if (axis == 0) {
          hTxx = hTxx + b1_1 * tc11 * d[3] - b1 * tc11 * av[3];
          hTyy = hTyy + b1_1 * tc12 * d[3] - b1 * tc12 * av[3];
          hTzz = hTzz + b1_1 * tc13 * d[3] - b1 * tc13 * av[3];
          h[3] = Dv * d[3] - ad * av[3];
          hTxy = hTxy + b1_1 * tc66 * d[4] - b1 * tc66 * av[4];
          h[4] = Dv * d[4] - ad * av[4];
          hTxz = hTxz + b1_1 * tc55 * d[5] - b1 * tc55 * av[5];
          h[5] = Dv * d[5] - ad * av[5];
          if (top) {  // mod_abs_npml.F90:1303-1333
            hTxx = hTxx - b1_1 * tc13 * tc13 / tc33 * d[3] + b1 * tc13 * tc13 / tc33 * av[3];
            hTyy = hTyy - b1_1 * tc23 * tc13 / tc33 * d[3] + b1 * tc23 * tc13 / tc33 * av[3];
          }
        } else if (axis == 1) {
          hTxy = hTxy + b1_1 * tc66 * d[3] - b1 * tc66 * av[3];
          h[3] = Dv * d[3] - ad * av[3];
          hTxx = hTxx + b1_1 * tc12 * d[4] - b1 * tc12 * av[4];
          hTyy = hTyy + b1_1 * tc22 * d[4] - b1 * tc22 * av[4];
          hTzz = hTzz + b1_1 * tc23 * d[4] - b1 * tc23 * av[4];
          h[4] = Dv * d[4] - ad * av[4];
          hTyz = hTyz + b1_1 * tc44 * d[5] - b1 * tc44 * av[5];
          h[5] = Dv * d[5] - ad * av[5];
          if (top) {  // mod_abs_npml.F90:1647-1677
            hTxx = hTxx - b1_1 * tc13 * tc23 / tc33 * d[4] + b1 * tc13 * tc23 / tc33 * av[4];
            hTyy = hTyy - b1_1 * tc23 * tc23 / tc33 * d[4] + b1 * tc23 * tc23 / tc33 * av[4];
          }
        } else {
          hTxz = hTxz + b1_1 * tc55 * d[3] - b1 * tc55 * av[3];
          h[3] = Dv * d[3] - ad * av[3];
          hTyz = hTyz + b1_1 * tc44 * d[4] - b1 * tc44 * av[4];
          h[4] = Dv * d[4] - ad * av[4];
          hTxx = hTxx + b1_1 * tc13 * d[5] - b1 * tc13 * av[5];
          hTyy = hTyy + b1_1 * tc23 * d[5] - b1 * tc23 * av[5];
          hTzz = hTzz + b1_1 * tc33 * d[5] - b1 * tc33 * av[5];
          h[5] = Dv * d[5] - ad * av[5];
        }
        // abs_RK_* (mod_abs_npml.F90:738-1105)
        float* __restrict__ ao = A.aout[sidx] + qa;
        float* __restrict__ at = A.at[sidx] + qa;
        if (NROLE_S > 0 && stg && !waited_s) {
          ok_p = mbar_wait(bar_pml, pml_ph & 1);
          waited_s = true;
        }
#pragma unroll
        for (int v = 0; v < 6 && ok_p; ++v) {
          if (RK == 0) {
            st_stream(ao + v * vs, av[v] + A.a * h[v], pol_stream);
            if (!NO_T) st_stream(at + v * vs, av[v] + A.b * h[v], pol_stream);
          } else if (RK == 1 && NO_T) {
            const float mv = stg ? PS(0, v) : ld_stream(A.am[sidx] + qa + v * vs, pol_stream);
            st_stream(ao + v * vs, mv + A.a * h[v], pol_stream);
          } else if (RK == 1 && RECON) {  // t-in (W2) is the output register set: read first
            const float mv = stg ? PS(0, v) : ld_stream(A.am[sidx] + qa + v * vs, pol_stream);
            const float w2 = stg ? PS(1, v) : ld_rw_stream(ao + v * vs, pol_stream);
            const float d = (w2 - mv) + 2.0f * (av[v] - mv) + A.a * h[v];  // increments, then m
            st_stream(ao + v * vs, mv + A.a * h[v], pol_stream);
            st_stream(at + v * vs, mv + d * (1.0f / 3.0f), pol_stream);
          } else if (RK == 1) {
            const float mv = stg ? PS(0, v) : ld_stream(A.am[sidx] + qa + v * vs, pol_stream);
            const float tv = stg ? PS(1, v) : ld_rw_stream(at + v * vs, pol_stream);
            st_stream(ao + v * vs, mv + A.a * h[v], pol_stream);
            st_stream(at + v * vs, tv + A.b * h[v], pol_stream);
          } else {
            const float tv = stg ? PB(v) : ld_rw_stream(at + v * vs, pol_stream);
            st_stream(at + v * vs, tv + A.b * h[v], pol_stream);
          }
        }
      }

      // ---- moment tensors (src_stress, mod_src.F90:207-273)
#pragma unroll 1
      for (int n = 0; cta_src && n < Src.nmom; ++n) {
        const int li = i - Src.mom_c[3 * n], lj = j - Src.mom_c[3 * n + 1], lk = k - Src.mom_c[3 * n + 2];
        if (li < -3 || li > 3 || lj < -3 || lj > 3 || lk < -3 || lk > 3) continue;
        const int e = n * 343 + (li + 3) + 7 * ((lj + 3) + 7 * (lk + 3));
        if (!Src.mom_on[e]) continue;
        const float dd = Src.mom_d[e], vol = Src.mom_vol[e];
        for (int m = 0; m < Src.ntwin_m; ++m) {
          const float rate = Src.mrate[(long long)gst * Src.nw_m + n * Src.ntwin_m + m];
          const float V = dd * rate / vol;
          const float* M = Src.mom_M + 6 * (n * Src.ntwin_m + m);
          hTxx = hTxx - M[0] * V; hTyy = hTyy - M[1] * V; hTzz = hTzz - M[2] * V;
          hTxy = hTxy - M[3] * V; hTxz = hTxz - M[4] * V; hTyz = hTyz - M[5] * V;
        }
      }
      // ---- body forces (src_force, mod_src.F90:275-345)
#pragma unroll 1
      for (int n = 0; cta_src && n < Src.nforce; ++n) {
        const int li = i - Src.force_c[3 * n], lj = j - Src.force_c[3 * n + 1], lk = k - Src.force_c[3 * n + 2];
        if (li < -3 || li > 3 || lj < -3 || lj > 3 || lk < -3 || lk > 3) continue;
        const int e = n * 343 + (li + 3) + 7 * ((lj + 3) + 7 * (lk + 3));
        if (!Src.force_on[e]) continue;
        const float V = Src.force_wt[e];
        for (int m = 0; m < Src.ntwin_f; ++m) {
          const float disp = Src.disp[(long long)gst * Src.nw_f + n * Src.ntwin_f + m];
          const float* F = Src.force_F + 3 * (n * Src.ntwin_f + m);
          const float fx0 = F[0] * disp, fy0 = F[1] * disp, fz0 = F[2] * disp;
          hVx = hVx + fx0 * V; hVy = hVy + fy0 * V; hVz = hVz + fz0 * V;
        }
      }

      // ---- RK update (mod_macdrp.F90:291-393); m of stage 1 is the stored input value
      if (LEAN && RK >= 1) ok_mt = mbar_wait(bar_mt, it & 1);
      if (SPLIT) ok_mt = mbar_wait(bar_rk(cur), (it >> 1) & 1);
      float hh[NF];
      hh[VX] = hVx; hh[VY] = hVy; hh[VZ] = hVz; hh[TZZ] = hTzz; hh[TXZ] = hTxz; hh[TYZ] = hTyz;
      hh[TXX] = hTxx; hh[TYY] = hTyy; hh[TXY] = hTxy;
#pragma unroll
      for (int f = 0; f < NF && ok_mt && ok_p; ++f) {
        const long long o = f * fs + p;
        if (RK == 0) {
          // the tile holds the stored input; on the surface the imaged components were
          // patched in shared memory, so read those three from global memory there
          const float m = (LEAN && f == TZZ) ? q[TZZ][TRAIL]
                          : dec((top && (f == TZZ || f == TXZ || f == TYZ)) ? W[o] : tl(f)[r0][c0], f);
          st_stream_s(Wout + o, enc(m + A.a * hh[f], f), pol_stream);
          if (!NO_T) st_stream_s(Wt + o, enc(m + A.b * hh[f], f), pol_stream);
        } else if (RK == 1 && NO_T) {
          st_stream_s(Wout + o, enc(dec(mbuf[f][ty][tx], f) + A.a * hh[f], f), pol_stream);
        } else if (RK == 1 && RECON) {
          // W3 at the point as RK_beg reads its m (the surface's imaged stresses from memory)
          const float w3 = (LEAN && f == TZZ) ? q[TZZ][TRAIL]
                           : dec((top && (f == TZZ || f == TXZ || f == TYZ)) ? W[o] : tl(f)[r0][c0], f);
          // t = m + (a1 h1 + 2 a2 h2 + a3 h3) / 3 from the increments W2 - m, W3 - m and a3 h3
          // (added before m, so that t rounds once at the magnitude of m)
          const float m = dec(mbuf[f][ty][tx], f), inc = A.a * hh[f];
          const float d = (dec(tbuf[f][ty][tx], f) - m) + 2.0f * (w3 - m) + inc;
          st_stream_s(Wout + o, enc(m + inc, f), pol_stream);
          st_stream_s(Wt + o, enc(m + d * (1.0f / 3.0f), f), pol_stream);
        } else if (RK == 1) {
          st_stream_s(Wout + o, enc(dec(mbuf[f][ty][tx], f) + A.a * hh[f], f), pol_stream);
          st_stream_s(Wt + o, enc(dec(tbuf[f][ty][tx], f) + A.b * hh[f], f), pol_stream);
        } else {
          st_stream_s(Wt + o, enc(dec(tbuf[f][ty][tx], f) + A.b * hh[f], f), pol_stream);
        }
      }
    }
    // all threads agree on a timeout before leaving the pipeline
    if (__syncthreads_or(!ok || !ok_mt || !ok_p)) {
      if (tid == 0) {
        atomicExch(A.err, DEVERR_TMA_TIMEOUT);
        if (k < ke) mbar_wait(bar0 + 8 * (cur ^ 1), ((it + 1) >> 1) & 1);  // copies still in flight
        if (NSLOT > 0 && pml_k) mbar_wait(bar_pml, pml_ph & 1);
        if (LEAN && RK >= 1) mbar_wait(bar_mt, it & 1);
        if (SPLIT) {
          mbar_wait(bar_rk(cur), (it >> 1) & 1);
          if (k < ke) mbar_wait(bar_rk(cur ^ 1), ((it + 1) >> 1) & 1);
        }
      }
      return false;
    }
    if (pml_k) ++pml_ph;
  }
  // every issued copy has been waited for (the last plane issues none)
  if (tid == 0) {
    mbar_inval(bar0);
    mbar_inval(bar0 + 8);
    if (NSLOT > 0 && NROLE_S > 0) mbar_inval(bar_pml);
    if (LEAN && RK >= 1) mbar_inval(bar_mt);
    if (SPLIT) {
      mbar_inval(bar_rk(0));
      mbar_inval(bar_rk(1));
    }
  }
  return true;
}

// Launch over a batch of simulations: the work items (tile x k-chunk, packed as
// bx | by << 10 | bz << 20) of all simulations are numbered simulation after simulation,
// and CTA b runs items b, b + gridDim.x, ... (one item each when the grid covers them
// all).  Lean launches get the interior items, full launches the others.
// Tile rows TY: 8 (the default, 256 threads; 3 interior-only or 2 full CTAs per SM) or 16
// (512 threads, one CTA per SM).
template <class S, bool EXACT, int FX, int FY, int FZ, int RK, bool LEAN, bool TOPO = false, int TY = STAGE_TY>
__global__ void __launch_bounds__(TX* TY, (LEAN ? 24 : 16) / TY > 0 ? (LEAN ? 24 : 16) / TY : 1)
    stage_batch_kernel(const __grid_constant__ BatchArgs B) {
  extern __shared__ __align__(1024) unsigned char smem[];
  for (int item = blockIdx.x; item < B.total; item += gridDim.x) {
    int s = 0;
    while (item >= B.off[s + 1]) ++s;
    const int packed = B.items[s][item - B.off[s]];
    const int bx = packed & 1023, by = (packed >> 10) & 1023, bz = int(unsigned(packed) >> 20);
    if (!stage_body<S, EXACT, FX, FY, FZ, RK, LEAN, TOPO, TY>(B.sims[s], bx, by, bz, smem)) return;
    __syncthreads();  // the next item re-initialises the barriers and reuses the buffers
  }
}

template <class S, bool EXACT, int FX, int FY, int FZ, int RK, bool LEAN, bool TOPO = false, int TY = STAGE_TY>
static int launch_batch_one(const BatchArgs& b, int ctas, cudaStream_t st) {
  stage_batch_kernel<S, EXACT, FX, FY, FZ, RK, LEAN, TOPO, TY>
      <<<ctas, dim3(TX, TY, 1), Lay<S, TOPO, TY>::smem_bytes(LEAN, RK), st>>>(b);
  return int(cudaGetLastError());
}

// Opt every instantiation of one (storage, form, RK) into the dynamic shared memory it
// needs; called once per device before any launch or stream capture.
template <class S, bool EXACT, int RK, int TY = STAGE_TY>
static int configure_rk() {
  cudaError_t e = cudaSuccess;
#define FW_CFG(FX, FY, FZ)                                                                               \
  if (e == cudaSuccess)                                                                                  \
    e = cudaFuncSetAttribute(stage_batch_kernel<S, EXACT, FX, FY, FZ, RK, false, false, TY>,             \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,                                \
                             Lay<S, false, TY>::smem_bytes(false, RK));                                  \
  if (e == cudaSuccess)                                                                                  \
    e = cudaFuncSetAttribute(stage_batch_kernel<S, EXACT, FX, FY, FZ, RK, true, false, TY>,              \
                             cudaFuncAttributeMaxDynamicSharedMemorySize, Lay<S, false, TY>::smem_bytes(true, RK));
  FW_CFG(0, 0, 0) FW_CFG(0, 0, 1) FW_CFG(0, 1, 0) FW_CFG(0, 1, 1)
  FW_CFG(1, 0, 0) FW_CFG(1, 0, 1) FW_CFG(1, 1, 0) FW_CFG(1, 1, 1)
#undef FW_CFG
  return int(e);
}

template <class S, bool EXACT, int RK, bool LEAN, int TY>
static int launch_batch_lean(const BatchArgs& b, int variant, int ctas, cudaStream_t st) {
  switch (variant) {
    case 0: return launch_batch_one<S, EXACT, 0, 0, 0, RK, LEAN, false, TY>(b, ctas, st);
    case 1: return launch_batch_one<S, EXACT, 0, 0, 1, RK, LEAN, false, TY>(b, ctas, st);
    case 2: return launch_batch_one<S, EXACT, 0, 1, 0, RK, LEAN, false, TY>(b, ctas, st);
    case 3: return launch_batch_one<S, EXACT, 0, 1, 1, RK, LEAN, false, TY>(b, ctas, st);
    case 4: return launch_batch_one<S, EXACT, 1, 0, 0, RK, LEAN, false, TY>(b, ctas, st);
    case 5: return launch_batch_one<S, EXACT, 1, 0, 1, RK, LEAN, false, TY>(b, ctas, st);
    case 6: return launch_batch_one<S, EXACT, 1, 1, 0, RK, LEAN, false, TY>(b, ctas, st);
    default: return launch_batch_one<S, EXACT, 1, 1, 1, RK, LEAN, false, TY>(b, ctas, st);
  }
}

template <class S, bool EXACT, int RK, int TY = STAGE_TY>
static int launch_batch_rk_variant(const BatchArgs& b, int variant, int lean, int ctas, cudaStream_t st) {
  return lean ? launch_batch_lean<S, EXACT, RK, true, TY>(b, variant, ctas, st)
              : launch_batch_lean<S, EXACT, RK, false, TY>(b, variant, ctas, st);
}

// Terrain form (FP32 storage, full form; EXACT selects the reference-order arithmetic):
// opt in and launch.
template <bool EXACT, int RK>
static int configure_topo_rk() {
  cudaError_t e = cudaSuccess;
#define FW_CFG(FX, FY, FZ)                                                                                 \
  if (e == cudaSuccess)                                                                                    \
    e = cudaFuncSetAttribute(stage_batch_kernel<float, EXACT, FX, FY, FZ, RK, false, true>,                \
                             cudaFuncAttributeMaxDynamicSharedMemorySize, Lay<float, true>::smem_bytes(false, RK));
  FW_CFG(0, 0, 0) FW_CFG(0, 0, 1) FW_CFG(0, 1, 0) FW_CFG(0, 1, 1)
  FW_CFG(1, 0, 0) FW_CFG(1, 0, 1) FW_CFG(1, 1, 0) FW_CFG(1, 1, 1)
#undef FW_CFG
  return int(e);
}

template <bool EXACT, int RK>
static int launch_batch_topo_variant(const BatchArgs& b, int variant, int ctas, cudaStream_t st) {
  switch (variant) {
    case 0: return launch_batch_one<float, EXACT, 0, 0, 0, RK, false, true>(b, ctas, st);
    case 1: return launch_batch_one<float, EXACT, 0, 0, 1, RK, false, true>(b, ctas, st);
    case 2: return launch_batch_one<float, EXACT, 0, 1, 0, RK, false, true>(b, ctas, st);
    case 3: return launch_batch_one<float, EXACT, 0, 1, 1, RK, false, true>(b, ctas, st);
    case 4: return launch_batch_one<float, EXACT, 1, 0, 0, RK, false, true>(b, ctas, st);
    case 5: return launch_batch_one<float, EXACT, 1, 0, 1, RK, false, true>(b, ctas, st);
    case 6: return launch_batch_one<float, EXACT, 1, 1, 0, RK, false, true>(b, ctas, st);
    default: return launch_batch_one<float, EXACT, 1, 1, 1, RK, false, true>(b, ctas, st);
  }
}

}  // namespace fw
