// Internal interface between the host driver (solver.cpp) and the CUDA kernels.
// Plain structs only: they are passed to kernels by value.
#pragma once
#include <cuda.h>

#include <cstddef>
#include <cstdint>

namespace fw {

constexpr int NF = 9;
// Storage order of the nine components inside a register set.  The six components
// differentiated along k come first so that one TMA box fetches exactly them.
enum { VX = 0, VY, VZ, TZZ, TXZ, TYZ, TXX, TYY, TXY };
// C-ABI component order (Vx Vy Vz Txx Tyy Tzz Txy Txz Tyz) -> storage index
constexpr int ABI2INT[NF] = {VX, VY, VZ, TXX, TYY, TZZ, TXY, TXZ, TYZ};
constexpr int LENFD = 3;
constexpr int PADL = 29;  // physical column of Fortran index i is (i-1)+PADL: interior starts at 32

// Geometry of one simulation in device memory.  Interior bounds are 0-based
// (Fortran index minus one).  Element (i,j,k) of a component lives at
// (i + PADL) + px*(j + ny*k).
struct Geom {
  int ni, nj, nk, nx, ny, nz;
  int px;                 // row pitch in elements (multiple of 32)
  long long plane;        // px*ny
  long long fstride;      // elements between components of one register set (multiple of 64)
  int i1, i2, j1, j2, k1, k2;  // interior, inclusive
  int freesurf;           // free surface on k = k2
};

// One PML slab (face x1 x2 y1 y2 z1 z2), points i1..i2 x j1..j2 x k1..k2.  Its six memory
// variables are stored as rows padded to 16 bytes: element (i,j,k) at
// (i-ox) + sx*((j-j1) + sy*(k-k1)), variables vstride apart, with the row origin ox <= i1
// congruent to the first interior column mod 4 and sx a multiple of 4, so that the part of
// a row under any 32-column tile is a 16-byte-aligned run of whole 16-byte units (the stage
// kernel copies it with cp.async.bulk).
struct Slab {
  int on;
  int i1, i2, j1, j2, k1, k2;
  int sx, sy;
  int ox;
  long long vstride;
};

// Sources resolved on the host into per-point weights.
struct Sources {
  // per-stage source-time tables: value at global stage g = ntime*4 + s for window w
  const float* disp;   // [G][nw_f]  src_stf of force windows
  const float* rate;   // [G][nw_f]  src_svf of force windows
  const float* mrate;  // [G][nw_m]  src_svf of moment windows
  int G;               // table length in stages
  int nw_f, nw_m;
  // surface forces (SrcSurface): entries in (n, m) order, last one wins at a node
  int nsurf;
  const int* surf_ij;     // [nsurf][2] 0-based (i, j)
  const float* surf_q;    // [nsurf][3] F/S of that window
  const int* surf_w;      // [nsurf] window index into disp/rate
  // body forces with 7^3 smoothing
  int nforce, ntwin_f;
  const int* force_c;     // [nforce][3] 0-based centre
  const float* force_wt;  // [nforce][343] 1/(V rho) d, 0 where skipped
  const unsigned char* force_on;  // [nforce][343]
  const float* force_F;   // [nforce][ntwin][3]
  // moment tensors with 7^3 smoothing
  int nmom, ntwin_m;
  const int* mom_c;
  const float* mom_d;     // [nmom][343] weights d
  const float* mom_vol;   // [nmom][343] cell volume V
  const unsigned char* mom_on;
  const float* mom_M;     // [nmom][ntwin][6] Mxx Myy Mzz Mxy Mxz Myz
};

// Stage-kernel tiling: a CTA owns TX x TY columns and marches along k.  TY = STAGE_TY is
// the default tile height; the FP32 forms also exist with TY = STAGE_TY_TALL (the tile
// shape is a tuning choice of the solver, fwant_set_tile_rows).
constexpr int STAGE_TX = 32, STAGE_TY = 8, STAGE_TY_TALL = 16;
// TMA boxes (x, y, 1 plane, components).  The halo'd tile starts tile_halo_x columns left
// of the CTA's first column so that its x origin stays 16-byte aligned: 4 columns for
// 4-byte storage, 8 for 2-byte storage.
constexpr int tile_halo_x(int elem_bytes) { return elem_bytes >= 4 ? 4 : 8; }
constexpr int tile_box_x(int elem_bytes) { return STAGE_TX + 2 * tile_halo_x(elem_bytes); }
// Rows of the halo'd tile: a one-sided y operator reads one row on one side and three on
// the other (forward: -1..+3, backward: -3..+1), so the box holds the CTA's rows plus
// four; its first row is tile_halo_y(FY) rows above the CTA's first row.
constexpr int tile_by(int ty) { return ty + 4; }
constexpr int TILE_BY = tile_by(STAGE_TY);
constexpr int tile_halo_y(int fwd) { return fwd ? 1 : 3; }
// wavefield storage kinds inside the kernels
enum { ST_F32 = 0, ST_BF16 = 1, ST_F16 = 2 };
constexpr int storage_bytes(int st) { return st == ST_F32 ? 4 : 2; }

// Everything one RK-stage launch needs.
struct StageArgs {
  CUtensorMap tm_tile;  // stage input W: box TILE_BX x TILE_BY x 1 x 9
  CUtensorMap tm_q;     // stage input W: box TX x TY x 1 x 6 (k-differentiated components)
  CUtensorMap tm_m;     // RK register m: box TX x TY x 1 x 9
  CUtensorMap tm_t;     // RK register t: box TX x TY x 1 x 9
  CUtensorMap tm_med;   // lambda, mu, rho: box TX x TY x 1 x 3
  // The lean form's tile boxes; the terrain form (never lean) uses the first slot for the
  // terrain-following grid's per-point 1/r, zeta_r, zeta_theta / r, zeta_phi / (r sin theta)
  // (box TX x TY x 1 x 4).
  union {
    CUtensorMap tm_tile_lo;  // stage input W, lean form: box TILE_BX x TILE_BY x 1 x 3 (Vx Vy Vz)
    CUtensorMap tm_topo;
  };
  CUtensorMap tm_tile_hi;  // stage input W, lean form: box TILE_BX x TILE_BY x 1 x 5 (Txz .. Txy)
  // terrain form: per surface column (padded plane layout, g.plane apart) m1, m2 of the
  // surface normal and the row-major 3x3 inverse of the traction condition (11 planes)
  const float* topo_sf;
  Geom g;
  const void* win;    // stage input W (9 components, storage type)
  void* wout;         // stage output W
  void* wt;           // RK accumulator t
  const void* wm;     // RK register m (W at the step start)
  // BF16/FP16 storage holds value * scale: velocities (sv) and stresses (st); 1/scale too
  float sv, st, isv, ist;
  // 1-D metric, 0-based Fortran index, with ghosts
  const float* xi_x;
  const float* eta_y;
  const float* zeta_z;
  const float* xsin;
  const float* xcot;
  const float* zc;
  const float* rzinv;  // 1/z (fast arithmetic)
  const float* rsinv;  // 1/xsin (fast arithmetic)
  // PML profile terms per axis, 0-based Fortran index: b1 = 1/B, b1 - 1, A + D, D (D = d/b)
  const float* pb1[3];
  const float* pb11[3];
  const float* pad[3];
  const float* pD[3];
  Slab slab[6];
  // TMA descriptors of the six faces' memory variables (device memory, one 5-D tensor per
  // face: x, y, z of the slab, variable, register set; null without PML) and the register
  // sets this stage reads as input, m and t
  const CUtensorMap* pml_map;
  int pml_set[3];
  const float* ain[6];
  const float* am[6];
  float* aout[6];
  float* at[6];
  float a, b;     // rka*stept, rkb*stept
  int stage;      // 0..3 inside the step
  int kc;         // planes per CTA along k
  int kz_lo, kz_hi;  // k-chunk boundaries (stage_chunk)
  const int* ntime;  // device step counter
  int* err;          // device error word (bounded-wait timeouts)
  Sources src;
};

// Batched launch: one stage of up to BATCH_PER_LAUNCH simulations in one grid, their
// arguments (tensor maps included) held in the kernel's parameter space (the 32 KB
// parameter limit bounds the count); larger batches use one launch per group.
constexpr int MAX_BATCH = 64;
constexpr int BATCH_PER_LAUNCH = 16;
struct BatchArgs {
  StageArgs sims[BATCH_PER_LAUNCH];
  const int* items[BATCH_PER_LAUNCH];  // per simulation: work items, bx | by << 10 | bz << 20
  int nsims, total;                    // simulations, work items
  int off[BATCH_PER_LAUNCH + 1];       // first work item of each simulation
};
static_assert(sizeof(BatchArgs) <= 32764, "kernel parameter space");

// RK kinds of the stage kernel.  0 RK_beg, 1 RK_inn, 2 RK_fin update the reference's
// registers (W, the stage start m and the accumulator t; mod_macdrp.F90:291-393).  The fast
// form also runs the classical RK4 step without carrying t through stages 1-3:
//   3  stage 1: W2 = m + a1 h                               (no t)
//   4  stage 2: W3 = m + a2 h                               (no t)
//   5  stage 3: W4 = m + a3 h, t = m + ((W2 - m) + 2 (W3 - m) + a3 h) / 3
//      (= m + b1 h1 + b2 h2 + b3 h3 of the reference's RK4 weights)
// and stage 4 is RK_fin (W = t + b4 h) as before: 129 instead of 156 floats moved per
// point and step, the same values up to FP32 rounding.  rk_base gives the reference kind
// whose data movement each one follows.
__host__ __device__ constexpr int rk_base(int rk) { return rk == 3 ? 0 : (rk >= 4 ? 1 : rk); }

// Stage launchers (stage_*.cu).  variant bit 2 = x, bit 1 = y, bit 0 = z; 1 = forward
// operator.  rk: the kinds above (3-5 in the fast form only).  exact = 1 selects the reference's
// operand order with IEEE division and no FMA (bit-reproducible against FP32 CPU runs
// of the same expressions); 0 the fast form (FMA, reciprocals).
// storage: ST_F32 / ST_BF16 / ST_F16 (the exact form exists for ST_F32 only).
// lean = 1: the interior-only form (items without PML points, sources or free surface).
// ty: tile rows (STAGE_TY, or STAGE_TY_TALL for FP32 storage); another value returns
// cudaErrorInvalidValue.
int launch_stage_batch(const BatchArgs& b, int variant, int rk, int exact, int storage, int lean, int ctas,
                       void* stream, int ty = STAGE_TY);
// The terrain form (FP32 storage, full form only; exact = 1 the reference-order arithmetic).
int launch_stage_batch_topo(const BatchArgs& b, int variant, int rk, int exact, int ctas, void* stream);
// FP64 metric of the terrain-following grid (r = z + h s): per point r, zeta_r,
// zeta_theta / r, zeta_phi / (r sin theta) into out (4 components fstride apart), from
// float heights h (nx*ny, i fastest), the 1-D arrays (0-based Fortran index with ghosts)
// and the double tables s(k), z_zeta(k).
struct TopoMetricArgs {
  Geom g;
  const float* h;        // [ny][nx]
  const double* hxi;     // [ny][nx] dh/dxi
  const double* heta;    // [ny][nx] dh/deta
  const float* z; const float* xi_x; const float* eta_y; const float* zeta_z; const float* xsin;
  const double* sk;      // [nz]
  const double* rzf;     // [nz]
  float* out;
};
void launch_topo_metric(const TopoMetricArgs& a, void* stream);
// Surface arrays (11 planes of the padded plane layout): m1, m2, the 3x3 inverse, from the
// metric at k = nk2 and the medium's lambda, mu there (FP64).
void launch_topo_surface(const Geom& g, const float* metric, const float* lam, const float* mu, float* out,
                         void* stream);
// dh/dxi, dh/deta of the heights (FP64, the metric's stencil with clamped ends)
void launch_topo_slopes(const Geom& g, const float* h, double* hxi, double* heta, void* stream);
// k-chunks of the work items.  The planes split into three bands at kz_lo (the first plane
// above the bottom PML slab, or k1) and kz_hi (the first plane of the free surface's band of
// four, or of the top PML slab, or k2 + 1), so that no chunk straddles a band edge: the
// chunks of the middle band then hold no slab or surface plane and can run in the
// interior-only form.  A band of len planes is cut into ceil(len / kc) chunks of nearly
// equal length (at most kc planes); chunk bz covers planes [kb, ke].
__host__ __device__ inline int stage_chunk_count(const Geom& g, int kc, int kz_lo, int kz_hi) {
  return (kz_lo - g.k1 + kc - 1) / kc + (kz_hi - kz_lo + kc - 1) / kc + (g.k2 + 1 - kz_hi + kc - 1) / kc;
}
__host__ __device__ inline void stage_chunk(const Geom& g, int kc, int kz_lo, int kz_hi, int bz, int* kb, int* ke) {
  int base = g.k1, len = kz_lo - g.k1, c = bz;
  int n = (len + kc - 1) / kc;
  if (c >= n) {
    c -= n;
    base = kz_lo;
    len = kz_hi - kz_lo;
    n = (len + kc - 1) / kc;
    if (c >= n) {
      c -= n;
      base = kz_hi;
      len = g.k2 + 1 - kz_hi;
      n = (len + kc - 1) / kc;
    }
  }
  // n >= 1 here for every bz below stage_chunk_count
  *kb = base + (c * len) / n;
  *ke = base + ((c + 1) * len) / n - 1;
}
// The band edges kz_lo, kz_hi of a simulation (absolute plane indices).
void stage_z_bands(const Geom& g, const Slab slab[6], int* kz_lo, int* kz_hi);
// Work items of one simulation split into the lean (interior) list and the full list.
// force_c / mom_c: 0-based source centres (3 per source).
void stage_items(const Geom& g, int kc, int ty, int kz_lo, int kz_hi, const Slab slab[6], const int* force_c,
                 int nforce, const int* mom_c, int nmom, int* lean, int* nlean, int* full, int* nfull);
long long stage_item_count(const Geom& g, int kc, int ty, int kz_lo, int kz_hi);
// Planes per CTA.  Short chunks keep the CTAs that share halo rows marching through the
// same planes at the same time, which is what lets L2 serve the halo and z-queue
// re-reads; measured on 400x400x200 (RK form 0): 16 planes 1.68 ms per RK_inn stage, 32
// planes 1.78, 64 planes 2.01, the whole column 3.04; with RK form 1 and concurrent
// interior-only / full launches, 24 planes per step 11.33 ms against 11.37 for 16 and 11.34
// for 20 (the autotuner picks 24 there too).  Small grids get shorter chunks so that there
// are at least ~4 CTAs per SM, down to 3 planes: on 100x100x60 (C1, its working set held in
// L2) 3 planes run 0.263 ms per step, 4 planes 0.280, 6 planes 0.278, 8 planes 0.297.
inline int stage_planes_per_cta(const Geom& g, int sm_count, int ty = STAGE_TY) {
  const long long tiles = (long long)((g.ni + STAGE_TX - 1) / STAGE_TX) * ((g.nj + ty - 1) / ty);
  const long long want = 4LL * sm_count * STAGE_TY / ty;  // ~4 CTAs of 256 threads per SM
  long long chunks = (want + tiles - 1) / tiles;
  if (chunks < 1) chunks = 1;
  int kc = int((g.nk + chunks - 1) / chunks);
  if (kc < 3) kc = 3;
  if (kc > 24) kc = 24;
  const int floor_chunks = (g.nk + 2046) / 2047;
  return kc > floor_chunks ? kc : floor_chunks;  // at most 2047 chunks, as fwant_set_planes_per_cta allows
}
int stage_configure();  // set the dynamic shared-memory attribute of every instantiation

struct RecvArgs {
  Geom g;
  const void* w;      // register set holding the step's result (storage type)
  int storage;        // ST_*; stored values are multiplied by isv / ist on reading
  float isv, ist;
  int npt;
  const int* idx;     // [npt][3] 0-based
  int tinv;
  float* seismo;      // [9][cap][npt], C-ABI component order
  int cap;
  int* ntime;
};
void launch_advance_record(const RecvArgs& a, void* stream);

// Strided sub-volume of one register set (snapshot frame).  start is 0-based (Fortran
// index minus one); comp holds storage indices; out is [ncomp][cnt2][cnt1][cnt0].
struct SnapArgs {
  Geom g;
  const void* w;
  int storage;
  float isv, ist;
  int start[3], cnt[3], stride[3];
  int ncomp;
  int comp[NF];
  float* out;
};
void launch_pack_snapshot(const SnapArgs& a, void* stream);
// Fixed staging array of fwant_get_snapshot_noalloc (floats) and its per-device address.
constexpr long long SNAPSHOT_NOALLOC_MAX = 4LL << 20;
int snapshot_noalloc_staging(int device, float** ptr);

// Strain-Green's-tensor recording: the six stresses of a strided sub-volume after every
// step whose counter is a multiple of tinv (frame ntime/tinv - 1), into
// out[6][max_frames][npts] (Txx Tyy Tzz Txy Txz Tyz, points i fastest).
struct SgtRecArgs {
  Geom g;
  const void* w;
  int storage;
  float isv, ist;
  int start[3], cnt[3], stride[3];
  int tinv, max_frames;
  long long npts;
  const int* ntime;
  float* out;
};
void launch_record_sgt(const SgtRecArgs& a, void* stream);

// Sensitivity-kernel accumulation (sgtker.cu).  Strains of the receiver-side SGTs
// (X, Y, Z force) and of the source-side SGT are formed from FP32 stresses in FP32
// (stress2strain); the time convolutions and window integrals accumulate in FP64.
struct ScatterArgs {
  long long npts;
  int knt;               // frames per series
  int nt1, nt2;          // 1-based output range
  double dt;
  const float* lam;      // [npts]
  const float* mu;       // [npts]
  const float* rsgt[3];  // receiver SGT per force component, [6][knt][npts] stresses (null: skipped)
  const float* ssgt;     // source SGT, [6][knt][npts]
  double* out;           // [6][knt][npts]: X -> (0, 3), Y -> (1, 5), Z -> (2, 4)
  int param;             // 0: Vp/Vs kernels, 1: lambda/mu kernels
};
int launch_sgt_scatter(const ScatterArgs& a, int sm_count, void* stream);
struct KernelArgs {
  long long npts;
  int knt, nt1, nt2;
  const double* ka;      // [knt][npts]
  const double* kb;
  const double* wv;      // [knt] trapezoid weight x V(n) (1-based n at index n-1)
  const double* wu;      // [knt] trapezoid weight x U(n)
  double v0, u0;         // normalisations: trapezoid integral of V^2 (U^2) x SGT_M0
  double* kap; double* kaq; double* kbp; double* kbq;  // [npts]
};
void launch_scatter_kernel(const KernelArgs& a, void* stream);
// SI_ker_pair (SI_ker_pair.F90:710-780): the strains of one receiver SGT and of the source
// SGT (stress2strain), then the single-precision scatter series of the pair over 1..knt
// (sgt2scatter), every operation rounded in the reference's order:
//   out[0] = Sa = x1 2 (lam + 2 mu), out[1] = Sb = 2 (x2 - x1) 2 mu   ([2][knt][npts], FP64
//   holding the FP32 values); strain scratch [14][knt][npts] floats.
struct PairArgs {
  long long npts;
  int knt;
  float dt;
  const float* lam;
  const float* mu;
  const float* rsgt;  // receiver SGT [6][knt][npts]
  const float* ssgt;  // source SGT [6][knt][npts]
  float* strain;      // scratch
  double* out;
};
int launch_pair_scatter(const PairArgs& a, void* stream);
// scatter2kernel of SI_ker_pair (:782-838) in single precision: the series rounded to FP32,
// trapezoid sums V(n) Ka(n) dt in order, divided by v0 / u0.
struct PairKernelArgs {
  long long npts;
  int nt1, nt2;
  float dt, v0, u0;
  const double* ka;  // [knt][npts]
  const double* kb;
  const float* v;    // [knt]
  const float* u;
  float* kap; float* kaq; float* kbp; float* kbq;
};
void launch_pair_kernel(const PairKernelArgs& a, void* stream);
// IIR filtering of npts series of knt samples ([knt][npts] FP64) as scatter_filter (mode 1)
// or scatter_filtfilt (mode 2) of SI_ker_sta.F90:1433-1558, or the forward-backward filter
// of SI_ker_pair (mode 3: zero padding, (nod1 - 1) samples in front and 2 nod1 behind,
// SI_ker_pair.F90:906-932); nod1 coefficients b[], a[]; scratch holds (knt + 6 (nod1-1))
// x npts doubles (modes 1, 2) or (knt + 3 (nod1-1) + 2) x npts (mode 3).
struct IirArgs {
  long long npts;
  int knt, mode, nod1;
  double b[16], a[16];
  const double* in;
  double* out;
  double* scratch;
};
constexpr int IIR_MAX_COEF = 16;
void launch_iir(const IirArgs& a, void* stream);
// Rotation of the three force components of the series: slots (0,1,2) and (3,5,4),
// new_c = sum_d rot[d + 3c] old_d (rot column-major, SI_ker_sta.F90:1339-1373).
void launch_rotate_series(double* series, long long slot_len, const double rot[9], void* stream);
// Kernel parameter conversion in place over n points (mode 1 lambda/mu -> kappa/mu, 2
// lambda/mu -> Vp/Vs, 3 Vp/Vs -> kappa/mu), phase and amplitude pairs (ka0, kb0), (ka1, kb1).
void launch_convert_kernel(int mode, long long n, const float* lam, const float* mu, float* ka0, float* ka1,
                           float* kb0, float* kb1, void* stream);

void launch_metric_fp64(int n, const float* coord, float* metric_out, int lo, int hi, void* stream);
void launch_sincot_fp64(int n, const float* x, float* xsin, float* xcot, void* stream);
// max |value| of each of the nine components (storage order) into out_bits[9]
void launch_maxabs(const Geom& g, const void* w, int storage, float isv, float ist, unsigned int* out_bits,
                   void* stream);
// count of the n values that are not > 0 (NaN included), added to *count
void launch_count_nonpositive(long long n, const float* v, unsigned int* count, void* stream);
// one component between storage type and FP32 (padded layout, scale applied)
void launch_convert_to_f32(const Geom& g, const void* src, int storage, float inv_scale, float* dst, void* stream);
void launch_convert_from_f32(const Geom& g, const float* src, int storage, float scale, void* dst, void* stream);

// a bounded wait on a barrier nothing completes: after `spins` polls it writes
// DEVERR_TMA_TIMEOUT to *err (the stage kernel's expired-wait path)
void launch_wait_timeout_probe(int spins, int* err, void* stream);

// device error codes written to StageArgs::err
enum { DEVERR_NONE = 0, DEVERR_TMA_TIMEOUT = 1 };

}  // namespace fw
