// Host driver of the GB300 forward solver: owns the device state of one simulation,
// resolves sources/receivers/PML into device tables, and runs the 8-step F/B LDDRK4
// cycle of seis3d_wave_8op_p3.F90 as fused stage launches, replayed from a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fwant_gb300.h"
#include "host_math.h"
#include "kernels.h"

namespace {

constexpr float RKA[4] = {0.5f, 0.5f, 1.0f, 0.0f};                        // firRKa (mod_macdrp.F90:205)
const float RKB[4] = {1.0f / 6.0f, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 6.0f};  // firRKb (mod_macdrp.F90:206)

// Stage-1/3 operator of each step of the 8-step cycle (seis3d_wave_8op_p3.F90:82-591);
// bit 2 = x, bit 1 = y, bit 0 = z, 1 = forward.  Stages 2/4 use the mirror.
constexpr int CYCLE[8] = {0b000, 0b110, 0b111, 0b001, 0b010, 0b100, 0b101, 0b011};

struct ForceDesc {
  int num = 0, ntwin = 0, stf_id = 200;
  std::vector<int> indx;  // 1-based
  std::vector<float> shift, t0, stf_time, stf_freq, fx, fy, fz;
};
struct MomentDesc {
  int num = 0, ntwin = 0, stf_id = 200;
  std::vector<int> indx;
  std::vector<float> shift, t0, stf_time, stf_freq, mom;  // mom: 6 blocks of ntwin*num
};

template <class T>
T* dalloc(size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
  return (T*)p;
}

// A second stream on which a stage's full-form launch runs beside its interior-only launch:
// the two cover disjoint work items (disjoint output points; both only read the stage
// input), so they may overlap, which overlaps their tails and lets an SM hold CTAs of both
// forms.  The side stream forks from the main stream before the stage's launches and joins
// it after them, eagerly and inside a captured graph alike.
struct FormFork {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  bool on = true;
  cudaError_t init() {
    if (const char* env = std::getenv("FWANT_CONCURRENT_FORMS")) on = std::atoi(env) != 0;  // measurement override
    cudaError_t e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    return e;
  }
  void destroy() {
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (side) cudaStreamDestroy(side);
    fork = join = nullptr;
    side = nullptr;
  }
  void begin(cudaStream_t main) {
    cudaEventRecord(fork, main);
    cudaStreamWaitEvent(side, fork, 0);
  }
  void end(cudaStream_t main) {
    cudaEventRecord(join, side);
    cudaStreamWaitEvent(main, join, 0);
  }
};

}  // namespace

struct fwant_solver {
  fwant_config cfg{};
  fw::Geom g{};
  float stept = 0.0f;
  cudaStream_t st = nullptr;
  FormFork fork;  // side stream of the full-form launches
  std::string err;

  // four register sets of nine components each (W ping-pong, m, t; see run_step)
  char* regs = nullptr;       // storage type given by `stor` (esz bytes per element)
  int stor = fw::ST_F32, esz = 4;
  // BF16/FP16 registers hold value * scale (velocities sv, stresses st)
  float sv = 1.0f, sc_t = 1.0f;
  float* d_conv = nullptr;    // FP32 staging for field import/export of 2-byte storage
  int rA = 0, rB = 1, rC = 2, rT = 3;
  float* med = nullptr;  // lambda, mu, rho, fstride apart (one TMA tensor)
  float *lam = nullptr, *mu = nullptr, *rho = nullptr;
  int* d_err = nullptr;  // device error word of the stage kernel (bounded waits)
  // TMA descriptors: per register set the halo'd tile, the z-queue plane and the point
  // box; one for the medium
  CUtensorMap tm_tile[4], tm_q[4], tm_pt[4], tm_med, tm_tile_lo[4], tm_tile_hi[4];
  // 1-D arrays, each with nx/ny/nz entries
  float *d_x = nullptr, *d_y = nullptr, *d_z = nullptr, *d_xsin = nullptr, *d_xcot = nullptr;
  float *d_xi = nullptr, *d_eta = nullptr, *d_zeta = nullptr;
  float* d_prof = nullptr;  // b1, b1-1, A+D, D for x (nx each), y (ny), z (nz)
  float *d_rzinv = nullptr, *d_rsinv = nullptr;
  int kc = 8;                // planes per CTA of the stage kernel
  int tile_ty = fw::STAGE_TY;  // rows of the stage kernel's 32-column tile (fw::STAGE_TY or STAGE_TY_TALL)
  int rk_scheme = 1;           // 1: stages 1-3 without t where the form allows it (RK kinds 3-5), 0: reference
  std::vector<float> hx, hy, hz, hxsin, hxcot;
  bool have_coord = false, have_metric = false, have_media = false;

  // PML
  int absn[6] = {0, 0, 0, 0, 0, 0};
  fw::Slab slab[6]{};
  float* aux[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // 4 sets each
  CUtensorMap* d_pml_map = nullptr;  // per face: x, y, z, variable, register set (device memory)
  long long aux_set[6] = {0, 0, 0, 0, 0, 0};                               // elements per set
  std::vector<float> hA[3], hB[3], hD[3];

  // sources
  ForceDesc forces;
  MomentDesc moments;
  bool src_dirty = true;
  fw::Sources S{};
  std::vector<void*> src_mem;
  int stf_cap_steps = 0;  // steps covered by the STF tables

  // receivers
  int npt = 0, tinv = 1, cap = 0, nsamp = 0;
  std::vector<int> rec_idx;  // 0-based
  int* d_rec = nullptr;
  float* d_seis = nullptr;

  int* d_ntime = nullptr;
  int ntime = 0, cycle_pos = 0;
  unsigned int* d_maxbits = nullptr;
  float* d_snap = nullptr;  // staging buffer of fwant_get_snapshot (grown on demand)
  size_t snap_cap = 0;
  // work items of the stage launches: lean (interior) items first, then the full ones
  int* d_items = nullptr;
  int n_lean = 0, n_full = 0;
  // RK kinds (bit 0 beg, 1 inn, 2 fin) whose interior items use the lean form.  Measured
  // on C2 (stage ms, full form -> split): beg 2.93 -> 2.66, fin 3.11 -> 3.08, inn 4.08 ->
  // 4.23 (the inn stage moves the most bytes and is DRAM-bound either way; the split only
  // adds a second launch and its tail).
  int lean_mask = -1;  // stages split into interior-only and full launches; -1: the form's default
  std::vector<int> h_items;
  std::vector<int> h_force_c, h_mom_c;  // 0-based source centres (item classification)
  // strain Green's tensor recording: sgt_ snapshot frames kept on the device
  float* d_sgt = nullptr;
  fw::SgtRecArgs sgt{};
  bool sgt_on = false;

  // terrain-following grid (Gaussian-hill extension): heights, their FP64 slopes, the
  // per-point metric (4 components, fstride apart) and the 11 surface planes
  bool topo_on = false, topo_sf_dirty = true;
  float* d_h = nullptr;
  double *d_hxi = nullptr, *d_heta = nullptr, *d_sk = nullptr, *d_rzf = nullptr;
  float* d_topo = nullptr;
  float* d_topo_sf = nullptr;
  CUtensorMap tm_topo{};

  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one per (rA,rT) assignment
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;

  ~fwant_solver() {
    cudaSetDevice(cfg.device);
    drop_graphs();
    free_sources();
    cudaFree(regs); cudaFree(med); cudaFree(d_err);
    cudaFree(d_x); cudaFree(d_y); cudaFree(d_z); cudaFree(d_xsin); cudaFree(d_xcot);
    cudaFree(d_xi); cudaFree(d_eta); cudaFree(d_zeta); cudaFree(d_prof); cudaFree(d_rzinv); cudaFree(d_rsinv);
    for (int f = 0; f < 6; ++f) cudaFree(aux[f]);
    cudaFree(d_pml_map);
    cudaFree(d_rec); cudaFree(d_seis); cudaFree(d_ntime); cudaFree(d_maxbits); cudaFree(d_snap); cudaFree(d_conv); cudaFree(d_sgt); cudaFree(d_items);
    cudaFree(d_h); cudaFree(d_hxi); cudaFree(d_heta); cudaFree(d_sk); cudaFree(d_rzf); cudaFree(d_topo); cudaFree(d_topo_sf);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    fork.destroy();
    if (st) cudaStreamDestroy(st);
  }

  fwant_status fail(fwant_status code, const std::string& m) {
    err = m;
    return code;
  }
  fwant_status cuda_fail(cudaError_t e, const char* where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return FWANT_ERR_CUDA;
  }

  void drop_graphs() {
    for (auto& ge : graph)
      if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
  }
  void free_sources() {
    for (void* p : src_mem) cudaFree(p);
    src_mem.clear();
    S = fw::Sources{};
    stf_cap_steps = 0;
  }
  template <class T>
  T* upload(const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    T* d = dalloc<T>(v.size());
    if (!d) return nullptr;
    src_mem.push_back(d);
    cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
  }

  long long off(int i, int j, int k) const {
    return (long long)(i + fw::PADL) + (long long)g.px * ((long long)j + (long long)g.ny * k);
  }
  void* set(int r) const { return regs + (long long)r * fw::NF * g.fstride * esz; }
  void* comp(int r, int f) const { return static_cast<char*>(set(r)) + (long long)f * g.fstride * esz; }
  float* aset(int f, int r) const { return aux[f] + (long long)r * aux_set[f]; }

  fwant_status init() {
    const int ni = cfg.ni, nj = cfg.nj, nk = cfg.nk;
    if (ni < 8 || nj < 8 || nk < 8) return fail(FWANT_ERR_INVALID_ARG, "ni, nj, nk must be >= 8");
    // work items pack the tile indices in 10 + 10 + 11 bits
    if (ni > 1024 * fw::STAGE_TX || nj > 1024 * fw::STAGE_TY || nk > 2047 * 4)
      return fail(FWANT_ERR_INVALID_ARG, "grid too large: ni <= 32768, nj <= 8192, nk <= 8188");
    if (!(cfg.stept > 0.0)) return fail(FWANT_ERR_INVALID_ARG, "stept must be > 0");
    if (cfg.storage == FWANT_STORAGE_FP32) stor = fw::ST_F32;
    else if (cfg.storage == FWANT_STORAGE_BF16) stor = fw::ST_BF16;
    else if (cfg.storage == FWANT_STORAGE_FP16) stor = fw::ST_F16;
    else return fail(FWANT_ERR_INVALID_ARG, "storage must be FP32, BF16 or FP16 (FP64 runs on the CPU solver)");
    if (stor != fw::ST_F32 && cfg.exact_arith)
      return fail(FWANT_ERR_INVALID_ARG, "exact_arith needs FP32 storage");
    esz = fw::storage_bytes(stor);
    cudaError_t e = cudaSetDevice(cfg.device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    stept = float(cfg.stept);
    g.ni = ni; g.nj = nj; g.nk = nk;
    g.nx = ni + 6; g.ny = nj + 6; g.nz = nk + 6;
    g.px = ((fw::PADL + g.nx + 31) / 32) * 32;
    g.plane = (long long)g.px * g.ny;
    g.fstride = ((g.plane * g.nz + 63) / 64) * 64;
    g.i1 = 3; g.i2 = 3 + ni - 1; g.j1 = 3; g.j2 = 3 + nj - 1; g.k1 = 3; g.k2 = 3 + nk - 1;
    g.freesurf = cfg.free_surface ? 1 : 0;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, cfg.device);
    kc = fw::stage_planes_per_cta(g, nsm > 0 ? nsm : 152);
    if (const char* env = std::getenv("FWANT_LEAN_STAGES")) {  // tuning override
      const int v = std::atoi(env);
      if (v >= 0 && v <= 7) lean_mask = v;
    }
    if (const char* env = std::getenv("FWANT_PLANES_PER_CTA")) {  // tuning override
      const int v = std::atoi(env);
      if (v >= 1 && (nk + v - 1) / v <= 2047) kc = v;
    }
    if (const char* env = std::getenv("FWANT_RK_SCHEME")) {  // measurement override
      const int v = std::atoi(env);
      if (v == 0 || v == 1) rk_scheme = v;
    }
    if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream");
    if ((e = fork.init()) != cudaSuccess) return cuda_fail(e, "side stream");
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    const size_t nreg = size_t(4) * fw::NF * g.fstride;
    regs = dalloc<char>(nreg * esz);
    med = dalloc<float>(3 * size_t(g.fstride));
    lam = med; mu = med + g.fstride; rho = med + 2 * g.fstride;
    d_err = dalloc<int>(1);
    d_x = dalloc<float>(g.nx); d_y = dalloc<float>(g.ny); d_z = dalloc<float>(g.nz);
    d_xsin = dalloc<float>(g.nx); d_xcot = dalloc<float>(g.nx); d_xi = dalloc<float>(g.nx);
    d_eta = dalloc<float>(g.ny); d_zeta = dalloc<float>(g.nz);
    d_prof = dalloc<float>(4 * size_t(g.nx + g.ny + g.nz));
    d_rzinv = dalloc<float>(g.nz); d_rsinv = dalloc<float>(g.nx);
    d_ntime = dalloc<int>(1); d_maxbits = dalloc<unsigned int>(fw::NF);
    if (!regs || !med || !d_err || !d_x || !d_y || !d_z || !d_xsin || !d_xcot || !d_xi || !d_eta ||
        !d_zeta || !d_prof || !d_rzinv || !d_rsinv || !d_ntime || !d_maxbits)
      return fail(FWANT_ERR_OOM, "device allocation failed");
    cudaMemset(regs, 0, nreg * esz);
    cudaMemset(med, 0, 3 * g.fstride * sizeof(float));
    cudaMemset(d_ntime, 0, sizeof(int));
    cudaMemset(d_err, 0, sizeof(int));
    fwant_status rc = make_tensor_maps();
    if (rc != FWANT_OK) return rc;
    if (int ce = fw::stage_configure()) return cuda_fail(cudaError_t(ce), "stage kernel configuration");
    for (int a = 0; a < 3; ++a) {
      const int n = a == 0 ? g.nx : a == 1 ? g.ny : g.nz;
      hA[a].assign(n, 0.0f); hB[a].assign(n, 1.0f); hD[a].assign(n, 0.0f);
    }
    if ((e = upload_profiles()) != cudaSuccess) return cuda_fail(e, "profiles");
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "init");
    return FWANT_OK;
  }

  // Per-index PML terms as the reference forms them at every point
  // (mod_abs_npml.F90:1168-1172): b1 = 1/B, b1_1 = b1 - 1, ad = A + D; and D.
  cudaError_t upload_profiles() {
    float* p = d_prof;
    for (int a = 0; a < 3; ++a) {
      const size_t n = hA[a].size();
      std::vector<float> b1(n), b11(n), ad(n);
      for (size_t q = 0; q < n; ++q) {
        b1[q] = 1.0f / hB[a][q];
        b11[q] = b1[q] - 1.0f;
        ad[q] = hA[a][q] + hD[a][q];
      }
      cudaMemcpy(p, b1.data(), n * 4, cudaMemcpyHostToDevice); p += n;
      cudaMemcpy(p, b11.data(), n * 4, cudaMemcpyHostToDevice); p += n;
      cudaMemcpy(p, ad.data(), n * 4, cudaMemcpyHostToDevice); p += n;
      cudaMemcpy(p, hD[a].data(), n * 4, cudaMemcpyHostToDevice); p += n;
    }
    return cudaGetLastError();
  }
  const float* prof(int axis, int which) const {
    const float* p = d_prof;
    for (int a = 0; a < axis; ++a) p += 4 * hA[a].size();
    return p + which * hA[axis].size();
  }
  // TMA descriptors over the padded layout: 4-D tensors (x: px, y: ny, z: nz,
  // component) with the component stride fstride.  Out-of-range box elements read 0.
  fwant_status make_tensor_maps() {
    using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess)
      return fail(FWANT_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    EncodeFn encode = reinterpret_cast<EncodeFn>(fn);
    // The halo'd tile's rows (160 B) start 16 B before a 128 B line: without promotion a
    // miss fetches only the 32 B sectors the row covers.  Override for tuning:
    // FWANT_TILE_L2_PROMOTION = 0, 64, 128 or 256.
    CUtensorMapL2promotion tile_promo = CU_TENSOR_MAP_L2_PROMOTION_NONE;
    if (const char* env = std::getenv("FWANT_TILE_L2_PROMOTION")) {
      const int v = std::atoi(env);
      tile_promo = v == 64 ? CU_TENSOR_MAP_L2_PROMOTION_L2_64B
                 : v == 128 ? CU_TENSOR_MAP_L2_PROMOTION_L2_128B
                 : v == 256 ? CU_TENSOR_MAP_L2_PROMOTION_L2_256B : CU_TENSOR_MAP_L2_PROMOTION_NONE;
    }
    const CUtensorMapDataType wtype = stor == fw::ST_F32    ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                      : stor == fw::ST_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                            : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    auto make = [&](CUtensorMap* m, void* base, CUtensorMapDataType dt, int es, int ncomp, cuuint32_t bx,
                    cuuint32_t by, cuuint32_t bc,
                    CUtensorMapL2promotion promo) {
      const cuuint64_t dims[4] = {cuuint64_t(g.px), cuuint64_t(g.ny), cuuint64_t(g.nz), cuuint64_t(ncomp)};
      const cuuint64_t strides[3] = {cuuint64_t(g.px) * es, cuuint64_t(g.plane) * es, cuuint64_t(g.fstride) * es};
      const cuuint32_t box[4] = {bx, by, 1, bc};
      const cuuint32_t el[4] = {1, 1, 1, 1};
      return encode(m, dt, 4, base, dims, strides, box, el, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, promo, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    };
    const CUtensorMapL2promotion line = CU_TENSOR_MAP_L2_PROMOTION_L2_128B;  // line-aligned boxes
    for (int r = 0; r < 4; ++r) {
      const cuuint32_t ty = cuuint32_t(tile_ty), tby = cuuint32_t(fw::tile_by(tile_ty));
      if (make(&tm_tile[r], set(r), wtype, esz, fw::NF, fw::tile_box_x(esz), tby, fw::NF, tile_promo) !=
              CUDA_SUCCESS ||
          make(&tm_q[r], set(r), wtype, esz, fw::NF, fw::STAGE_TX, ty, 6, line) != CUDA_SUCCESS ||
          make(&tm_pt[r], set(r), wtype, esz, fw::NF, fw::STAGE_TX, ty, fw::NF, line) != CUDA_SUCCESS ||
          make(&tm_tile_lo[r], set(r), wtype, esz, fw::NF, fw::tile_box_x(esz), tby, 3, tile_promo) !=
              CUDA_SUCCESS ||
          make(&tm_tile_hi[r], set(r), wtype, esz, fw::NF, fw::tile_box_x(esz), tby, 5, tile_promo) !=
              CUDA_SUCCESS)
        return fail(FWANT_ERR_CUDA, "tensor map encoding failed");
    }
    if (make(&tm_med, med, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 3, fw::STAGE_TX, cuuint32_t(tile_ty), 3, line) !=
        CUDA_SUCCESS)
      return fail(FWANT_ERR_CUDA, "tensor map encoding failed");
    return FWANT_OK;
  }

  // Tile shape of the stage kernel: rows 8 (every storage and form) or 16 (FP32 storage,
  // flat grid); the tensor maps' boxes follow it.
  bool tile_rows_allowed(int rows) const {
    return rows == fw::STAGE_TY || (rows == fw::STAGE_TY_TALL && stor == fw::ST_F32 && !topo_on);
  }
  fwant_status set_tile_rows(int rows) {
    if (!tile_rows_allowed(rows))
      return fail(FWANT_ERR_INVALID_ARG, "tile rows: 8, or 16 with FP32 storage and no topography");
    if (rows == tile_ty) return FWANT_OK;
    tile_ty = rows;
    fwant_status rc = make_tensor_maps();
    if (rc == FWANT_OK) rc = make_pml_maps();
    drop_graphs();
    return rc;
  }

  // TMA descriptors of the PML faces, in device memory: per face a 5-D tensor over its four
  // register sets (x: sx, y: sy, z: the slab's planes, the six variables vstride apart, the
  // sets 6 vstride apart); the stage kernel loads TX x TY x 1 x 6 x 1 boxes of them.
  fwant_status make_pml_maps() {
    using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess)
      return fail(FWANT_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    CUtensorMap maps[6];
    std::memset(maps, 0, sizeof(maps));
    bool any = false;
    for (int f = 0; f < 6; ++f) {
      const fw::Slab& s = slab[f];
      if (!s.on) continue;
      any = true;
      const cuuint64_t sz = cuuint64_t(s.k2 - s.k1 + 1), vs = cuuint64_t(s.vstride);
      const cuuint64_t dims[5] = {cuuint64_t(s.sx), cuuint64_t(s.sy), sz, 6, 4};
      const cuuint64_t strides[4] = {cuuint64_t(s.sx) * 4, cuuint64_t(s.sx) * s.sy * 4, vs * 4, 6 * vs * 4};
      const cuuint32_t box[5] = {fw::STAGE_TX, cuuint32_t(tile_ty), 1, 6, 1};
      const cuuint32_t el[5] = {1, 1, 1, 1, 1};
      if (reinterpret_cast<EncodeFn>(fn)(&maps[f], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, aux[f], dims, strides, box, el,
                                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return fail(FWANT_ERR_CUDA, "PML tensor map encoding failed");
    }
    if (!any) return FWANT_OK;
    if (!d_pml_map) {
      void* p = nullptr;
      if (cudaMalloc(&p, sizeof(maps)) != cudaSuccess) {
        cudaGetLastError();
        return fail(FWANT_ERR_OOM, "PML descriptors");
      }
      d_pml_map = static_cast<CUtensorMap*>(p);
    }
    e = cudaMemcpy(d_pml_map, maps, sizeof(maps), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "PML descriptors");
    return FWANT_OK;
  }

  // 1/z and 1/xsin for the fast arithmetic form
  cudaError_t upload_reciprocals() {
    std::vector<float> rz(g.nz), rs(g.nx);
    for (int k = 0; k < g.nz; ++k) rz[k] = 1.0f / hz[k];
    for (int i = 0; i < g.nx; ++i) rs[i] = 1.0f / hxsin[i];
    cudaMemcpy(d_rzinv, rz.data(), g.nz * 4, cudaMemcpyHostToDevice);
    return cudaMemcpy(d_rsinv, rs.data(), g.nx * 4, cudaMemcpyHostToDevice);
  }

  // Fortran (nx,ny,nz) host array -> padded device array
  cudaError_t put3(float* dst, const float* src) {
    return cudaMemcpy2D(dst + fw::PADL, size_t(g.px) * 4, src, size_t(g.nx) * 4, size_t(g.nx) * 4,
                        size_t(g.ny) * g.nz, cudaMemcpyHostToDevice);
  }
  // rho of the 7^3 box around (si, sj, sk) from the device medium; entries outside the
  // arrays stay 0 (the source weights use interior points only)
  cudaError_t fetch_rho_box(int si, int sj, int sk, float* box) {
    std::fill(box, box + 343, 0.0f);
    const int i0 = std::max(si - 3, 0), i1 = std::min(si + 3, g.nx - 1);
    if (i0 > i1) return cudaSuccess;
    for (int lk = -3; lk <= 3; ++lk)
      for (int lj = -3; lj <= 3; ++lj) {
        const int j = sj + lj, k = sk + lk;
        if (j < 0 || j >= g.ny || k < 0 || k >= g.nz) continue;
        const float* src = rho + fw::PADL + i0 + size_t(g.px) * (size_t(j) + size_t(g.ny) * k);
        const cudaError_t e = cudaMemcpy(box + (i0 - (si - 3)) + 7 * ((lj + 3) + 7 * (lk + 3)), src,
                                         size_t(i1 - i0 + 1) * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return e;
      }
    return cudaSuccess;
  }
  cudaError_t get3(float* dst, const float* src) {
    return cudaMemcpy2D(dst, size_t(g.nx) * 4, src + fw::PADL, size_t(g.px) * 4, size_t(g.nx) * 4,
                        size_t(g.ny) * g.nz, cudaMemcpyDeviceToHost);
  }

  // abs_init (mod_abs_npml.F90:135-616), isotropic build.
  fwant_status set_pml(const int* number, const float* vel, const float* bmax, const float* amax) {
    if (!have_coord) return fail(FWANT_ERR_STATE, "fwant_set_pml needs fwant_set_coord first");
    for (int f = 0; f < 6; ++f) {
      absn[f] = number[f] > 0 ? number[f] : 0;
      if (absn[f] > 0 && bmax[f] < 1.0f) return fail(FWANT_ERR_INVALID_ARG, "CFS_bmax should be >= 1");
    }
    if (absn[0] + absn[1] + 2 > cfg.ni || absn[2] + absn[3] + 2 > cfg.nj)
      return fail(FWANT_ERR_INVALID_ARG, "PML thicker than the grid");
    if (absn[5] > 0) g.freesurf = 0;  // mod_abs_npml.F90:182-184
    if (g.freesurf && absn[4] + 5 > cfg.nk)
      return fail(FWANT_ERR_INVALID_ARG, "the z1 PML must stay below the top four planes");
    for (int a = 0; a < 3; ++a) {
      std::fill(hA[a].begin(), hA[a].end(), 0.0f);
      std::fill(hB[a].begin(), hB[a].end(), 1.0f);
      std::fill(hD[a].begin(), hD[a].end(), 0.0f);
    }
    // Fortran 1-based indexing helpers on the 0-based host copies
    auto X = [&](int i) { return hx[i - 1]; };
    auto Y = [&](int j) { return hy[j - 1]; };
    auto Z = [&](int k) { return hz[k - 1]; };
    const int ni1 = 4, ni2 = 3 + cfg.ni, nj1 = 4, nj2 = 3 + cfg.nj, nk1 = 4, nk2 = 3 + cfg.nk;
    auto face = [&](int f, int axis, int lo, int hi, float L0, float dmax, auto dist) {
      for (int q = lo; q <= hi; ++q) {
        const float L = dist(q);
        hD[axis][q - 1] = fw::hm::pml_d(L, L0, dmax);
        hA[axis][q - 1] = fw::hm::pml_a(L, L0, amax[f]);
        hB[axis][q - 1] = fw::hm::pml_b(L, L0, bmax[f]);
      }
    };
    if (absn[0] > 0) {
      const float x0 = X(absn[0] + ni1), L0 = Z(nk2) * (x0 - X(ni1));
      const float dm = fw::hm::pml_dmax(L0, vel[0], fw::hm::pml_R(absn[0]));
      face(0, 0, ni1, absn[0] + ni1, L0, dm, [&](int i) { return Z(nk2) * (x0 - X(i)); });
    }
    if (absn[1] > 0) {
      const float x0 = X(ni2 - absn[1]), L0 = Z(nk2) * (X(ni2) - x0);
      const float dm = fw::hm::pml_dmax(L0, vel[1], fw::hm::pml_R(absn[1]));
      face(1, 0, ni2 - absn[1], ni2, L0, dm, [&](int i) { return Z(nk2) * (X(i) - x0); });
    }
    if (absn[2] > 0) {
      const float y0 = Y(absn[2] + nj1), L0 = Z(nk2) * (y0 - Y(nj1));
      const float dm = fw::hm::pml_dmax(L0, vel[2], fw::hm::pml_R(absn[2]));
      face(2, 1, nj1, absn[2] + nj1, L0, dm, [&](int j) { return Z(nk2) * (y0 - Y(j)); });
    }
    if (absn[3] > 0) {
      const float y0 = Y(nj2 - absn[3]), L0 = Z(nk2) * (Y(nj2) - y0);
      const float dm = fw::hm::pml_dmax(L0, vel[3], fw::hm::pml_R(absn[3]));
      face(3, 1, nj2 - absn[3], nj2, L0, dm, [&](int j) { return Z(nk2) * (Y(j) - y0); });
    }
    if (absn[4] > 0) {
      const float z0 = Z(absn[4] + nk1), L0 = z0 - Z(nk1);
      const float dm = fw::hm::pml_dmax(L0, vel[4], fw::hm::pml_R(absn[4]));
      face(4, 2, nk1, nk1 + absn[4], L0, dm, [&](int k) { return z0 - Z(k); });
    }
    if (absn[5] > 0) {
      const float z0 = Z(nk2 - absn[5]), L0 = Z(nk2) - z0;
      const float dm = fw::hm::pml_dmax(L0, vel[5], fw::hm::pml_R(absn[5]));
      face(5, 2, nk2 - absn[5], nk2, L0, dm, [&](int k) { return Z(k) - z0; });
    }
    for (int a = 0; a < 3; ++a)
      for (size_t q = 0; q < hD[a].size(); ++q) hD[a][q] = hD[a][q] / hB[a][q];  // D := d/b
    cudaError_t e = upload_profiles();
    if (e != cudaSuccess) return cuda_fail(e, "pml profiles");
    // slabs (0-based bounds)
    const int i1 = g.i1, i2 = g.i2, j1 = g.j1, j2 = g.j2, k1 = g.k1, k2 = g.k2;
    const int b[6][6] = {{i1, i1 + absn[0], j1, j2, k1, k2}, {i2 - absn[1], i2, j1, j2, k1, k2},
                         {i1, i2, j1, j1 + absn[2], k1, k2}, {i1, i2, j2 - absn[3], j2, k1, k2},
                         {i1, i2, j1, j2, k1, k1 + absn[4]}, {i1, i2, j1, j2, k2 - absn[5], k2}};
    for (int f = 0; f < 6; ++f) {
      cudaFree(aux[f]);
      aux[f] = nullptr;
      fw::Slab& s = slab[f];
      s = fw::Slab{};
      if (absn[f] <= 0) continue;
      s.on = 1;
      s.i1 = b[f][0]; s.i2 = b[f][1]; s.j1 = b[f][2]; s.j2 = b[f][3]; s.k1 = b[f][4]; s.k2 = b[f][5];
      s.ox = s.i1 - ((s.i1 - g.i1) & 3);                 // rows start 16-byte aligned under every tile
      s.sx = ((s.i2 - s.ox + 1) + 3) / 4 * 4; s.sy = s.j2 - s.j1 + 1;
      const long long n = (long long)s.sx * s.sy * (s.k2 - s.k1 + 1);
      s.vstride = ((n + 31) / 32) * 32;
      aux_set[f] = 6 * s.vstride;
      aux[f] = dalloc<float>(size_t(4) * aux_set[f]);
      if (!aux[f]) return fail(FWANT_ERR_OOM, "PML allocation failed");
      cudaMemset(aux[f], 0, size_t(4) * aux_set[f] * sizeof(float));
    }
    if (fwant_status rc = make_pml_maps(); rc != FWANT_OK) return rc;
    drop_graphs();
    src_dirty = true;  // the surface-source list depends on the free-surface flag
    return FWANT_OK;
  }

  // Resolve sources into device tables covering at least `steps` steps.
  fwant_status prepare_sources(int steps) {
    if (!src_dirty && steps <= stf_cap_steps) return FWANT_OK;
    drop_graphs();
    free_sources();
    if (upload_reciprocals() != cudaSuccess) return fail(FWANT_ERR_CUDA, "reciprocal tables");
    const int cap_steps = std::max(steps + 8, 1024);
    const int G = cap_steps * 4;
    const float incr[4] = {0.0f, RKA[0], RKA[1], RKA[2]};  // set_cur_time(ntime, firRKa(s))
    const bool surf_rate = g.freesurf && cfg.src_surface;
    const ForceDesc& F = forces;
    const MomentDesc& Mo = moments;
    const int nwf = F.num * F.ntwin, nwm = Mo.num * Mo.ntwin;
    std::vector<float> disp(size_t(G) * std::max(nwf, 1), 0.0f), rate(size_t(G) * std::max(nwf, 1), 0.0f);
    std::vector<float> mrate(size_t(G) * std::max(nwm, 1), 0.0f);
    for (int n = 0; n < cap_steps; ++n)
      for (int s = 0; s < 4; ++s) {
        const int gs = n * 4 + s;
        const float t = (float(n) + incr[s]) * stept;
        for (int q = 0; q < F.num; ++q)
          for (int m = 0; m < F.ntwin; ++m) {
            // src_surface evaluates both functions of every force, and only under a free
            // surface (mod_src.F90:384-396); src_force needs the STF alone (:312)
            float dv, rv = 0.0f;
            if (!fw::hm::stf(t - F.t0[q], F.stf_time[m], F.stf_freq[m], F.stf_id, n, stept, &dv) ||
                (surf_rate && !fw::hm::svf(t - F.t0[q], F.stf_time[m], F.stf_freq[m], F.stf_id, n, stept, &rv)))
              return fail(FWANT_ERR_INVALID_ARG, "unknown force stf id");
            disp[size_t(gs) * nwf + q * F.ntwin + m] = dv;
            rate[size_t(gs) * nwf + q * F.ntwin + m] = rv;
          }
        for (int q = 0; q < Mo.num; ++q)
          for (int m = 0; m < Mo.ntwin; ++m) {
            float rv;
            if (!fw::hm::svf(t - Mo.t0[q], Mo.stf_time[m], Mo.stf_freq[m], Mo.stf_id, n, stept, &rv))
              return fail(FWANT_ERR_INVALID_ARG, "unknown moment stf id");
            mrate[size_t(gs) * nwm + q * Mo.ntwin + m] = rv;
          }
      }
    auto X = [&](int i) { return hx[i]; };  // 0-based
    auto Y = [&](int j) { return hy[j]; };
    auto Z = [&](int k) { return hz[k]; };
    auto interior = [&](int i, int j, int k) {
      return i >= g.i1 && i <= g.i2 && j >= g.j1 && j <= g.j2 && k >= g.k1 && k <= g.k2;
    };
    // surface forces (src_surface, mod_src.F90:373-414)
    std::vector<int> surf_ij, surf_w;
    std::vector<float> surf_q;
    if (g.freesurf && cfg.src_surface)
      for (int q = 0; q < F.num; ++q) {
        const int i = F.indx[3 * q] - 1, j = F.indx[3 * q + 1] - 1, k = F.indx[3 * q + 2] - 1;
        if (!(i >= g.i1 && i <= g.i2 && j >= g.j1 && j <= g.j2 && k == g.k2)) continue;
        const float Sa = (X(i + 1) - X(i - 1)) * (Y(j + 1) - Y(j - 1)) / 4.0f * (Z(k) * Z(k)) * hxsin[i];
        for (int m = 0; m < F.ntwin; ++m) {
          const size_t w = m + size_t(F.ntwin) * q;
          surf_ij.push_back(i); surf_ij.push_back(j);
          surf_q.push_back(F.fx[w] / Sa); surf_q.push_back(F.fy[w] / Sa); surf_q.push_back(F.fz[w] / Sa);
          surf_w.push_back(q * F.ntwin + m);
        }
      }
    // body forces (src_force, mod_src.F90:275-345)
    std::vector<int> fc;
    std::vector<float> fwt, fF;
    std::vector<unsigned char> fon;
    float nd[343], rbox[343];
    for (int q = 0; q < F.num; ++q) {
      const int si = F.indx[3 * q] - 1, sj = F.indx[3 * q + 1] - 1, sk = F.indx[3 * q + 2] - 1;
      {
        const cudaError_t re = fetch_rho_box(si, sj, sk, rbox);
        if (re != cudaSuccess) return cuda_fail(re, "source weights: rho");
      }
      if (!fw::hm::norm_delt(nd, F.shift[3 * q], F.shift[3 * q + 1], F.shift[3 * q + 2]))
        return fail(FWANT_ERR_INVALID_ARG, "cal_norm_delt is zero");
      if (g.freesurf && sk + 3 > g.k2) {
        float s = 0.0f;
        for (int lk = -3; lk <= g.k2 - sk; ++lk)
          for (int lj = -3; lj <= 3; ++lj)
            for (int li = -3; li <= 3; ++li) s += nd[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))];
        for (int e = 0; e < 343; ++e) nd[e] = nd[e] / s;
      }
      fc.push_back(si); fc.push_back(sj); fc.push_back(sk);
      for (int lk = -3; lk <= 3; ++lk)
        for (int lj = -3; lj <= 3; ++lj)
          for (int li = -3; li <= 3; ++li) {
            const int i = si + li, j = sj + lj, k = sk + lk;
            const float d = nd[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))];
            float wv = 0.0f;
            unsigned char on = 0;
            if (interior(i, j, k)) {
              float V = (X(i + 1) - X(i - 1)) * (Y(j + 1) - Y(j - 1)) * (Z(k + 1) - Z(k - 1)) / 8.0f * (Z(k) * Z(k)) * hxsin[i];
              V = 1.0f / (V * rbox[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))]) * d;
              on = 1;
              wv = V;
              if (g.freesurf && k == g.k2) {
                if (cfg.src_surface) on = 0;
                else wv = 2.0f * V;  // exact: fx*2 == fx0*(2V) in binary floating point
              }
            }
            fwt.push_back(wv);
            fon.push_back(on);
          }
      for (int m = 0; m < F.ntwin; ++m) {
        const size_t w = m + size_t(F.ntwin) * q;
        fF.push_back(F.fx[w]); fF.push_back(F.fy[w]); fF.push_back(F.fz[w]);
      }
    }
    // moment tensors (src_stress, mod_src.F90:207-273)
    std::vector<int> mc;
    std::vector<float> md, mvol, mM;
    std::vector<unsigned char> mon;
    for (int q = 0; q < Mo.num; ++q) {
      const int si = Mo.indx[3 * q] - 1, sj = Mo.indx[3 * q + 1] - 1, sk = Mo.indx[3 * q + 2] - 1;
      if (!fw::hm::norm_delt(nd, Mo.shift[3 * q], Mo.shift[3 * q + 1], Mo.shift[3 * q + 2]))
        return fail(FWANT_ERR_INVALID_ARG, "cal_norm_delt is zero");
      if (g.freesurf && sk + 3 > g.k2) {
        float s = 0.0f;
        for (int lk = -3; lk <= g.k2 - sk; ++lk)
          for (int lj = -3; lj <= 3; ++lj)
            for (int li = -3; li <= 3; ++li) s += nd[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))];
        for (int e = 0; e < 343; ++e) nd[e] = nd[e] / s;
      }
      mc.push_back(si); mc.push_back(sj); mc.push_back(sk);
      for (int lk = -3; lk <= 3; ++lk)
        for (int lj = -3; lj <= 3; ++lj)
          for (int li = -3; li <= 3; ++li) {
            const int i = si + li, j = sj + lj, k = sk + lk;
            const bool in = interior(i, j, k);
            md.push_back(nd[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))]);
            mvol.push_back(in ? (X(i + 1) - X(i - 1)) * (Y(j + 1) - Y(j - 1)) * (Z(k + 1) - Z(k - 1)) / 8.0f * (Z(k) * Z(k)) * hxsin[i]
                              : 1.0f);
            mon.push_back(in ? 1 : 0);
          }
      const size_t nb = size_t(Mo.ntwin) * Mo.num;
      for (int m = 0; m < Mo.ntwin; ++m)
        for (int c = 0; c < 6; ++c) mM.push_back(Mo.mom[c * nb + m + size_t(Mo.ntwin) * q]);
    }
    S.G = G;
    S.nw_f = nwf; S.nw_m = nwm;
    S.disp = upload(disp); S.rate = upload(rate); S.mrate = upload(mrate);
    S.nsurf = int(surf_w.size());
    S.surf_ij = upload(surf_ij); S.surf_q = upload(surf_q); S.surf_w = upload(surf_w);
    h_force_c = fc;
    h_mom_c = mc;
    S.nforce = F.num; S.ntwin_f = F.ntwin;
    S.force_c = upload(fc); S.force_wt = upload(fwt); S.force_on = upload(fon); S.force_F = upload(fF);
    S.nmom = Mo.num; S.ntwin_m = Mo.ntwin;
    S.mom_c = upload(mc); S.mom_d = upload(md); S.mom_vol = upload(mvol); S.mom_on = upload(mon);
    S.mom_M = upload(mM);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "source tables");
    stf_cap_steps = cap_steps;
    src_dirty = false;
    return FWANT_OK;
  }

  fwant_status prepare_receivers(int end_step) {
    if (npt <= 0) return FWANT_OK;
    const int need = end_step / tinv + 1;
    if (need <= cap && d_rec) return FWANT_OK;
    drop_graphs();
    const int ncap = std::max(need + 64, 2 * cap);
    float* ns = dalloc<float>(size_t(fw::NF) * ncap * npt);
    if (!ns) return fail(FWANT_ERR_OOM, "seismogram buffer");
    cudaMemset(ns, 0, size_t(fw::NF) * ncap * npt * sizeof(float));
    if (d_seis && cap > 0)
      for (int f = 0; f < fw::NF; ++f)
        cudaMemcpy(ns + size_t(f) * ncap * npt, d_seis + size_t(f) * cap * npt, size_t(cap) * npt * 4,
                   cudaMemcpyDeviceToDevice);
    cudaFree(d_seis);
    d_seis = ns;
    cap = ncap;
    if (!d_rec) {
      d_rec = dalloc<int>(rec_idx.size());
      if (!d_rec) return fail(FWANT_ERR_OOM, "receiver index");
      cudaMemcpy(d_rec, rec_idx.data(), rec_idx.size() * sizeof(int), cudaMemcpyHostToDevice);
    }
    return FWANT_OK;
  }

  fw::StageArgs base_args() const {
    fw::StageArgs a{};
    a.g = g;
    a.tm_med = tm_med;
    a.err = d_err;
    a.sv = sv; a.st = sc_t; a.isv = 1.0f / sv; a.ist = 1.0f / sc_t;
    a.xi_x = d_xi; a.eta_y = d_eta; a.zeta_z = d_zeta; a.xsin = d_xsin; a.xcot = d_xcot; a.zc = d_z;
    a.rzinv = d_rzinv; a.rsinv = d_rsinv;
    for (int ax = 0; ax < 3; ++ax) {
      a.pb1[ax] = prof(ax, 0); a.pb11[ax] = prof(ax, 1); a.pad[ax] = prof(ax, 2); a.pD[ax] = prof(ax, 3);
    }
    a.kc = kc;
    fw::stage_z_bands(g, slab, &a.kz_lo, &a.kz_hi);
    for (int f = 0; f < 6; ++f) a.slab[f] = slab[f];
    a.ntime = d_ntime;
    a.src = S;
    return a;
  }

  // One time step: four fused stage launches and the receiver/counter kernel.
  // Register-set roles: A holds W at the step start (and is the RK "m" register), T is
  // the RK "t" accumulator; B and C are the stage outputs.  Stage 4 writes W(n+1) into
  // T in place, after which A and T swap roles.
  // Work-item lists of the stage launches for the current k-chunk, PML and sources
  // (rebuilt, and the graphs dropped, when they change).
  fwant_status ensure_items() {
    int kz_lo, kz_hi;
    fw::stage_z_bands(g, slab, &kz_lo, &kz_hi);
    const long long n = fw::stage_item_count(g, kc, tile_ty, kz_lo, kz_hi);
    std::vector<int> lean(static_cast<size_t>(n)), full(static_cast<size_t>(n));
    int nl = 0, nf = 0;
    fw::stage_items(g, kc, tile_ty, kz_lo, kz_hi, slab, h_force_c.data(), int(h_force_c.size() / 3),
                    h_mom_c.data(), int(h_mom_c.size() / 3), lean.data(), &nl, full.data(), &nf);
    // lean items, full items, then every item in launch order (x fastest, then y, k)
    std::vector<int> all(lean.begin(), lean.begin() + nl);
    all.insert(all.end(), full.begin(), full.begin() + nf);
    {
      const int nbx = (g.ni + fw::STAGE_TX - 1) / fw::STAGE_TX, nby = (g.nj + tile_ty - 1) / tile_ty;
      const int nbz = fw::stage_chunk_count(g, kc, kz_lo, kz_hi);
      for (int bz = 0; bz < nbz; ++bz)
        for (int by = 0; by < nby; ++by)
          for (int bx = 0; bx < nbx; ++bx) all.push_back(int(unsigned(bx) | unsigned(by) << 10 | unsigned(bz) << 20));
    }
    if (d_items && nl == n_lean && all == h_items) return FWANT_OK;
    cudaFree(d_items);
    d_items = dalloc<int>(all.size());
    if (!d_items) return fail(FWANT_ERR_OOM, "work items");
    cudaError_t e = cudaMemcpy(d_items, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "work items");
    h_items = std::move(all);
    n_lean = nl;
    n_full = nf;
    drop_graphs();
    return FWANT_OK;
  }
  // Items of one launch of RK kind rk: lean = 1 the interior items, lean = 0 the others,
  // or all items in launch order when the lean form is off for rk.
  // Default split: stages 1 and 4 (mask 5); with the stages without t also stages 2 and 3
  // (7: stage 2 then moves 30 floats per point and gains from the interior-only form).
  int lean_stages() const { return lean_mask >= 0 ? lean_mask : (recon_on() ? 7 : 5); }
  bool lean_on(int rk) const { return !topo_on && (lean_stages() >> fw::rk_base(rk) & 1) != 0; }
  const int* items(bool lean, int rk) const {
    if (!lean_on(rk)) return d_items + n_lean + n_full;
    return d_items + (lean ? 0 : n_lean);
  }
  int item_count(bool lean, int rk) const {
    if (!lean_on(rk)) return lean ? 0 : n_lean + n_full;
    return lean ? n_lean : n_full;
  }

  // Arguments of stage s (0..3) of a step that starts with W in register set ra (the
  // other of sets 0 and 3 is the accumulator T).
  fw::StageArgs stage_args(int s, int ra) const {
    const int rt = 3 - ra;
    fw::StageArgs a = base_args();
    const int in_of[4] = {ra, rB, rC, rB};
    const int out_of[4] = {rB, rC, rB, rt};
    a.win = set(in_of[s]); a.wout = set(out_of[s]); a.wt = set(rt); a.wm = set(ra);
    a.tm_tile = tm_tile[in_of[s]]; a.tm_q = tm_q[in_of[s]]; a.tm_m = tm_pt[ra]; a.tm_t = tm_pt[rt];
    a.tm_tile_lo = tm_tile_lo[in_of[s]]; a.tm_tile_hi = tm_tile_hi[in_of[s]];
    if (topo_on) {  // the terrain form queues all nine components
      a.tm_q = tm_pt[in_of[s]];
      a.tm_topo = tm_topo;
      a.topo_sf = d_topo_sf;
    }
    a.pml_map = d_pml_map;
    a.pml_set[0] = in_of[s]; a.pml_set[1] = ra; a.pml_set[2] = rt;
    if (s == 2 && recon_on()) {  // stage 3 reads W2 (register set rB, its output) as t-in
      a.tm_t = tm_pt[rB];
      a.pml_set[2] = rB;
    }
    for (int f = 0; f < 6; ++f) {
      if (!slab[f].on) continue;
      a.ain[f] = aset(f, in_of[s]); a.am[f] = aset(f, ra); a.aout[f] = aset(f, out_of[s]); a.at[f] = aset(f, rt);
    }
    a.a = RKA[s] * stept;
    a.b = RKB[s] * stept;
    a.stage = s;
    return a;
  }
  static int stage_variant(int cpos, int s) {
    const int X = CYCLE[cpos & 7];
    return (s % 2 == 0) ? X : (~X & 7);
  }
  // The classical RK4 step without carrying t through stages 1-3 (RK kinds 3, 4, 5, then
  // RK_fin): the fast form, every storage.
  bool recon_on() const { return rk_scheme == 1 && !cfg.exact_arith; }
  int stage_rk(int s) const {
    if (recon_on()) return s == 0 ? 3 : (s == 1 ? 4 : (s == 2 ? 5 : 2));
    return s == 0 ? 0 : (s == 3 ? 2 : 1);
  }

  // Step-end work of one simulation: receivers, step counter, SGT frame.
  fw::RecvArgs recv_args(int rt) const {
    fw::RecvArgs r{};
    r.g = g; r.w = set(rt); r.npt = npt; r.idx = d_rec; r.tinv = tinv; r.seismo = d_seis; r.cap = cap;
    r.storage = stor; r.isv = 1.0f / sv; r.ist = 1.0f / sc_t;
    r.ntime = d_ntime;
    return r;
  }
  fw::SgtRecArgs sgt_args(int rt) const {
    fw::SgtRecArgs q = sgt;
    q.w = set(rt);
    return q;
  }
  // Returns the number of kernels launched.
  int enqueue_step_end(cudaStream_t stream) const {
    fw::launch_advance_record(recv_args(rT), stream);
    if (sgt_on) fw::launch_record_sgt(sgt_args(rT), stream);
    return sgt_on ? 2 : 1;
  }
  // Bytes of every launch argument of a step for both register-role assignments: equal
  // signatures mean a captured graph of this simulation's launches is still valid.
  void append_signature(std::vector<unsigned char>& sig) const {
    auto put = [&](const void* p, size_t n) {
      const auto* c = static_cast<const unsigned char*>(p);
      sig.insert(sig.end(), c, c + n);
    };
    for (int ra : {0, 3}) {
      for (int s = 0; s < 4; ++s) {
        const fw::StageArgs a = stage_args(s, ra);
        put(&a, sizeof(a));
      }
      const fw::RecvArgs r = recv_args(3 - ra);
      put(&r, sizeof(r));
      if (sgt_on) {
        const fw::SgtRecArgs q = sgt_args(3 - ra);
        put(&q, sizeof(q));
      }
    }
    put(&kc, sizeof(kc));
    put(&d_items, sizeof(d_items));
    put(&n_lean, sizeof(n_lean));
    put(&n_full, sizeof(n_full));
    put(&lean_mask, sizeof(lean_mask));
    put(&topo_on, sizeof(topo_on));
    put(&rk_scheme, sizeof(rk_scheme));
  }
  void finish_step_host() {
    std::swap(rA, rT);
    cycle_pos = (cycle_pos + 1) & 7;
    ntime += 1;
  }

  // One time step: per RK stage the lean launch over the interior items and the full
  // launch over the others, then the step-end kernels.
  int enqueue_step(cudaEvent_t* ev = nullptr) {
    int lerr = 0;
    static thread_local fw::BatchArgs b;  // 30 KB: kept off the stack
    for (int s = 0; s < 4; ++s) {
      if (ev) cudaEventRecord(ev[s], st);
      b.sims[0] = stage_args(s, rA);
      b.nsims = 1;
      const int rk = stage_rk(s);
      const bool both = fork.on && item_count(true, rk) > 0 && item_count(false, rk) > 0;
      if (both) fork.begin(st);
      for (int lean = 0; lean <= 1; ++lean) {  // the full form first, on the side stream
        const int cnt = item_count(lean, rk);
        if (cnt == 0) continue;
        b.items[0] = items(lean, rk);
        b.off[0] = 0;
        b.off[1] = cnt;
        b.total = cnt;
        cudaStream_t ls = (both && !lean) ? fork.side : st;
        const int le = topo_on ? fw::launch_stage_batch_topo(b, stage_variant(cycle_pos, s), rk, cfg.exact_arith,
                                                             cnt, ls)
                               : fw::launch_stage_batch(b, stage_variant(cycle_pos, s), rk, cfg.exact_arith, stor,
                                                        lean, cnt, ls, tile_ty);
        if (le && !lerr) lerr = le;
      }
      if (both) fork.end(st);
    }
    if (ev) cudaEventRecord(ev[4], st);
    enqueue_step_end(st);
    if (ev) cudaEventRecord(ev[5], st);
    finish_step_host();
    return lerr;
  }

  // Validate a snapshot request (io_snap_read/corr_indx, mod_io.F90:180-300: the
  // sub-volume lies in the interior) and fill the pack-kernel arguments; n = floats out.
  fwant_status snap_setup(const int* subs, const int* subc, const int* subt, int ncomp, const int* comps,
                          fw::SnapArgs& a, size_t& n) {
    if (!subs || !subc || !subt || !comps || ncomp < 1 || ncomp > fw::NF)
      return fail(FWANT_ERR_INVALID_ARG, "snapshot: bad arguments");
    a = fw::SnapArgs{};
    a.g = g;
    a.w = set(rA);
    a.storage = stor; a.isv = 1.0f / sv; a.ist = 1.0f / sc_t;
    const int lo[3] = {g.i1, g.j1, g.k1}, hi[3] = {g.i2, g.j2, g.k2};
    for (int d = 0; d < 3; ++d) {
      if (subc[d] < 1 || subt[d] < 1) return fail(FWANT_ERR_INVALID_ARG, "snapshot: counts and strides must be >= 1");
      // 64-bit end index: a large stride x count must not wrap back into the interior
      const long long s0 = (long long)subs[d] - 1;
      const long long e0 = s0 + (long long)subt[d] * ((long long)subc[d] - 1);
      if (s0 < lo[d] || e0 > hi[d]) return fail(FWANT_ERR_INVALID_ARG, "snapshot: sub-volume outside the interior");
      a.start[d] = s0; a.cnt[d] = subc[d]; a.stride[d] = subt[d];
    }
    for (int c = 0; c < ncomp; ++c) {
      if (comps[c] < 0 || comps[c] >= fw::NF) return fail(FWANT_ERR_INVALID_ARG, "snapshot: bad component id");
      a.comp[c] = fw::ABI2INT[comps[c]];
    }
    a.ncomp = ncomp;
    n = size_t(subc[0]) * subc[1] * subc[2] * ncomp;
    return FWANT_OK;
  }

  // device error word written by the stage kernel's bounded waits
  fwant_status check_device_error() {
    int h = 0;
    cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (h == fw::DEVERR_TMA_TIMEOUT) {
      cudaMemset(d_err, 0, sizeof(int));
      return fail(FWANT_ERR_TIMEOUT, "stage kernel: TMA copy did not complete within the wait bound");
    }
    return FWANT_OK;
  }

  // ---- terrain-following grid (Gaussian-hill extension) ----------------------------------
  // Metric of r = z(k) + h(i,j) s(k) from the current coordinates and 1-D metric (FP64 on
  // the device); s(k) and z_zeta(k) are formed here in double, in the order the CPU
  // restatement uses.
  fwant_status topo_compute() {
    const int nz = g.nz;
    std::vector<double> zd(nz), sk(nz), rzf(nz);
    for (int k = 0; k < nz; ++k) zd[k] = double(hz[k]);
    const double cF[5] = {-0.30874, -0.6326, 1.2330, -0.3334, 0.04168};
    const double cB[5] = {-0.04168, 0.3334, -1.2330, 0.6326, 0.30874};
    for (int k = 0; k < nz; ++k) {
      sk[k] = (zd[k] - zd[0]) / (zd[g.k2] - zd[0]);
      const int kk = std::min(std::max(k, g.k1), g.k2);
      double sb = 0.0, sf = 0.0;
      for (int q = 0; q < 5; ++q) {
        sb = sb + zd[kk - 3 + q] * cB[q];
        sf = sf + zd[kk - 1 + q] * cF[q];
      }
      rzf[k] = (sb + sf) * 0.5;
    }
    cudaError_t e = cudaMemcpy(d_sk, sk.data(), nz * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_rzf, rzf.data(), nz * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "topography tables");
    fw::launch_topo_slopes(g, d_h, d_hxi, d_heta, st);
    fw::TopoMetricArgs a{};
    a.g = g; a.h = d_h; a.hxi = d_hxi; a.heta = d_heta;
    a.z = d_z; a.xi_x = d_xi; a.eta_y = d_eta; a.zeta_z = d_zeta; a.xsin = d_xsin;
    a.sk = d_sk; a.rzf = d_rzf; a.out = d_topo;
    fw::launch_topo_metric(a, st);
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "topography metric");
    topo_sf_dirty = true;
    drop_graphs();
    return FWANT_OK;
  }

  fwant_status set_topography(const float* h) {
    if (!have_coord || !have_metric)
      return fail(FWANT_ERR_STATE, "fwant_set_topography needs the coordinates and the metric first");
    if (stor != fw::ST_F32) return fail(FWANT_ERR_INVALID_ARG, "the terrain-following grid runs with FP32 storage");
    if (tile_ty != fw::STAGE_TY) return fail(FWANT_ERR_INVALID_ARG, "the terrain-following grid runs with 32 x 8 tiles");
    for (size_t q = 0; q < size_t(g.nx) * g.ny; ++q)
      if (!std::isfinite(h[q])) return fail(FWANT_ERR_INVALID_ARG, "topography: non-finite height");
    const size_t n2 = size_t(g.nx) * g.ny;
    if (!d_topo) {
      d_h = dalloc<float>(n2); d_hxi = dalloc<double>(n2); d_heta = dalloc<double>(n2);
      d_sk = dalloc<double>(g.nz); d_rzf = dalloc<double>(g.nz);
      d_topo = dalloc<float>(4 * size_t(g.fstride));
      d_topo_sf = dalloc<float>(11 * size_t(g.plane));
      if (!d_h || !d_hxi || !d_heta || !d_sk || !d_rzf || !d_topo || !d_topo_sf)
        return fail(FWANT_ERR_OOM, "topography arrays");
      cudaMemset(d_topo, 0, 4 * size_t(g.fstride) * sizeof(float));
      cudaMemset(d_topo_sf, 0, 11 * size_t(g.plane) * sizeof(float));
      using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult qr;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr) !=
              cudaSuccess || !fn || qr != cudaDriverEntryPointSuccess)
        return fail(FWANT_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
      const cuuint64_t dims[4] = {cuuint64_t(g.px), cuuint64_t(g.ny), cuuint64_t(g.nz), 4};
      const cuuint64_t strides[3] = {cuuint64_t(g.px) * 4, cuuint64_t(g.plane) * 4, cuuint64_t(g.fstride) * 4};
      const cuuint32_t box[4] = {fw::STAGE_TX, fw::STAGE_TY, 1, 4};
      const cuuint32_t el[4] = {1, 1, 1, 1};
      if (reinterpret_cast<EncodeFn>(fn)(&tm_topo, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, d_topo, dims, strides, box, el,
                                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return fail(FWANT_ERR_CUDA, "tensor map encoding failed");
    }
    cudaError_t e = cudaMemcpy(d_h, h, n2 * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "topography upload");
    topo_on = true;
    return topo_compute();
  }

  // surface arrays of the terrain form (they need the medium)
  fwant_status topo_prepare() {
    if (!topo_on || !topo_sf_dirty) return FWANT_OK;
    fw::launch_topo_surface(g, d_topo, lam, mu, d_topo_sf, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "topography surface arrays");
    topo_sf_dirty = false;
    return FWANT_OK;
  }

  fwant_status run(int nsteps) {
    if (nsteps < 0) return fail(FWANT_ERR_INVALID_ARG, "nsteps < 0");
    if (!have_coord || !have_metric || !have_media)
      return fail(FWANT_ERR_STATE, "coordinates, metric and media must be set before fwant_run");
    cudaSetDevice(cfg.device);
    fwant_status rc = prepare_sources(ntime + nsteps);
    if (rc != FWANT_OK) return rc;
    if ((rc = prepare_receivers(ntime + nsteps)) != FWANT_OK) return rc;
    if ((rc = ensure_items()) != FWANT_OK) return rc;
    if ((rc = topo_prepare()) != FWANT_OK) return rc;
    cudaEventRecord(ev0, st);
    int left = nsteps;
    while (left > 0) {
      if (cycle_pos == 0 && left >= 8) {
        const int gi = rA == 0 ? 0 : 1;
        if (!graph[gi]) {
          const int save_ntime = ntime;
          cudaGraph_t gr;
          cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
          if (e != cudaSuccess) return cuda_fail(e, "begin capture");
          int lerr = 0;
          for (int q = 0; q < 8; ++q) lerr |= enqueue_step();
          e = cudaStreamEndCapture(st, &gr);
          if (e == cudaSuccess && lerr) e = cudaError_t(lerr);
          if (e != cudaSuccess) return cuda_fail(e, "end capture");
          ntime = save_ntime;
          e = cudaGraphInstantiate(&graph[gi], gr, 0);
          cudaGraphDestroy(gr);
          if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
        }
        cudaError_t e = cudaGraphLaunch(graph[gi], st);
        if (e != cudaSuccess) return cuda_fail(e, "graph launch");
        ntime += 8;
        left -= 8;
      } else {
        const int le = enqueue_step();
        if (le) return cuda_fail(cudaError_t(le), "stage launch");
        left -= 1;
      }
    }
    cudaEventRecord(ev1, st);
    cudaError_t e = cudaEventSynchronize(ev1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "run");
    if ((rc = check_device_error()) != FWANT_OK) return rc;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    last_ms = ms;
    if (npt > 0) nsamp = std::max(nsamp, std::min(ntime / tinv, cap));
    return FWANT_OK;
  }

  // Back to the state before the first step (zero wavefield, memory variables, records),
  // keeping the model, sources and receivers.
  cudaError_t reset_state() {
    cudaError_t e = cudaMemsetAsync(regs, 0, size_t(4) * fw::NF * g.fstride * esz, st);
    for (int f = 0; f < 6 && e == cudaSuccess; ++f)
      if (aux[f]) e = cudaMemsetAsync(aux[f], 0, size_t(4) * aux_set[f] * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_ntime, 0, sizeof(int), st);
    if (e == cudaSuccess && d_seis) e = cudaMemsetAsync(d_seis, 0, size_t(fw::NF) * cap * npt * sizeof(float), st);
    if (e == cudaSuccess && sgt_on)
      e = cudaMemsetAsync(d_sgt, 0, size_t(6) * sgt.max_frames * sgt.npts * sizeof(float), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ntime = 0; cycle_pos = 0; rA = 0; rT = 3; nsamp = 0;
    return e;
  }

  // Eager steps with CUDA events around every launch: average device time of the four
  // stage launches (index = stage inside the step) and of the step-end kernel.
  fwant_status profile(int nsteps, double* stage_ms, double* other_ms) {
    if (nsteps <= 0) return fail(FWANT_ERR_INVALID_ARG, "nsteps <= 0");
    if (!have_coord || !have_metric || !have_media)
      return fail(FWANT_ERR_STATE, "coordinates, metric and media must be set before profiling");
    cudaSetDevice(cfg.device);
    fwant_status rc = prepare_sources(ntime + nsteps);
    if (rc != FWANT_OK) return rc;
    if ((rc = prepare_receivers(ntime + nsteps)) != FWANT_OK) return rc;
    if ((rc = ensure_items()) != FWANT_OK) return rc;
    if ((rc = topo_prepare()) != FWANT_OK) return rc;
    std::vector<cudaEvent_t> ev(size_t(6) * nsteps);
    for (auto& e : ev) cudaEventCreate(&e);
    int lerr = 0;
    for (int q = 0; q < nsteps; ++q) lerr |= enqueue_step(&ev[size_t(6) * q]);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    double acc[5] = {0, 0, 0, 0, 0};
    if (e == cudaSuccess)
      for (int q = 0; q < nsteps; ++q)
        for (int k = 0; k < 5; ++k) {
          float ms = 0.0f;
          cudaEventElapsedTime(&ms, ev[size_t(6) * q + k], ev[size_t(6) * q + k + 1]);
          acc[k] += ms;
        }
    for (auto& x : ev) cudaEventDestroy(x);
    if (e == cudaSuccess && lerr) e = cudaError_t(lerr);
    if (e != cudaSuccess) return cuda_fail(e, "profile");
    if ((rc = check_device_error()) != FWANT_OK) return rc;
    for (int k = 0; k < 4; ++k) stage_ms[k] = acc[k] / nsteps;
    *other_ms = acc[4] / nsteps;
    if (npt > 0) nsamp = std::max(nsamp, std::min(ntime / tinv, cap));
    return FWANT_OK;
  }
};

extern "C" {

const char* fwant_version(void) { return "fwant_gb300 0.1 (sm_103a)"; }

fwant_status fwant_source_time_function(int which, int stf_id, float t, float t0, float f0, int ntime, float stept,
                                        float* out) {
  if (!out || (which != 0 && which != 1)) return FWANT_ERR_INVALID_ARG;
  const bool ok = which == 0 ? fw::hm::stf(t, t0, f0, stf_id, ntime, stept, out)
                             : fw::hm::svf(t, t0, f0, stf_id, ntime, stept, out);
  return ok ? FWANT_OK : FWANT_ERR_INVALID_ARG;
}

fwant_status fwant_create(const fwant_config* cfg, fwant_solver** out) {
  if (!cfg || !out) return FWANT_ERR_INVALID_ARG;
  *out = nullptr;
  fwant_solver* s = new (std::nothrow) fwant_solver;
  if (!s) return FWANT_ERR_OOM;
  s->cfg = *cfg;
  fwant_status rc = s->init();
  if (rc != FWANT_OK) {
    std::fprintf(stderr, "fwant_create: %s\n", s->err.c_str());
    delete s;
    return rc;
  }
  *out = s;
  return FWANT_OK;
}

void fwant_destroy(fwant_solver* s) { delete s; }

const char* fwant_last_error(const fwant_solver* s) { return s ? s->err.c_str() : "null handle"; }

fwant_status fwant_set_coord(fwant_solver* s, const float* x, const float* y, const float* z) {
  if (!s || !x || !y || !z) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  s->hx.assign(x, x + s->g.nx); s->hy.assign(y, y + s->g.ny); s->hz.assign(z, z + s->g.nz);
  cudaMemcpy(s->d_x, x, s->g.nx * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->d_y, y, s->g.ny * 4, cudaMemcpyHostToDevice);
  cudaError_t e = cudaMemcpy(s->d_z, z, s->g.nz * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return s->cuda_fail(e, "set_coord");
  s->have_coord = true;
  s->src_dirty = true;
  return (s->topo_on && s->have_metric) ? s->topo_compute() : FWANT_OK;
}

fwant_status fwant_set_metric(fwant_solver* s, const float* xsin, const float* xcot, const float* xi_x,
                              const float* eta_y, const float* zeta_z) {
  if (!s || !xsin || !xcot || !xi_x || !eta_y || !zeta_z) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  const auto& g = s->g;
  s->hxsin.assign(xsin, xsin + g.nx); s->hxcot.assign(xcot, xcot + g.nx);
  cudaMemcpy(s->d_xsin, xsin, g.nx * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->d_xcot, xcot, g.nx * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->d_xi, xi_x, g.nx * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->d_eta, eta_y, g.ny * 4, cudaMemcpyHostToDevice);
  cudaError_t e = cudaMemcpy(s->d_zeta, zeta_z, g.nz * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return s->cuda_fail(e, "set_metric");
  s->have_metric = true;
  s->src_dirty = true;
  return s->topo_on ? s->topo_compute() : FWANT_OK;
}

fwant_status fwant_compute_metric(fwant_solver* s) {
  if (!s) return FWANT_ERR_INVALID_ARG;
  if (!s->have_coord) return s->fail(FWANT_ERR_STATE, "fwant_compute_metric needs fwant_set_coord first");
  cudaSetDevice(s->cfg.device);
  const auto& g = s->g;
  fw::launch_sincot_fp64(g.nx, s->d_x, s->d_xsin, s->d_xcot, s->st);
  fw::launch_metric_fp64(g.nx, s->d_x, s->d_xi, g.i1, g.i2, s->st);
  fw::launch_metric_fp64(g.ny, s->d_y, s->d_eta, g.j1, g.j2, s->st);
  fw::launch_metric_fp64(g.nz, s->d_z, s->d_zeta, g.k1, g.k2, s->st);
  cudaError_t e = cudaStreamSynchronize(s->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return s->cuda_fail(e, "compute_metric");
  s->hxsin.resize(g.nx); s->hxcot.resize(g.nx);
  cudaMemcpy(s->hxsin.data(), s->d_xsin, g.nx * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(s->hxcot.data(), s->d_xcot, g.nx * 4, cudaMemcpyDeviceToHost);
  s->have_metric = true;
  s->src_dirty = true;
  return s->topo_on ? s->topo_compute() : FWANT_OK;
}

fwant_status fwant_set_topography(fwant_solver* s, const float* h) {
  if (!s || !h) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  return s->set_topography(h);
}

fwant_status fwant_get_topography_array(fwant_solver* s, int which, float* out) {
  if (!s || !out || which < 0 || which > 14) return FWANT_ERR_INVALID_ARG;
  if (!s->topo_on) return s->fail(FWANT_ERR_STATE, "no topography set");
  cudaSetDevice(s->cfg.device);
  fwant_status rc = s->topo_prepare();
  if (rc != FWANT_OK) return rc;
  const auto& g = s->g;
  cudaError_t e;
  if (which < 4) {
    e = s->get3(out, s->d_topo + size_t(which) * g.fstride);
  } else {
    e = cudaMemcpy2D(out, size_t(g.nx) * 4, s->d_topo_sf + size_t(which - 4) * g.plane + fw::PADL, size_t(g.px) * 4,
                     size_t(g.nx) * 4, size_t(g.ny), cudaMemcpyDeviceToHost);
  }
  return e == cudaSuccess ? FWANT_OK : s->cuda_fail(e, "get_topography_array");
}

fwant_status fwant_metric_arrays(int ni, int nj, int nk, const float* x, const float* y, const float* z, int device,
                                 float* xsin, float* xcot, float* xi_x, float* eta_y, float* zeta_z) {
  if (ni < 2 || nj < 2 || nk < 2 || !x || !y || !z || !xsin || !xcot || !xi_x || !eta_y || !zeta_z)
    return FWANT_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return FWANT_ERR_CUDA;
  const int nx = ni + 6, ny = nj + 6, nz = nk + 6;
  // one buffer: x, y, z, then xsin, xcot, xi_x, eta_y, zeta_z
  const size_t n = size_t(3) * nx + 2 * size_t(ny) + 2 * size_t(nz) + 2 * size_t(nx);
  float* d = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaMalloc(&d, n * sizeof(float));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  float *dx = d, *dy = dx + nx, *dz = dy + ny, *dsin = dz + nz, *dcot = dsin + nx, *dxi = dcot + nx,
        *deta = dxi + nx, *dzeta = deta + ny;
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, nx * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y, ny * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z, nz * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    fw::launch_sincot_fp64(nx, dx, dsin, dcot, st);
    fw::launch_metric_fp64(nx, dx, dxi, 3, 3 + ni - 1, st);
    fw::launch_metric_fp64(ny, dy, deta, 3, 3 + nj - 1, st);
    fw::launch_metric_fp64(nz, dz, dzeta, 3, 3 + nk - 1, st);
    e = cudaGetLastError();
  }
  const std::pair<float*, std::pair<const float*, int>> outs[] = {
      {xsin, {dsin, nx}}, {xcot, {dcot, nx}}, {xi_x, {dxi, nx}}, {eta_y, {deta, ny}}, {zeta_z, {dzeta, nz}}};
  for (const auto& o : outs)
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(o.first, o.second.first, o.second.second * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (st) cudaStreamDestroy(st);
  if (d) cudaFree(d);
  return e == cudaSuccess ? FWANT_OK : FWANT_ERR_CUDA;
}

fwant_status fwant_get_metric(fwant_solver* s, float* xsin, float* xcot, float* xi_x, float* eta_y,
                              float* zeta_z) {
  if (!s || !xsin || !xcot || !xi_x || !eta_y || !zeta_z) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  const auto& g = s->g;
  cudaMemcpy(xsin, s->d_xsin, g.nx * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(xcot, s->d_xcot, g.nx * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(xi_x, s->d_xi, g.nx * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(eta_y, s->d_eta, g.ny * 4, cudaMemcpyDeviceToHost);
  cudaError_t e = cudaMemcpy(zeta_z, s->d_zeta, g.nz * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return s->cuda_fail(e, "get_metric");
  return FWANT_OK;
}

// Medium from host arrays (through a device staging buffer, one large copy each) or from
// device arrays; rho is checked on the device before anything is overwritten, then each
// array goes into the padded layout.
static fwant_status load_media(fwant_solver* s, const float* lambda, const float* mu, const float* rho,
                               bool on_device) {
  if (!s || !lambda || !mu || !rho) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  const auto& g = s->g;
  const size_t n = size_t(g.nx) * g.ny * g.nz;
  float* staging = nullptr;
  const size_t bytes = on_device ? 256 : n * sizeof(float) + 256;
  cudaError_t e = cudaMalloc(&staging, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return s->fail(FWANT_ERR_OOM, "set_media: no device memory for the staging buffer");
  }
  unsigned int* bad = reinterpret_cast<unsigned int*>(reinterpret_cast<char*>(staging) + bytes - 128);
  unsigned int hbad = 0;
  const float* drho = rho;
  if (!on_device) {
    e = cudaMemcpy(staging, rho, n * sizeof(float), cudaMemcpyHostToDevice);
    drho = staging;
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s->st);
  if (e == cudaSuccess) {
    fw::launch_count_nonpositive((long long)n, drho, bad, s->st);
    e = cudaMemcpyAsync(&hbad, bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, s->st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  if (e == cudaSuccess && hbad) {
    cudaFree(staging);
    return s->fail(FWANT_ERR_INVALID_ARG, "rho must be > 0 everywhere (ghosts included)");
  }
  auto pad = [&](float* dst, const float* src) {
    return cudaMemcpy2D(dst + fw::PADL, size_t(g.px) * 4, src, size_t(g.nx) * 4, size_t(g.nx) * 4,
                        size_t(g.ny) * g.nz, cudaMemcpyDeviceToDevice);
  };
  if (on_device) {
    if (e == cudaSuccess) e = pad(s->rho, rho);
    if (e == cudaSuccess) e = pad(s->lam, lambda);
    if (e == cudaSuccess) e = pad(s->mu, mu);
  } else {
    if (e == cudaSuccess) e = pad(s->rho, staging);
    if (e == cudaSuccess) e = cudaMemcpy(staging, lambda, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = pad(s->lam, staging);
    if (e == cudaSuccess) e = cudaMemcpy(staging, mu, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = pad(s->mu, staging);
  }
  cudaFree(staging);
  if (e != cudaSuccess) return s->cuda_fail(e, "set_media");
  s->have_media = true;
  s->topo_sf_dirty = true;
  s->src_dirty = true;
  return FWANT_OK;
}

fwant_status fwant_set_media(fwant_solver* s, const float* lambda, const float* mu, const float* rho) {
  return load_media(s, lambda, mu, rho, false);
}

fwant_status fwant_set_media_device(fwant_solver* s, const float* d_lambda, const float* d_mu, const float* d_rho) {
  return load_media(s, d_lambda, d_mu, d_rho, true);
}

fwant_status fwant_set_pml(fwant_solver* s, const int number[6], const float velocity[6], const float bmax[6],
                           const float amax[6]) {
  if (!s || !number || !velocity || !bmax || !amax) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  return s->set_pml(number, velocity, bmax, amax);
}

static bool check_idx(const fwant_solver* s, const int* indx, int num) {
  for (int q = 0; q < num; ++q) {
    const int i = indx[3 * q], j = indx[3 * q + 1], k = indx[3 * q + 2];
    if (i < 1 || i > s->g.nx || j < 1 || j > s->g.ny || k < 1 || k > s->g.nz) return false;
  }
  return true;
}

fwant_status fwant_set_forces(fwant_solver* s, int num, int ntwin, const int* indx, const float* shift,
                              const float* start_time, const float* stf_time, const float* stf_freq,
                              const float* fx, const float* fy, const float* fz, int stf_id) {
  if (!s || num < 0 || (num > 0 && (ntwin <= 0 || !indx || !shift || !start_time || !stf_time || !stf_freq || !fx ||
                                    !fy || !fz)))
    return FWANT_ERR_INVALID_ARG;
  if (num > 0 && !check_idx(s, indx, num)) return s->fail(FWANT_ERR_INVALID_ARG, "force index outside the grid");
  auto& F = s->forces;
  F.num = num; F.ntwin = num > 0 ? ntwin : 0; F.stf_id = stf_id;
  F.indx.assign(indx, indx + 3 * num);
  F.shift.assign(shift, shift + 3 * num);
  F.t0.assign(start_time, start_time + num);
  F.stf_time.assign(stf_time, stf_time + F.ntwin);
  F.stf_freq.assign(stf_freq, stf_freq + F.ntwin);
  F.fx.assign(fx, fx + size_t(F.ntwin) * num);
  F.fy.assign(fy, fy + size_t(F.ntwin) * num);
  F.fz.assign(fz, fz + size_t(F.ntwin) * num);
  s->src_dirty = true;
  return FWANT_OK;
}

fwant_status fwant_set_moments(fwant_solver* s, int num, int ntwin, const int* indx, const float* shift,
                               const float* start_time, const float* stf_time, const float* stf_freq,
                               const float* mom, int stf_id) {
  if (!s || num < 0 || (num > 0 && (ntwin <= 0 || !indx || !shift || !start_time || !stf_time || !stf_freq || !mom)))
    return FWANT_ERR_INVALID_ARG;
  if (num > 0 && !check_idx(s, indx, num)) return s->fail(FWANT_ERR_INVALID_ARG, "moment index outside the grid");
  auto& M = s->moments;
  M.num = num; M.ntwin = num > 0 ? ntwin : 0; M.stf_id = stf_id;
  M.indx.assign(indx, indx + 3 * num);
  M.shift.assign(shift, shift + 3 * num);
  M.t0.assign(start_time, start_time + num);
  M.stf_time.assign(stf_time, stf_time + M.ntwin);
  M.stf_freq.assign(stf_freq, stf_freq + M.ntwin);
  M.mom.assign(mom, mom + 6 * size_t(M.ntwin) * num);
  s->src_dirty = true;
  return FWANT_OK;
}

fwant_status fwant_set_receivers(fwant_solver* s, int num, const int* indx, int tinv) {
  if (!s || num < 0 || (num > 0 && !indx)) return FWANT_ERR_INVALID_ARG;
  for (int q = 0; q < num; ++q) {
    const int i = indx[3 * q] - 1, j = indx[3 * q + 1] - 1, k = indx[3 * q + 2] - 1;
    if (i < s->g.i1 || i > s->g.i2 || j < s->g.j1 || j > s->g.j2 || k < s->g.k1 || k > s->g.k2)
      return s->fail(FWANT_ERR_INVALID_ARG, "receiver outside the interior");
  }
  cudaSetDevice(s->cfg.device);
  s->drop_graphs();
  s->npt = num;
  s->tinv = tinv > 0 ? tinv : 1;
  s->rec_idx.resize(3 * size_t(num));
  for (int q = 0; q < 3 * num; ++q) s->rec_idx[q] = indx[q] - 1;
  cudaFree(s->d_rec); s->d_rec = nullptr;
  cudaFree(s->d_seis); s->d_seis = nullptr;
  s->cap = 0; s->nsamp = 0;
  return FWANT_OK;
}

fwant_status fwant_run(fwant_solver* s, int nsteps) {
  if (!s) return FWANT_ERR_INVALID_ARG;
  return s->run(nsteps);
}

int fwant_reference_steps(int nt) { return nt < 0 ? 0 : 8 * (nt / 8 + 1); }

fwant_status fwant_get_ntime(fwant_solver* s, int* ntime) {
  if (!s || !ntime) return FWANT_ERR_INVALID_ARG;
  *ntime = s->ntime;
  return FWANT_OK;
}

fwant_status fwant_get_seismo(fwant_solver* s, float* out, int max_samples, int* nsamp) {
  if (!s || !nsamp || (max_samples > 0 && !out)) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  const int ns = std::min(s->nsamp, std::max(max_samples, 0));
  *nsamp = ns;
  if (ns == 0 || s->npt == 0) return FWANT_OK;
  for (int f = 0; f < fw::NF; ++f) {
    cudaError_t e = cudaMemcpy(out + size_t(f) * ns * s->npt, s->d_seis + size_t(f) * s->cap * s->npt,
                               size_t(ns) * s->npt * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return s->cuda_fail(e, "get_seismo");
  }
  return FWANT_OK;
}

// FP32 staging array for converting one component of 2-byte storage
static fwant_status conv_buffer(fwant_solver* s) {
  if (s->d_conv) return FWANT_OK;
  s->d_conv = dalloc<float>(s->g.fstride);
  if (!s->d_conv) return s->fail(FWANT_ERR_OOM, "conversion buffer");
  cudaMemset(s->d_conv, 0, s->g.fstride * sizeof(float));
  return FWANT_OK;
}

fwant_status fwant_get_field(fwant_solver* s, int component, float* out) {
  if (!s || !out || component < 0 || component >= fw::NF) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  const int f = fw::ABI2INT[component];
  const float* src = static_cast<const float*>(s->comp(s->rA, f));
  if (s->stor != fw::ST_F32) {
    fwant_status rc = conv_buffer(s);
    if (rc != FWANT_OK) return rc;
    fw::launch_convert_to_f32(s->g, s->comp(s->rA, f), s->stor, 1.0f / (f < 3 ? s->sv : s->sc_t), s->d_conv, s->st);
    cudaStreamSynchronize(s->st);
    src = s->d_conv;
  }
  cudaError_t e = s->get3(out, src);
  if (e != cudaSuccess) return s->cuda_fail(e, "get_field");
  return FWANT_OK;
}

fwant_status fwant_set_field(fwant_solver* s, int component, const float* in) {
  if (!s || !in || component < 0 || component >= fw::NF) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  const auto& g = s->g;
  std::vector<float> tmp(in, in + size_t(g.nx) * g.ny * g.nz);
  for (int k = 0; k < g.nz; ++k)
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nx; ++i)
        if (i < g.i1 || i > g.i2 || j < g.j1 || j > g.j2 || k < g.k1 || k > g.k2)
          tmp[size_t(i) + size_t(g.nx) * (size_t(j) + size_t(g.ny) * k)] = 0.0f;
  const int f = fw::ABI2INT[component];
  cudaError_t e;
  if (s->stor == fw::ST_F32) {
    e = s->put3(static_cast<float*>(s->comp(s->rA, f)), tmp.data());
  } else {
    fwant_status rc = conv_buffer(s);
    if (rc != FWANT_OK) return rc;
    e = s->put3(s->d_conv, tmp.data());
    fw::launch_convert_from_f32(s->g, s->d_conv, s->stor, f < 3 ? s->sv : s->sc_t, s->comp(s->rA, f), s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  }
  if (e != cudaSuccess) return s->cuda_fail(e, "set_field");
  return FWANT_OK;
}

fwant_status fwant_set_storage_scale(fwant_solver* s, float velocity_scale, float stress_scale) {
  if (!s || !(velocity_scale > 0.0f) || !(stress_scale > 0.0f) || !std::isfinite(velocity_scale) ||
      !std::isfinite(stress_scale))
    return FWANT_ERR_INVALID_ARG;
  int ev = 0, et = 0;
  if (std::frexp(velocity_scale, &ev) != 0.5f || std::frexp(stress_scale, &et) != 0.5f)
    return s->fail(FWANT_ERR_INVALID_ARG, "storage scales must be powers of two");
  if (s->ntime != 0) return s->fail(FWANT_ERR_STATE, "storage scales must be set before the first step");
  s->sv = velocity_scale;
  s->sc_t = stress_scale;
  s->drop_graphs();
  return FWANT_OK;
}

fwant_status fwant_max_abs(fwant_solver* s, float out[9]) {
  if (!s || !out) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  cudaMemsetAsync(s->d_maxbits, 0, fw::NF * sizeof(unsigned int), s->st);
  fw::launch_maxabs(s->g, s->set(s->rA), s->stor, 1.0f / s->sv, 1.0f / s->sc_t, s->d_maxbits, s->st);
  unsigned int bits[fw::NF];
  cudaMemcpyAsync(bits, s->d_maxbits, sizeof(bits), cudaMemcpyDeviceToHost, s->st);
  cudaError_t e = cudaStreamSynchronize(s->st);
  if (e != cudaSuccess) return s->cuda_fail(e, "max_abs");
  for (int c = 0; c < fw::NF; ++c) std::memcpy(&out[c], &bits[fw::ABI2INT[c]], sizeof(float));
  return FWANT_OK;
}

fwant_status fwant_get_snapshot(fwant_solver* s, const int subs[3], const int subc[3], const int subt[3], int ncomp,
                                const int* comps, float* out) {
  if (!s || !out) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  fw::SnapArgs a;
  size_t n = 0;
  fwant_status rc = s->snap_setup(subs, subc, subt, ncomp, comps, a, n);
  if (rc != FWANT_OK) return rc;
  if (n > s->snap_cap) {
    cudaFree(s->d_snap);
    s->d_snap = dalloc<float>(n);
    s->snap_cap = s->d_snap ? n : 0;
    if (!s->d_snap) return s->fail(FWANT_ERR_OOM, "snapshot staging buffer");
  }
  a.out = s->d_snap;
  fw::launch_pack_snapshot(a, s->st);
  cudaError_t e = cudaMemcpyAsync(out, s->d_snap, n * sizeof(float), cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return s->cuda_fail(e, "get_snapshot");
  return FWANT_OK;
}

fwant_status fwant_get_snapshot_noalloc(fwant_solver* s, const int subs[3], const int subc[3], const int subt[3],
                                        int ncomp, const int* comps, float* out) {
  if (!s || !out) return FWANT_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(s->cfg.device);
  if (e != cudaSuccess) return s->cuda_fail(e, "get_snapshot_noalloc");
  fw::SnapArgs a;
  size_t n = 0;
  fwant_status rc = s->snap_setup(subs, subc, subt, ncomp, comps, a, n);
  if (rc != FWANT_OK) return rc;
  if (n > size_t(fw::SNAPSHOT_NOALLOC_MAX)) {
    char b[160];
    std::snprintf(b, sizeof(b), "get_snapshot_noalloc: %zu values requested, the fixed staging buffer holds %lld",
                  n, fw::SNAPSHOT_NOALLOC_MAX);
    return s->fail(FWANT_ERR_INVALID_ARG, b);
  }
  float* staging = nullptr;
  if (int ge = fw::snapshot_noalloc_staging(s->cfg.device, &staging))
    return s->cuda_fail(cudaError_t(ge), "get_snapshot_noalloc: staging address");
  a.out = staging;
  fw::launch_pack_snapshot(a, s->st);
  e = cudaMemcpyAsync(out, staging, n * sizeof(float), cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return s->cuda_fail(e, "get_snapshot_noalloc");
  return FWANT_OK;
}

// ---- checkpoint / resume -----------------------------------------------------------------
// File: a fixed header (magic, version, the configuration the state belongs to, counters,
// section sizes, FNV-1a 64 checksum of the payload) followed by the payload: the
// wavefield register set holding W (padded layout, storage type), the PML memory variables
// of that set per active slab, the recorded seismogram samples and the recorded SGT frames.
namespace {
constexpr char CKPT_MAGIC[8] = {'F', 'W', 'A', 'N', 'T', 'C', 'K', '1'};
struct CkptHeader {
  char magic[8];
  uint32_t version;
  int32_t ni, nj, nk, px, storage, freesurf;
  int64_t fstride;
  int32_t ntime, cycle_pos;
  float sv, st;
  int32_t slab_on[6];
  int64_t aux_set[6];
  int32_t npt, tinv, nsamp;
  int32_t sgt_on, sgt_frames, sgt_max_frames;
  int64_t sgt_npts;
  uint64_t payload_bytes;
  uint64_t checksum;
};
uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h) {
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ULL;
  }
  return h;
}
}  // namespace

fwant_status fwant_save_checkpoint(fwant_solver* s, const char* path) {
  if (!s || !path) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, CKPT_MAGIC, 8);
  h.version = 1;
  h.ni = s->g.ni; h.nj = s->g.nj; h.nk = s->g.nk; h.px = s->g.px; h.storage = s->stor; h.freesurf = s->g.freesurf;
  h.fstride = s->g.fstride;
  h.ntime = s->ntime; h.cycle_pos = s->cycle_pos;
  h.sv = s->sv; h.st = s->sc_t;
  for (int f = 0; f < 6; ++f) { h.slab_on[f] = s->slab[f].on; h.aux_set[f] = s->slab[f].on ? s->aux_set[f] : 0; }
  h.npt = s->npt; h.tinv = s->tinv; h.nsamp = s->npt > 0 ? std::min(s->nsamp, s->cap) : 0;
  h.sgt_on = s->sgt_on;
  h.sgt_frames = s->sgt_on ? std::min(s->ntime / s->sgt.tinv, s->sgt.max_frames) : 0;
  h.sgt_max_frames = s->sgt_on ? s->sgt.max_frames : 0;
  h.sgt_npts = s->sgt_on ? s->sgt.npts : 0;
  // payload
  std::vector<unsigned char> pay;
  auto append_dev = [&](const void* d, size_t bytes) -> cudaError_t {
    const size_t o = pay.size();
    pay.resize(o + bytes);
    return bytes ? cudaMemcpy(pay.data() + o, d, bytes, cudaMemcpyDeviceToHost) : cudaSuccess;
  };
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = append_dev(s->set(s->rA), size_t(fw::NF) * s->g.fstride * s->esz);
  for (int f = 0; f < 6 && e == cudaSuccess; ++f)
    if (h.slab_on[f]) e = append_dev(s->aset(f, s->rA), size_t(h.aux_set[f]) * sizeof(float));
  for (int c = 0; c < fw::NF && e == cudaSuccess; ++c)
    e = append_dev(s->d_seis + size_t(c) * s->cap * s->npt, size_t(h.nsamp) * s->npt * sizeof(float));
  for (int c = 0; c < 6 && e == cudaSuccess && h.sgt_on; ++c)
    e = append_dev(s->d_sgt + size_t(c) * h.sgt_max_frames * h.sgt_npts, size_t(h.sgt_frames) * h.sgt_npts * 4);
  if (e != cudaSuccess) return s->cuda_fail(e, "save_checkpoint");
  h.payload_bytes = pay.size();
  h.checksum = fnv1a(pay.data(), pay.size(), 1469598103934665603ULL);
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return s->fail(FWANT_ERR_INVALID_ARG, std::string("save_checkpoint: cannot open ") + path);
  const bool ok = std::fwrite(&h, sizeof(h), 1, fp) == 1 && std::fwrite(pay.data(), 1, pay.size(), fp) == pay.size();
  if (std::fclose(fp) != 0 || !ok) return s->fail(FWANT_ERR_INVALID_ARG, "save_checkpoint: write failed");
  return FWANT_OK;
}

fwant_status fwant_load_checkpoint(fwant_solver* s, const char* path) {
  if (!s || !path) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return s->fail(FWANT_ERR_INVALID_ARG, std::string("load_checkpoint: cannot open ") + path);
  CkptHeader h;
  std::vector<unsigned char> pay;
  bool ok = std::fread(&h, sizeof(h), 1, fp) == 1 && std::memcmp(h.magic, CKPT_MAGIC, 8) == 0 && h.version == 1 &&
            h.payload_bytes < (uint64_t(1) << 44);
  if (ok) {
    pay.resize(size_t(h.payload_bytes));
    ok = std::fread(pay.data(), 1, pay.size(), fp) == pay.size();
  }
  std::fclose(fp);
  if (!ok) return s->fail(FWANT_ERR_INVALID_ARG, "load_checkpoint: not a checkpoint file or truncated");
  if (fnv1a(pay.data(), pay.size(), 1469598103934665603ULL) != h.checksum)
    return s->fail(FWANT_ERR_INVALID_ARG, "load_checkpoint: checksum mismatch (corrupt file)");
  // the state must belong to this solver's configuration
  bool same = h.ni == s->g.ni && h.nj == s->g.nj && h.nk == s->g.nk && h.px == s->g.px && h.storage == s->stor &&
              h.freesurf == s->g.freesurf && h.fstride == s->g.fstride && h.npt == s->npt && h.tinv == s->tinv &&
              h.sgt_on == int(s->sgt_on) && h.cycle_pos >= 0 && h.cycle_pos < 8 && h.ntime >= 0 &&
              h.cycle_pos == (h.ntime & 7);
  for (int f = 0; f < 6; ++f)
    same = same && h.slab_on[f] == s->slab[f].on && (!h.slab_on[f] || h.aux_set[f] == s->aux_set[f]);
  if (h.sgt_on) same = same && h.sgt_npts == s->sgt.npts && h.sgt_max_frames == s->sgt.max_frames;
  if (!same) return s->fail(FWANT_ERR_STATE, "load_checkpoint: the file belongs to another configuration");
  size_t need = size_t(fw::NF) * h.fstride * s->esz;
  for (int f = 0; f < 6; ++f) need += size_t(h.aux_set[f]) * sizeof(float);
  need += size_t(fw::NF) * h.nsamp * h.npt * sizeof(float) + size_t(6) * h.sgt_frames * h.sgt_npts * 4;
  if (need != pay.size()) return s->fail(FWANT_ERR_INVALID_ARG, "load_checkpoint: section sizes disagree");
  if (h.npt > 0) {
    fwant_status rc = s->prepare_receivers(h.nsamp * h.tinv);
    if (rc != FWANT_OK) return rc;
  }
  // W into set 0 (roles A = 0, T = 3), memory variables likewise
  size_t o = 0;
  auto put_dev = [&](void* d, size_t bytes) -> cudaError_t {
    const cudaError_t e = bytes ? cudaMemcpy(d, pay.data() + o, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    o += bytes;
    return e;
  };
  s->drop_graphs();
  s->rA = 0; s->rT = 3;
  cudaError_t e = put_dev(s->set(0), size_t(fw::NF) * h.fstride * s->esz);
  for (int f = 0; f < 6 && e == cudaSuccess; ++f)
    if (h.slab_on[f]) e = put_dev(s->aset(f, 0), size_t(h.aux_set[f]) * sizeof(float));
  if (e == cudaSuccess && s->d_seis)
    e = cudaMemset(s->d_seis, 0, size_t(fw::NF) * s->cap * s->npt * sizeof(float));
  for (int c = 0; c < fw::NF && e == cudaSuccess; ++c)
    e = put_dev(s->d_seis + size_t(c) * s->cap * s->npt, size_t(h.nsamp) * h.npt * sizeof(float));
  if (e == cudaSuccess && h.sgt_on) e = cudaMemset(s->d_sgt, 0, size_t(6) * h.sgt_max_frames * h.sgt_npts * 4);
  for (int c = 0; c < 6 && e == cudaSuccess && h.sgt_on; ++c)
    e = put_dev(s->d_sgt + size_t(c) * h.sgt_max_frames * h.sgt_npts, size_t(h.sgt_frames) * h.sgt_npts * 4);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_ntime, &h.ntime, sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return s->cuda_fail(e, "load_checkpoint");
  s->ntime = h.ntime;
  s->cycle_pos = h.cycle_pos;
  s->nsamp = h.nsamp;
  s->sv = h.sv;
  s->sc_t = h.st;
  return FWANT_OK;
}

fwant_status fwant_set_sgt_record(fwant_solver* s, const int subs[3], const int subc[3], const int subt[3], int tinv,
                                  int max_frames) {
  if (!s) return FWANT_ERR_INVALID_ARG;
  if (tinv < 1 || max_frames < 1) return s->fail(FWANT_ERR_INVALID_ARG, "sgt record: tinv and max_frames must be >= 1");
  if (s->ntime != 0) return s->fail(FWANT_ERR_STATE, "sgt record: set before the first time step");
  cudaSetDevice(s->cfg.device);
  static const int comps[1] = {3};
  fw::SnapArgs a;
  size_t n = 0;
  fwant_status rc = s->snap_setup(subs, subc, subt, 1, comps, a, n);
  if (rc != FWANT_OK) return rc;
  const size_t total = n * 6 * size_t(max_frames);
  cudaFree(s->d_sgt);
  s->d_sgt = dalloc<float>(total);
  s->sgt_on = false;
  if (!s->d_sgt) return s->fail(FWANT_ERR_OOM, "sgt record buffer");
  cudaMemset(s->d_sgt, 0, total * sizeof(float));
  fw::SgtRecArgs& r = s->sgt;
  r = fw::SgtRecArgs{};
  r.g = s->g;
  r.storage = s->stor;
  r.isv = 1.0f / s->sv; r.ist = 1.0f / s->sc_t;
  for (int d = 0; d < 3; ++d) { r.start[d] = a.start[d]; r.cnt[d] = a.cnt[d]; r.stride[d] = a.stride[d]; }
  r.tinv = tinv;
  r.max_frames = max_frames;
  r.npts = (long long)n;
  r.ntime = s->d_ntime;
  r.out = s->d_sgt;
  s->sgt_on = true;
  s->drop_graphs();
  return FWANT_OK;
}

fwant_status fwant_get_sgt(fwant_solver* s, float* out, int max_frames, int* nframes) {
  if (!s || !out || !nframes || max_frames < 0) return FWANT_ERR_INVALID_ARG;
  if (!s->sgt_on) return s->fail(FWANT_ERR_STATE, "get_sgt: no sgt record configured");
  cudaSetDevice(s->cfg.device);
  const int have = std::min(s->ntime / s->sgt.tinv, s->sgt.max_frames);
  const int nf = std::min(have, max_frames);
  const size_t npts = size_t(s->sgt.npts);
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < 6 && e == cudaSuccess && nf > 0; ++c)
    e = cudaMemcpy(out + size_t(c) * nf * npts, s->d_sgt + size_t(c) * s->sgt.max_frames * npts,
                   size_t(nf) * npts * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return s->cuda_fail(e, "get_sgt");
  *nframes = nf;
  return FWANT_OK;
}

extern "C++" {
namespace fw {
// Device view of a solver's SGT record for the sensitivity-kernel object.
int solver_sgt_view(fwant_solver* s, const float** data, long long* npts, int* max_frames, int* nframes,
                    int* device) {
  if (!s || !s->sgt_on) return 1;
  *data = s->d_sgt;
  *npts = s->sgt.npts;
  *max_frames = s->sgt.max_frames;
  *nframes = std::min(s->ntime / s->sgt.tinv, s->sgt.max_frames);
  *device = s->cfg.device;
  return 0;
}
}  // namespace fw
}  // extern "C++"

fwant_status fwant_check(fwant_solver* s) {
  if (!s) return FWANT_ERR_INVALID_ARG;
  float m[fw::NF];
  fwant_status rc = fwant_max_abs(s, m);
  if (rc != FWANT_OK) return rc;
  static const char* const names[fw::NF] = {"Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz"};
  for (int c = 0; c < fw::NF; ++c) {
    if (!(m[c] < 3.4028234663852886e38f)) {  // huge(1.0), NaN and Inf all fail this test
      char b[128];
      std::snprintf(b, sizeof(b), "overflow: max |%s| = %g at ntime %d", names[c], double(m[c]), s->ntime);
      return s->fail(FWANT_ERR_NUMERIC_OVERFLOW, b);
    }
  }
  return FWANT_OK;
}

fwant_status fwant_profile_stages(fwant_solver* s, int nsteps, double* stage_ms, double* other_ms) {
  if (!s || !stage_ms || !other_ms) return FWANT_ERR_INVALID_ARG;
  return s->profile(nsteps, stage_ms, other_ms);
}

fwant_status fwant_last_run_ms(fwant_solver* s, double* ms) {
  if (!s || !ms) return FWANT_ERR_INVALID_ARG;
  *ms = s->last_ms;
  return FWANT_OK;
}

// ---- autotuning -------------------------------------------------------------------------
// Candidates are timed with CUDA events on eager steps (fwant_profile_stages) from the
// initial state, which is restored afterwards; results are cached per process by the
// shape of the problem.
namespace {
struct TuneKey {
  int ni, nj, nk, storage, exact, device;
  int pml[6];
  bool operator<(const TuneKey& o) const { return std::memcmp(this, &o, sizeof(TuneKey)) < 0; }
};
std::mutex g_tune_mutex;
std::map<TuneKey, std::pair<int, int>> g_tune_cache;  // planes per CTA, tile rows

TuneKey tune_key(const fwant_solver* s) {
  TuneKey k;
  std::memset(&k, 0, sizeof(k));
  k.ni = s->cfg.ni; k.nj = s->cfg.nj; k.nk = s->cfg.nk; k.storage = s->stor; k.exact = s->cfg.exact_arith;
  k.device = s->cfg.device;
  for (int f = 0; f < 6; ++f) k.pml[f] = s->slab[f].on ? (s->slab[f].i2 - s->slab[f].i1 + 1) * 1000000 +
                                                          (s->slab[f].j2 - s->slab[f].j1 + 1) * 1000 +
                                                          (s->slab[f].k2 - s->slab[f].k1 + 1) : 0;
  return k;
}
}  // namespace

fwant_status fwant_autotune(fwant_solver* s, int trial_steps, int* planes_out) {
  if (!s || trial_steps < 1) return FWANT_ERR_INVALID_ARG;
  if (s->ntime != 0) return s->fail(FWANT_ERR_STATE, "autotune: call before the first time step");
  const TuneKey key = tune_key(s);
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      s->kc = it->second.first;
      if (fwant_status rc = s->set_tile_rows(it->second.second); rc != FWANT_OK) return rc;
      s->drop_graphs();
      if (planes_out) *planes_out = s->kc;
      return FWANT_OK;
    }
  }
  // tile shape (32 x 8, and 32 x 16 where the storage and grid allow it) x planes per CTA
  std::vector<int> shapes = {fw::STAGE_TY};
  if (s->tile_rows_allowed(fw::STAGE_TY_TALL)) shapes.push_back(fw::STAGE_TY_TALL);
  const int cand[] = {3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128};
  double best = 1e30;
  int best_kc = s->kc, best_ty = s->tile_ty;
  for (int ty : shapes) {
    if (fwant_status rc = s->set_tile_rows(ty); rc != FWANT_OK) return rc;
    for (int kc : cand) {
      if (kc > s->cfg.nk && kc != cand[0]) break;
      s->kc = kc;
      s->drop_graphs();
      double st[4], other;
      fwant_status rc = s->profile(1, st, &other);  // first touch of this configuration
      if (rc == FWANT_OK) rc = s->profile(trial_steps, st, &other);
      cudaError_t e = s->reset_state();
      if (rc != FWANT_OK) return rc;
      if (e != cudaSuccess) return s->cuda_fail(e, "autotune reset");
      const double t = st[0] + st[1] + st[2] + st[3];
      if (t < best) { best = t; best_kc = kc; best_ty = ty; }
    }
  }
  s->kc = best_kc;
  if (fwant_status rc = s->set_tile_rows(best_ty); rc != FWANT_OK) return rc;
  s->drop_graphs();
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = {best_kc, best_ty};
  }
  if (planes_out) *planes_out = best_kc;
  return FWANT_OK;
}

fwant_status fwant_set_tile_rows(fwant_solver* s, int rows) {
  if (!s) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  return s->set_tile_rows(rows);
}

fwant_status fwant_get_tile_rows(fwant_solver* s, int* rows) {
  if (!s || !rows) return FWANT_ERR_INVALID_ARG;
  *rows = s->tile_ty;
  return FWANT_OK;
}

fwant_status fwant_set_planes_per_cta(fwant_solver* s, int planes) {
  if (!s || planes < 1 || planes > 4096) return FWANT_ERR_INVALID_ARG;
  if ((s->cfg.nk + planes - 1) / planes > 2047)
    return s->fail(FWANT_ERR_INVALID_ARG, "planes per CTA: at most 2047 k-chunks");
  s->kc = planes;
  s->drop_graphs();
  return FWANT_OK;
}

fwant_status fwant_get_planes_per_cta(fwant_solver* s, int* planes) {
  if (!s || !planes) return FWANT_ERR_INVALID_ARG;
  *planes = s->kc;
  return FWANT_OK;
}

fwant_status fwant_check_wait_timeout(fwant_solver* s, int spins) {
  if (!s || spins < 1 || spins > (1 << 20)) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(s->cfg.device);
  fw::launch_wait_timeout_probe(spins, s->d_err, s->st);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  if (e != cudaSuccess) return s->cuda_fail(e, "wait timeout check");
  return s->check_device_error();
}

fwant_status fwant_set_lean_stages(fwant_solver* s, int mask) {
  if (!s || (mask & ~7) != 0) return FWANT_ERR_INVALID_ARG;
  s->lean_mask = mask;
  s->drop_graphs();
  return FWANT_OK;
}

fwant_status fwant_get_lean_stages(fwant_solver* s, int* mask) {
  if (!s || !mask) return FWANT_ERR_INVALID_ARG;
  *mask = s->lean_stages();
  return FWANT_OK;
}

fwant_status fwant_set_rk_scheme(fwant_solver* s, int scheme) {
  if (!s || (scheme != 0 && scheme != 1)) return FWANT_ERR_INVALID_ARG;
  s->rk_scheme = scheme;  // t lives within a step only: switching between steps is safe
  s->drop_graphs();
  return FWANT_OK;
}

fwant_status fwant_get_rk_scheme(fwant_solver* s, int* scheme) {
  if (!s || !scheme) return FWANT_ERR_INVALID_ARG;
  *scheme = s->recon_on() ? 1 : 0;
  return FWANT_OK;
}

}  // extern "C"

// ---- batches of simulations stepped together -------------------------------------------
// Each stage of up to BATCH_PER_LAUNCH members runs in one launch (stage_batch_kernel);
// the members' step-end kernels follow.  Members advance in lockstep, so they share the
// F/B variant of every stage and the register-role assignment.
struct fwant_batch {
  std::vector<fwant_solver*> sims;
  int device = 0;
  int ctas = 0;                              // persistent CTAs per launch (0: 2 per SM)
  int sm_count = 152;
  cudaStream_t st = nullptr;
  FormFork fork;  // side stream of the full-form launches
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  std::vector<unsigned char> graph_sig;      // launch arguments the graphs were captured with
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  int launches_per_step = 0;                 // kernels of the last enqueued step
  std::string err;

  ~fwant_batch() {
    cudaSetDevice(device);
    drop_graphs();
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    fork.destroy();
    if (st) cudaStreamDestroy(st);
  }
  fwant_status fail(fwant_status c, const std::string& m) {
    err = m;
    return c;
  }
  fwant_status cuda_fail(cudaError_t e, const char* where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return FWANT_ERR_CUDA;
  }
  void drop_graphs() {
    for (auto& ge : graph)
      if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
  }
  int n() const { return int(sims.size()); }

  // Arguments of stage s for members [first, first+count) (count <= BATCH_PER_LAUNCH),
  // lean or full items.
  void batch_args(fw::BatchArgs& b, int first, int count, int ra, int s, bool lean) const {
    b.nsims = count;
    int off = 0;
    const int rk = sims[0]->stage_rk(s);
    for (int q = 0; q < count; ++q) {
      const fwant_solver* m = sims[first + q];
      b.sims[q] = m->stage_args(s, ra);
      b.items[q] = m->items(lean, rk);
      b.off[q] = off;
      off += m->item_count(lean, rk);
    }
    b.off[count] = off;
    b.total = off;
  }

  // ev (optional, 6 events): recorded before each stage, after the stages and after the
  // step-end kernels.
  int enqueue_step(cudaEvent_t* ev = nullptr) {
    fwant_solver* s0 = sims[0];
    int lerr = 0, nlaunch = 0;
    static thread_local fw::BatchArgs b;  // 30 KB: kept off the stack
    for (int s = 0; s < 4; ++s) {
      if (ev) cudaEventRecord(ev[s], st);
      for (int first = 0; first < n(); first += fw::BATCH_PER_LAUNCH) {
        const int count = std::min(fw::BATCH_PER_LAUNCH, n() - first);
        int cnt[2] = {0, 0};  // full, interior-only items of the group
        for (int q = 0; q < count; ++q)
          for (int lean = 0; lean <= 1; ++lean) cnt[lean] += sims[first + q]->item_count(lean != 0, s0->stage_rk(s));
        const bool both = fork.on && cnt[0] > 0 && cnt[1] > 0;
        if (both) fork.begin(st);
        for (int lean = 0; lean <= 1; ++lean) {  // the full form first, on the side stream
          batch_args(b, first, count, s0->rA, s, lean != 0);
          if (b.total == 0) continue;
          const int nct = ctas > 0 ? std::min(b.total, ctas) : b.total;
          const int le = fw::launch_stage_batch(b, fwant_solver::stage_variant(s0->cycle_pos, s),
                                                s0->stage_rk(s), s0->cfg.exact_arith, s0->stor, lean,
                                                std::max(1, nct), (both && !lean) ? fork.side : st, s0->tile_ty);
          if (le && !lerr) lerr = le;
          ++nlaunch;
        }
        if (both) fork.end(st);
      }
    }
    if (ev) cudaEventRecord(ev[4], st);
    for (fwant_solver* m : sims) nlaunch += m->enqueue_step_end(st);
    launches_per_step = nlaunch;
    if (ev) cudaEventRecord(ev[5], st);
    for (fwant_solver* m : sims) m->finish_step_host();
    return lerr;
  }

  fwant_status prepare(int nsteps) {
    fwant_solver* s0 = sims[0];
    for (fwant_solver* m : sims) {
      if (m->ntime != s0->ntime || m->cycle_pos != s0->cycle_pos || m->rA != s0->rA)
        return fail(FWANT_ERR_STATE, "batch members must be at the same time step");
      if (m->rk_scheme != s0->rk_scheme) return fail(FWANT_ERR_STATE, "batch members must share the RK scheme");
      if (!m->have_coord || !m->have_metric || !m->have_media)
        return fail(FWANT_ERR_STATE, "coordinates, metric and media must be set for every member");
      fwant_status rc = m->prepare_sources(m->ntime + nsteps);
      if (rc == FWANT_OK) rc = m->prepare_receivers(m->ntime + nsteps);
      if (rc == FWANT_OK) rc = m->ensure_items();
      if (rc != FWANT_OK) return fail(rc, "member: " + m->err);
    }
    return FWANT_OK;
  }
  fwant_status finish() {
    for (fwant_solver* m : sims) {
      fwant_status rc = m->check_device_error();
      if (rc != FWANT_OK) return fail(rc, "member: " + m->err);
      if (m->npt > 0) m->nsamp = std::max(m->nsamp, std::min(m->ntime / m->tinv, m->cap));
    }
    return FWANT_OK;
  }

  // Eager steps with events around every stage: average device time per stage launch
  // group and of the step-end kernels.
  fwant_status profile(int nsteps, double* stage_ms, double* other_ms) {
    if (nsteps <= 0) return fail(FWANT_ERR_INVALID_ARG, "nsteps <= 0");
    cudaSetDevice(device);
    fwant_status rc = prepare(nsteps);
    if (rc != FWANT_OK) return rc;
    std::vector<cudaEvent_t> ev(size_t(6) * nsteps);
    for (auto& x : ev) cudaEventCreate(&x);
    int lerr = 0;
    for (int q = 0; q < nsteps; ++q) lerr |= enqueue_step(&ev[size_t(6) * q]);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    double acc[5] = {0, 0, 0, 0, 0};
    if (e == cudaSuccess)
      for (int q = 0; q < nsteps; ++q)
        for (int k = 0; k < 5; ++k) {
          float ms = 0.0f;
          cudaEventElapsedTime(&ms, ev[size_t(6) * q + k], ev[size_t(6) * q + k + 1]);
          acc[k] += ms;
        }
    for (auto& x : ev) cudaEventDestroy(x);
    if (e == cudaSuccess && lerr) e = cudaError_t(lerr);
    if (e != cudaSuccess) return cuda_fail(e, "batch profile");
    if ((rc = finish()) != FWANT_OK) return rc;
    for (int k = 0; k < 4; ++k) stage_ms[k] = acc[k] / nsteps;
    *other_ms = acc[4] / nsteps;
    return FWANT_OK;
  }

  // Capture the graph of an 8-step block that starts with W in register set ra.
  fwant_status capture(int gi) {
    std::vector<int> save_nt, save_ra, save_cp;
    for (fwant_solver* m : sims) {
      save_nt.push_back(m->ntime); save_ra.push_back(m->rA); save_cp.push_back(m->cycle_pos);
      m->rA = gi == 0 ? 0 : 3; m->rT = 3 - m->rA; m->cycle_pos = 0;
    }
    cudaGraph_t gr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    int lerr = 0;
    if (e == cudaSuccess) {
      for (int q = 0; q < 8; ++q) lerr |= enqueue_step();
      e = cudaStreamEndCapture(st, &gr);
    }
    if (e == cudaSuccess && lerr) e = cudaError_t(lerr);
    for (int q = 0; q < n(); ++q) {
      sims[q]->ntime = save_nt[q]; sims[q]->rA = save_ra[q]; sims[q]->rT = 3 - save_ra[q];
      sims[q]->cycle_pos = save_cp[q];
    }
    if (e != cudaSuccess) return cuda_fail(e, "graph capture");
    e = cudaGraphInstantiate(&graph[gi], gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
    return FWANT_OK;
  }

  fwant_status run(int nsteps) {
    if (nsteps < 0) return fail(FWANT_ERR_INVALID_ARG, "nsteps < 0");
    cudaSetDevice(device);
    fwant_solver* s0 = sims[0];
    fwant_status rc = prepare(nsteps);
    if (rc != FWANT_OK) return rc;
    // graphs hold the launch arguments: keep them only while those are unchanged (source
    // tables and receiver buffers may have been reallocated above)
    std::vector<unsigned char> sig;
    for (const fwant_solver* m : sims) m->append_signature(sig);
    sig.insert(sig.end(), reinterpret_cast<const unsigned char*>(&ctas),
               reinterpret_cast<const unsigned char*>(&ctas) + sizeof(ctas));
    if (sig != graph_sig) {
      drop_graphs();
      graph_sig = sig;
    }
    // the graph that the 8-step blocks of this call will use, built before timing starts
    const int pre = (8 - s0->cycle_pos) & 7;
    if (nsteps - pre >= 8) {
      const int gi = ((s0->rA == 0 ? 0 : 1) ^ (pre & 1));
      if (!graph[gi] && (rc = capture(gi)) != FWANT_OK) return rc;
    }
    cudaError_t e = cudaSuccess;
    cudaEventRecord(ev0, st);
    int left = nsteps;
    while (left > 0) {
      if (s0->cycle_pos == 0 && left >= 8) {
        const int gi = s0->rA == 0 ? 0 : 1;
        if (!graph[gi] && (rc = capture(gi)) != FWANT_OK) return rc;
        e = cudaGraphLaunch(graph[gi], st);
        if (e != cudaSuccess) return cuda_fail(e, "graph launch");
        for (int q = 0; q < 8; ++q)
          for (fwant_solver* m : sims) m->finish_step_host();
        left -= 8;
      } else {
        const int le = enqueue_step();
        if (le) return cuda_fail(cudaError_t(le), "batch stage launch");
        left -= 1;
      }
    }
    cudaEventRecord(ev1, st);
    e = cudaEventSynchronize(ev1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "batch run");
    if ((rc = finish()) != FWANT_OK) return rc;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    last_ms = ms;
    return FWANT_OK;
  }
};

extern "C" {

fwant_status fwant_batch_create(fwant_solver* const* sims, int n, fwant_batch** out) {
  if (!out) return FWANT_ERR_INVALID_ARG;
  *out = nullptr;
  if (!sims || n < 1 || n > fw::MAX_BATCH) return FWANT_ERR_INVALID_ARG;
  for (int q = 0; q < n; ++q) {
    if (!sims[q]) return FWANT_ERR_INVALID_ARG;
    for (int r = 0; r < q; ++r)
      if (sims[r] == sims[q]) return FWANT_ERR_INVALID_ARG;
    if (sims[q]->cfg.device != sims[0]->cfg.device || sims[q]->stor != sims[0]->stor ||
        sims[q]->cfg.exact_arith != sims[0]->cfg.exact_arith)
      return FWANT_ERR_INVALID_ARG;
    if (sims[q]->topo_on) return FWANT_ERR_INVALID_ARG;  // terrain-following grids step alone
    if (sims[q]->tile_ty != sims[0]->tile_ty) return FWANT_ERR_INVALID_ARG;  // one tile shape per launch
  }
  auto* b = new fwant_batch();
  b->sims.assign(sims, sims + n);
  b->device = sims[0]->cfg.device;
  cudaError_t e = cudaSetDevice(b->device);
  int nsm = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device);
  if (nsm > 0) b->sm_count = nsm;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = b->fork.init();
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return FWANT_ERR_CUDA;
  }
  *out = b;
  return FWANT_OK;
}

void fwant_batch_destroy(fwant_batch* b) { delete b; }

const char* fwant_batch_last_error(fwant_batch* b) { return b ? b->err.c_str() : "null handle"; }

fwant_status fwant_batch_set_ctas(fwant_batch* b, int ctas) {
  if (!b || ctas < 0) return FWANT_ERR_INVALID_ARG;
  b->ctas = ctas;
  b->drop_graphs();
  return FWANT_OK;
}

fwant_status fwant_batch_run(fwant_batch* b, int nsteps) {
  if (!b) return FWANT_ERR_INVALID_ARG;
  return b->run(nsteps);
}

fwant_status fwant_batch_autotune(fwant_batch* b, int trial_steps, int* ctas_out) {
  if (!b || trial_steps < 1) return FWANT_ERR_INVALID_ARG;
  for (fwant_solver* m : b->sims)
    if (m->ntime != 0) return b->fail(FWANT_ERR_STATE, "batch autotune: call before the first time step");
  // one timed trial of the batch as configured: the four stage times of trial_steps steps
  // after one step of first touch, then every member back to its initial state
  auto trial = [&](double* t) -> fwant_status {
    b->drop_graphs();
    double st[4], other;
    fwant_status rc = b->profile(1, st, &other);
    if (rc == FWANT_OK) rc = b->profile(trial_steps, st, &other);
    cudaError_t e = cudaSuccess;
    for (fwant_solver* m : b->sims)
      if (e == cudaSuccess) e = m->reset_state();
    if (rc != FWANT_OK) return rc;
    if (e != cudaSuccess) return b->cuda_fail(e, "batch autotune reset");
    *t = st[0] + st[1] + st[2] + st[3];
    return FWANT_OK;
  };
  // planes per CTA: one value for every member, timed on the batch itself (the members'
  // items share each launch, so a member's fastest value alone is not the batch's)
  int min_nk = b->sims[0]->cfg.nk;
  for (fwant_solver* m : b->sims) min_nk = std::min(min_nk, m->cfg.nk);
  // tile shape (32 x 8, and 32 x 16 where every member allows it) x planes per CTA
  std::vector<int> shapes = {fw::STAGE_TY};
  bool tall = true;
  for (fwant_solver* m : b->sims) tall = tall && m->tile_rows_allowed(fw::STAGE_TY_TALL);
  if (tall) shapes.push_back(fw::STAGE_TY_TALL);
  const int kcand[] = {3, 4, 6, 8, 12, 16, 24, 32};
  double best_t = 1e30;
  int best_kc = b->sims[0]->kc, best_ty = b->sims[0]->tile_ty;
  b->ctas = 0;
  for (int ty : shapes) {
    for (fwant_solver* m : b->sims)
      if (fwant_status rc = m->set_tile_rows(ty); rc != FWANT_OK) return b->fail(rc, "member: " + m->err);
    for (int kc : kcand) {
      if (kc > min_nk && kc != kcand[0]) break;
      for (fwant_solver* m : b->sims) {
        m->kc = kc;
        m->drop_graphs();
      }
      double t = 0.0;
      fwant_status rc = trial(&t);
      if (rc != FWANT_OK) return rc;
      if (t < best_t) { best_t = t; best_kc = kc; best_ty = ty; }
    }
  }
  for (fwant_solver* m : b->sims) {
    if (fwant_status rc = m->set_tile_rows(best_ty); rc != FWANT_OK) return b->fail(rc, "member: " + m->err);
    m->kc = best_kc;
    m->drop_graphs();
  }
  // CTA schedule: one CTA per work item, or persistent grids of 1, 2 and 4 CTAs per SM
  const int cand[] = {0, b->sm_count, 2 * b->sm_count, 4 * b->sm_count};
  double best = 1e30;
  int best_ctas = 0;
  for (int c : cand) {
    b->ctas = c;
    double t = 0.0;
    fwant_status rc = trial(&t);
    if (rc != FWANT_OK) return rc;
    if (t < best) { best = t; best_ctas = c; }
  }
  b->ctas = best_ctas;
  // interior-only launches for every stage (7), for stages 1 and 4 (5), for one of them, or
  // none: on small grids most items touch a boundary and the extra launches can cost more
  // than they save
  const int masks[] = {7, 5, 1, 4, 0};
  int best_mask = b->sims[0]->lean_stages();
  double best_m = 1e30;
  for (int mk : masks) {
    for (fwant_solver* m : b->sims) {
      m->lean_mask = mk;
      m->drop_graphs();
    }
    double t = 0.0;
    fwant_status rc = trial(&t);
    if (rc != FWANT_OK) return rc;
    if (t < best_m) { best_m = t; best_mask = mk; }
  }
  for (fwant_solver* m : b->sims) {
    m->lean_mask = best_mask;
    m->drop_graphs();
  }
  b->drop_graphs();
  if (ctas_out) *ctas_out = best_ctas;
  return FWANT_OK;
}

fwant_status fwant_batch_profile_stages(fwant_batch* b, int nsteps, double* stage_ms, double* other_ms) {
  if (!b || !stage_ms || !other_ms) return FWANT_ERR_INVALID_ARG;
  return b->profile(nsteps, stage_ms, other_ms);
}

fwant_status fwant_batch_last_run_ms(fwant_batch* b, double* ms) {
  if (!b || !ms) return FWANT_ERR_INVALID_ARG;
  *ms = b->last_ms;
  return FWANT_OK;
}

fwant_status fwant_batch_launches_per_step(fwant_batch* b, int* n) {
  if (!b || !n) return FWANT_ERR_INVALID_ARG;
  *n = b->launches_per_step;
  return FWANT_OK;
}

}  // extern "C"
