// Sensitivity-kernel statistics (SI_ker2info, code/srcF.kernel/SI_ker2info.F90:268-353):
// per-point sums of |K|, per-event counts of |K| above a threshold, the number of events
// that reached each point and the per-record (station, event, count) entries.  C ABI in
// include/fwant_kerinfo.h.
//
// Layout: every per-slot quantity is (4, npts), slot slowest, so that a warp's loads of one
// slot are consecutive points.  The records are one device buffer each, (3, 4, npts) ints:
// M, station tag, event tag; record r exists once some point's N_ap reaches r + 1, and one
// spare record is kept allocated so that an event never writes past the allocated ones (an
// event raises the largest N_ap by at most one).
//
// Both passes are element-wise and bound by HBM traffic: a pick moves 16 B of kernel values
// in and 32 B of S and M in and out per point (plus its host-to-device copy, which is the
// larger cost), an event end reads M and N and writes N, M and the sparse record entries.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fwant_kerinfo.h"

namespace {

constexpr int KI_THREADS = 256;

struct Thresholds {
  float k0[4];
};

// S_q += |K_q| (each add rounded to single precision, as the reference's REAL arrays), and
// M_q += 1 where |K_q| > K0_q (SI_ker2info.F90:276-289).
__global__ void __launch_bounds__(KI_THREADS) pick_kernel(long long npts, const float* __restrict__ K,
                                                          float* __restrict__ S, int* __restrict__ M,
                                                          Thresholds th) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npts; p += stride) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long o = q * npts + p;
      const float a = fabsf(__ldg(K + o));
      S[o] = __fadd_rn(S[o], a);
      if (a > th.k0[q]) M[o] += 1;
    }
  }
}

// The event end (SI_ker2info.F90:294-334): N_q += 1 where M_q >= 1; the record of index
// N_ap (after its increment) takes M_q and the tags for every slot with M_q >= 1, provided
// N_ap >= 1; then M is reset.  The largest N_ap goes to *maxrec.
__global__ void __launch_bounds__(KI_THREADS) event_kernel(long long npts, int* __restrict__ M,
                                                           int* __restrict__ N, int* const* __restrict__ rec,
                                                           int sta, int evt, int* __restrict__ maxrec) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  int top = 0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npts; p += stride) {
    int m[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) m[q] = M[q * npts + p];
    int nap = N[p];
    if (m[0] >= 1) N[p] = ++nap;
    int* r = nap >= 1 ? rec[nap - 1] : nullptr;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (m[q] < 1) continue;
      if (q > 0) N[q * npts + p] += 1;
      if (r) {
        r[q * npts + p] = m[q];
        if (sta > 0) r[(4 + q) * npts + p] = sta;
        if (evt > 0) r[(8 + q) * npts + p] = evt;
      }
      M[q * npts + p] = 0;
    }
    top = max(top, nap);
  }
  for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(0xffffffffu, top, o));
  if ((threadIdx.x & 31) == 0 && top > 0) atomicMax(maxrec, top);
}

int grid_for(long long npts, int device) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1) sms = 1;
  const long long need = (npts + KI_THREADS - 1) / KI_THREADS;
  return int(std::max(1LL, std::min(need, (long long)sms * 8)));
}

}  // namespace

struct fwant_kerinfo {
  long long npts = 0;
  int device = 0, grid = 1, nrec = 0;
  Thresholds th{};
  float* d_K = nullptr;   // (4, npts) staging of the pick's volumes
  float* d_S = nullptr;   // (4, npts)
  int* d_M = nullptr;     // (4, npts)
  int* d_N = nullptr;     // (4, npts)
  int* d_max = nullptr;   // largest N_ap
  std::vector<int*> recs; // record buffers, (3, 4, npts) ints each
  int** d_recs = nullptr; // device copy of recs
  size_t recs_cap = 0, recs_synced = 0;  // capacity of d_recs, entries copied to it
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float last_ms = 0.0f;
  std::string err;

  fwant_status fail(fwant_status rc, const std::string& m) {
    err = m;
    return rc;
  }
  fwant_status cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return FWANT_ERR_CUDA;
  }
  size_t vol_bytes(size_t elem) const { return size_t(4) * size_t(npts) * elem; }
  ~fwant_kerinfo() {
    cudaSetDevice(device);
    if (st) cudaStreamSynchronize(st);
    for (void* p : {static_cast<void*>(d_K), static_cast<void*>(d_S), static_cast<void*>(d_M),
                    static_cast<void*>(d_N), static_cast<void*>(d_max), static_cast<void*>(d_recs)})
      if (p) cudaFree(p);
    for (int* r : recs) cudaFree(r);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
  }

  // records 0 .. n-1 allocated (zeroed) and listed in d_recs
  cudaError_t ensure_records(size_t n) {
    cudaError_t e = cudaSuccess;
    while (recs.size() < n && e == cudaSuccess) {
      int* r = nullptr;
      e = cudaMalloc(&r, size_t(3) * vol_bytes(sizeof(int)));
      if (e != cudaSuccess) break;
      recs.push_back(r);
      e = cudaMemsetAsync(r, 0, size_t(3) * vol_bytes(sizeof(int)), st);
    }
    if (e != cudaSuccess) return e;
    if (recs_cap < recs.size()) {
      size_t cap = std::max<size_t>(16, recs_cap * 2);
      while (cap < recs.size()) cap *= 2;
      int** d = nullptr;
      e = cudaMalloc(&d, cap * sizeof(int*));
      if (e != cudaSuccess) return e;
      if (d_recs) {
        e = cudaStreamSynchronize(st);
        cudaFree(d_recs);
      }
      d_recs = d;
      recs_cap = cap;
      recs_synced = 0;
    }
    if (e == cudaSuccess && recs_synced < recs.size()) {
      e = cudaMemcpyAsync(d_recs, recs.data(), recs.size() * sizeof(int*), cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // recs.data() is pageable host memory
      if (e == cudaSuccess) recs_synced = recs.size();
    }
    return e;
  }
};

extern "C" {

fwant_status fwant_kerinfo_create(long long npts, const float thresholds[4], int device, fwant_kerinfo** out) {
  if (!out) return FWANT_ERR_INVALID_ARG;
  *out = nullptr;
  if (npts < 1 || !thresholds) return FWANT_ERR_INVALID_ARG;
  auto* k = new fwant_kerinfo();
  *out = k;
  k->npts = npts;
  k->device = device;
  for (int q = 0; q < 4; ++q) k->th.k0[q] = thresholds[q];
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&k->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&k->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&k->e1);
  if (e == cudaSuccess) e = cudaMalloc(&k->d_K, k->vol_bytes(sizeof(float)));
  if (e == cudaSuccess) e = cudaMalloc(&k->d_S, k->vol_bytes(sizeof(float)));
  if (e == cudaSuccess) e = cudaMalloc(&k->d_M, k->vol_bytes(sizeof(int)));
  if (e == cudaSuccess) e = cudaMalloc(&k->d_N, k->vol_bytes(sizeof(int)));
  if (e == cudaSuccess) e = cudaMalloc(&k->d_max, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(k->d_S, 0, k->vol_bytes(sizeof(float)), k->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(k->d_M, 0, k->vol_bytes(sizeof(int)), k->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(k->d_N, 0, k->vol_bytes(sizeof(int)), k->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(k->d_max, 0, sizeof(int), k->st);
  if (e == cudaSuccess) e = k->ensure_records(1);
  if (e != cudaSuccess) return k->cuda_fail(e, "create");
  k->grid = grid_for(npts, device);
  return FWANT_OK;
}

void fwant_kerinfo_destroy(fwant_kerinfo* k) { delete k; }

const char* fwant_kerinfo_last_error(fwant_kerinfo* k) { return k ? k->err.c_str() : "null handle"; }

fwant_status fwant_kerinfo_add_pick(fwant_kerinfo* k, const float* const kernels[4]) {
  if (!k || !kernels) return FWANT_ERR_INVALID_ARG;
  for (int q = 0; q < 4; ++q)
    if (!kernels[q]) return k->fail(FWANT_ERR_INVALID_ARG, "null kernel volume");
  cudaError_t e = cudaSetDevice(k->device);
  for (int q = 0; q < 4 && e == cudaSuccess; ++q)
    e = cudaMemcpyAsync(k->d_K + size_t(q) * k->npts, kernels[q], size_t(k->npts) * sizeof(float),
                        cudaMemcpyHostToDevice, k->st);
  if (e == cudaSuccess) e = cudaEventRecord(k->e0, k->st);
  if (e == cudaSuccess) {
    pick_kernel<<<k->grid, KI_THREADS, 0, k->st>>>(k->npts, k->d_K, k->d_S, k->d_M, k->th);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(k->e1, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);  // the caller may reuse its buffers
  if (e == cudaSuccess) e = cudaEventElapsedTime(&k->last_ms, k->e0, k->e1);
  return e == cudaSuccess ? FWANT_OK : k->cuda_fail(e, "add_pick");
}

fwant_status fwant_kerinfo_end_event(fwant_kerinfo* k, int station_tag, int event_tag) {
  if (!k || station_tag < 0 || event_tag < 0) return FWANT_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(k->device);
  if (e == cudaSuccess) e = k->ensure_records(size_t(k->nrec) + 1);
  if (e == cudaSuccess) {
    event_kernel<<<k->grid, KI_THREADS, 0, k->st>>>(k->npts, k->d_M, k->d_N, k->d_recs, station_tag, event_tag,
                                                     k->d_max);
    e = cudaGetLastError();
  }
  int top = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&top, k->d_max, sizeof(int), cudaMemcpyDeviceToHost, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  if (e != cudaSuccess) return k->cuda_fail(e, "end_event");
  if (top < k->nrec || top > k->nrec + 1) return k->fail(FWANT_ERR_CUDA, "end_event: record count out of step");
  k->nrec = top;
  return FWANT_OK;
}

fwant_status fwant_kerinfo_records(fwant_kerinfo* k, int* nrec) {
  if (!k || !nrec) return FWANT_ERR_INVALID_ARG;
  *nrec = k->nrec;
  return FWANT_OK;
}

fwant_status fwant_kerinfo_totals(fwant_kerinfo* k, float* sums, int* counts) {
  if (!k || (!sums && !counts)) return FWANT_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(k->device);
  if (e == cudaSuccess && sums)
    e = cudaMemcpyAsync(sums, k->d_S, k->vol_bytes(sizeof(float)), cudaMemcpyDeviceToHost, k->st);
  if (e == cudaSuccess && counts)
    e = cudaMemcpyAsync(counts, k->d_N, k->vol_bytes(sizeof(int)), cudaMemcpyDeviceToHost, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  return e == cudaSuccess ? FWANT_OK : k->cuda_fail(e, "totals");
}

fwant_status fwant_kerinfo_record(fwant_kerinfo* k, int r, int* m, int* station, int* event) {
  if (!k || r < 0 || (!m && !station && !event)) return FWANT_ERR_INVALID_ARG;
  if (r >= k->nrec) return k->fail(FWANT_ERR_INVALID_ARG, "record " + std::to_string(r) + " not written");
  cudaError_t e = cudaSetDevice(k->device);
  int* const dst[3] = {m, station, event};
  for (int w = 0; w < 3 && e == cudaSuccess; ++w)
    if (dst[w])
      e = cudaMemcpyAsync(dst[w], k->recs[size_t(r)] + size_t(w) * 4 * size_t(k->npts), k->vol_bytes(sizeof(int)),
                          cudaMemcpyDeviceToHost, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  return e == cudaSuccess ? FWANT_OK : k->cuda_fail(e, "record");
}

fwant_status fwant_kerinfo_last_ms(fwant_kerinfo* k, double* ms) {
  if (!k || !ms) return FWANT_ERR_INVALID_ARG;
  *ms = k->last_ms;
  return FWANT_OK;
}

}  // extern "C"
