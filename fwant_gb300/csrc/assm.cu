// Kernel assembly onto inversion blocks (SI_ker2assm / SI_ker_kamu2assm,
// code/srcF.kernel/SI_ker2assm.F90:306-323): B(n) = sum over block n's pixels of K * volume,
// S(n) += |B(n)|.  C ABI in include/fwant_assm.h.
//
// Layout: the pixel lists are stored transposed, (max_pix, num_blk) with the block index
// fastest, as linear offsets into the Fortran-order kernel volume, so that the threads of a
// warp (consecutive blocks) read their m-th pixel with one coalesced load; the kernel values
// themselves are gathers.  One thread sums one block in the file's pixel order, each product
// rounded before the add (__fmul_rn / __fadd_rn), which is the reference's single-precision
// arithmetic; the sweep over all blocks reads every kernel point about once, so the launch is
// bound by the gathers' DRAM traffic.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "fwant_assm.h"

namespace {

constexpr int AS_THREADS = 256;
constexpr int AS_MAXQ = 4;

struct KPtrs {
  const float* p[AS_MAXQ];
};

template <int NQ>
__global__ void __launch_bounds__(AS_THREADS) project_kernel(int nblk, const int* __restrict__ npix,
                                                             const int* __restrict__ lin,
                                                             const float* __restrict__ vol, KPtrs K,
                                                             float* __restrict__ B, float* __restrict__ S) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nblk) return;
  float b[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) b[q] = 0.0f;
  const int np = npix[n];
  const int* lp = lin + n;
  const float* vp = vol + n;
#pragma unroll 4
  for (int m = 0; m < np; ++m) {
    const int idx = __ldg(lp);
    const float v = __ldg(vp);
    lp += nblk;
    vp += nblk;
#pragma unroll
    for (int q = 0; q < NQ; ++q) b[q] = __fadd_rn(b[q], __fmul_rn(__ldg(K.p[q] + idx), v));
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    B[size_t(q) * nblk + n] = b[q];
    S[size_t(q) * nblk + n] = __fadd_rn(S[size_t(q) * nblk + n], fabsf(b[q]));
  }
}

void launch_project(int nq, int nblk, const int* npix, const int* lin, const float* vol, const KPtrs& K, float* B,
                    float* S, cudaStream_t st) {
  const int grid = (nblk + AS_THREADS - 1) / AS_THREADS;
  switch (nq) {
    case 1: project_kernel<1><<<grid, AS_THREADS, 0, st>>>(nblk, npix, lin, vol, K, B, S); break;
    case 2: project_kernel<2><<<grid, AS_THREADS, 0, st>>>(nblk, npix, lin, vol, K, B, S); break;
    case 3: project_kernel<3><<<grid, AS_THREADS, 0, st>>>(nblk, npix, lin, vol, K, B, S); break;
    default: project_kernel<4><<<grid, AS_THREADS, 0, st>>>(nblk, npix, lin, vol, K, B, S); break;
  }
}

}  // namespace

struct fwant_assm {
  int ki = 0, kj = 0, kk = 0, nblk = 0, maxpix = 0, device = 0;
  size_t nvol = 0;
  int* d_npix = nullptr;
  int* d_lin = nullptr;
  float* d_vol = nullptr;
  float* d_S = nullptr;  // (num_blk, 4)
  float* d_B = nullptr;  // (num_blk, 4)
  float* d_K = nullptr;  // staging of host kernel volumes, (nvol, 4)
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
  ~fwant_assm() {
    cudaSetDevice(device);
    for (void* p : {static_cast<void*>(d_npix), static_cast<void*>(d_lin), static_cast<void*>(d_vol),
                    static_cast<void*>(d_S), static_cast<void*>(d_B), static_cast<void*>(d_K)})
      if (p) cudaFree(p);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
  }

  fwant_status run(int nq, const KPtrs& K, float* blocks) {
    cudaError_t e = cudaEventRecord(e0, st);
    launch_project(nq, nblk, d_npix, d_lin, d_vol, K, d_B, d_S, st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(blocks, d_B, size_t(nq) * nblk * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&last_ms, e0, e1);
    return e == cudaSuccess ? FWANT_OK : cuda_fail(e, "projection");
  }
};

extern "C" {

fwant_status fwant_assm_create(int ki, int kj, int kk, int num_blk, int max_pix, const float* volume,
                               const int* num_of_pix, const int* indx_of_pix, int device, fwant_assm** out) {
  if (!out) return FWANT_ERR_INVALID_ARG;
  *out = nullptr;
  if (ki < 1 || kj < 1 || kk < 1 || num_blk < 1 || max_pix < 1 || !volume || !num_of_pix || !indx_of_pix)
    return FWANT_ERR_INVALID_ARG;
  const size_t nvol = size_t(ki) * kj * kk;
  if (nvol > size_t(0x7fffffff)) return FWANT_ERR_INVALID_ARG;
  auto* a = new fwant_assm();
  a->ki = ki; a->kj = kj; a->kk = kk; a->nblk = num_blk; a->maxpix = max_pix; a->device = device;
  a->nvol = nvol;
  // transpose the pixel lists to (max_pix, num_blk) linear offsets, checking every used index
  const size_t np = size_t(max_pix) * num_blk;
  std::vector<int> lin(np, 0);
  std::vector<float> vol(np, 0.0f);
  for (int n = 0; n < num_blk; ++n) {
    const int cnt = num_of_pix[n];
    if (cnt < 0 || cnt > max_pix) {
      *out = a;
      return a->fail(FWANT_ERR_INVALID_ARG, "num_of_pix of block " + std::to_string(n + 1) + " outside 0..max_pix");
    }
    for (int m = 0; m < cnt; ++m) {
      const int* p = indx_of_pix + 3 * (size_t(n) * max_pix + m);
      if (p[0] < 1 || p[0] > ki || p[1] < 1 || p[1] > kj || p[2] < 1 || p[2] > kk) {
        *out = a;
        return a->fail(FWANT_ERR_INVALID_ARG, "pixel " + std::to_string(m + 1) + " of block " + std::to_string(n + 1) +
                                                  " lies outside the kernel volume");
      }
      lin[size_t(m) * num_blk + n] = (p[0] - 1) + ki * ((p[1] - 1) + kj * (p[2] - 1));
      vol[size_t(m) * num_blk + n] = volume[size_t(n) * max_pix + m];
    }
  }
  *out = a;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&a->e1);
  if (e == cudaSuccess) e = cudaMalloc(&a->d_npix, size_t(num_blk) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&a->d_lin, np * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&a->d_vol, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->d_S, size_t(AS_MAXQ) * num_blk * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->d_B, size_t(AS_MAXQ) * num_blk * sizeof(float));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(a->d_npix, num_of_pix, size_t(num_blk) * sizeof(int), cudaMemcpyHostToDevice, a->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->d_lin, lin.data(), np * sizeof(int), cudaMemcpyHostToDevice, a->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->d_vol, vol.data(), np * sizeof(float), cudaMemcpyHostToDevice, a->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(a->d_S, 0, size_t(AS_MAXQ) * num_blk * sizeof(float), a->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(a->st);
  if (e != cudaSuccess) return a->cuda_fail(e, "create");
  return FWANT_OK;
}

void fwant_assm_destroy(fwant_assm* a) { delete a; }

const char* fwant_assm_last_error(fwant_assm* a) { return a ? a->err.c_str() : "null handle"; }

fwant_status fwant_assm_project(fwant_assm* a, int nq, const float* const* kernels, float* blocks) {
  if (!a || nq < 1 || nq > AS_MAXQ || !kernels || !blocks) return FWANT_ERR_INVALID_ARG;
  for (int q = 0; q < nq; ++q)
    if (!kernels[q]) return a->fail(FWANT_ERR_INVALID_ARG, "null kernel volume");
  cudaError_t e = cudaSetDevice(a->device);
  if (e == cudaSuccess && !a->d_K) e = cudaMalloc(&a->d_K, size_t(AS_MAXQ) * a->nvol * sizeof(float));
  KPtrs K{};
  for (int q = 0; q < nq && e == cudaSuccess; ++q) {
    K.p[q] = a->d_K + size_t(q) * a->nvol;
    e = cudaMemcpyAsync(const_cast<float*>(K.p[q]), kernels[q], a->nvol * sizeof(float), cudaMemcpyHostToDevice,
                        a->st);
  }
  if (e != cudaSuccess) return a->cuda_fail(e, "kernel upload");
  return a->run(nq, K, blocks);
}

// Bytes from p to the end of the device allocation holding it (driver entry point
// cuMemGetAddressRange, looked up through the runtime so the library needs no -lcuda).
static int device_room(const void* p, size_t* room) {
  using RangeFn = CUresult (*)(CUdeviceptr*, size_t*, CUdeviceptr);
  static RangeFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<RangeFn>(f);
  }();
  if (!fn) return -1;
  CUdeviceptr base = 0;
  size_t size = 0;
  const CUresult r = fn(&base, &size, reinterpret_cast<CUdeviceptr>(p));
  if (r != CUDA_SUCCESS) return int(r);
  *room = size_t(base + size - reinterpret_cast<CUdeviceptr>(p));
  return 0;
}

fwant_status fwant_assm_project_device(fwant_assm* a, int nq, const float* const* d_kernels, float* blocks) {
  if (!a || nq < 1 || nq > AS_MAXQ || !d_kernels || !blocks) return FWANT_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(a->device);
  if (e != cudaSuccess) return a->cuda_fail(e, "set device");
  KPtrs K{};
  for (int q = 0; q < nq; ++q) {
    cudaPointerAttributes at{};
    if (!d_kernels[q] || cudaPointerGetAttributes(&at, d_kernels[q]) != cudaSuccess ||
        at.type != cudaMemoryTypeDevice || at.device != a->device) {
      cudaGetLastError();
      return a->fail(FWANT_ERR_INVALID_ARG, "kernel volumes must be device memory of the handle's GPU");
    }
    // the allocation must hold the whole volume from the given pointer on: the gather
    // kernel reads any of its ki*kj*kk values
    size_t room = 0;
    if (int ce = device_room(d_kernels[q], &room))
      return a->fail(FWANT_ERR_INVALID_ARG, "kernel volume: cuMemGetAddressRange failed (" + std::to_string(ce) + ")");
    if (room < a->nvol * sizeof(float))
      return a->fail(FWANT_ERR_INVALID_ARG, "kernel volume " + std::to_string(q) + ": its allocation holds " +
                                                std::to_string(room / sizeof(float)) + " floats past the pointer, " +
                                                std::to_string(a->nvol) + " needed");
    K.p[q] = d_kernels[q];
  }
  return a->run(nq, K, blocks);
}

fwant_status fwant_assm_sums(fwant_assm* a, float* sums) {
  if (!a || !sums) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(a->device);
  const cudaError_t e = cudaMemcpy(sums, a->d_S, size_t(AS_MAXQ) * a->nblk * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? FWANT_OK : a->cuda_fail(e, "sums");
}

fwant_status fwant_assm_last_ms(fwant_assm* a, double* ms) {
  if (!a || !ms) return FWANT_ERR_INVALID_ARG;
  *ms = a->last_ms;
  return FWANT_OK;
}

}  // extern "C"
