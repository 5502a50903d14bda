// Strided sub-volume extraction of the wavefield: the data of one snapshot frame of
// io_wave_export (mod_io.F90:505-645), packed on the device into a staging buffer and
// copied to the host.
#include <cuda_runtime.h>

#include "kernels.h"
#include "storage.cuh"

namespace fw {

__global__ void pack_snapshot_kernel(const SnapArgs a) {
  const long long n = (long long)a.cnt[0] * a.cnt[1] * a.cnt[2];
  const long long tot = n * a.ncomp;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int c = int(e / n);
    long long r = e - (long long)c * n;
    const int ii = int(r % a.cnt[0]);
    r /= a.cnt[0];
    const int jj = int(r % a.cnt[1]);
    const int kk = int(r / a.cnt[1]);
    const int i = a.start[0] + ii * a.stride[0], j = a.start[1] + jj * a.stride[1], k = a.start[2] + kk * a.stride[2];
    const long long p = (long long)(i + PADL) + (long long)a.g.px * ((long long)j + (long long)a.g.ny * k);
    a.out[e] = load_component(a.w, a.storage, a.g.fstride, a.comp[c], p, a.isv, a.ist);
  }
}

void launch_pack_snapshot(const SnapArgs& a, void* stream) {
  const long long tot = (long long)a.cnt[0] * a.cnt[1] * a.cnt[2] * a.ncomp;
  long long blocks = (tot + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  if (blocks < 1) blocks = 1;
  pack_snapshot_kernel<<<int(blocks), 256, 0, (cudaStream_t)stream>>>(a);
}

// Stress components of an SGT frame in storage order: Txx Tyy Tzz Txy Txz Tyz.
__constant__ int kSgtComp[6] = {6, 7, 3, 8, 4, 5};

__global__ void record_sgt_kernel(const SgtRecArgs a) {
  const int nt = *a.ntime;
  if (nt <= 0 || nt % a.tinv != 0) return;
  const int frame = nt / a.tinv - 1;
  if (frame >= a.max_frames) return;
  const long long tot = a.npts * 6;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int c = int(e / a.npts);
    long long r = e - (long long)c * a.npts;
    const long long pt = r;
    const int ii = int(r % a.cnt[0]);
    r /= a.cnt[0];
    const int jj = int(r % a.cnt[1]);
    const int kk = int(r / a.cnt[1]);
    const int i = a.start[0] + ii * a.stride[0], j = a.start[1] + jj * a.stride[1], k = a.start[2] + kk * a.stride[2];
    const long long p = (long long)(i + PADL) + (long long)a.g.px * ((long long)j + (long long)a.g.ny * k);
    a.out[((long long)c * a.max_frames + frame) * a.npts + pt] =
        load_component(a.w, a.storage, a.g.fstride, kSgtComp[c], p, a.isv, a.ist);
  }
}

void launch_record_sgt(const SgtRecArgs& a, void* stream) {
  long long blocks = (a.npts * 6 + 255) / 256;
  if (blocks > 152LL * 8) blocks = 152LL * 8;
  if (blocks < 1) blocks = 1;
  record_sgt_kernel<<<int(blocks), 256, 0, (cudaStream_t)stream>>>(a);
}

// Staging buffer of fwant_get_snapshot_noalloc, for callers that must not allocate
// device memory.  It is a module-scope device array, so it exists on every device that
// loads this library, for as long as the library stays loaded; every call on a device
// shares it.  The pack kernel writes every element that is copied out, so nothing in it
// needs clearing between calls.
static __device__ __align__(256) float g_snapshot_staging[SNAPSHOT_NOALLOC_MAX];

// Device address of the staging array on the current device.  It is resolved on every
// call (cudaGetSymbolAddress allocates nothing and is cheap), so a device reset or a
// re-created primary context, after which the module may load at another address, never
// leaves a stale pointer behind.
int snapshot_noalloc_staging(int device, float** ptr) {
  (void)device;  // the caller has made `device` current
  float* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_snapshot_staging);
  if (e != cudaSuccess) return int(e);
  *ptr = p;
  return 0;
}

}  // namespace fw
