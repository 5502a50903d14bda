// Small kernels around the stage kernel: receiver sampling with the step counter,
// the FP64 metric, and the overflow check.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>

#include "kernels.h"
#include "storage.cuh"

namespace fw {

// io_seismo_put (mod_io.F90:461-497) fused with ntime = ntime + 1
// (seis3d_wave_8op_p3.F90:152): one block; every thread reads the counter before
// thread 0 advances it.
__global__ void advance_record_kernel(const RecvArgs a) {
  const int n = *a.ntime;
  const int nn = n + 1;
  if (a.npt > 0 && nn % a.tinv == 0) {
    const int m = nn / a.tinv - 1;
    if (m < a.cap) {
      for (int e = threadIdx.x; e < a.npt * NF; e += blockDim.x) {
        const int pt = e % a.npt, f = e / a.npt;  // f in the output order Vx Vy Vz Txx Tyy Tzz Txy Txz Tyz
        const int fi = f < 3 ? f : (f == 3 ? TXX : (f == 4 ? TYY : (f == 5 ? TZZ : (f == 6 ? TXY : (f == 7 ? TXZ : TYZ)))));
        const int i = a.idx[3 * pt], j = a.idx[3 * pt + 1], k = a.idx[3 * pt + 2];
        const long long p = (long long)(i + PADL) + (long long)a.g.px * ((long long)j + (long long)a.g.ny * k);
        a.seismo[((long long)f * a.cap + m) * a.npt + pt] = load_component(a.w, a.storage, a.g.fstride, fi, p, a.isv, a.ist);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *a.ntime = nn;
}

void launch_advance_record(const RecvArgs& a, void* stream) {
  advance_record_kernel<<<1, 256, 0, (cudaStream_t)stream>>>(a);
}

// seis3d_metric (seis3d_metric.F90:83-112) in FP64: x_xi is the mean of the backward
// and forward DRP/opt derivatives of the coordinate, xi_x its reciprocal rounded to
// FP32; the ghost entries copy the nearest interior value.
__global__ void metric_kernel(int n, const float* __restrict__ g, float* __restrict__ out, int lo, int hi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ii = i < lo ? lo : (i > hi ? hi : i);
  const double cF[5] = {-0.30874, -0.6326, 1.2330, -0.3334, 0.04168};
  const double cB[5] = {-0.04168, 0.3334, -1.2330, 0.6326, 0.30874};
  double sb = 0.0, sf = 0.0;
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    sb += double(g[ii - 3 + q]) * cB[q];
    sf += double(g[ii - 1 + q]) * cF[q];
  }
  out[i] = float(1.0 / ((sb + sf) * 0.5));
}

void launch_metric_fp64(int n, const float* coord, float* out, int lo, int hi, void* stream) {
  metric_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(n, coord, out, lo, hi);
}

__global__ void sincot_kernel(int n, const float* __restrict__ x, float* __restrict__ xsin, float* __restrict__ xcot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = double(x[i]);
  xsin[i] = float(sin(v));
  xcot[i] = float(1.0 / tan(v));
}

void launch_sincot_fp64(int n, const float* x, float* xsin, float* xcot, void* stream) {
  sincot_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(n, x, xsin, xcot);
}

// macdrp_check (mod_macdrp.F90:228-264): maximum of |value| over the interior of each
// of the nine components.  The bit pattern of a non-negative float orders like the value,
// and NaN (0x7fc00000 after fabs) orders above Inf, so an atomicMax on the bits yields
// max|v| with NaN and Inf detectable on the host.
__global__ void maxabs_kernel(const Geom g, const void* __restrict__ w, int storage, float isv, float ist,
                              unsigned int* out) {
  unsigned int best[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) best[f] = 0;
  const long long tot = (long long)g.ni * g.nj * g.nk;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = g.i1 + int(e % g.ni);
    const long long r = e / g.ni;
    const int j = g.j1 + int(r % g.nj);
    const int k = g.k1 + int(r / g.nj);
    const long long p = (long long)(i + PADL) + (long long)g.px * ((long long)j + (long long)g.ny * k);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const unsigned int b = __float_as_uint(fabsf(load_component(w, storage, g.fstride, f, p, isv, ist)));
      best[f] = b > best[f] ? b : best[f];
    }
  }
#pragma unroll
  for (int f = 0; f < NF; ++f) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned int v = __shfl_xor_sync(0xffffffffu, best[f], o);
      best[f] = v > best[f] ? v : best[f];
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out + f, best[f]);
  }
}

void launch_maxabs(const Geom& g, const void* w, int storage, float isv, float ist, unsigned int* out_bits,
                   void* stream) {
  maxabs_kernel<<<152 * 4, 256, 0, (cudaStream_t)stream>>>(g, w, storage, isv, ist, out_bits);
}

// One component between its storage type and FP32 over the whole padded array.
__global__ void convert_kernel(long long n, const void* __restrict__ src, int src_st, float scale, void* __restrict__ dst,
                               int dst_st) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    float v;
    if (src_st == ST_F32) v = static_cast<const float*>(src)[e];
    else if (src_st == ST_BF16) v = __bfloat162float(static_cast<const __nv_bfloat16*>(src)[e]);
    else v = __half2float(static_cast<const __half*>(src)[e]);
    v = v * scale;
    if (dst_st == ST_F32) static_cast<float*>(dst)[e] = v;
    else if (dst_st == ST_BF16) static_cast<__nv_bfloat16*>(dst)[e] = __float2bfloat16_rn(v);
    else static_cast<__half*>(dst)[e] = __float2half_rn(v);
  }
}

// number of elements that are not > 0 (NaN included) into *count
__global__ void count_nonpositive_kernel(long long n, const float* __restrict__ v, unsigned int* count) {
  unsigned int c = 0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    c += !(v[e] > 0.0f);
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

void launch_count_nonpositive(long long n, const float* v, unsigned int* count, void* stream) {
  count_nonpositive_kernel<<<152 * 4, 256, 0, (cudaStream_t)stream>>>(n, v, count);
}

void launch_convert_to_f32(const Geom& g, const void* src, int storage, float inv_scale, float* dst, void* stream) {
  convert_kernel<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(g.plane * g.nz, src, storage, inv_scale, dst, ST_F32);
}

void launch_convert_from_f32(const Geom& g, const float* src, int storage, float scale, void* dst, void* stream) {
  convert_kernel<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(g.plane * g.nz, src, ST_F32, scale, dst, storage);
}

}  // namespace fw
