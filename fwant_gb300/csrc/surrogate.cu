// Kernels of the waveform surrogate: a small 3-D convolutional network (3x3x3
// convolutions, dense layers, leaky ReLU) with BF16 weights and FP32 activations,
// accumulation and gradients, trained with Adam on FP32 master weights.  Every kernel is
// deterministic (fixed reduction order), so training runs repeat bit for bit.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/fwant_surrogate.h"

namespace {

__device__ __forceinline__ float bf(const uint16_t v) { return __uint_as_float(uint32_t(v) << 16); }

inline int grid_for(long long n, int threads, int cap = 152 * 32) {
  long long b = (n + threads - 1) / threads;
  if (b > cap) b = cap;
  return int(b < 1 ? 1 : b);
}

// ---- 3x3x3 convolution, padding 1, stride s; layouts NCDHW, weights [Cout][Cin][27] ----
struct ConvDims {
  int B, Ci, D, H, W, Co, s, Do, Ho, Wo;
};

__global__ void conv_fwd_kernel(const float* __restrict__ x, const uint16_t* __restrict__ w,
                                const float* __restrict__ bias, float* __restrict__ y, ConvDims c) {
  const long long n = (long long)c.B * c.Co * c.Do * c.Ho * c.Wo;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    long long r = e;
    const int wo = int(r % c.Wo); r /= c.Wo;
    const int ho = int(r % c.Ho); r /= c.Ho;
    const int d0 = int(r % c.Do); r /= c.Do;
    const int co = int(r % c.Co);
    const int b = int(r / c.Co);
    float acc = bias ? bias[co] : 0.0f;
    for (int ci = 0; ci < c.Ci; ++ci) {
      const float* xp = x + ((long long)b * c.Ci + ci) * c.D * c.H * c.W;
      const uint16_t* wp = w + ((long long)co * c.Ci + ci) * 27;
      for (int kd = 0; kd < 3; ++kd) {
        const int di = d0 * c.s + kd - 1;
        if (di < 0 || di >= c.D) continue;
        for (int kh = 0; kh < 3; ++kh) {
          const int hi = ho * c.s + kh - 1;
          if (hi < 0 || hi >= c.H) continue;
          for (int kw = 0; kw < 3; ++kw) {
            const int wi = wo * c.s + kw - 1;
            if (wi < 0 || wi >= c.W) continue;
            acc = fmaf(bf(wp[(kd * 3 + kh) * 3 + kw]), xp[((long long)di * c.H + hi) * c.W + wi], acc);
          }
        }
      }
    }
    y[e] = acc;
  }
}

// dx[b,ci,di,hi,wi] = sum over co, k with di = do*s + kd - 1 of dy[b,co,do,..] w[co,ci,k]
__global__ void conv_bwd_data_kernel(const float* __restrict__ dy, const uint16_t* __restrict__ w,
                                     float* __restrict__ dx, ConvDims c) {
  const long long n = (long long)c.B * c.Ci * c.D * c.H * c.W;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    long long r = e;
    const int wi = int(r % c.W); r /= c.W;
    const int hi = int(r % c.H); r /= c.H;
    const int di = int(r % c.D); r /= c.D;
    const int ci = int(r % c.Ci);
    const int b = int(r / c.Ci);
    float acc = 0.0f;
    for (int co = 0; co < c.Co; ++co) {
      const float* dp = dy + ((long long)b * c.Co + co) * c.Do * c.Ho * c.Wo;
      const uint16_t* wp = w + ((long long)co * c.Ci + ci) * 27;
      for (int kd = 0; kd < 3; ++kd) {
        const int t = di + 1 - kd;
        if (t < 0 || t % c.s) continue;
        const int d0 = t / c.s;
        if (d0 >= c.Do) continue;
        for (int kh = 0; kh < 3; ++kh) {
          const int u = hi + 1 - kh;
          if (u < 0 || u % c.s) continue;
          const int ho = u / c.s;
          if (ho >= c.Ho) continue;
          for (int kw = 0; kw < 3; ++kw) {
            const int v = wi + 1 - kw;
            if (v < 0 || v % c.s) continue;
            const int wo = v / c.s;
            if (wo >= c.Wo) continue;
            acc = fmaf(bf(wp[(kd * 3 + kh) * 3 + kw]), dp[((long long)d0 * c.Ho + ho) * c.Wo + wo], acc);
          }
        }
      }
    }
    dx[e] = acc;
  }
}

// dw[co,ci,k] = sum over b and output positions of dy * x; one CTA per weight, fixed-order
// block reduction.  db[co] likewise (ci == 0, k == 0 CTAs).
__global__ void conv_bwd_weight_kernel(const float* __restrict__ x, const float* __restrict__ dy,
                                       float* __restrict__ dw, float* __restrict__ db, ConvDims c) {
  const int widx = blockIdx.x;  // co*Ci*27 + ci*27 + k
  const int k = widx % 27, ci = (widx / 27) % c.Ci, co = widx / (27 * c.Ci);
  const int kd = k / 9, kh = (k / 3) % 3, kw = k % 3;
  const long long per = (long long)c.Do * c.Ho * c.Wo;
  const long long n = (long long)c.B * per;
  float acc = 0.0f, accb = 0.0f;
  for (long long e = threadIdx.x; e < n; e += blockDim.x) {
    const int b = int(e / per);
    long long r = e - (long long)b * per;
    const int wo = int(r % c.Wo); r /= c.Wo;
    const int ho = int(r % c.Ho);
    const int d0 = int(r / c.Ho);
    const float g = dy[((long long)b * c.Co + co) * per + (long long)(d0 * c.Ho + ho) * c.Wo + wo];
    accb += g;
    const int di = d0 * c.s + kd - 1, hi = ho * c.s + kh - 1, wi = wo * c.s + kw - 1;
    if (di < 0 || di >= c.D || hi < 0 || hi >= c.H || wi < 0 || wi >= c.W) continue;
    acc = fmaf(g, x[(((long long)b * c.Ci + ci) * c.D + di) * c.H * c.W + (long long)hi * c.W + wi], acc);
  }
  __shared__ float red[2][256];
  red[0][threadIdx.x] = acc;
  red[1][threadIdx.x] = accb;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    dw[widx] = red[0][0];
    if (db && ci == 0 && k == 0) db[co] = red[1][0];
  }
}

// ---- dense layers: tiled C = A * B with strided operands (B optionally BF16) ----------
// C[m][n] (row-major, ldc) = sum_k A(m,k) B(k,n) (+ bias[n]); A(m,k) = A[m*sam + k*sak],
// B(k,n) = B[k*sbk + n*sbn].  64x64 tile, 256 threads of 4x4 outputs, k-step 16.
// Split K: blockIdx.z takes k in [z*kchunk, min(K, (z+1)*kchunk)) and, with more than one
// split, writes its partial tile to C + z*M*ldc (a workspace) for splitk_reduce_kernel.
template <bool BBF16>
__global__ void __launch_bounds__(256) gemm_kernel(const float* __restrict__ A, long long sam, long long sak,
                                                   const void* __restrict__ Bv, long long sbk, long long sbn,
                                                   const float* __restrict__ bias, float* __restrict__ C,
                                                   long long ldc, int M, int N, int K, int kchunk) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64 + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  if (gridDim.z > 1) {
    C += (long long)blockIdx.z * M * ldc;
    bias = nullptr;
  }
  float acc[4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += 16) {
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const int kk = e / 64, mm = e % 64;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < ke) ? A[m * sam + k * sak] : 0.0f;
    }
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const int kk = e / 64, nn = e % 64;
      const int n = n0 + nn, k = k0 + kk;
      float v = 0.0f;
      if (n < N && k < ke) {
        if (BBF16) v = bf(static_cast<const uint16_t*>(Bv)[k * sbk + n * sbn]);
        else v = static_cast<const float*>(Bv)[k * sbk + n * sbn];
      }
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][ty * 4 + q];
        b[q] = Bs[kk][tx * 4 + q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int m = m0 + ty * 4 + p;
    if (m >= M) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int n = n0 + tx * 4 + q;
      if (n >= N) continue;
      C[m * ldc + n] = acc[p][q] + (bias ? bias[n] : 0.0f);
    }
  }
}

// C[m][n] = sum_z W[z][m][n] (+ bias[n]) in split order
__global__ void splitk_reduce_kernel(const float* __restrict__ W, int splits, const float* __restrict__ bias,
                                     float* __restrict__ C, int M, int N) {
  const long long n_el = (long long)M * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_el; e += (long long)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int z = 0; z < splits; ++z) s += W[(long long)z * n_el + e];
    C[e] = s + (bias ? bias[e % N] : 0.0f);
  }
}

// Workspace of the split-K partial tiles, grown on demand (one per process and device).
float* splitk_workspace(size_t floats, int* err) {
  static float* ws[64] = {};
  static size_t cap[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) { *err = int(cudaErrorInvalidDevice); return nullptr; }
  if (cap[dev] < floats) {
    cudaFree(ws[dev]);
    ws[dev] = nullptr;
    cap[dev] = 0;
    if (cudaMalloc(&ws[dev], floats * sizeof(float)) != cudaSuccess) {
      *err = int(cudaGetLastError());
      return nullptr;
    }
    cap[dev] = floats;
  }
  return ws[dev];
}

template <bool BBF16>
int gemm(const float* A, long long sam, long long sak, const void* B, long long sbk, long long sbn, const float* bias,
         float* C, long long ldc, int M, int N, int K, cudaStream_t st) {
  const int tiles = ((N + 63) / 64) * ((M + 63) / 64);
  // split K when the tiles alone cannot fill the GPU (contiguous C only)
  int splits = 1;
  if (ldc == N && tiles < 304 && K >= 512) {
    splits = (304 + tiles - 1) / tiles;
    if (splits > K / 256) splits = K / 256;
    if (splits < 1) splits = 1;
  }
  const int kchunk = ((K + splits - 1) / splits + 15) / 16 * 16;
  splits = (K + kchunk - 1) / kchunk;
  const dim3 grid((N + 63) / 64, (M + 63) / 64, splits);
  if (splits == 1) {
    gemm_kernel<BBF16><<<grid, 256, 0, st>>>(A, sam, sak, B, sbk, sbn, bias, C, ldc, M, N, K, kchunk);
    return int(cudaGetLastError());
  }
  int err = 0;
  float* ws = splitk_workspace(size_t(splits) * M * N, &err);
  if (!ws) return err;
  gemm_kernel<BBF16><<<grid, 256, 0, st>>>(A, sam, sak, B, sbk, sbn, bias, ws, N, M, N, K, kchunk);
  splitk_reduce_kernel<<<grid_for((long long)M * N, 256), 256, 0, st>>>(ws, splits, bias, C, M, N);
  return int(cudaGetLastError());
}

// column sums: out[n] = sum_m A[m][n] (bias gradients), fixed order
__global__ void colsum_kernel(const float* __restrict__ A, float* __restrict__ out, int M, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.0f;
  for (int m = 0; m < M; ++m) s += A[(long long)m * N + n];
  out[n] = s;
}

__global__ void lrelu_fwd_kernel(float* y, long long n, float slope) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float v = y[e];
    y[e] = v > 0.0f ? v : slope * v;
  }
}
// dy *= f'(y) with y the activation output (positive iff the input was)
__global__ void lrelu_bwd_kernel(const float* y, float* dy, long long n, float slope) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    if (!(y[e] > 0.0f)) dy[e] *= slope;
}

// loss = sum (y - t)^2 / n, dy = 2 (y - t) / n; per-block partial sums then a fixed-order
// final sum by one block
__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy,
                           float* __restrict__ partial, long long n) {
  __shared__ float red[256];
  float s = 0.0f;
  const float inv = 1.0f / float(n);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float d = y[e] - t[e];
    s = fmaf(d, d, s);
    if (dy) dy[e] = 2.0f * d * inv;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}
__global__ void sum_partials_kernel(const float* partial, int nb, long long n, float* loss) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += partial[b];
  *loss = float(s / double(n));
}

// Adam with decoupled weight decay on FP32 master weights; refreshes the BF16 copy
__global__ void adam_kernel(float* w, uint16_t* w16, const float* g, float* m, float* v, long long n, float lr,
                            float b1, float b2, float eps, float wd, float c1, float c2) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float gg = g[e];
    const float mm = b1 * m[e] + (1.0f - b1) * gg;
    const float vv = b2 * v[e] + (1.0f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    float ww = w[e] * (1.0f - lr * wd);
    ww -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    w[e] = ww;
    if (w16) w16[e] = __bfloat16_as_ushort(__float2bfloat16_rn(ww));
  }
}

__global__ void to_bf16_kernel(const float* w, uint16_t* w16, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    w16[e] = __bfloat16_as_ushort(__float2bfloat16_rn(w[e]));
}

// y[e] = a[e] + s * b[e]
__global__ void axpby_kernel(const float* a, const float* b, float s, float* y, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    y[e] = a[e] + s * b[e];
}

// out[b][g][t] = sum_k coef[b][g][k] basis[g][k][t]
__global__ void basis_fwd_kernel(const float* __restrict__ coef, const float* __restrict__ basis,
                                 float* __restrict__ out, int B, int G, int K, int T) {
  const long long n = (long long)B * G * T;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int t = int(e % T);
    const long long bg = e / T;
    const int g = int(bg % G);
    const float* c = coef + bg * K;
    const float* bs = basis + (long long)g * K * T + t;
    float acc = 0.0f;
    for (int k = 0; k < K; ++k) acc = fmaf(c[k], bs[(long long)k * T], acc);
    out[e] = acc;
  }
}
// dcoef[b][g][k] = sum_t dout[b][g][t] basis[g][k][t]
__global__ void basis_bwd_kernel(const float* __restrict__ dout, const float* __restrict__ basis,
                                 float* __restrict__ dcoef, int B, int G, int K, int T) {
  const long long n = (long long)B * G * K;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int k = int(e % K);
    const long long bg = e / K;
    const int g = int(bg % G);
    const float* d = dout + bg * T;
    const float* bs = basis + ((long long)g * K + k) * T;
    float acc = 0.0f;
    for (int t = 0; t < T; ++t) acc = fmaf(d[t], bs[t], acc);
    dcoef[e] = acc;
  }
}

ConvDims dims(int B, int Ci, int D, int H, int W, int Co, int s) {
  ConvDims c{B, Ci, D, H, W, Co, s, (D - 1) / s + 1, (H - 1) / s + 1, (W - 1) / s + 1};
  return c;
}

}  // namespace

extern "C" {

int fwant_nn_conv3d_fwd(const float* x, const uint16_t* w, const float* bias, float* y, int B, int Ci, int D, int H,
                        int W, int Co, int stride, void* stream) {
  if (stride < 1 || B < 1 || Ci < 1 || Co < 1) return int(cudaErrorInvalidValue);
  const ConvDims c = dims(B, Ci, D, H, W, Co, stride);
  const long long n = (long long)B * Co * c.Do * c.Ho * c.Wo;
  conv_fwd_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(x, w, bias, y, c);
  return int(cudaGetLastError());
}

int fwant_nn_conv3d_bwd(const float* x, const uint16_t* w, const float* dy, float* dx, float* dw, float* db, int B,
                        int Ci, int D, int H, int W, int Co, int stride, void* stream) {
  if (stride < 1 || B < 1 || Ci < 1 || Co < 1) return int(cudaErrorInvalidValue);
  const ConvDims c = dims(B, Ci, D, H, W, Co, stride);
  cudaStream_t st = (cudaStream_t)stream;
  if (dx) {
    const long long n = (long long)B * Ci * D * H * W;
    conv_bwd_data_kernel<<<grid_for(n, 256), 256, 0, st>>>(dy, w, dx, c);
  }
  if (dw) conv_bwd_weight_kernel<<<Co * Ci * 27, 256, 0, st>>>(x, dy, dw, db, c);
  return int(cudaGetLastError());
}

int fwant_nn_linear_fwd(const float* x, const uint16_t* w, const float* bias, float* y, int B, int In, int Out,
                        void* stream) {
  // y[b][o] = sum_i x[b][i] w[o][i] + bias[o]
  return gemm<true>(x, In, 1, w, 1, In, bias, y, Out, B, Out, In, (cudaStream_t)stream);
}

int fwant_nn_linear_bwd(const float* x, const uint16_t* w, const float* dy, float* dx, float* dw, float* db, int B,
                        int In, int Out, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  int e = 0;
  // dx[b][i] = sum_o dy[b][o] w[o][i]
  if (dx) e = gemm<true>(dy, Out, 1, w, In, 1, nullptr, dx, In, B, In, Out, st);
  // dw[o][i] = sum_b dy[b][o] x[b][i]
  if (!e && dw) e = gemm<false>(dy, 1, Out, x, In, 1, nullptr, dw, In, Out, In, B, st);
  if (!e && db) {
    colsum_kernel<<<(Out + 255) / 256, 256, 0, st>>>(dy, db, B, Out);
    e = int(cudaGetLastError());
  }
  return e;
}

int fwant_nn_lrelu_fwd(float* y, long long n, float slope, void* stream) {
  lrelu_fwd_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(y, n, slope);
  return int(cudaGetLastError());
}

int fwant_nn_lrelu_bwd(const float* y, float* dy, long long n, float slope, void* stream) {
  lrelu_bwd_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(y, dy, n, slope);
  return int(cudaGetLastError());
}

int fwant_nn_mse(const float* y, const float* t, float* dy, float* loss, float* scratch, long long n, void* stream) {
  // scratch: at least FWANT_NN_MSE_BLOCKS floats
  const int nb = grid_for(n, 256, FWANT_NN_MSE_BLOCKS);
  cudaStream_t st = (cudaStream_t)stream;
  mse_kernel<<<nb, 256, 0, st>>>(y, t, dy, scratch, n);
  sum_partials_kernel<<<1, 32, 0, st>>>(scratch, nb, n, loss);
  return int(cudaGetLastError());
}

int fwant_nn_adam(float* w, uint16_t* w16, const float* g, float* m, float* v, long long n, float lr, float b1,
                  float b2, float eps, float wd, int t, void* stream) {
  if (t < 1) return int(cudaErrorInvalidValue);
  const float c1 = 1.0f - powf(b1, float(t)), c2 = 1.0f - powf(b2, float(t));
  adam_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(w, w16, g, m, v, n, lr, b1, b2, eps, wd, c1, c2);
  return int(cudaGetLastError());
}

int fwant_nn_to_bf16(const float* w, uint16_t* w16, long long n, void* stream) {
  to_bf16_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(w, w16, n);
  return int(cudaGetLastError());
}

int fwant_nn_basis_fwd(const float* coef, const float* basis, float* out, int B, int G, int K, int T, void* stream) {
  basis_fwd_kernel<<<grid_for((long long)B * G * T, 256), 256, 0, (cudaStream_t)stream>>>(coef, basis, out, B, G, K, T);
  return int(cudaGetLastError());
}

int fwant_nn_basis_bwd(const float* dout, const float* basis, float* dcoef, int B, int G, int K, int T, void* stream) {
  basis_bwd_kernel<<<grid_for((long long)B * G * K, 256), 256, 0, (cudaStream_t)stream>>>(dout, basis, dcoef, B, G, K,
                                                                                        T);
  return int(cudaGetLastError());
}

int fwant_nn_axpby(const float* a, const float* b, float s, float* y, long long n, void* stream) {
  axpby_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(a, b, s, y, n);
  return int(cudaGetLastError());
}

}  // extern "C"
