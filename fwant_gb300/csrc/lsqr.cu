// LSQR on the GPU (inv.LSQR/mod_LSQR.f90: lsqr_init / lldrow :44-135, slsqr :137-268,
// lgtsol :270-285, lnrliz / lupdat / dotp / lax / laty :287-413).
//
// Layout in HBM: A in compressed rows (row offsets int64, columns int32, values FP64) and
// the same entries in compressed columns (built once on the host, rows ascending within a
// column), so both products are gathers: A v over rows, A^T u over columns, with the rows
// (columns) split by length into four classes handled one thread, eight lanes, a warp or a
// block per row, each summing its entries in a fixed order.  Vectors u (nrow) and v, w, x, sig
// (ncol) are FP64.
//
// One iteration is seven launches: rows (u = A v - alpha u, partial |u|^2), normalise u
// (beta), columns (v = A^T u - beta v, partial |v|^2), normalise v (alpha), the scalar
// recurrences (rho, c, s, theta, rhobar, phi, phibar; one thread), the vector update
// (x, w, sig; partial |x|^2) and the convergence test (test1, test2, iteration count,
// done flag).  Norms are sums of per-block partial sums in a fixed order, so results do not
// depend on the GPU's scheduling.  The scalars live in device memory; iterations run as a
// CUDA graph of ITERS_PER_GRAPH iterations whose kernels return at once when the done flag
// is set, and the host reads the flag once per replay.
//
// Roofline: HBM.  Per iteration both products read 12 B per entry (value + column or row
// index) plus the vectors (gathered from L2 for vectors that fit it): 24 B per stored entry.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fwant_lsqr.h"

namespace {

constexpr int LS_THREADS = 256;
constexpr int LS_WARPS = LS_THREADS / 32;
constexpr int ITERS_PER_GRAPH = 32;
// Blocks of every grid-stride launch = number of partial sums: fixed (8 blocks of 256
// threads on each of 152 SMs fill a GB300 once), so the summation order, and with it every
// result, is the same on any device.
constexpr int LS_BLOCKS = 1216;
constexpr double CONS_EQ = 1.0e-20;  // lnrliz leaves a vector of norm <= CONS_EQ unscaled

struct Scal {
  double alpha, beta, phibar, rhobar, anorm;
  double rho, c, s, theta, phi;
  double test1, test2, res2, xnorm;
  double atol, btol;
  long long itct, maxit;
  int done;  // 0 running; 1 converged or maxit (res2 set); 2 rho == 0 (returned early)
};

// Sum over the block; the result is valid in thread 0.  Fixed order: shuffle tree within
// each warp, then warp 0 adds the warps' sums in warp order.
__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < LS_WARPS; ++q) t += sh[q];
  __syncthreads();
  return t;
}

// Compressed rows (or columns) with their rows split by length into four classes, each a
// list of row numbers: short rows (<= SHORT_ROW_MAX entries) one thread per row, medium
// rows eight lanes per row, long rows (>= LONG_ROW_MIN) a warp per row, very long rows
// (>= BLOCK_ROW_MIN) a whole block per row; every lane keeps four independent accumulators.
// Row lengths of an inversion system are bimodal (measurement rows with thousands of kernel
// entries, damping and smoothing rows with one or two).  GB300 issues FP64 at a rate close
// to its HBM rate for this product (one FMA per 12-byte entry), so the classes keep the
// reduction's extra FP64 adds per row small against the row's FMAs: eight lanes up to 64
// entries a lane, and a block per row only where a warp per row would leave the GPU with
// fewer rows than warps.
constexpr int SHORT_ROW_MAX = 4;
constexpr int LONG_ROW_MIN = 512;
constexpr int BLOCK_ROW_MIN = 4096;
constexpr int NCLS = 4;

struct Sparse {
  const long long* ptr;
  const int* idx;
  const double* val;
  const int* cls[NCLS];  // row numbers of the short, medium, long and very long classes
  long long ncls[NCLS];
};

// y = sum over row r's entries of val * in[idx] by W lanes (lane `sub` of the group takes
// entries sub, sub + W, ...), combined in a fixed order.  IT: entry-offset type, 32-bit
// when every offset fits (fewer 64-bit integer instructions in the loop), else 64-bit.
template <int W, typename IT>
__device__ __forceinline__ double row_dot(const Sparse& A, int r, int sub, const double* __restrict__ in) {
  const IT e0 = IT(A.ptr[r]), e1 = IT(A.ptr[r + 1]);
  double y0 = 0.0, y1 = 0.0, y2 = 0.0, y3 = 0.0;
  IT e = e0 + sub;
  // two groups of four loaded before either is summed (more loads in flight); each
  // accumulator still takes its entries in the same order as one group at a time
  for (; e + 7 * W < e1; e += 8 * W) {
    double a[8], x[8];
    int c[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      a[q] = A.val[e + q * W];
      c[q] = A.idx[e + q * W];
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = in[c[q]];
    y0 = fma(a[0], x[0], y0);
    y1 = fma(a[1], x[1], y1);
    y2 = fma(a[2], x[2], y2);
    y3 = fma(a[3], x[3], y3);
    y0 = fma(a[4], x[4], y0);
    y1 = fma(a[5], x[5], y1);
    y2 = fma(a[6], x[6], y2);
    y3 = fma(a[7], x[7], y3);
  }
  for (; e + 3 * W < e1; e += 4 * W) {
    y0 = fma(A.val[e], in[A.idx[e]], y0);
    y1 = fma(A.val[e + W], in[A.idx[e + W]], y1);
    y2 = fma(A.val[e + 2 * W], in[A.idx[e + 2 * W]], y2);
    y3 = fma(A.val[e + 3 * W], in[A.idx[e + 3 * W]], y3);
  }
  for (; e < e1; e += W) y0 = fma(A.val[e], in[A.idx[e]], y0);
  return (y0 + y1) + (y2 + y3);
}

// One length class: groups of W lanes take the class's rows grid-stride; the group's first
// lane writes out[r] (y, or y - out[r] * factor) and adds out[r]^2 to sq.
template <int W, typename IT>
__device__ __forceinline__ void gather_class(const Sparse& A, int c, const double* __restrict__ in,
                                             double* __restrict__ out, double factor, bool subtract, double& sq) {
  const long long tid = (long long)blockIdx.x * LS_THREADS + threadIdx.x;
  const long long groups = (long long)gridDim.x * (LS_THREADS / W);
  const int sub = threadIdx.x % W;
  const int lane = threadIdx.x & 31;
  const unsigned mask = W == 32 ? 0xffffffffu : (((1u << W) - 1u) << (lane & ~(W - 1)));
  for (long long g = tid / W; g < A.ncls[c]; g += groups) {
    const int r = A.cls[c][g];
    double y = row_dot<W, IT>(A, r, sub, in);
    if (W > 1)
      for (int o = W / 2; o > 0; o >>= 1) y += __shfl_down_sync(mask, y, o, W);
    if (sub == 0) {
      const double o = subtract ? __dsub_rn(y, __dmul_rn(out[r], factor)) : y;
      out[r] = o;
      sq = fma(o, o, sq);
    }
  }
}

// out[r] = (A in)[r] for every row r, then out[r] = y - out[r] * factor (which 0: alpha,
// u = A v - alpha u; which 1: beta, v = A^T u - beta v; which 2: out = A in), and the
// block's sum of out[r]^2 into partial[blockIdx.x].
template <typename IT>
__global__ void __launch_bounds__(LS_THREADS) gather_kernel(const Sparse A, const double* __restrict__ in,
                                                            double* __restrict__ out, const Scal* __restrict__ S,
                                                            int which, int check_done, double* __restrict__ partial) {
  __shared__ double sh[LS_WARPS];
  if (check_done && S->done) return;
  const double factor = which == 0 ? S->alpha : which == 1 ? S->beta : 0.0;
  const bool subtract = which != 2;
  double sq = 0.0;
  // very long rows: a block per row (the loop is uniform over the block)
  for (long long g = blockIdx.x; g < A.ncls[3]; g += gridDim.x) {
    const int r = A.cls[3][g];
    const double y = block_sum(row_dot<LS_THREADS, IT>(A, r, threadIdx.x, in), sh);
    if (threadIdx.x == 0) {
      const double o = subtract ? __dsub_rn(y, __dmul_rn(out[r], factor)) : y;
      out[r] = o;
      sq = fma(o, o, sq);
    }
  }
  gather_class<32, IT>(A, 2, in, out, factor, subtract, sq);
  gather_class<8, IT>(A, 1, in, out, factor, subtract, sq);
  gather_class<1, IT>(A, 0, in, out, factor, subtract, sq);
  const double t = block_sum(sq, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// entry offsets up to this bound run the 32-bit form (e + 4 W stays below 2^31)
constexpr long long I32_NNZ_MAX = 0x7fffffffLL - 8 * LS_THREADS;

void launch_gather(const Sparse& A, long long nnz, const double* in, double* out, const Scal* S, int which,
                   int check_done, double* partial, int nblk, cudaStream_t st) {
  if (nnz <= I32_NNZ_MAX)
    gather_kernel<int><<<nblk, LS_THREADS, 0, st>>>(A, in, out, S, which, check_done, partial);
  else
    gather_kernel<long long><<<nblk, LS_THREADS, 0, st>>>(A, in, out, S, which, check_done, partial);
}

// lnrliz: norm = sqrt(sum of the partials) (every block sums them in the same order), the
// vector divided by it unless it is <= CONS_EQ; block 0 stores it as beta (which 0) or
// alpha (which 1).
__global__ void __launch_bounds__(LS_THREADS) normalise_kernel(double* __restrict__ vec, long long n,
                                                               const double* __restrict__ partial, int npart,
                                                               Scal* __restrict__ S, int which, int check_done) {
  __shared__ double sh[LS_WARPS];
  __shared__ double nrm_s;
  if (check_done && S->done) return;
  double t = 0.0;
  for (int i = threadIdx.x; i < npart; i += LS_THREADS) t += partial[i];
  t = block_sum(t, sh);
  if (threadIdx.x == 0) nrm_s = sqrt(t);
  __syncthreads();
  const double nrm = nrm_s;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (which == 0) S->beta = nrm;
    else S->alpha = nrm;
  }
  if (fabs(nrm) <= CONS_EQ) return;
  for (long long i = (long long)blockIdx.x * LS_THREADS + threadIdx.x; i < n; i += (long long)gridDim.x * LS_THREADS)
    vec[i] = vec[i] / nrm;
}

// steps (a)-(g) of Paige and Saunders (slsqr :196-205)
__global__ void scalar_kernel(Scal* S) {
  if (S->done) return;
  const double rho = sqrt(__dadd_rn(__dmul_rn(S->rhobar, S->rhobar), __dmul_rn(S->beta, S->beta)));
  S->rho = rho;
  if (rho == 0.0) {
    S->done = 2;
    return;
  }
  const double c = S->rhobar / rho, s = S->beta / rho;
  S->c = c;
  S->s = s;
  S->theta = __dmul_rn(s, S->alpha);
  S->rhobar = -__dmul_rn(c, S->alpha);
  S->phi = __dmul_rn(c, S->phibar);
  S->phibar = __dmul_rn(s, S->phibar);
}

// x += phi w / rho; w = v - theta w / rho; sig += (w / rho)^2 (slsqr :207-212)
__global__ void __launch_bounds__(LS_THREADS) update_kernel(double* __restrict__ x, double* __restrict__ w,
                                                            const double* __restrict__ v, double* __restrict__ sig,
                                                            long long n, const Scal* __restrict__ S,
                                                            double* __restrict__ partial) {
  __shared__ double sh[LS_WARPS];
  if (S->done) return;
  const double rho = S->rho, phi = S->phi, theta = S->theta;
  double sq = 0.0;
  for (long long i = (long long)blockIdx.x * LS_THREADS + threadIdx.x; i < n; i += (long long)gridDim.x * LS_THREADS) {
    const double temp = w[i] / rho;
    const double xi = __dadd_rn(x[i], __dmul_rn(phi, temp));
    x[i] = xi;
    w[i] = __dsub_rn(v[i], __dmul_rn(theta, temp));
    sig[i] = __dadd_rn(sig[i], __dmul_rn(temp, temp));
    sq = fma(xi, xi, sq);
  }
  const double t = block_sum(sq, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// convergence test (slsqr :221-250)
__global__ void __launch_bounds__(LS_THREADS) finish_kernel(Scal* __restrict__ S, const double* __restrict__ partial,
                                                            int npart) {
  __shared__ double sh[LS_WARPS];
  if (S->done) return;
  double t = 0.0;
  for (int i = threadIdx.x; i < npart; i += LS_THREADS) t += partial[i];
  t = block_sum(t, sh);
  if (threadIdx.x != 0) return;
  const double xnorm = sqrt(t);
  const double rnorm = S->phibar;
  S->xnorm = xnorm;
  S->test1 = rnorm / S->anorm / xnorm;
  S->test2 = __dmul_rn(S->alpha, fabs(S->c)) / S->anorm;
  S->itct += 1;
  if (S->test1 <= S->atol || S->test2 <= S->btol || S->itct == S->maxit) {
    S->res2 = S->phibar;
    S->done = 1;
  }
}

// sum of val^2 over all entries into per-block partials (|A|_F)
__global__ void __launch_bounds__(LS_THREADS) sumsq_kernel(const double* __restrict__ val, long long n,
                                                           double* __restrict__ partial) {
  __shared__ double sh[LS_WARPS];
  double sq = 0.0;
  for (long long i = (long long)blockIdx.x * LS_THREADS + threadIdx.x; i < n; i += (long long)gridDim.x * LS_THREADS)
    sq = fma(val[i], val[i], sq);
  const double t = block_sum(sq, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void __launch_bounds__(LS_THREADS) anorm_kernel(Scal* __restrict__ S, const double* __restrict__ partial,
                                                           int npart) {
  __shared__ double sh[LS_WARPS];
  double t = 0.0;
  for (int i = threadIdx.x; i < npart; i += LS_THREADS) t += partial[i];
  t = block_sum(t, sh);
  if (threadIdx.x == 0) S->anorm = sqrt(t);
}

// start of slsqr (:160-190) after u = b: w = v, x = sig = 0, phibar = beta, rhobar = alpha
__global__ void start_kernel(double* __restrict__ w, const double* __restrict__ v, double* __restrict__ x,
                             double* __restrict__ sig, long long n, Scal* __restrict__ S) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    w[i] = v[i];
    x[i] = 0.0;
    sig[i] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S->phibar = S->beta;
    S->rhobar = S->alpha;
  }
}

}  // namespace

struct fwant_lsqr {
  int device = 0;
  int nblk = 0;  // blocks of every grid-stride launch (= number of partial sums): LS_BLOCKS
  cudaStream_t st = nullptr;
  long long nrow = 0, ncol = 0, nnz = 0;
  long long *rp = nullptr, *cp = nullptr;
  int *ci = nullptr, *ri = nullptr;
  int* cls_rows = nullptr;  // row numbers by length class (short, medium, long), concatenated
  int* cls_cols = nullptr;  // column numbers likewise
  Sparse A{}, At{};         // the two layouts with their class lists
  double *va = nullptr, *vt = nullptr;
  double *b = nullptr, *u = nullptr, *v = nullptr, *w = nullptr, *x = nullptr, *sig = nullptr, *partial = nullptr;
  double* tmp = nullptr;  // ncol scratch (multiply)
  Scal* S = nullptr;
  Scal* hS = nullptr;     // pinned
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  bool solved = false;
  std::string err;

  ~fwant_lsqr() {
    cudaSetDevice(device);
    if (graph) cudaGraphExecDestroy(graph);
    for (void* p : {(void*)rp, (void*)cp, (void*)ci, (void*)ri, (void*)va, (void*)vt, (void*)b, (void*)u, (void*)v,
                    (void*)w, (void*)x, (void*)sig, (void*)partial, (void*)tmp, (void*)S, (void*)cls_rows,
                    (void*)cls_cols})
      cudaFree(p);
    if (hS) cudaFreeHost(hS);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
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
  template <class T>
  fwant_status alloc(T** p, size_t n, const char* what) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return fail(FWANT_ERR_OOM, std::string("out of device memory: ") + what);
    }
    *p = static_cast<T*>(q);
    return FWANT_OK;
  }
  // one LSQR iteration (slsqr's loop body)
  void enqueue_iteration() {
    launch_gather(A, nnz, v, u, S, 0, 1, partial, nblk, st);
    normalise_kernel<<<nblk, LS_THREADS, 0, st>>>(u, nrow, partial, nblk, S, 0, 1);
    launch_gather(At, nnz, u, v, S, 1, 1, partial, nblk, st);
    normalise_kernel<<<nblk, LS_THREADS, 0, st>>>(v, ncol, partial, nblk, S, 1, 1);
    scalar_kernel<<<1, 1, 0, st>>>(S);
    update_kernel<<<nblk, LS_THREADS, 0, st>>>(x, w, v, sig, ncol, S, partial);
    finish_kernel<<<1, LS_THREADS, 0, st>>>(S, partial, nblk);
  }
};

extern "C" {

fwant_status fwant_lsqr_create(long long nrow, long long ncol, const long long* row_ptr, const int* col,
                               const double* val, const double* rhs, int device, fwant_lsqr** out) {
  if (!out) return FWANT_ERR_INVALID_ARG;
  *out = nullptr;
  if (nrow < 1 || ncol < 1 || ncol > 0x7fffffffLL || nrow > 0x7fffffffLL || !row_ptr || !rhs)
    return FWANT_ERR_INVALID_ARG;
  if (row_ptr[0] != 0) return FWANT_ERR_INVALID_ARG;
  for (long long r = 0; r < nrow; ++r)
    if (row_ptr[r + 1] < row_ptr[r]) return FWANT_ERR_INVALID_ARG;
  const long long nnz = row_ptr[nrow];
  if (nnz > 0 && (!col || !val)) return FWANT_ERR_INVALID_ARG;
  // host work in T threads, each over a contiguous range of rows holding about nnz / T
  // entries (the column check, then the counting sort into compressed columns)
  const int T = int(std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
  std::vector<long long> rb(size_t(T) + 1, nrow);
  rb[0] = 0;
  for (int t = 1; t < T; ++t)
    rb[size_t(t)] = std::lower_bound(row_ptr, row_ptr + nrow + 1, nnz / T * t) - row_ptr;
  auto parallel = [T](const std::function<void(int)>& body) {
    std::vector<std::thread> th;
    for (int t = 1; t < T; ++t) th.emplace_back(body, t);
    body(0);
    for (auto& x : th) x.join();
  };
  {
    std::vector<char> bad_col(size_t(T), 0);
    parallel([&](int t) {
      for (long long e = row_ptr[rb[size_t(t)]]; e < row_ptr[rb[size_t(t) + 1]]; ++e)
        if (col[e] < 0 || col[e] >= ncol) bad_col[size_t(t)] = 1;
    });
    for (char b : bad_col)
      if (b) return FWANT_ERR_INVALID_ARG;
  }
  auto* l = new fwant_lsqr();
  l->device = device;
  l->nrow = nrow;
  l->ncol = ncol;
  l->nnz = nnz;
  auto bad = [&](fwant_status rc) {
    delete l;
    return rc;
  };
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return bad(FWANT_ERR_CUDA);
  }
  l->nblk = LS_BLOCKS;
  // compressed columns: counting sort by column.  Thread t counts its rows' entries per
  // column; a column's entries from thread t follow those of threads 0..t-1, so rows stay
  // ascending within every column, whatever the thread count.
  std::vector<long long> cp(size_t(ncol) + 1, 0);
  std::vector<std::vector<long long>> pos(static_cast<size_t>(T));
  parallel([&](int t) {
    std::vector<long long>& c = pos[size_t(t)];
    c.assign(size_t(ncol), 0);
    for (long long e = row_ptr[rb[size_t(t)]]; e < row_ptr[rb[size_t(t) + 1]]; ++e) ++c[size_t(col[e])];
  });
  for (long long j = 0; j < ncol; ++j) {
    long long acc = cp[size_t(j)];
    for (int t = 0; t < T; ++t) {
      const long long c = pos[size_t(t)][size_t(j)];
      pos[size_t(t)][size_t(j)] = acc;
      acc += c;
    }
    cp[size_t(j) + 1] = acc;
  }
  std::unique_ptr<int[]> ri(new int[size_t(std::max(nnz, 1LL))]);
  std::unique_ptr<double[]> vt(new double[size_t(std::max(nnz, 1LL))]);
  parallel([&](int t) {
    std::vector<long long>& c = pos[size_t(t)];
    for (long long r = rb[size_t(t)]; r < rb[size_t(t) + 1]; ++r)
      for (long long e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
        const long long p = c[size_t(col[e])]++;
        ri[size_t(p)] = int(r);
        vt[size_t(p)] = val[e];
      }
  });
  pos.clear();
  // length classes of the rows and of the columns, each list ascending
  auto classes = [](const long long* ptr, long long n, std::vector<int>& lst, long long cnt[NCLS]) {
    lst.clear();
    for (int c = 0; c < NCLS; ++c) {
      cnt[c] = 0;
      for (long long r = 0; r < n; ++r) {
        const long long len = ptr[r + 1] - ptr[r];
        const int k = len <= SHORT_ROW_MAX ? 0 : len < LONG_ROW_MIN ? 1 : len < BLOCK_ROW_MIN ? 2 : 3;
        if (k == c) {
          lst.push_back(int(r));
          ++cnt[c];
        }
      }
    }
  };
  std::vector<int> rows_cls, cols_cls;
  long long nrc[NCLS], ncc[NCLS];
  classes(row_ptr, nrow, rows_cls, nrc);
  classes(cp.data(), ncol, cols_cls, ncc);
  fwant_status rc = FWANT_OK;
  const size_t nr = size_t(nrow), nc = size_t(ncol), ne = size_t(nnz);
  if ((rc = l->alloc(&l->rp, nr + 1, "row offsets")) || (rc = l->alloc(&l->cp, nc + 1, "column offsets")) ||
      (rc = l->alloc(&l->ci, ne, "columns")) || (rc = l->alloc(&l->ri, ne, "rows")) ||
      (rc = l->alloc(&l->va, ne, "values")) || (rc = l->alloc(&l->vt, ne, "transposed values")) ||
      (rc = l->alloc(&l->b, nr, "b")) || (rc = l->alloc(&l->u, nr, "u")) || (rc = l->alloc(&l->v, nc, "v")) ||
      (rc = l->alloc(&l->w, nc, "w")) || (rc = l->alloc(&l->x, nc, "x")) || (rc = l->alloc(&l->sig, nc, "sig")) ||
      (rc = l->alloc(&l->tmp, nc, "scratch")) || (rc = l->alloc(&l->partial, size_t(l->nblk), "partial sums")) ||
      (rc = l->alloc(&l->S, 1, "scalars")) || (rc = l->alloc(&l->cls_rows, nr, "row classes")) ||
      (rc = l->alloc(&l->cls_cols, nc, "column classes"))) {
    const std::string m = l->err;
    delete l;
    (void)m;
    return rc;
  }
  cudaError_t e = cudaMallocHost(&l->hS, sizeof(Scal));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&l->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&l->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&l->ev1);
  if (e == cudaSuccess) e = cudaMemcpy(l->rp, row_ptr, (nr + 1) * sizeof(long long), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(l->cp, cp.data(), (nc + 1) * sizeof(long long), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ne) e = cudaMemcpy(l->ci, col, ne * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ne) e = cudaMemcpy(l->va, val, ne * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ne) e = cudaMemcpy(l->ri, ri.get(), ne * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ne) e = cudaMemcpy(l->vt, vt.get(), ne * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(l->b, rhs, nr * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(l->cls_rows, rows_cls.data(), nr * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(l->cls_cols, cols_cls.data(), nc * sizeof(int), cudaMemcpyHostToDevice);
  {
    l->A = Sparse{l->rp, l->ci, l->va, {}, {}};
    l->At = Sparse{l->cp, l->ri, l->vt, {}, {}};
    long long ro = 0, co = 0;
    for (int c = 0; c < NCLS; ++c) {
      l->A.cls[c] = l->cls_rows + ro;
      l->A.ncls[c] = nrc[c];
      ro += nrc[c];
      l->At.cls[c] = l->cls_cols + co;
      l->At.ncls[c] = ncc[c];
      co += ncc[c];
    }
  }
  if (e == cudaSuccess) {
    // |A|_F once (slsqr :157-158)
    Scal s0{};
    e = cudaMemcpy(l->S, &s0, sizeof(Scal), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      sumsq_kernel<<<l->nblk, LS_THREADS, 0, l->st>>>(l->va, nnz, l->partial);
      anorm_kernel<<<1, LS_THREADS, 0, l->st>>>(l->S, l->partial, l->nblk);
      e = cudaStreamSynchronize(l->st);
      if (e == cudaSuccess) e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete l;
    return FWANT_ERR_CUDA;
  }
  *out = l;
  return FWANT_OK;
}

void fwant_lsqr_destroy(fwant_lsqr* l) { delete l; }

const char* fwant_lsqr_last_error(fwant_lsqr* l) { return l ? l->err.c_str() : "null handle"; }

fwant_status fwant_lsqr_solve(fwant_lsqr* l, double atol, double btol, long long maxit, long long* itct) {
  if (!l) return FWANT_ERR_INVALID_ARG;
  if (maxit < 1) return l->fail(FWANT_ERR_INVALID_ARG, "lsqr_solve: maxit must be >= 1");
  cudaSetDevice(l->device);
  l->solved = false;
  // state of the start of slsqr, keeping |A|_F
  cudaError_t e = cudaMemcpy(l->hS, l->S, sizeof(Scal), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_solve");
  Scal s0{};
  s0.anorm = l->hS->anorm;
  s0.atol = atol;
  s0.btol = btol;
  s0.maxit = maxit;
  e = cudaMemcpyAsync(l->S, &s0, sizeof(Scal), cudaMemcpyHostToDevice, l->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(l->u, l->b, size_t(l->nrow) * sizeof(double), cudaMemcpyDeviceToDevice, l->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(l->v, 0, size_t(l->ncol) * sizeof(double), l->st);
  if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_solve");
  cudaEventRecord(l->ev0, l->st);
  // u = b / |b|; v = A^T u / |A^T u|; w = v; x = sig = 0
  const int nb = l->nblk;
  sumsq_kernel<<<nb, LS_THREADS, 0, l->st>>>(l->u, l->nrow, l->partial);
  normalise_kernel<<<nb, LS_THREADS, 0, l->st>>>(l->u, l->nrow, l->partial, nb, l->S, 0, 0);
  launch_gather(l->At, l->nnz, l->u, l->v, l->S, 2, 0, l->partial, nb, l->st);
  normalise_kernel<<<nb, LS_THREADS, 0, l->st>>>(l->v, l->ncol, l->partial, nb, l->S, 1, 0);
  start_kernel<<<nb, LS_THREADS, 0, l->st>>>(l->w, l->v, l->x, l->sig, l->ncol, l->S);
  e = cudaGetLastError();
  if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_solve start");
  if (!l->graph) {
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(l->st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      for (int i = 0; i < ITERS_PER_GRAPH; ++i) l->enqueue_iteration();
      e = cudaStreamEndCapture(l->st, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&l->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_solve graph");
  }
  // replay until the done flag is set; the flag is read once per replay
  const long long max_replays = maxit / ITERS_PER_GRAPH + 2;
  for (long long rep = 0;; ++rep) {
    e = cudaGraphLaunch(l->graph, l->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(l->hS, l->S, sizeof(Scal), cudaMemcpyDeviceToHost, l->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(l->st);
    if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_solve");
    if (l->hS->done) break;
    if (rep >= max_replays) return l->fail(FWANT_ERR_STATE, "lsqr_solve: iteration count passed maxit");
  }
  cudaEventRecord(l->ev1, l->st);
  cudaEventSynchronize(l->ev1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, l->ev0, l->ev1);
  l->last_ms = ms;
  l->solved = true;
  if (itct) *itct = l->hS->itct;
  return FWANT_OK;
}

fwant_status fwant_lsqr_solution(fwant_lsqr* l, long long nvar, double* x, double* serr) {
  if (!l || !x || !serr) return FWANT_ERR_INVALID_ARG;
  if (!l->solved) return l->fail(FWANT_ERR_STATE, "lsqr_solution: no solve yet");
  if (nvar < 1 || nvar > l->ncol) return l->fail(FWANT_ERR_INVALID_ARG, "lsqr_solution: nvar outside 1..ncol");
  cudaSetDevice(l->device);
  std::vector<double> sig(static_cast<size_t>(nvar));
  cudaError_t e = cudaMemcpy(x, l->x, size_t(nvar) * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sig.data(), l->sig, size_t(nvar) * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_solution");
  const double temp = l->hS->res2 / double(std::max(l->nrow - nvar, 1LL));
  for (long long i = 0; i < nvar; ++i) serr[i] = std::sqrt(temp * sig[size_t(i)]);
  return FWANT_OK;
}

fwant_status fwant_lsqr_info(fwant_lsqr* l, double* info) {
  if (!l || !info) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(l->device);
  cudaError_t e = cudaMemcpy(l->hS, l->S, sizeof(Scal), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_info");
  const Scal& s = *l->hS;
  const double v[6] = {s.anorm, s.res2, s.test1, s.test2, s.phibar, s.xnorm};
  std::memcpy(info, v, sizeof(v));
  return FWANT_OK;
}

fwant_status fwant_lsqr_multiply(fwant_lsqr* l, const double* x, double* y) {
  if (!l || !x || !y) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(l->device);
  double* yd = nullptr;
  fwant_status rc = l->alloc(&yd, size_t(l->nrow), "product");
  if (rc != FWANT_OK) return rc;
  cudaError_t e = cudaMemcpyAsync(l->tmp, x, size_t(l->ncol) * sizeof(double), cudaMemcpyHostToDevice, l->st);
  if (e == cudaSuccess) {
    launch_gather(l->A, l->nnz, l->tmp, yd, l->S, 2, 0, l->partial, l->nblk, l->st);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, yd, size_t(l->nrow) * sizeof(double), cudaMemcpyDeviceToHost, l->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(l->st);
  cudaFree(yd);
  if (e != cudaSuccess) return l->cuda_fail(e, "lsqr_multiply");
  return FWANT_OK;
}

fwant_status fwant_lsqr_last_solve_ms(fwant_lsqr* l, double* ms) {
  if (!l || !ms) return FWANT_ERR_INVALID_ARG;
  *ms = l->last_ms;
  return FWANT_OK;
}

}  // extern "C"
