// Host side of the sensitivity-kernel accumulation: one fwant_sgtker holds the strain
// Green's tensors of one block of kernel points (the receiver station's X/Y/Z force
// simulations and the source station's simulation, as the sgt_ snapshot files that
// SI_ker_sta.F90 reads at :411-622), the media of those points, the scattering series
// and the window kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/fwant_gb300.h"
#include "kernels.h"

namespace fw {
int solver_sgt_view(fwant_solver* s, const float** data, long long* npts, int* max_frames, int* nframes,
                    int* device);
}

struct fwant_sgtker {
  long long npts = 0;
  int knt = 0;
  double kdt = 0.0;
  int device = 0;
  cudaStream_t st = nullptr;
  float* lam = nullptr;
  float* mu = nullptr;
  float* sgt[4] = {nullptr, nullptr, nullptr, nullptr};  // X, Y, Z receiver SGT; source SGT
  double* series = nullptr;                              // [6][knt][npts]
  int scatter_nt1 = 0, scatter_nt2 = 0, scatter_flags = 0;
  int param = 0;                                         // 0 Vp/Vs, 1 lambda/mu kernels
  double* wts = nullptr;                                 // wv[knt], wu[knt]
  double* kout = nullptr;                                // 4 x [npts]
  double* filtered = nullptr;                            // 2 x [knt][npts]: filtered Ka, Kb
  double* iir_scratch = nullptr;                         // [knt + 6 nod][npts]
  size_t iir_scratch_len = 0;
  float* pstrain = nullptr;                              // SI_ker_pair strains [14][knt][npts]
  float* pvu = nullptr;                                  // SI_ker_pair V, U [2][knt]
  bool pair_done = false;                                // series slots 0, 1 hold the pair's Sa, Sb
  bool have_media = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  std::string err;

  ~fwant_sgtker() {
    cudaSetDevice(device);
    cudaFree(lam); cudaFree(mu);
    for (float* p : sgt) cudaFree(p);
    cudaFree(series); cudaFree(wts); cudaFree(kout); cudaFree(filtered); cudaFree(iir_scratch);
    cudaFree(pstrain); cudaFree(pvu);
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
  size_t series_len() const { return size_t(knt) * size_t(npts); }
  template <class T>
  fwant_status alloc(T** p, size_t n, const char* what) {
    if (*p) return FWANT_OK;
    void* q = nullptr;
    if (cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return fail(FWANT_ERR_OOM, std::string("out of device memory: ") + what);
    }
    *p = static_cast<T*>(q);
    return FWANT_OK;
  }
};

extern "C" {

fwant_status fwant_sgtker_create(long long npts, int knt, double kdt, int device, fwant_sgtker** out) {
  if (!out) return FWANT_ERR_INVALID_ARG;
  *out = nullptr;
  if (npts < 1 || npts > 0x7fffffffLL || knt < 2 || !(kdt > 0.0)) return FWANT_ERR_INVALID_ARG;
  auto* k = new fwant_sgtker();
  k->npts = npts;
  k->knt = knt;
  k->kdt = kdt;
  k->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&k->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&k->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&k->ev1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete k;
    return FWANT_ERR_CUDA;
  }
  *out = k;
  return FWANT_OK;
}

void fwant_sgtker_destroy(fwant_sgtker* k) { delete k; }

const char* fwant_sgtker_last_error(fwant_sgtker* k) { return k ? k->err.c_str() : "null handle"; }

fwant_status fwant_sgtker_set_media(fwant_sgtker* k, const float* lam, const float* mu) {
  if (!k || !lam || !mu) return FWANT_ERR_INVALID_ARG;
  for (long long p = 0; p < k->npts; ++p)
    if (!(mu[p] > 0.0f) || !(lam[p] + mu[p] > 0.0f))
      return k->fail(FWANT_ERR_INVALID_ARG, "sgtker media: mu must be > 0 at every kernel point (stress2strain)");
  cudaSetDevice(k->device);
  fwant_status rc;
  if ((rc = k->alloc(&k->lam, size_t(k->npts), "lambda")) != FWANT_OK) return rc;
  if ((rc = k->alloc(&k->mu, size_t(k->npts), "mu")) != FWANT_OK) return rc;
  cudaError_t e = cudaMemcpy(k->lam, lam, size_t(k->npts) * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(k->mu, mu, size_t(k->npts) * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_set_media");
  k->have_media = true;
  return FWANT_OK;
}

fwant_status fwant_sgtker_set_sgt(fwant_sgtker* k, int which, const float* stress) {
  if (!k || !stress || which < 0 || which > 3) return FWANT_ERR_INVALID_ARG;
  cudaSetDevice(k->device);
  fwant_status rc = k->alloc(&k->sgt[which], 6 * k->series_len(), "sgt");
  if (rc != FWANT_OK) return rc;
  cudaError_t e = cudaMemcpy(k->sgt[which], stress, 6 * k->series_len() * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_set_sgt");
  return FWANT_OK;
}

fwant_status fwant_sgtker_take_sgt(fwant_sgtker* k, int which, fwant_solver* s) {
  if (!k || !s || which < 0 || which > 3) return FWANT_ERR_INVALID_ARG;
  const float* src = nullptr;
  long long npts = 0;
  int maxf = 0, nf = 0, dev = -1;
  if (fw::solver_sgt_view(s, &src, &npts, &maxf, &nf, &dev))
    return k->fail(FWANT_ERR_STATE, "sgtker_take_sgt: the solver records no SGT");
  if (dev != k->device) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_take_sgt: solver on another device");
  if (npts != k->npts) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_take_sgt: point count differs");
  if (nf < k->knt) {
    char b[128];
    std::snprintf(b, sizeof(b), "sgtker_take_sgt: the solver has recorded %d frames, %d needed", nf, k->knt);
    return k->fail(FWANT_ERR_STATE, b);
  }
  cudaSetDevice(k->device);
  fwant_status rc = k->alloc(&k->sgt[which], 6 * k->series_len(), "sgt");
  if (rc != FWANT_OK) return rc;
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < 6 && e == cudaSuccess; ++c)
    e = cudaMemcpyAsync(k->sgt[which] + size_t(c) * k->series_len(), src + size_t(c) * size_t(maxf) * size_t(npts),
                        k->series_len() * sizeof(float), cudaMemcpyDeviceToDevice, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_take_sgt");
  return FWANT_OK;
}

fwant_status fwant_sgtker_set_param(fwant_sgtker* k, int param) {
  if (!k) return FWANT_ERR_INVALID_ARG;
  if (param != 0 && param != 1) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_set_param: param must be 0 or 1");
  k->param = param;
  return FWANT_OK;
}

fwant_status fwant_sgtker_scatter(fwant_sgtker* k, int flags, int nt1, int nt2) {
  if (!k) return FWANT_ERR_INVALID_ARG;
  if ((flags & 7) == 0 || (flags & ~7)) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_scatter: flags must be 1..7");
  if (nt1 < 1 || nt2 > k->knt || nt1 > nt2) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_scatter: bad nt1/nt2");
  if (!k->have_media) return k->fail(FWANT_ERR_STATE, "sgtker_scatter: media not set");
  if (!k->sgt[3]) return k->fail(FWANT_ERR_STATE, "sgtker_scatter: source SGT not set");
  for (int c = 0; c < 3; ++c)
    if ((flags >> c & 1) && !k->sgt[c]) return k->fail(FWANT_ERR_STATE, "sgtker_scatter: receiver SGT not set");
  cudaSetDevice(k->device);
  fwant_status rc = k->alloc(&k->series, 6 * k->series_len(), "scatter series");
  if (rc != FWANT_OK) return rc;
  k->pair_done = false;
  k->scatter_flags = 0;  // until this scatter completes
  cudaMemsetAsync(k->series, 0, 6 * k->series_len() * sizeof(double), k->st);
  fw::ScatterArgs a{};
  a.npts = k->npts;
  a.knt = k->knt;
  a.nt1 = nt1;
  a.nt2 = nt2;
  a.dt = k->kdt;
  a.lam = k->lam;
  a.mu = k->mu;
  for (int c = 0; c < 3; ++c) a.rsgt[c] = (flags >> c & 1) ? k->sgt[c] : nullptr;
  a.ssgt = k->sgt[3];
  a.out = k->series;
  a.param = k->param;
  cudaEventRecord(k->ev0, k->st);
  int le = fw::launch_sgt_scatter(a, 0, k->st);
  cudaEventRecord(k->ev1, k->st);
  cudaError_t e = le ? cudaError_t(le) : cudaStreamSynchronize(k->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_scatter");
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, k->ev0, k->ev1);
  k->last_ms = ms;
  k->scatter_nt1 = nt1;
  k->scatter_nt2 = nt2;
  k->scatter_flags = flags;
  k->pair_done = false;  // the series are now this scatter's
  return FWANT_OK;
}

fwant_status fwant_sgtker_get_scatter(fwant_sgtker* k, int slot, double* out) {
  if (!k || !out || slot < 0 || slot > 5) return FWANT_ERR_INVALID_ARG;
  if (!k->series) return k->fail(FWANT_ERR_STATE, "sgtker_get_scatter: no scatter computed");
  cudaSetDevice(k->device);
  cudaError_t e = cudaMemcpy(out, k->series + size_t(slot) * k->series_len(), k->series_len() * sizeof(double),
                             cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_get_scatter");
  return FWANT_OK;
}

namespace {
// filter / filtfilt of SI_ker_sta.F90:1491-1558 on one host series (the synthetic V or U),
// in double, operands in the reference's order
std::vector<double> host_iir(const float* w0, int nt, int mode, int nod1, const double* b, const double* a) {
  const int nod = nod1 - 1, nfact = 3 * nod, nel = nt + 2 * nfact;
  std::vector<double> x(nel + 1), y(nel + 1), w(nel + 1);
  for (int n = 1; n <= nt; ++n) x[nfact + n] = w0[n - 1];
  for (int n = 1; n <= nfact; ++n) {
    x[n] = mode == 1 ? 0.0 : 2.0 * x[nfact + 1] - x[2 * nfact + 1 - (n - 1)];
    x[nel - nfact + n] = 2.0 * x[nel - nfact] - x[nel - nfact - n];
  }
  auto filter = [&](const std::vector<double>& in, std::vector<double>& out) {
    for (int n = 1; n <= nel; ++n) {
      double yy = b[0] * in[n];
      for (int m = 2; m <= std::min(nod + 1, n); ++m) yy = (yy + b[m - 1] * in[n - m + 1]) - a[m - 1] * out[n - m + 1];
      out[n] = yy / a[0];
    }
  };
  filter(x, y);
  if (mode == 2) {
    for (int n = 1; n <= nel; ++n) w[n] = y[nel + 1 - n];
    filter(w, x);
    for (int n = 1; n <= nel; ++n) y[n] = x[nel + 1 - n];
  }
  return std::vector<double>(y.begin() + nfact + 1, y.begin() + nfact + 1 + nt);
}

// syn_filter / syn_filtfilt of SI_ker_pair (SI_ker_pair.F90:882-932): the series between
// zero padding (NOD samples in front, 2 (NOD + 1) behind), each pass with y(1:NOD) = 0, in
// FP64; the result rounded to FP32.
std::vector<float> host_pair_filter(const float* w0, int nt, int mode, int nod1, const double* b, const double* a) {
  const int nod = nod1 - 1, nel = nt + 3 * nod + 2;
  std::vector<double> x(nel + 1, 0.0), y(nel + 1, 0.0), w(nel + 1, 0.0);
  for (int n = 1; n <= nt; ++n) x[nod + n] = w0[n - 1];
  auto filter = [&](const std::vector<double>& in, std::vector<double>& out) {
    for (int n = 1; n <= nod; ++n) out[n] = 0.0;
    for (int n = nod + 1; n <= nel; ++n) {
      double yy = b[0] * in[n];
      for (int m = 2; m <= nod + 1; ++m) yy = (yy + b[m - 1] * in[n - m + 1]) - a[m - 1] * out[n - m + 1];
      out[n] = yy / a[0];
    }
  };
  filter(x, y);
  if (mode == 2) {
    for (int n = 1; n <= nel; ++n) w[n] = y[nel + 1 - n];
    filter(w, x);
    for (int n = 1; n <= nel; ++n) y[n] = x[nel + 1 - n];
  }
  std::vector<float> out(static_cast<size_t>(nt));
  for (int n = 1; n <= nt; ++n) out[size_t(n - 1)] = float(y[nod + n]);
  return out;
}
}  // namespace

fwant_status fwant_sgtker_scatter_pair(fwant_sgtker* k) {
  if (!k) return FWANT_ERR_INVALID_ARG;
  if (!k->have_media) return k->fail(FWANT_ERR_STATE, "sgtker_scatter_pair: media not set");
  if (!k->sgt[0] || !k->sgt[3])
    return k->fail(FWANT_ERR_STATE, "sgtker_scatter_pair: the receiver SGT (slot 0) and the source SGT (slot 3) are needed");
  cudaSetDevice(k->device);
  fwant_status rc = k->alloc(&k->series, 6 * k->series_len(), "scatter series");
  if (rc == FWANT_OK) rc = k->alloc(&k->pstrain, 14 * k->series_len(), "pair strains");
  if (rc != FWANT_OK) return rc;
  k->pair_done = false;  // until this scatter completes
  k->scatter_flags = 0;
  fw::PairArgs pa{};
  pa.npts = k->npts;
  pa.knt = k->knt;
  pa.dt = float(k->kdt);
  pa.lam = k->lam;
  pa.mu = k->mu;
  pa.rsgt = k->sgt[0];
  pa.ssgt = k->sgt[3];
  pa.strain = k->pstrain;
  pa.out = k->series;
  cudaError_t e = cudaEventRecord(k->ev0, k->st);
  if (e == cudaSuccess) e = cudaError_t(fw::launch_pair_scatter(pa, k->st));
  if (e == cudaSuccess) e = cudaEventRecord(k->ev1, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, k->ev0, k->ev1);
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_scatter_pair");
  k->last_ms = ms;
  k->scatter_flags = 0;  // the series now hold the pair's Sa, Sb
  k->pair_done = true;
  return FWANT_OK;
}

fwant_status fwant_sgtker_kernel_pair(fwant_sgtker* k, const float* v, const float* u, int nt1, int nt2, float sgt_m0,
                                      int mode, int nod1, const double* b, const double* a, float* kap, float* kaq,
                                      float* kbp, float* kbq) {
  if (!k || !v || !u || !kap || !kaq || !kbp || !kbq) return FWANT_ERR_INVALID_ARG;
  if (mode < 0 || mode > 2) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel_pair: filter mode must be 0, 1 or 2");
  if (mode != 0 && (!b || !a || nod1 < 1 || nod1 > fw::IIR_MAX_COEF || !(a[0] != 0.0)))
    return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel_pair: filter needs 1..16 coefficients with a[0] != 0");
  if (!k->pair_done) return k->fail(FWANT_ERR_STATE, "sgtker_kernel_pair: fwant_sgtker_scatter_pair first");
  if (nt1 < 1 || nt2 > k->knt || nt1 > nt2)
    return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel_pair: window outside 1..knt");
  const double* ser_a = k->series;
  const double* ser_b = k->series + k->series_len();
  std::vector<float> vf(v, v + k->knt), uf(u, u + k->knt);
  cudaSetDevice(k->device);
  if (mode != 0) {  // syn_filter(filtfilt) of V, U on the host; scatter_filter(filtfilt) on the device
    vf = host_pair_filter(v, k->knt, mode, nod1, b, a);
    uf = host_pair_filter(u, k->knt, mode, nod1, b, a);
    const size_t nel = size_t(k->knt) + 3 * size_t(nod1 - 1) + 2;
    fwant_status rc = k->alloc(&k->filtered, 2 * k->series_len(), "filtered series");
    if (rc != FWANT_OK) return rc;
    if (k->iir_scratch_len < nel * size_t(k->npts)) {
      cudaFree(k->iir_scratch);
      k->iir_scratch = nullptr;
      k->iir_scratch_len = 0;
      if ((rc = k->alloc(&k->iir_scratch, nel * size_t(k->npts), "filter scratch")) != FWANT_OK) return rc;
      k->iir_scratch_len = nel * size_t(k->npts);
    }
    fw::IirArgs ia{};
    ia.npts = k->npts;
    ia.knt = k->knt;
    ia.mode = mode == 1 ? 1 : 3;
    ia.nod1 = nod1;
    for (int q = 0; q < nod1; ++q) { ia.b[q] = b[q]; ia.a[q] = a[q]; }
    ia.scratch = k->iir_scratch;
    for (int s = 0; s < 2; ++s) {
      ia.in = s == 0 ? ser_a : ser_b;
      ia.out = k->filtered + size_t(s) * k->series_len();
      fw::launch_iir(ia, k->st);
    }
    ser_a = k->filtered;
    ser_b = k->filtered + k->series_len();
  }
  // normalisation (SI_ker_pair.F90:802-808), FP32 in the reference's order
  const float dt = float(k->kdt);
  float v0 = (0.5f * (vf[size_t(nt1 - 1)] * vf[size_t(nt1 - 1)]) + 0.5f * (vf[size_t(nt2 - 1)] * vf[size_t(nt2 - 1)])) * dt;
  float u0 = (0.5f * (uf[size_t(nt1 - 1)] * uf[size_t(nt1 - 1)]) + 0.5f * (uf[size_t(nt2 - 1)] * uf[size_t(nt2 - 1)])) * dt;
  for (int n = nt1 + 1; n <= nt2 - 1; ++n) {
    v0 = v0 + (vf[size_t(n - 1)] * vf[size_t(n - 1)]) * dt;
    u0 = u0 + (uf[size_t(n - 1)] * uf[size_t(n - 1)]) * dt;
  }
  v0 = v0 * sgt_m0;
  u0 = u0 * sgt_m0;
  if (!(v0 != 0.0f) || !(u0 != 0.0f)) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel_pair: zero normalisation");
  fwant_status rc = k->alloc(&k->pvu, 2 * size_t(k->knt), "pair synthetics");
  if (rc == FWANT_OK) rc = k->alloc(&k->kout, 4 * size_t(k->npts), "kernels");
  if (rc != FWANT_OK) return rc;
  cudaError_t e = cudaMemcpyAsync(k->pvu, vf.data(), size_t(k->knt) * sizeof(float), cudaMemcpyHostToDevice, k->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(k->pvu + k->knt, uf.data(), size_t(k->knt) * sizeof(float), cudaMemcpyHostToDevice, k->st);
  float* ko = reinterpret_cast<float*>(k->kout);
  const size_t np = size_t(k->npts);
  fw::PairKernelArgs pk{};
  pk.npts = k->npts;
  pk.nt1 = nt1;
  pk.nt2 = nt2;
  pk.dt = dt;
  pk.v0 = v0;
  pk.u0 = u0;
  pk.ka = ser_a;
  pk.kb = ser_b;
  pk.v = k->pvu;
  pk.u = k->pvu + k->knt;
  pk.kap = ko;
  pk.kaq = ko + np;
  pk.kbp = ko + 2 * np;
  pk.kbq = ko + 3 * np;
  if (e == cudaSuccess) {
    fw::launch_pair_kernel(pk, k->st);
    e = cudaGetLastError();
  }
  float* const host[4] = {kap, kaq, kbp, kbq};
  for (int q = 0; q < 4 && e == cudaSuccess; ++q)
    e = cudaMemcpyAsync(host[q], ko + q * np, np * sizeof(float), cudaMemcpyDeviceToHost, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_kernel_pair");
  return FWANT_OK;
}

fwant_status fwant_sgtker_rotate(fwant_sgtker* k, const double rot[9]) {
  if (!k || !rot) return FWANT_ERR_INVALID_ARG;
  if (!k->series || (k->scatter_flags & 7) != 7)
    return k->fail(FWANT_ERR_STATE, "sgtker_rotate: the scatter of all three components is needed");
  cudaSetDevice(k->device);
  fw::launch_rotate_series(k->series, (long long)k->series_len(), rot, k->st);
  cudaError_t e = cudaStreamSynchronize(k->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_rotate");
  return FWANT_OK;
}

fwant_status fwant_sgtker_kernel_filtered(fwant_sgtker* k, int ncmp, const float* v, const float* u, int nt1,
                                          int nt2, double sgt_m0, int mode, int nod1, const double* b,
                                          const double* a, double* kap, double* kaq, double* kbp, double* kbq);

fwant_status fwant_sgtker_convert(fwant_sgtker* k, int mode, float* kap, float* kaq, float* kbp, float* kbq) {
  if (!k || !kap || !kaq || !kbp || !kbq) return FWANT_ERR_INVALID_ARG;
  if (mode < 1 || mode > 3) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_convert: mode must be 1, 2 or 3");
  if (!k->have_media) return k->fail(FWANT_ERR_STATE, "sgtker_convert: media not set");
  cudaSetDevice(k->device);
  // the four arrays share one device buffer (the window-kernel outputs' FP64 space holds them)
  fwant_status rc = k->alloc(&k->kout, 4 * size_t(k->npts), "kernel outputs");
  if (rc != FWANT_OK) return rc;
  float* d = reinterpret_cast<float*>(k->kout);
  const size_t n = size_t(k->npts), bytes = n * sizeof(float);
  float* const host[4] = {kap, kaq, kbp, kbq};
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < 4 && e == cudaSuccess; ++q)
    e = cudaMemcpyAsync(d + q * n, host[q], bytes, cudaMemcpyHostToDevice, k->st);
  if (e == cudaSuccess) {
    fw::launch_convert_kernel(mode, k->npts, k->lam, k->mu, d, d + n, d + 2 * n, d + 3 * n, k->st);
    e = cudaGetLastError();
  }
  for (int q = 0; q < 4 && e == cudaSuccess; ++q)
    e = cudaMemcpyAsync(host[q], d + q * n, bytes, cudaMemcpyDeviceToHost, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_convert");
  return FWANT_OK;
}

fwant_status fwant_sgtker_kernel(fwant_sgtker* k, int ncmp, const float* v, const float* u, int nt1, int nt2,
                                 double sgt_m0, double* kap, double* kaq, double* kbp, double* kbq) {
  return fwant_sgtker_kernel_filtered(k, ncmp, v, u, nt1, nt2, sgt_m0, 0, 0, nullptr, nullptr, kap, kaq, kbp, kbq);
}

fwant_status fwant_sgtker_kernel_filtered(fwant_sgtker* k, int ncmp, const float* v, const float* u, int nt1,
                                          int nt2, double sgt_m0, int mode, int nod1, const double* b,
                                          const double* a, double* kap, double* kaq, double* kbp, double* kbq) {
  if (!k || !v || !u || !kap || !kaq || !kbp || !kbq) return FWANT_ERR_INVALID_ARG;
  if (mode < 0 || mode > 2) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel: filter mode must be 0, 1 or 2");
  if (mode != 0 && (!b || !a || nod1 < 1 || nod1 > fw::IIR_MAX_COEF || !(a[0] != 0.0)))
    return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel: filter needs 1..16 coefficients with a[0] != 0");
  // the reflected padding of 3 (order) samples at each end lies inside the series
  if (mode != 0 && k->knt <= 3 * (nod1 - 1))
    return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel: series shorter than the filter padding");
  if (ncmp < 1 || ncmp > 3) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel: ncmp must be 1, 2 or 3");
  if (!k->series || !(k->scatter_flags >> (ncmp - 1) & 1))
    return k->fail(FWANT_ERR_STATE, "sgtker_kernel: scatter of this component not computed");
  if (nt1 < k->scatter_nt1 || nt2 > k->scatter_nt2 || nt1 > nt2)
    return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel: window outside the scatter range");
  // filtering of the synthetics (syn_filter / syn_filtfilt) and of the two series
  // (scatter_filter / scatter_filtfilt), SI_ker_sta.F90:756-773
  static const int slot_a[3] = {0, 1, 2}, slot_b[3] = {3, 5, 4};
  const double* ser_a = k->series + size_t(slot_a[ncmp - 1]) * k->series_len();
  const double* ser_b = k->series + size_t(slot_b[ncmp - 1]) * k->series_len();
  std::vector<double> vd(k->knt), ud(k->knt);
  if (mode != 0) {
    const std::vector<double> fv = host_iir(v, k->knt, mode, nod1, b, a), fu = host_iir(u, k->knt, mode, nod1, b, a);
    vd = fv;
    ud = fu;
    cudaSetDevice(k->device);
    const size_t nel = size_t(k->knt) + 6 * size_t(nod1 - 1);
    fwant_status rc = k->alloc(&k->filtered, 2 * k->series_len(), "filtered series");
    if (rc != FWANT_OK) return rc;
    if (k->iir_scratch_len < nel * size_t(k->npts)) {
      cudaFree(k->iir_scratch);
      k->iir_scratch = nullptr;
      k->iir_scratch_len = 0;
      if ((rc = k->alloc(&k->iir_scratch, nel * size_t(k->npts), "filter scratch")) != FWANT_OK) return rc;
      k->iir_scratch_len = nel * size_t(k->npts);
    }
    fw::IirArgs ia{};
    ia.npts = k->npts;
    ia.knt = k->knt;
    ia.mode = mode;
    ia.nod1 = nod1;
    for (int q = 0; q < nod1; ++q) { ia.b[q] = b[q]; ia.a[q] = a[q]; }
    ia.scratch = k->iir_scratch;
    for (int s = 0; s < 2; ++s) {
      ia.in = s == 0 ? ser_a : ser_b;
      ia.out = k->filtered + size_t(s) * k->series_len();
      fw::launch_iir(ia, k->st);
    }
    ser_a = k->filtered;
    ser_b = k->filtered + k->series_len();
  } else {
    for (int n = 0; n < k->knt; ++n) { vd[n] = v[n]; ud[n] = u[n]; }
  }
  // normalisation (SI_ker_sta.F90:1397-1402): trapezoid integral of V^2 and U^2 times SGT_M0
  const double dt = k->kdt;
  const double v1 = vd[nt1 - 1], v2 = vd[nt2 - 1], u1 = ud[nt1 - 1], u2 = ud[nt2 - 1];
  double v0 = (0.5 * v1 * v1 + 0.5 * v2 * v2) * dt, u0 = (0.5 * u1 * u1 + 0.5 * u2 * u2) * dt;
  for (int n = nt1 + 1; n <= nt2 - 1; ++n) {
    const double vn = vd[n - 1], un = ud[n - 1];
    v0 += vn * vn * dt;
    u0 += un * un * dt;
  }
  v0 *= sgt_m0;
  u0 *= sgt_m0;
  if (!(v0 != 0.0) || !(u0 != 0.0)) return k->fail(FWANT_ERR_INVALID_ARG, "sgtker_kernel: zero normalisation");
  std::vector<double> w(2 * size_t(k->knt), 0.0);
  for (int n = nt1; n <= nt2; ++n) {
    const double wt = (n == nt1 || n == nt2) ? 0.5 * dt : dt;
    w[n - 1] = wt * vd[n - 1];
    w[k->knt + n - 1] = wt * ud[n - 1];
  }
  cudaSetDevice(k->device);
  fwant_status rc = k->alloc(&k->wts, 2 * size_t(k->knt), "weights");
  if (rc == FWANT_OK) rc = k->alloc(&k->kout, 4 * size_t(k->npts), "kernels");
  if (rc != FWANT_OK) return rc;
  cudaError_t e = cudaMemcpyAsync(k->wts, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, k->st);
  fw::KernelArgs ka{};
  ka.npts = k->npts;
  ka.knt = k->knt;
  ka.nt1 = nt1;
  ka.nt2 = nt2;
  ka.ka = ser_a;
  ka.kb = ser_b;
  ka.wv = k->wts;
  ka.wu = k->wts + k->knt;
  ka.v0 = v0;
  ka.u0 = u0;
  const size_t np = size_t(k->npts);
  ka.kap = k->kout; ka.kaq = k->kout + np; ka.kbp = k->kout + 2 * np; ka.kbq = k->kout + 3 * np;
  fw::launch_scatter_kernel(ka, k->st);
  double* dst[4] = {kap, kaq, kbp, kbq};
  for (int q = 0; q < 4 && e == cudaSuccess; ++q)
    e = cudaMemcpyAsync(dst[q], k->kout + q * np, np * sizeof(double), cudaMemcpyDeviceToHost, k->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(k->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return k->cuda_fail(e, "sgtker_kernel");
  return FWANT_OK;
}

fwant_status fwant_sgtker_last_scatter_ms(fwant_sgtker* k, double* ms) {
  if (!k || !ms) return FWANT_ERR_INVALID_ARG;
  *ms = k->last_ms;
  return FWANT_OK;
}

}  // extern "C"
