// Sensitivity-kernel accumulation on the device: the strain Green's tensor convolution
// of sgt2scatter3 (SI_ker_sta.F90:1257-1337) with the strains of stress2strain
// (SI_ker_sta.F90:1185-1211), and the window integrals of scatter2kernel
// (SI_ker_sta.F90:1375-1431).
//
// Strains are formed from the FP32 stresses with the reference's FP32 expressions
// (round-to-nearest intrinsics: no contraction, IEEE division).  Products of two strains
// are exact in FP64 and every sum runs in FP64 in a fixed order (ascending lag m, then the
// six components Exx Eyy Ezz Exy Exz Eyz), so the results do not depend on the launch shape.
#include <cuda_runtime.h>

#include "kernels.h"

namespace fw {

namespace {

constexpr int SC_THREADS = 256;  // outputs n per CTA
constexpr int SC_MCHUNK = 512;   // lags m staged per pass
// per time index: trace (FP64) + six strains (FP64, shear components doubled on the receiver side)
constexpr int SC_VALS = 7;

struct Compliance {
  float e1, e2, e3;
};

__device__ __forceinline__ Compliance compliance(float lam, float miu) {
  // E1 = (lam+miu)/(miu*(3 lam+2 miu)), E2 = -lam/(2 miu (3 lam+2 miu)), E3 = 1/miu
  const float s = __fadd_rn(__fmul_rn(3.0f, lam), __fmul_rn(2.0f, miu));
  Compliance c;
  c.e1 = __fdiv_rn(__fadd_rn(lam, miu), __fmul_rn(miu, s));
  c.e2 = -__fdiv_rn(lam, __fmul_rn(__fmul_rn(2.0f, miu), s));
  c.e3 = __fdiv_rn(1.0f, miu);
  return c;
}

// Strains of one time index from the six stresses (Txx Tyy Tzz Txy Txz Tyz); FP32 as in
// stress2strain.  Writes the FP64 trace and the six strains, shear scaled by `shear`.
__device__ __forceinline__ void strain_at(const float* __restrict__ sgt, long long cstride, long long o,
                                          const Compliance& c, double shear, double* dst, int ld) {
  const float txx = sgt[o], tyy = sgt[o + cstride], tzz = sgt[o + 2 * cstride];
  const float txy = sgt[o + 3 * cstride], txz = sgt[o + 4 * cstride], tyz = sgt[o + 5 * cstride];
  const float e0 = __fmul_rn(c.e2, __fadd_rn(__fadd_rn(txx, tyy), tzz));
  const float d = __fsub_rn(c.e2, c.e1);
  const float h = __fmul_rn(0.5f, c.e3);
  const float exx = __fsub_rn(e0, __fmul_rn(d, txx));
  const float eyy = __fsub_rn(e0, __fmul_rn(d, tyy));
  const float ezz = __fsub_rn(e0, __fmul_rn(d, tzz));
  dst[0] = ((double)exx + (double)eyy) + (double)ezz;
  dst[ld] = exx;
  dst[2 * ld] = eyy;
  dst[3 * ld] = ezz;
  dst[4 * ld] = shear * (double)__fmul_rn(h, txy);
  dst[5 * ld] = shear * (double)__fmul_rn(h, txz);
  dst[6 * ld] = shear * (double)__fmul_rn(h, tyz);
}

// grid: x = point, y = receiver force component (0 X, 1 Y, 2 Z), z = chunk of outputs.
// Output n (1-based) of thread t is nt1 + z*SC_THREADS + t.
__global__ void __launch_bounds__(SC_THREADS) sgt_scatter_kernel(const ScatterArgs a) {
  extern __shared__ double sm[];
  const int comp = blockIdx.y;
  const float* __restrict__ rs = comp == 0 ? a.rsgt[0] : (comp == 1 ? a.rsgt[1] : a.rsgt[2]);
  if (!rs) return;
  const long long p = blockIdx.x;
  const int n_lo = a.nt1 + blockIdx.z * SC_THREADS;
  const int n_hi = min(a.nt2, n_lo + SC_THREADS - 1);
  const int n = n_lo + threadIdx.x;
  const long long cs = (long long)a.knt * a.npts;  // stride between stress components
  const Compliance cm = compliance(a.lam[p], a.mu[p]);

  // R chunk: lags [m0, m0+SC_MCHUNK), ld = SC_MCHUNK; S window: indices n - m for the
  // CTA's outputs and the chunk's lags, ld = SC_THREADS + SC_MCHUNK.
  constexpr int LDR = SC_MCHUNK, LDS = SC_THREADS + SC_MCHUNK;
  double* R = sm;
  double* Sw = sm + SC_VALS * LDR;

  double x1 = 0.0, x2 = 0.0;
  for (int m0 = 1; m0 <= n_hi - 1; m0 += SC_MCHUNK) {
    const int m1 = min(m0 + SC_MCHUNK, n_hi);  // exclusive
    // S indices needed: [max(1, n_lo - m1 + 1), n_hi - m0]
    const int s_lo = max(1, n_lo - m1 + 1);
    const int s_hi = n_hi - m0;
    __syncthreads();
    for (int m = m0 + threadIdx.x; m < m1; m += SC_THREADS)
      strain_at(rs, cs, (long long)(m - 1) * a.npts + p, cm, 2.0, R + (m - m0), LDR);
    for (int s = s_lo + threadIdx.x; s <= s_hi; s += SC_THREADS)
      strain_at(a.ssgt, cs, (long long)(s - 1) * a.npts + p, cm, 1.0, Sw + (s - s_lo), LDS);
    __syncthreads();
    if (n <= n_hi) {
      const int mend = min(m1, n);  // m < n
      for (int m = m0; m < mend; ++m) {
        const double* r = R + (m - m0);
        const double* q = Sw + (n - m - s_lo);
        x1 = fma(r[0], q[0], x1);
        x2 = fma(r[LDR], q[LDS], x2);
        x2 = fma(r[2 * LDR], q[2 * LDS], x2);
        x2 = fma(r[3 * LDR], q[3 * LDS], x2);
        x2 = fma(r[4 * LDR], q[4 * LDS], x2);
        x2 = fma(r[5 * LDR], q[5 * LDS], x2);
        x2 = fma(r[6 * LDR], q[6 * LDS], x2);
      }
    }
  }
  if (n > n_hi) return;
  const double lam = a.lam[p], mu = a.mu[p];
  // Vp/Vs: Ka = x1 2 (lam + 2 mu), Kb = 2 (x2 - x1) 2 mu (SI_ker_sta.F90:1297-1298);
  // lambda/mu: Ka = x1 lam, Kb = 2 x2 mu (SI_ker_sta_lamu.F90:1299-1300)
  double ka, kb;
  if (a.param == 1) {
    ka = (x1 * a.dt) * lam;
    kb = (2.0 * (x2 * a.dt)) * mu;
  } else {
    ka = (x1 * a.dt) * (2.0 * (lam + 2.0 * mu));
    kb = ((x2 - x1) * a.dt) * (4.0 * mu);
  }
  // X -> (Exx, Exy), Y -> (Eyy, Eyz), Z -> (Ezz, Exz); component slots Exx Eyy Ezz Exy Exz Eyz
  const int slot_a = comp, slot_b = comp == 0 ? 3 : (comp == 1 ? 5 : 4);
  const long long o = (long long)(n - 1) * a.npts + p;
  a.out[(long long)slot_a * cs + o] = ka;
  a.out[(long long)slot_b * cs + o] = kb;
}

// scatter2kernel: trapezoid integrals of the two series against V and U, per point.
__global__ void window_integral_kernel(const KernelArgs a) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= a.npts) return;
  const double* ka = a.ka + p;
  const double* kb = a.kb + p;
  const long long ld = a.npts;
  double sap = 0.0, saq = 0.0, sbp = 0.0, sbq = 0.0;
  // trapezoid: both end points (weights carry the 1/2), then the interior in order
  auto add = [&](int n) {
    const double va = ka[(long long)(n - 1) * ld], vb = kb[(long long)(n - 1) * ld];
    const double wv = a.wv[n - 1], wu = a.wu[n - 1];
    sap = fma(wv, va, sap);
    saq = fma(wu, va, saq);
    sbp = fma(wv, vb, sbp);
    sbq = fma(wu, vb, sbq);
  };
  add(a.nt1);
  add(a.nt2);
  for (int n = a.nt1 + 1; n < a.nt2; ++n) add(n);
  a.kap[p] = sap / a.v0;
  a.kaq[p] = saq / a.u0;
  a.kbp[p] = sbp / a.v0;
  a.kbq[p] = sbq / a.u0;
}

// One thread per point.  The padded series (NFACT = 3 NOD values reflected about the end
// samples, or zeros in front for the one-pass filter) is generated on the fly; the forward
// pass stores its output in scratch ([NEL][npts]), the backward pass of filtfilt reads it
// in reverse and writes only the unpadded range.  Operands in the reference's order, no
// contraction: y(n) = ((b1 x(n) + b2 x(n-1) - a2 y(n-1)) + ...) / a1.
__global__ void iir_kernel(const IirArgs A) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= A.npts) return;
  const int nod = A.nod1 - 1, nt = A.knt;
  // padding in front / behind: 3 nod reflected samples (modes 1, 2), or zeros: nod in
  // front, 2 (nod + 1) behind (mode 3)
  const int nfact = A.mode == 3 ? nod : 3 * nod;
  const int nel = A.mode == 3 ? nt + 3 * nod + 2 : nt + 2 * nfact;
  const long long ld = A.npts;
  const double* in = A.in + p;
  auto x_at = [&](int n) -> double {  // 1-based padded input
    if (A.mode == 3) return (n > nfact && n <= nfact + nt) ? in[(long long)(n - nfact - 1) * ld] : 0.0;
    if (n <= nfact) {
      if (A.mode == 1) return 0.0;
      return __dsub_rn(__dmul_rn(2.0, in[0]), in[(long long)(nfact + 1 - n) * ld]);
    }
    if (n <= nfact + nt) return in[(long long)(n - nfact - 1) * ld];
    const int m = n - nfact - nt;
    return __dsub_rn(__dmul_rn(2.0, in[(long long)(nt - 1) * ld]), in[(long long)(nt - 1 - m) * ld]);
  };
  double xs[IIR_MAX_COEF], ys[IIR_MAX_COEF];  // x(n-1..n-nod), y(n-1..n-nod)
  for (int m = 0; m < IIR_MAX_COEF; ++m) xs[m] = ys[m] = 0.0;
  double* scr = A.scratch + p;
  double* out = A.out + p;
  auto step = [&](double x, int n) -> double {
    if (A.mode == 3 && n <= nod) {  // SI_ker_pair's filter sets y(1:NOD) = 0 (:924)
      for (int m = nod - 1; m > 0; --m) { xs[m] = xs[m - 1]; ys[m] = ys[m - 1]; }
      xs[0] = x;
      ys[0] = 0.0;
      return 0.0;
    }
    double y = __dmul_rn(A.b[0], x);
    const int mm = min(nod + 1, n);
    for (int m = 2; m <= mm; ++m) y = __dsub_rn(__dadd_rn(y, __dmul_rn(A.b[m - 1], xs[m - 2])), __dmul_rn(A.a[m - 1], ys[m - 2]));
    y = __ddiv_rn(y, A.a[0]);
    for (int m = nod - 1; m > 0; --m) { xs[m] = xs[m - 1]; ys[m] = ys[m - 1]; }
    xs[0] = x;
    ys[0] = y;
    return y;
  };
  for (int n = 1; n <= nel; ++n) {
    const double y = step(x_at(n), n);
    if (A.mode == 1) {
      if (n > nfact && n <= nfact + nt) out[(long long)(n - nfact - 1) * ld] = y;
    } else {
      scr[(long long)(n - 1) * ld] = y;
    }
  }
  if (A.mode == 1) return;
  for (int m = 0; m < IIR_MAX_COEF; ++m) xs[m] = ys[m] = 0.0;
  for (int m = 1; m <= nel; ++m) {
    const double y = step(scr[(long long)(nel - m) * ld], m);
    const int n = nel + 1 - m;  // position in the final (reversed) series
    if (n > nfact && n <= nfact + nt) out[(long long)(n - nfact - 1) * ld] = y;
  }
}

__global__ void rotate_series_kernel(double* s, long long len, const double r0, const double r1, const double r2,
                                     const double r3, const double r4, const double r5, const double r6,
                                     const double r7, const double r8) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= len) return;
  const double rot[9] = {r0, r1, r2, r3, r4, r5, r6, r7, r8};
  const int slots[2][3] = {{0, 1, 2}, {3, 5, 4}};
  for (int g = 0; g < 2; ++g) {
    double v[3];
    for (int d = 0; d < 3; ++d) v[d] = s[slots[g][d] * len + e];
    for (int c = 0; c < 3; ++c)
      s[slots[g][c] * len + e] =
          __dadd_rn(__dadd_rn(__dmul_rn(v[0], rot[3 * c]), __dmul_rn(v[1], rot[3 * c + 1])), __dmul_rn(v[2], rot[3 * c + 2]));
  }
}

// Kernel parameter conversions of the kernel-file programs, one thread per point, FP32
// with every operation rounded separately in the reference's operand order (no
// contraction), so the device equals the reference's single-precision loops.
//   mode 1 SI_ker_lamu2kamu.F90:823-830, 2 SI_ker_lamu2vpvs.F90:823-830,
//   3 SI_ker_vpvs2kamu.F90:823-831.
__global__ void convert_kernel_kernel(int mode, long long n, const float* __restrict__ lam,
                                      const float* __restrict__ mu, float* __restrict__ ka0, float* __restrict__ ka1,
                                      float* __restrict__ kb0, float* __restrict__ kb1) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float l = lam[e], m = mu[e];
  float* const ka[2] = {ka0, ka1};
  float* const kb[2] = {kb0, kb1};
  for (int q = 0; q < 2; ++q) {  // phase (p) then amplitude (q) pair
    float a = ka[q][e], b = kb[q][e];
    if (mode == 1) {
      a = __fdiv_rn(a, l);
      b = __fdiv_rn(__fdiv_rn(b, m), 2.0f);
      b = __fmul_rn(__fsub_rn(__fmul_rn(2.0f, b), __fdiv_rn(__fmul_rn(2.0f, a), 3.0f)), m);
      a = __fmul_rn(a, __fadd_rn(l, __fdiv_rn(__fmul_rn(2.0f, m), 3.0f)));
    } else if (mode == 2) {
      a = __fdiv_rn(a, l);
      b = __fdiv_rn(__fdiv_rn(b, m), 2.0f);
      b = __fmul_rn(__fmul_rn(__fmul_rn(2.0f, __fsub_rn(b, a)), 2.0f), m);
      a = __fmul_rn(__fmul_rn(a, 2.0f), __fadd_rn(l, __fmul_rn(2.0f, m)));
    } else {
      a = __fdiv_rn(a, __fmul_rn(2.0f, __fadd_rn(l, __fmul_rn(2.0f, m))));
      b = __fadd_rn(__fdiv_rn(__fdiv_rn(b, m), 4.0f), a);
      b = __fmul_rn(__fsub_rn(__fmul_rn(2.0f, b), __fdiv_rn(__fmul_rn(2.0f, a), 3.0f)), m);
      a = __fmul_rn(a, __fadd_rn(l, __fdiv_rn(__fmul_rn(2.0f, m), 3.0f)));
    }
    ka[q][e] = a;
    kb[q][e] = b;
  }
}

// stress2strain of SI_ker_pair (:710-736, the same FP32 expressions as SI_ker_sta's) for
// one (frame, point) of the receiver and the source SGT; stores per side the trace
// (E11 + E22) + E33 and the six strains, the receiver's shear strains doubled
// (2 E12R E12S in sgt2scatter is (2 E12R) E12S).  Layout [14][knt][npts].
__global__ void pair_strain_kernel(const PairArgs a) {
  const long long len = (long long)a.knt * a.npts;
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= len) return;
  const long long p = e % a.npts;
  const Compliance c = compliance(a.lam[p], a.mu[p]);
  for (int side = 0; side < 2; ++side) {
    const float* g = side == 0 ? a.rsgt : a.ssgt;
    const float txx = g[e], tyy = g[e + len], tzz = g[e + 2 * len];
    const float txy = g[e + 3 * len], txz = g[e + 4 * len], tyz = g[e + 5 * len];
    const float e0 = __fmul_rn(c.e2, __fadd_rn(__fadd_rn(txx, tyy), tzz));
    const float d = __fsub_rn(c.e2, c.e1);
    const float h = __fmul_rn(0.5f, c.e3);
    const float exx = __fsub_rn(e0, __fmul_rn(d, txx));
    const float eyy = __fsub_rn(e0, __fmul_rn(d, tyy));
    const float ezz = __fsub_rn(e0, __fmul_rn(d, tzz));
    const float sh = side == 0 ? 2.0f : 1.0f;
    float* o = a.strain + (long long)side * 7 * len + e;
    o[0] = __fadd_rn(__fadd_rn(exx, eyy), ezz);
    o[len] = exx;
    o[2 * len] = eyy;
    o[3 * len] = ezz;
    o[4 * len] = __fmul_rn(sh, __fmul_rn(h, txy));
    o[5 * len] = __fmul_rn(sh, __fmul_rn(h, txz));
    o[6 * len] = __fmul_rn(sh, __fmul_rn(h, tyz));
  }
}

// sgt2scatter of SI_ker_pair (:738-780): for every output n, in order of the lag m = 1 ..
// n-1, x1 += (dt trR(m)) trS(n-m) and x2 += dt (E11R E11S + E22R E22S + E33R E33S +
// 2E12R E12S + 2E13R E13S + 2E23R E23S), FP32 with each operation rounded.  One CTA per
// point, one thread per output n; the receiver's lags and the source's window are staged
// in shared memory chunk by chunk (lags ascend across chunks, so each thread's sums keep
// the reference's order).
constexpr int PS_THREADS = 256, PS_MCHUNK = 512;
__global__ void __launch_bounds__(PS_THREADS) pair_scatter_kernel(const PairArgs a) {
  extern __shared__ float psm[];
  const long long p = blockIdx.x;
  const int n_lo = 1 + blockIdx.y * PS_THREADS;
  const int n_hi = min(a.knt, n_lo + PS_THREADS - 1);
  const int n = n_lo + threadIdx.x;
  const long long len = (long long)a.knt * a.npts;
  constexpr int LDR = PS_MCHUNK, LDS = PS_THREADS + PS_MCHUNK;
  float* R = psm;
  float* Sw = psm + 7 * LDR;
  const float* rs = a.strain;
  const float* ss = a.strain + 7 * len;
  float x1 = 0.0f, x2 = 0.0f;
  for (int m0 = 1; m0 <= n_hi - 1; m0 += PS_MCHUNK) {
    const int m1 = min(m0 + PS_MCHUNK, n_hi);  // exclusive
    const int s_lo = max(1, n_lo - m1 + 1);
    const int s_hi = n_hi - m0;
    __syncthreads();
    for (int m = m0 + threadIdx.x; m < m1; m += PS_THREADS)
      for (int q = 0; q < 7; ++q) R[q * LDR + (m - m0)] = rs[q * len + (long long)(m - 1) * a.npts + p];
    for (int t = s_lo + threadIdx.x; t <= s_hi; t += PS_THREADS)
      for (int q = 0; q < 7; ++q) Sw[q * LDS + (t - s_lo)] = ss[q * len + (long long)(t - 1) * a.npts + p];
    __syncthreads();
    if (n <= n_hi) {
      const int mend = min(m1, n);  // m < n
      for (int m = m0; m < mend; ++m) {
        const float* r = R + (m - m0);
        const float* q = Sw + (n - m - s_lo);
        x1 = __fadd_rn(x1, __fmul_rn(__fmul_rn(a.dt, r[0]), q[0]));
        float sum = __fmul_rn(r[LDR], q[LDS]);
        sum = __fadd_rn(sum, __fmul_rn(r[2 * LDR], q[2 * LDS]));
        sum = __fadd_rn(sum, __fmul_rn(r[3 * LDR], q[3 * LDS]));
        sum = __fadd_rn(sum, __fmul_rn(r[4 * LDR], q[4 * LDS]));
        sum = __fadd_rn(sum, __fmul_rn(r[5 * LDR], q[5 * LDS]));
        sum = __fadd_rn(sum, __fmul_rn(r[6 * LDR], q[6 * LDS]));
        x2 = __fadd_rn(x2, __fmul_rn(a.dt, sum));
      }
    }
  }
  if (n > n_hi) return;
  const float lam = a.lam[p], mu = a.mu[p];
  const float sa = __fmul_rn(__fmul_rn(x1, 2.0f), __fadd_rn(lam, __fmul_rn(2.0f, mu)));
  const float sb = __fmul_rn(__fmul_rn(__fmul_rn(2.0f, __fsub_rn(x2, x1)), 2.0f), mu);
  const long long o = (long long)(n - 1) * a.npts + p;
  a.out[o] = sa;
  a.out[len + o] = sb;
}

// scatter2kernel of SI_ker_pair (:782-838), FP32, one thread per point.
__global__ void pair_kernel_kernel(const PairKernelArgs a) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= a.npts) return;
  const long long ld = a.npts;
  auto ka = [&](int n) { return float(a.ka[(long long)(n - 1) * ld + p]); };
  auto kb = [&](int n) { return float(a.kb[(long long)(n - 1) * ld + p]); };
  const int n1 = a.nt1, n2 = a.nt2;
  const float hdt = __fmul_rn(0.5f, a.dt);
  const float v1 = a.v[n1 - 1], v2 = a.v[n2 - 1], u1 = a.u[n1 - 1], u2 = a.u[n2 - 1];
  const float ka1 = ka(n1), ka2 = ka(n2), kb1 = kb(n1), kb2 = kb(n2);
  float sap = __fmul_rn(hdt, __fadd_rn(__fmul_rn(v1, ka1), __fmul_rn(v2, ka2)));
  float saq = __fmul_rn(hdt, __fadd_rn(__fmul_rn(u1, ka1), __fmul_rn(u2, ka2)));
  float sbp = __fmul_rn(hdt, __fadd_rn(__fmul_rn(v1, kb1), __fmul_rn(v2, kb2)));
  float sbq = __fmul_rn(hdt, __fadd_rn(__fmul_rn(u1, kb1), __fmul_rn(u2, kb2)));
  for (int n = n1 + 1; n < n2; ++n) {
    const float vn = a.v[n - 1], un = a.u[n - 1], an = ka(n), bn = kb(n);
    sap = __fadd_rn(sap, __fmul_rn(__fmul_rn(vn, an), a.dt));
    saq = __fadd_rn(saq, __fmul_rn(__fmul_rn(un, an), a.dt));
    sbp = __fadd_rn(sbp, __fmul_rn(__fmul_rn(vn, bn), a.dt));
    sbq = __fadd_rn(sbq, __fmul_rn(__fmul_rn(un, bn), a.dt));
  }
  a.kap[p] = __fdiv_rn(sap, a.v0);
  a.kaq[p] = __fdiv_rn(saq, a.u0);
  a.kbp[p] = __fdiv_rn(sbp, a.v0);
  a.kbq[p] = __fdiv_rn(sbq, a.u0);
}

}  // namespace

int launch_pair_scatter(const PairArgs& a, void* stream) {
  if (a.npts <= 0 || a.knt <= 0) return 0;
  const long long len = (long long)a.knt * a.npts;
  pair_strain_kernel<<<(unsigned)((len + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a);
  const size_t smem = sizeof(float) * 7 * (PS_MCHUNK + PS_THREADS + PS_MCHUNK);
  cudaError_t e = cudaFuncSetAttribute(pair_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return int(e);
  dim3 grid((unsigned)a.npts, (unsigned)((a.knt + PS_THREADS - 1) / PS_THREADS));
  pair_scatter_kernel<<<grid, PS_THREADS, smem, (cudaStream_t)stream>>>(a);
  return int(cudaGetLastError());
}

void launch_pair_kernel(const PairKernelArgs& a, void* stream) {
  if (a.npts <= 0) return;
  pair_kernel_kernel<<<(unsigned)((a.npts + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a);
}

void launch_iir(const IirArgs& a, void* stream) {
  iir_kernel<<<(unsigned)((a.npts + 127) / 128), 128, 0, (cudaStream_t)stream>>>(a);
}

void launch_rotate_series(double* series, long long slot_len, const double rot[9], void* stream) {
  rotate_series_kernel<<<(unsigned)((slot_len + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      series, slot_len, rot[0], rot[1], rot[2], rot[3], rot[4], rot[5], rot[6], rot[7], rot[8]);
}

int launch_sgt_scatter(const ScatterArgs& a, int /*sm_count*/, void* stream) {
  const size_t smem = sizeof(double) * SC_VALS * (SC_MCHUNK + SC_THREADS + SC_MCHUNK);
  const cudaError_t e =
      cudaFuncSetAttribute(sgt_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return int(e);
  const int nout = a.nt2 - a.nt1 + 1;
  if (a.npts <= 0 || nout <= 0) return 0;
  dim3 grid((unsigned)a.npts, 3, (unsigned)((nout + SC_THREADS - 1) / SC_THREADS));
  sgt_scatter_kernel<<<grid, SC_THREADS, smem, (cudaStream_t)stream>>>(a);
  return int(cudaGetLastError());
}

void launch_convert_kernel(int mode, long long n, const float* lam, const float* mu, float* ka0, float* ka1,
                           float* kb0, float* kb1, void* stream) {
  if (n <= 0) return;
  convert_kernel_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(mode, n, lam, mu, ka0, ka1,
                                                                                      kb0, kb1);
}

void launch_scatter_kernel(const KernelArgs& a, void* stream) {
  const long long blocks = (a.npts + 255) / 256;
  if (blocks < 1) return;
  window_integral_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(a);
}

}  // namespace fw
