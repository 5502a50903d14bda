// ORACLE — test infrastructure, never the product.
//
// CPU restatement of the sensitivity-kernel accumulation of SI_ker_sta.F90:
// stress2strain (:1185-1211), sgt2scatter3 (:1257-1337) and scatter2kernel (:1375-1431).
// Only the tests and the precision study load it, as the checker.
//
// Two arithmetic modes:
//   mode 0 — the reference's single-precision program: every value and accumulator is
//            FP32, dt multiplies every term, operand order as the Fortran expressions;
//   mode 1 — FP64 accumulation as the device computes it: FP32 strains (as mode 0), trace
//            summed in FP64, exact FP64 products accumulated with fma in ascending lag
//            order (trace product first, then Exx Eyy Ezz and the doubled Exy Exz Eyz
//            products), dt applied once after the sum.
// Layout of every series: [component][frame][point], point fastest (the (I,J,K,time)
// layout of one sgt_ file variable per component).  Build with -ffp-contract=off.

#include <cmath>
#include <cstddef>

namespace {

struct Compliance {
  float e1, e2, e3;
};

// E1 = (lam+miu)/(miu*(3.0*lam+2.0*miu)), E2 = -lam/(2.0*miu*(3.0*lam+2.0*miu)), E3 = 1.0/miu
Compliance compliance(float lam, float miu) {
  const float s = 3.0f * lam + 2.0f * miu;
  Compliance c;
  c.e1 = (lam + miu) / (miu * s);
  c.e2 = -(lam / ((2.0f * miu) * s));
  c.e3 = 1.0f / miu;
  return c;
}

// Strains (Exx Eyy Ezz Exy Exz Eyz) of point p, frame n from the six stresses.
void strain(const float* sgt, long long npts, int knt, long long p, int n, const Compliance& c, float e[6]) {
  const size_t cs = size_t(knt) * size_t(npts);
  const size_t o = size_t(n) * size_t(npts) + size_t(p);
  const float txx = sgt[o], tyy = sgt[o + cs], tzz = sgt[o + 2 * cs];
  const float txy = sgt[o + 3 * cs], txz = sgt[o + 4 * cs], tyz = sgt[o + 5 * cs];
  const float e0 = c.e2 * ((txx + tyy) + tzz);
  const float d = c.e2 - c.e1;
  e[0] = e0 - d * txx;
  e[1] = e0 - d * tyy;
  e[2] = e0 - d * tzz;
  const float h = 0.5f * c.e3;
  e[3] = h * txy;
  e[4] = h * txz;
  e[5] = h * tyz;
}

}  // namespace

extern "C" {

// stress2strain on [6][knt][npts] stresses -> strains (same layout).
void orc_stress2strain(long long npts, int knt, const float* lam, const float* mu, const float* stress,
                       float* out) {
  const size_t cs = size_t(knt) * size_t(npts);
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < npts; ++p) {
    const Compliance c = compliance(lam[p], mu[p]);
    for (int n = 0; n < knt; ++n) {
      float e[6];
      strain(stress, npts, knt, p, n, c, e);
      for (int q = 0; q < 6; ++q) out[q * cs + size_t(n) * size_t(npts) + size_t(p)] = e[q];
    }
  }
}

// sgt2scatter3: rsgt[3] receiver SGT stresses (null = flag off), ssgt source SGT; out
// [6][knt][npts] FP64 (slots X -> 0, 3; Y -> 1, 5; Z -> 2, 4); nt1, nt2 1-based.
// param 0: Vp/Vs kernels, Ka = x1 2 (lambda + 2 mu), Kb = 2 (x2 - x1) 2 mu (SI_ker_sta.F90:1297-1298);
// param 1: lambda/mu kernels, Ka = x1 lambda, Kb = 2 x2 mu (SI_ker_sta_lamu.F90:1299-1300).
void orc_sgt2scatter3(long long npts, int knt, int nt1, int nt2, double dt, const float* lam, const float* mu,
                      const float* rx, const float* ry, const float* rz, const float* ssgt, int mode, int param,
                      double* out) {
  const float* rs[3] = {rx, ry, rz};
  const int slot_b[3] = {3, 5, 4};
  const size_t cs = size_t(knt) * size_t(npts);
#pragma omp parallel for schedule(dynamic, 16)
  for (long long p = 0; p < npts; ++p) {
    const Compliance c = compliance(lam[p], mu[p]);
    float* es = new float[size_t(knt) * 6];
    float* er = new float[size_t(knt) * 6];
    for (int n = 0; n < knt; ++n) strain(ssgt, npts, knt, p, n, c, es + 6 * n);
    for (int comp = 0; comp < 3; ++comp) {
      if (!rs[comp]) continue;
      for (int n = 0; n < knt; ++n) strain(rs[comp], npts, knt, p, n, c, er + 6 * n);
      for (int n = nt1; n <= nt2; ++n) {  // 1-based output index
        double ka, kb;
        if (mode == 0) {
          const float fdt = float(dt);
          float x1 = 0.0f, x2 = 0.0f;
          for (int m = 1; m <= n - 1; ++m) {
            const float* R = er + 6 * (m - 1);
            const float* S = es + 6 * (n - m - 1);
            x1 = x1 + ((1.0f * fdt) * ((R[0] + R[1]) + R[2])) * ((S[0] + S[1]) + S[2]);
            x2 = x2 + (1.0f * fdt) * (((((R[0] * S[0] + R[1] * S[1]) + R[2] * S[2]) + (2.0f * R[3]) * S[3]) +
                                       (2.0f * R[4]) * S[4]) +
                                      (2.0f * R[5]) * S[5]);
          }
          if (param == 1) {
            ka = x1 * lam[p];
            kb = (2.0f * x2) * mu[p];
          } else {
            ka = (x1 * 2.0f) * (lam[p] + 2.0f * mu[p]);
            kb = ((2.0f * (x2 - x1)) * 2.0f) * mu[p];
          }
        } else {
          double x1 = 0.0, x2 = 0.0;
          for (int m = 1; m <= n - 1; ++m) {
            const float* R = er + 6 * (m - 1);
            const float* S = es + 6 * (n - m - 1);
            const double trr = (double(R[0]) + double(R[1])) + double(R[2]);
            const double trs = (double(S[0]) + double(S[1])) + double(S[2]);
            x1 = std::fma(trr, trs, x1);
            x2 = std::fma(double(R[0]), double(S[0]), x2);
            x2 = std::fma(double(R[1]), double(S[1]), x2);
            x2 = std::fma(double(R[2]), double(S[2]), x2);
            x2 = std::fma(2.0 * double(R[3]), double(S[3]), x2);
            x2 = std::fma(2.0 * double(R[4]), double(S[4]), x2);
            x2 = std::fma(2.0 * double(R[5]), double(S[5]), x2);
          }
          const double l = lam[p], u = mu[p];
          if (param == 1) {
            ka = (x1 * dt) * l;
            kb = (2.0 * (x2 * dt)) * u;
          } else {
            ka = (x1 * dt) * (2.0 * (l + 2.0 * u));
            kb = ((x2 - x1) * dt) * (4.0 * u);
          }
        }
        const size_t o = size_t(n - 1) * size_t(npts) + size_t(p);
        out[size_t(comp) * cs + o] = ka;
        out[size_t(slot_b[comp]) * cs + o] = kb;
      }
    }
    delete[] es;
    delete[] er;
  }
}

// FP64 accumulation of scatter2kernel (SI_ker_sta.F90:1375-1431): trapezoid weights
// times the synthetic, one fma per frame in the order nt1, nt2, nt1+1 .. nt2-1.
extern "C++" {
template <typename T>
static void scatter2kernel_fp64(long long npts, int nt1, int nt2, double dt, const T* v, const T* u, const double* ka,
                                const double* kb, double sgt_m0, double* kap, double* kaq, double* kbp, double* kbq) {
  const double v1 = v[nt1 - 1], v2 = v[nt2 - 1], u1 = u[nt1 - 1], u2 = u[nt2 - 1];
  double v0 = (0.5 * v1 * v1 + 0.5 * v2 * v2) * dt, u0 = (0.5 * u1 * u1 + 0.5 * u2 * u2) * dt;
  for (int n = nt1 + 1; n <= nt2 - 1; ++n) {
    const double vn = v[n - 1], un = u[n - 1];
    v0 += vn * vn * dt;
    u0 += un * un * dt;
  }
  v0 *= sgt_m0;
  u0 *= sgt_m0;
  auto wv = [&](int n) { return ((n == nt1 || n == nt2) ? 0.5 * dt : dt) * double(v[n - 1]); };
  auto wu = [&](int n) { return ((n == nt1 || n == nt2) ? 0.5 * dt : dt) * double(u[n - 1]); };
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < npts; ++p) {
    double sap = 0.0, saq = 0.0, sbp = 0.0, sbq = 0.0;
    auto add = [&](int n) {
      const double a = ka[size_t(n - 1) * size_t(npts) + size_t(p)];
      const double b = kb[size_t(n - 1) * size_t(npts) + size_t(p)];
      sap = std::fma(wv(n), a, sap);
      saq = std::fma(wu(n), a, saq);
      sbp = std::fma(wv(n), b, sbp);
      sbq = std::fma(wu(n), b, sbq);
    };
    add(nt1);
    add(nt2);
    for (int n = nt1 + 1; n < nt2; ++n) add(n);
    kap[p] = sap / v0;
    kaq[p] = saq / u0;
    kbp[p] = sbp / v0;
    kbq[p] = sbq / u0;
  }
}
}  // extern "C++"

// scatter2kernel over frames nt1..nt2 (1-based) of the series ka, kb ([knt][npts]).
void orc_scatter2kernel(long long npts, int knt, int nt1, int nt2, double dt, const float* v, const float* u,
                        const double* ka, const double* kb, double sgt_m0, int mode, double* kap, double* kaq,
                        double* kbp, double* kbq) {
  (void)knt;
  if (mode == 0) {
    const float fdt = float(dt), m0 = float(sgt_m0);
    const float v1 = v[nt1 - 1], v2 = v[nt2 - 1], u1 = u[nt1 - 1], u2 = u[nt2 - 1];
    float v0 = ((0.5f * (v1 * v1)) + (0.5f * (v2 * v2))) * fdt;
    float u0 = ((0.5f * (u1 * u1)) + (0.5f * (u2 * u2))) * fdt;
    for (int n = nt1 + 1; n <= nt2 - 1; ++n) {
      v0 = v0 + (v[n - 1] * v[n - 1]) * fdt;
      u0 = u0 + (u[n - 1] * u[n - 1]) * fdt;
    }
    v0 = v0 * m0;
    u0 = u0 * m0;
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < npts; ++p) {
      auto A = [&](int n) { return float(ka[size_t(n - 1) * size_t(npts) + size_t(p)]); };
      auto B = [&](int n) { return float(kb[size_t(n - 1) * size_t(npts) + size_t(p)]); };
      float sap = (0.5f * fdt) * (v1 * A(nt1) + v2 * A(nt2));
      float saq = (0.5f * fdt) * (u1 * A(nt1) + u2 * A(nt2));
      float sbp = (0.5f * fdt) * (v1 * B(nt1) + v2 * B(nt2));
      float sbq = (0.5f * fdt) * (u1 * B(nt1) + u2 * B(nt2));
      for (int n = nt1 + 1; n <= nt2 - 1; ++n) {
        sap = sap + (v[n - 1] * A(n)) * fdt;
        saq = saq + (u[n - 1] * A(n)) * fdt;
        sbp = sbp + (v[n - 1] * B(n)) * fdt;
        sbq = sbq + (u[n - 1] * B(n)) * fdt;
      }
      kap[p] = sap / v0;
      kaq[p] = saq / u0;
      kbp[p] = sbp / v0;
      kbq[p] = sbq / u0;
    }
    return;
  }
  scatter2kernel_fp64(npts, nt1, nt2, dt, v, u, ka, kb, sgt_m0, kap, kaq, kbp, kbq);
}

// scatter2kernel with the synthetics already in double (after filter / filtfilt), FP64
// accumulation as in mode 1 of orc_scatter2kernel.
void orc_scatter2kernel_dv(long long npts, int knt, int nt1, int nt2, double dt, const double* v, const double* u,
                           const double* ka, const double* kb, double sgt_m0, double* kap, double* kaq, double* kbp,
                           double* kbq) {
  (void)knt;
  scatter2kernel_fp64(npts, nt1, nt2, dt, v, u, ka, kb, sgt_m0, kap, kaq, kbp, kbq);
}

// filter (mode 1) / filtfilt (mode 2) of SI_ker_sta.F90:1433-1558 on one series of nt
// samples, double arithmetic in the reference's operand order, padding of NFACT = 3 NOD
// samples at each end (zeros in front for the one-pass filter, reflections otherwise).
void orc_iir(const double* w0, int nt, int mode, int nod1, const double* b, const double* a, double* out) {
  const int nod = nod1 - 1, nfact = 3 * nod, nel = nt + 2 * nfact;
  double* x = new double[nel + 1];
  double* y = new double[nel + 1];
  double* w = new double[nel + 1];
  for (int n = 1; n <= nt; ++n) x[nfact + n] = w0[n - 1];
  for (int n = 1; n <= nfact; ++n) {
    x[n] = mode == 1 ? 0.0 : 2.0 * x[nfact + 1] - x[2 * nfact + 1 - (n - 1)];
    x[nel - nfact + n] = 2.0 * x[nel - nfact] - x[nel - nfact - n];
  }
  auto filter = [&](const double* in, double* o) {
    for (int n = 1; n <= nel; ++n) {
      double yy = b[0] * in[n];
      const int mm = nod + 1 < n ? nod + 1 : n;
      for (int m = 2; m <= mm; ++m) yy = (yy + b[m - 1] * in[n - m + 1]) - a[m - 1] * o[n - m + 1];
      o[n] = yy / a[0];
    }
  };
  filter(x, y);
  if (mode == 2) {
    for (int n = 1; n <= nel; ++n) w[n] = y[nel + 1 - n];
    filter(w, x);
    for (int n = 1; n <= nel; ++n) y[n] = x[nel + 1 - n];
  }
  for (int n = 1; n <= nt; ++n) out[n - 1] = y[nfact + n];
  delete[] x;
  delete[] y;
  delete[] w;
}

}  // extern "C"
