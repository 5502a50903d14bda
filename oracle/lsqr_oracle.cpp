// TEST INFRASTRUCTURE ONLY (the oracle).  CPU restatement of the reference's LSQR
// (inv.LSQR/mod_LSQR.f90): slsqr :137-268 with lnrliz :287-300, lupdat :320-335, dotp
// :337-345, lax :347-365, laty :367-388, and lgtsol :270-285.  Sequential, every sum in the
// reference's order, no contraction (compiled with -ffp-contract=off).  Used by the tests
// and the benchmark's CPU baseline to check and time the GPU solver; never by the product.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr double CONS_EQ = 1.0e-20;

double dotp(const double* a, const double* b, long long n) {
  double s = 0.0;
  for (long long i = 0; i < n; ++i) s = s + a[i] * b[i];
  return s;
}

// lnrliz: returns the norm; scales only when it exceeds CONS_EQ
double lnrliz(double* v, long long n) {
  const double v0 = std::sqrt(dotp(v, v, n));
  if (std::fabs(v0) <= CONS_EQ) return v0;
  for (long long i = 0; i < n; ++i) v[i] = v[i] / v0;
  return v0;
}

}  // namespace

extern "C" {

// A in compressed rows (0-based); returns the iteration count.  info[6] = |A|_F, res2,
// test1, test2, phibar, |x|; flag: 1 stopped by a test or maxit, 2 rho == 0.
long long orc_lsqr(long long nrow, long long ncol, const long long* rp, const int* ci, const double* va,
                   const double* b, double atol, double btol, long long maxit, double* x, double* sig, double* info,
                   int* flag) {
  std::vector<double> u(static_cast<size_t>(nrow)), v(static_cast<size_t>(ncol)), w(static_cast<size_t>(ncol)),
      q(static_cast<size_t>(std::max(nrow, ncol)));
  const long long nel = rp[nrow];
  const double anorm = std::sqrt(dotp(va, va, nel));
  auto lax = [&](double* yy, const double* xx) {  // yy = A xx
    for (long long i = 0; i < nrow; ++i) {
      double y0 = 0.0;
      for (long long l = rp[i]; l < rp[i + 1]; ++l) y0 = y0 + va[l] * xx[ci[l]];
      yy[i] = y0;
    }
  };
  auto laty = [&](double* xx, const double* yy) {  // xx = A^T yy, rows in order
    for (long long i = 0; i < ncol; ++i) xx[i] = 0.0;
    for (long long i = 0; i < nrow; ++i) {
      const double yi = yy[i];
      for (long long l = rp[i]; l < rp[i + 1]; ++l) xx[ci[l]] = xx[ci[l]] + va[l] * yi;
    }
  };
  for (long long i = 0; i < nrow; ++i) u[size_t(i)] = b[i];
  double beta = lnrliz(u.data(), nrow);
  laty(v.data(), u.data());
  double alpha = lnrliz(v.data(), ncol);
  for (long long i = 0; i < ncol; ++i) {
    w[size_t(i)] = v[size_t(i)];
    x[i] = 0.0;
    sig[i] = 0.0;
  }
  double phibar = beta, rhobar = alpha, res2 = 0.0, test1 = 0.0, test2 = 0.0, xnorm = 0.0;
  long long itct = 0;
  *flag = 1;
  for (;;) {
    lax(q.data(), v.data());
    for (long long i = 0; i < nrow; ++i) u[size_t(i)] = q[size_t(i)] - u[size_t(i)] * alpha;
    beta = lnrliz(u.data(), nrow);
    laty(q.data(), u.data());
    for (long long i = 0; i < ncol; ++i) v[size_t(i)] = q[size_t(i)] - v[size_t(i)] * beta;
    alpha = lnrliz(v.data(), ncol);
    const double rho = std::sqrt(rhobar * rhobar + beta * beta);
    if (rho == 0.0) {
      *flag = 2;
      break;
    }
    const double c = rhobar / rho, s = beta / rho, theta = s * alpha;
    rhobar = -c * alpha;
    const double phi = c * phibar;
    phibar = s * phibar;
    for (long long i = 0; i < ncol; ++i) {
      const double temp = w[size_t(i)] / rho;
      x[i] = x[i] + phi * temp;
      w[size_t(i)] = v[size_t(i)] - theta * temp;
      sig[i] = sig[i] + temp * temp;
    }
    const double rnorm = phibar;
    xnorm = std::sqrt(dotp(x, x, ncol));
    test1 = rnorm / anorm / xnorm;
    test2 = alpha * std::fabs(c) / anorm;
    itct = itct + 1;
    if (test1 <= atol || test2 <= btol || itct == maxit) {
      res2 = phibar;
      break;
    }
  }
  const double out[6] = {anorm, res2, test1, test2, phibar, xnorm};
  std::memcpy(info, out, sizeof(out));
  return itct;
}

// lgtsol: standard errors sqrt(res2 / max(nrow - nvar, 1) * sig)
void orc_lgtsol(long long nrow, long long nvar, double res2, const double* sig, double* serr) {
  const double temp = res2 / double(nrow - nvar > 1 ? nrow - nvar : 1);
  for (long long i = 0; i < nvar; ++i) serr[i] = std::sqrt(temp * sig[i]);
}

}  // extern "C"
