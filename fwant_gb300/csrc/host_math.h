// Host-side scalar math of the solver set-up: source time functions, smoothing
// weights and CFS-PML profiles.  These run once per stage (STF tables) or once per
// set-up, in FP32 with the reference's operand order, so that the device kernels see
// the same source amplitudes and damping profiles as the reference computes.
#pragma once
#include <cmath>

namespace fw {
namespace hm {

constexpr double PI = 3.141592653589793;  // mod_constants.F90:27 (DP parameter)

// fun_gauss (mod_src.F90:533-541)
inline float gauss(float t, float a, float t0) {
  if (std::fabs(t0) >= 1.0e-20f && (t <= 0.0f || t >= 2.0f * t0)) return 0.0f;
  const float q = (t - t0) * (t - t0);
  const float e = std::exp(-(q / (a * a)));
  return float(double(e) / (std::sqrt(PI) * double(a)));
}
// fun_gauss_deriv (mod_src.F90:542-550)
inline float gauss_deriv(float t, float a, float t0) {
  if (std::fabs(t0) >= 1.0e-20f && (t <= 0.0f || t >= 2.0f * t0)) return 0.0f;
  const float q = (t - t0) * (t - t0);
  const float e = std::exp(-(q / (a * a)));
  const double g = double(e) / (std::sqrt(PI) * double(a));
  return float(g * double(-2.0f * (t - t0) / (a * a)));
}
// fun_ricker / fun_ricker_deriv (mod_src.F90:509-530): u is formed in DP because PI is DP.
inline float ricker(float t, float fc, float t0) {
  if (t <= 0.0f) return 0.0f;
  const float f0 = float(std::sqrt(PI) / 2.0);
  const float u = float(double((t - t0) * 2.0f) * PI * double(fc));
  const float u2 = u * u;
  return ((u2 / 4.0f - 0.5f) * std::exp(-(u2 / 4.0f))) * f0;
}
inline float ricker_deriv(float t, float fc, float t0) {
  if (t <= 0.0f) return 0.0f;
  const float f0 = float(std::sqrt(PI) / 2.0);
  const float u = float(double((t - t0) * 2.0f) * PI * double(fc));
  const float u2 = u * u;
  const float v = ((u * (1.5f - u2 / 4.0f)) * std::exp(-(u2 / 4.0f))) * f0;
  return float(double(v) * PI * double(fc));
}
// bell family and triangle (mod_src.F90:552-592)
inline float bell(float t, float r) {
  if (t > 0.0f && t < r) return float((1.0 - std::cos(2 * PI * double(t) / double(r))) / double(r));
  return 0.0f;
}
inline float bell_deriv(float t, float r) {
  if (t > 0.0f && t < r) return float(2.0 * PI * std::sin(2 * PI * double(t) / double(r)) / double(r));
  return 0.0f;
}
inline float bell_int(float t, float r) {
  if (t <= 0.0f) return 0.0f;
  if (t < r) return float(double(t / r) - std::sin(2 * PI * double(t) / double(r)) / (2.0 * PI));
  return 1.0f;
}
inline float triangle(float t, float r) {
  const float t0 = r / 2.0f;
  if (t > r) return 0.0f;
  if (t > t0) return 2.0f / t0 - t / (t0 * t0);
  if (t > 0.0f) return t / (t0 * t0);
  return 0.0f;
}

// src_stf (mod_src.F90:464-487)
inline bool stf(float t, float t0, float f0, int id, int ntime, float stept, float* out) {
  switch (id) {
    case 220: *out = gauss(t, f0, t0); return true;
    case 200: *out = ricker(t, f0, t0); return true;
    case 230: *out = bell(t - t0, f0); return true;
    case 100: *out = bell_int(t - t0, f0); return true;
    case 240: *out = 1.0f; return true;
    case 250: *out = ntime == 0 ? 1.0f / stept : 0.0f; return true;
    default: return false;
  }
}
// src_svf (mod_src.F90:438-463)
inline bool svf(float t, float t0, float f0, int id, int ntime, float stept, float* out) {
  float r;
  switch (id) {
    case 120: r = gauss(t, f0, t0); break;
    case 220: r = gauss_deriv(t, f0, t0); break;
    case 200: r = ricker_deriv(t, f0, t0); break;
    case 100: r = bell(t - t0, f0); break;
    case 230: r = bell_deriv(t - t0, f0); break;
    case 110: r = triangle(t - t0, f0); break;
    case 240: r = ntime == 0 ? 1.0f / stept : 0.0f; break;
    default: return false;
  }
  if (std::fabs(r) < 1.0e-20f) r = 0.0f;
  *out = r;
  return true;
}

// cal_norm_delt (mod_src.F90:419-437): 7^3 separable Gaussian, radius 1.5 cells,
// index (li+3) + 7*((lj+3) + 7*(lk+3)).
inline bool norm_delt(float* d, float x0, float y0, float z0) {
  int n = 0;
  for (int k = -3; k <= 3; ++k)
    for (int j = -3; j <= 3; ++j)
      for (int i = -3; i <= 3; ++i)
        d[n++] = gauss(float(i) - x0, 1.5f, 0.0f) * gauss(float(j) - y0, 1.5f, 0.0f) *
                 gauss(float(k) - z0, 1.5f, 0.0f);
  float s = 0.0f;
  for (int q = 0; q < 343; ++q) s += d[q];
  if (s < 1.0e-20f) return false;
  for (int q = 0; q < 343; ++q) d[q] = d[q] / s;
  return true;
}

// CFS-PML profiles (mod_abs_npml.F90:9070-9124).  The exponents are the integer
// parameters CONSPD = CONSPB = 2 and CONSPA = 1.
inline float pml_dmax(float L, float Vp, float R) { return -((((Vp / 2.0f) / L) * std::log(R)) * 3.0f); }
inline float pml_d(float x, float L, float dmax) {
  if (x < 0.0f) return 0.0f;
  const float q = x / L;
  return dmax * (q * q);
}
inline float pml_a(float x, float L, float amax) {
  if (x < 0.0f) return 0.0f;
  return amax * (1.0f - (x / L));
}
inline float pml_b(float x, float L, float bmax) {
  if (x < 0.0f) return 1.0f;
  const float q = x / L;
  return 1.0f + (bmax - 1.0f) * (q * q);
}
inline float pml_R(int n) {
  return float(std::pow(10.0, -(std::log10(double(n)) - 1.0) / std::log10(2.0) - 3.0));
}

}  // namespace hm
}  // namespace fw
