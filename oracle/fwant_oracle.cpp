// ORACLE — test infrastructure, never the product.
//
// CPU restatement of the FWANT forward solver `seis3d_wave` (LDDRK4 velocity-stress
// finite differences in spherical coordinates) in the reference's build configuration
// (cpp flags STATIC USEPML SrcSmooth SrcSurface CondFreeTIMG CondFreeVLOW, WATER on).
// Only the tests, `__graft_entry__.smoke()` and the `cpu_baseline` leg of `bench.py`
// load this library, and only as the checker.
//
// Parity status: the reference (Fortran 90 + MPI + NetCDF) cannot be compiled in this
// environment and ships no golden vectors, so this restatement follows the source text
// line by line (citations below) and is pinned by known-answer tests of its primitives
// and by physics checks: "parity unpinned" against reference outputs.
//
// The solver is templated on the real kind T: float reproduces the reference's
// single-precision build, double its `-DDataTypeDouble` build (the FP64 oracle run).
// Every expression keeps the reference's operand order and association so that the
// float instantiation rounds the way the Fortran source says it does.  Build with
// -ffp-contract=off.
//
// Array layout: Fortran column-major (nx1:nx2, ny1:ny2, nz1:nz2) with 1-based indices,
// LenFD=3 ghost cells on every side (code/srcF/mod_para.F90:79-82).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

constexpr int LenFD = 3;
constexpr double PI_DP = 3.141592653589793;  // constants_mod PI (mod_constants.F90:27)

// Source time function ids (mod_src.F90:48-57).
enum {
  SIG_SVF_BELL = 100, SIG_SVF_TRIANGLE = 110, SIG_SVF_GAUSS = 120,
  SIG_STF_RICKER = 200, SIG_STF_BSHIFT = 210, SIG_STF_GAUSS = 220,
  SIG_STF_BELL = 230, SIG_STF_STEP = 240, SIG_STF_DELTA = 250
};

// Field order used at the C boundary: the receiver output order of io_seismo_put
// (mod_io.F90:461-497): Vx Vy Vz Txx Tyy Tzz Txy Txz Tyz.
enum { VX = 0, VY, VZ, TXX, TYY, TZZ, TXY, TXZ, TYZ, NF };

template <class T> struct Coef;
// DRP/opt MacCormack weights (mod_macdrp.h:19), 2-4 and 2-2 MacCormack weights
// (mod_macdrp.h:230,250), classical RK4 weights (mod_macdrp.h:39-40).
template <> struct Coef<float> {
  static constexpr float MCA_1 = -0.30874f, MCA0 = -0.6326f, MCA1 = 1.233f,
                         MCA2 = -0.3334f, MCA3 = 0.04168f;
  static float A24_0() { return -7.0f / 6.0f; }
  static float A24_1() { return 8.0f / 6.0f; }
  static float A24_2() { return -1.0f / 6.0f; }
  static constexpr float A22_0 = -1.0f, A22_1 = 1.0f;
  static float rkb(int s) {
    const float v[4] = {1.0f / 6.0f, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 6.0f};
    return v[s];
  }
  static float rka(int s) {
    const float v[4] = {0.5f, 0.5f, 1.0f, 0.0f};
    return v[s];
  }
};
template <> struct Coef<double> {
  static constexpr double MCA_1 = -0.30874, MCA0 = -0.6326, MCA1 = 1.233, MCA2 = -0.3334,
                          MCA3 = 0.04168;
  static double A24_0() { return -7.0 / 6.0; }
  static double A24_1() { return 8.0 / 6.0; }
  static double A24_2() { return -1.0 / 6.0; }
  static constexpr double A22_0 = -1.0, A22_1 = 1.0;
  static double rkb(int s) {
    const double v[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    return v[s];
  }
  static double rka(int s) {
    const double v[4] = {0.5, 0.5, 1.0, 0.0};
    return v[s];
  }
};

template <class T> static inline T t_exp(T v) { return std::exp(v); }
template <class T> static inline T t_log(T v) { return std::log(v); }

// ---------------------------------------------------------------------------
// Source time functions, mod_src.F90:438-622.  Mixed-kind expressions follow the
// Fortran promotion rules: anything multiplied by PI (a DP parameter) is evaluated in
// double and rounded back to T on assignment.
// ---------------------------------------------------------------------------
template <class T> T fun_gauss(T t, T a, T t0) {  // mod_src.F90:533-541
  const T SEIS_ZERO = T(1.0e-20f);
  if (std::fabs(t0) >= SEIS_ZERO && (t <= T(0) || t >= T(2) * t0)) return T(0);
  T q = (t - t0) * (t - t0);
  T e = t_exp<T>(-(q / (a * a)));
  return T(double(e) / (std::sqrt(PI_DP) * double(a)));
}
template <class T> T fun_gauss_deriv(T t, T a, T t0) {  // mod_src.F90:542-550
  const T SEIS_ZERO = T(1.0e-20f);
  if (std::fabs(t0) >= SEIS_ZERO && (t <= T(0) || t >= T(2) * t0)) return T(0);
  T q = (t - t0) * (t - t0);
  T e = t_exp<T>(-(q / (a * a)));
  double g = double(e) / (std::sqrt(PI_DP) * double(a));
  return T(g * double(-2 * (t - t0) / (a * a)));
}
template <class T> T fun_ricker(T t, T fc, T t0) {  // mod_src.F90:509-519
  if (t <= T(0)) return T(0);
  T f0 = T(std::sqrt(PI_DP) / 2.0);
  T u = T(double((t - t0) * T(2)) * PI_DP * double(fc));
  T u2 = u * u;
  return ((u2 / T(4) - T(0.5)) * t_exp<T>(-(u2 / T(4)))) * f0;
}
template <class T> T fun_ricker_deriv(T t, T fc, T t0) {  // mod_src.F90:520-530
  if (t <= T(0)) return T(0);
  T f0 = T(std::sqrt(PI_DP) / 2.0);
  T u = T(double((t - t0) * T(2)) * PI_DP * double(fc));
  T u2 = u * u;
  T v = ((u * (T(1.5) - u2 / T(4))) * t_exp<T>(-(u2 / T(4)))) * f0;
  return T(double(v) * PI_DP * double(fc));
}
template <class T> T fun_bell(T t, T riset) {  // mod_src.F90:552-559
  if (t > T(0) && t < riset)
    return T((1.0 - std::cos(2 * PI_DP * double(t) / double(riset))) / double(riset));
  return T(0);
}
template <class T> T fun_bell_deriv(T t, T riset) {  // mod_src.F90:560-567
  if (t > T(0) && t < riset)
    return T(2.0 * PI_DP * std::sin(2 * PI_DP * double(t) / double(riset)) / double(riset));
  return T(0);
}
template <class T> T fun_bell_int(T t, T riset) {  // mod_src.F90:568-577
  if (t <= T(0)) return T(0);
  if (t < riset)
    return T(double(t / riset) -
             std::sin(2 * PI_DP * double(t) / double(riset)) / (2.0 * PI_DP));
  return T(1);
}
template <class T> T fun_triangle(T t, T riset) {  // mod_src.F90:579-592
  T t0 = riset / T(2);
  if (t > riset) return T(0);
  if (t > t0) return T(2) / t0 - t / (t0 * t0);
  if (t > T(0)) return t / (t0 * t0);
  return T(0);
}
template <class T> T fun_delta(T stept, int ntime) {  // mod_src.F90:617-622
  return ntime == 0 ? T(1) / stept : T(0);
}

// src_stf (mod_src.F90:464-487); returns false on an unknown id (the reference stops).
template <class T> bool src_stf(T t, T t0, T f0, int id, int ntime, T stept, T* out) {
  switch (id) {
    case SIG_STF_GAUSS: *out = fun_gauss<T>(t, f0, t0); return true;
    case SIG_STF_RICKER: *out = fun_ricker<T>(t, f0, t0); return true;
    case SIG_STF_BELL: *out = fun_bell<T>(t - t0, f0); return true;
    case SIG_SVF_BELL: *out = fun_bell_int<T>(t - t0, f0); return true;
    case SIG_STF_STEP: *out = T(1); return true;
    case SIG_STF_DELTA: *out = fun_delta<T>(stept, ntime); return true;
    default: return false;
  }
}
// src_svf (mod_src.F90:438-463)
template <class T> bool src_svf(T t, T t0, T f0, int id, int ntime, T stept, T* out) {
  T r;
  switch (id) {
    case SIG_SVF_GAUSS: r = fun_gauss<T>(t, f0, t0); break;
    case SIG_STF_GAUSS: r = fun_gauss_deriv<T>(t, f0, t0); break;
    case SIG_STF_RICKER: r = fun_ricker_deriv<T>(t, f0, t0); break;
    case SIG_SVF_BELL: r = fun_bell<T>(t - t0, f0); break;
    case SIG_STF_BELL: r = fun_bell_deriv<T>(t - t0, f0); break;
    case SIG_SVF_TRIANGLE: r = fun_triangle<T>(t - t0, f0); break;
    case SIG_STF_STEP: r = fun_delta<T>(stept, ntime); break;
    default: return false;
  }
  if (std::fabs(r) < T(1.0e-20f)) r = T(0);
  *out = r;
  return true;
}

// cal_norm_delt (mod_src.F90:419-437): separable Gaussian weights on the 7^3 box,
// radius LenFD/2 = 1.5 cells, normalised to unit sum.  Index (li,lj,lk) in -3..3,
// stored i fastest.  Returns false when the sum is below SEIS_ZERO (the reference aborts).
template <class T> bool cal_norm_delt(T* delt, T x0, T y0, T z0, T rx0, T ry0, T rz0) {
  int n = 0;
  for (int k = -LenFD; k <= LenFD; ++k)
    for (int j = -LenFD; j <= LenFD; ++j)
      for (int i = -LenFD; i <= LenFD; ++i) {
        T D1 = fun_gauss<T>(T(i) - x0, rx0, T(0));
        T D2 = fun_gauss<T>(T(j) - y0, ry0, T(0));
        T D3 = fun_gauss<T>(T(k) - z0, rz0, T(0));
        delt[n++] = D1 * D2 * D3;
      }
  T s = T(0);
  for (int q = 0; q < 343; ++q) s += delt[q];
  if (s < T(1.0e-20f)) return false;
  for (int q = 0; q < 343; ++q) delt[q] = delt[q] / s;
  return true;
}

// PML profile functions, mod_abs_npml.F90:9070-9124.  CONSPD and CONSPB are declared
// integer (value 2) and CONSPA integer 1 (mod_abs_npml.F90:88-90), so the powers are
// integer powers.
template <class T> T cal_pml_dmax(T L, T Vp, T Rpp) {
  return -((((Vp / T(2)) / L) * t_log<T>(Rpp)) * (T(2) + T(1)));
}
template <class T> T cal_pml_d(T x, T L, T dmax) {
  if (x < T(0)) return T(0);
  T q = x / L;
  return dmax * (q * q);
}
template <class T> T cal_pml_a(T x, T L, T amax) {
  if (x < T(0)) return T(0);
  return amax * (T(1) - (x / L));
}
template <class T> T cal_pml_b(T x, T L, T bmax) {
  if (x < T(0)) return T(1);
  T q = x / L;
  return T(1) + (bmax - T(1)) * (q * q);
}
template <class T> T cal_pml_R(int n) {
  return T(std::pow(10.0, -(std::log10(double(n)) - 1.0) / std::log10(2.0) - 3.0));
}

// ---------------------------------------------------------------------------
// The solver.
// ---------------------------------------------------------------------------
template <class T> struct Solver {
  using C = Coef<T>;
  int ni, nj, nk, nx, ny, nz;
  int ni1, ni2, nj1, nj2, nk1, nk2;  // 1-based interior bounds (mod_para.F90:79-81)
  T stept;
  bool freenode;        // top face is the free surface
  bool srcsurface = true;  // -DSrcSurface
  int ntime = 0;        // completed steps
  int cycle_pos = 0;    // position inside the 8-step F/B cycle since the run started
  std::string err;

  std::vector<T> x, y, z, xsin, xcot, xi_x, eta_y, zeta_z;  // 1-D, index 1..n (slot 0 unused)
  std::vector<T> lam, mu, rho;
  std::vector<T> W[NF], H[NF], M[NF], R[NF];  // wavefield, rhs, RK "m" and "t" registers
  std::vector<T> TxSrc, TySrc, TzSrc, VxSrc, VySrc, VzSrc;  // (nx,ny)

  // PML (abs_mod)
  int absn[6] = {0, 0, 0, 0, 0, 0};  // x1 x2 y1 y2 z1 z2
  std::vector<T> Ax, Bx, Dx, Ay, By, Dy, Az, Bz, Dz;
  struct Slab {
    bool on = false;
    int i1, i2, j1, j2, k1, k2;
    std::vector<T> v[6], h[6], m[6], t[6];
    size_t id(int i, int j, int k) const {
      return size_t(i - i1) + size_t(i2 - i1 + 1) * (size_t(j - j1) + size_t(j2 - j1 + 1) * size_t(k - k1));
    }
    size_t size() const { return size_t(i2 - i1 + 1) * (j2 - j1 + 1) * (k2 - k1 + 1); }
  } slab[6];

  // sources (src_mod)
  int num_force = 0, ntwin_force = 0, frcstf_id = SIG_STF_RICKER;
  std::vector<int> force_indx;  // 3*num
  std::vector<T> force_shift, force_t0, frcstf_time, frcstf_freq, ForceX, ForceY, ForceZ;
  int num_moment = 0, ntwin_moment = 0, momstf_id = SIG_STF_RICKER;
  std::vector<int> moment_indx;
  std::vector<T> moment_shift, moment_t0, momstf_time, momstf_freq, MomTxx, MomTyy, MomTzz,
      MomTxy, MomTxz, MomTyz;

  // receivers (io_mod)
  int num_pt = 0, pt_tinv = 1;
  std::vector<int> pt_indx;
  std::vector<T> seismo;  // [var][sample][pt]
  int nsamp = 0, nsamp_cap = 0;

  // Gaussian-hill extension (no counterpart in the reference, whose grid is orthogonal
  // spherical with a flat top): terrain-following radius r(i,j,k) = z(k) + h(i,j) s(k),
  // s(k) = (z(k) - z(1)) / (z(nk2) - z(1)), so the free surface k = nk2 follows h and the
  // bottom of the grid stays flat.
  bool topo_on = false, topo_bc_dirty = true;
  std::vector<double> topo_h, topo_hx, topo_hy;  // (nx,ny): heights (m), d/dxi, d/deta
  std::vector<T> t_r, t_az, t_bx, t_by;  // (nx,ny,nz): r, zeta_r, zeta_theta / r, zeta_phi / (r sin theta)
  std::vector<T> t_m1, t_m2, t_minv;     // (nx,ny): surface normal / its radial part; 3x3 inverse (x 9)
  std::vector<unsigned char> t_slope;    // (nx,ny): the column's surface has a non-zero slope

  size_t id(int i, int j, int k) const {
    return size_t(i - 1) + size_t(nx) * (size_t(j - 1) + size_t(ny) * size_t(k - 1));
  }
  size_t id2(int i, int j) const { return size_t(i - 1) + size_t(nx) * size_t(j - 1); }

  Solver(int ni_, int nj_, int nk_, T stept_, bool freenode_)
      : ni(ni_), nj(nj_), nk(nk_), stept(stept_), freenode(freenode_) {
    ni1 = 1 + LenFD; ni2 = ni1 + ni - 1; nx = ni2 + LenFD;
    nj1 = 1 + LenFD; nj2 = nj1 + nj - 1; ny = nj2 + LenFD;
    nk1 = 1 + LenFD; nk2 = nk1 + nk - 1; nz = nk2 + LenFD;
    size_t n3 = size_t(nx) * ny * nz;
    for (int f = 0; f < NF; ++f) {
      W[f].assign(n3, T(0)); H[f].assign(n3, T(0)); M[f].assign(n3, T(0)); R[f].assign(n3, T(0));
    }
    lam.assign(n3, T(0)); mu.assign(n3, T(0)); rho.assign(n3, T(1));
    x.assign(nx + 1, T(0)); y.assign(ny + 1, T(0)); z.assign(nz + 1, T(0));
    xsin.assign(nx + 1, T(0)); xcot.assign(nx + 1, T(0)); xi_x.assign(nx + 1, T(0));
    eta_y.assign(ny + 1, T(0)); zeta_z.assign(nz + 1, T(0));
    size_t n2 = size_t(nx) * ny;
    TxSrc.assign(n2, T(0)); TySrc.assign(n2, T(0)); TzSrc.assign(n2, T(0));
    VxSrc.assign(n2, T(0)); VySrc.assign(n2, T(0)); VzSrc.assign(n2, T(0));
    Ax.assign(nx + 1, T(0)); Bx.assign(nx + 1, T(1)); Dx.assign(nx + 1, T(0));
    Ay.assign(ny + 1, T(0)); By.assign(ny + 1, T(1)); Dy.assign(ny + 1, T(0));
    Az.assign(nz + 1, T(0)); Bz.assign(nz + 1, T(1)); Dz.assign(nz + 1, T(0));
  }

  // abs_init (mod_abs_npml.F90:135-616) for the isotropic build.
  bool set_pml(const int* number, const double* vel, const double* bmax_in, const double* amax_in) {
    for (int f = 0; f < 6; ++f) absn[f] = number[f] > 0 ? number[f] : 0;
    T Rpp[6], dmax[6], Vs[6], bmax[6], amax[6];
    for (int f = 0; f < 6; ++f) {
      Vs[f] = T(vel[f]); bmax[f] = T(bmax_in[f]); amax[f] = T(amax_in[f]);
      if (absn[f] > 0) {
        if (bmax[f] < T(1)) { err = "CFS_bmax should be large or equal to 1"; return false; }
        Rpp[f] = cal_pml_R<T>(absn[f]);
      }
    }
    if (absn[5] > 0 && freenode) freenode = false;  // mod_abs_npml.F90:182-184
    if (absn[0] > 0) {
      T x0 = x[absn[0] + ni1];
      T L0 = z[nk2] * (x0 - x[ni1]);
      dmax[0] = cal_pml_dmax<T>(L0, Vs[0], Rpp[0]);
      for (int i = ni1; i <= absn[0] + ni1; ++i) {
        T Lx = z[nk2] * (x0 - x[i]);
        Dx[i] = cal_pml_d<T>(Lx, L0, dmax[0]); Ax[i] = cal_pml_a<T>(Lx, L0, amax[0]);
        Bx[i] = cal_pml_b<T>(Lx, L0, bmax[0]);
      }
    }
    if (absn[1] > 0) {
      T x0 = x[ni2 - absn[1]];
      T L0 = z[nk2] * (x[ni2] - x0);
      dmax[1] = cal_pml_dmax<T>(L0, Vs[1], Rpp[1]);
      for (int i = ni2 - absn[1]; i <= ni2; ++i) {
        T Lx = z[nk2] * (x[i] - x0);
        Dx[i] = cal_pml_d<T>(Lx, L0, dmax[1]); Ax[i] = cal_pml_a<T>(Lx, L0, amax[1]);
        Bx[i] = cal_pml_b<T>(Lx, L0, bmax[1]);
      }
    }
    if (absn[2] > 0) {
      T y0 = y[absn[2] + nj1];
      T L0 = z[nk2] * (y0 - y[nj1]);
      dmax[2] = cal_pml_dmax<T>(L0, Vs[2], Rpp[2]);
      for (int j = nj1; j <= absn[2] + nj1; ++j) {
        T Ly = z[nk2] * (y0 - y[j]);
        Dy[j] = cal_pml_d<T>(Ly, L0, dmax[2]); Ay[j] = cal_pml_a<T>(Ly, L0, amax[2]);
        By[j] = cal_pml_b<T>(Ly, L0, bmax[2]);
      }
    }
    if (absn[3] > 0) {
      T y0 = y[nj2 - absn[3]];
      T L0 = z[nk2] * (y[nj2] - y0);
      dmax[3] = cal_pml_dmax<T>(L0, Vs[3], Rpp[3]);
      for (int j = nj2 - absn[3]; j <= nj2; ++j) {
        T Ly = z[nk2] * (y[j] - y0);
        Dy[j] = cal_pml_d<T>(Ly, L0, dmax[3]); Ay[j] = cal_pml_a<T>(Ly, L0, amax[3]);
        By[j] = cal_pml_b<T>(Ly, L0, bmax[3]);
      }
    }
    if (absn[4] > 0) {
      T z0 = z[absn[4] + nk1];
      T L0 = z0 - z[nk1];
      dmax[4] = cal_pml_dmax<T>(L0, Vs[4], Rpp[4]);
      for (int k = nk1; k <= nk1 + absn[4]; ++k) {
        T Lz = z0 - z[k];
        Dz[k] = cal_pml_d<T>(Lz, L0, dmax[4]); Az[k] = cal_pml_a<T>(Lz, L0, amax[4]);
        Bz[k] = cal_pml_b<T>(Lz, L0, bmax[4]);
      }
    }
    if (absn[5] > 0) {
      T z0 = z[nk2 - absn[5]];
      T L0 = z[nk2] - z0;
      dmax[5] = cal_pml_dmax<T>(L0, Vs[5], Rpp[5]);
      for (int k = nk2 - absn[5]; k <= nk2; ++k) {
        T Lz = z[k] - z0;
        Dz[k] = cal_pml_d<T>(Lz, L0, dmax[5]); Az[k] = cal_pml_a<T>(Lz, L0, amax[5]);
        Bz[k] = cal_pml_b<T>(Lz, L0, bmax[5]);
      }
    }
    for (int i = 1; i <= nx; ++i) Dx[i] = Dx[i] / Bx[i];  // mod_abs_npml.F90:282-284
    for (int j = 1; j <= ny; ++j) Dy[j] = Dy[j] / By[j];
    for (int k = 1; k <= nz; ++k) Dz[k] = Dz[k] / Bz[k];
    // slab extents (mod_abs_npml.F90:286-470)
    const int b[6][6] = {
        {ni1, ni1 + absn[0], nj1, nj2, nk1, nk2}, {ni2 - absn[1], ni2, nj1, nj2, nk1, nk2},
        {ni1, ni2, nj1, nj1 + absn[2], nk1, nk2}, {ni1, ni2, nj2 - absn[3], nj2, nk1, nk2},
        {ni1, ni2, nj1, nj2, nk1, nk1 + absn[4]}, {ni1, ni2, nj1, nj2, nk2 - absn[5], nk2}};
    for (int f = 0; f < 6; ++f) {
      Slab& s = slab[f];
      s.on = absn[f] > 0;
      if (!s.on) continue;
      s.i1 = b[f][0]; s.i2 = b[f][1]; s.j1 = b[f][2]; s.j2 = b[f][3]; s.k1 = b[f][4]; s.k2 = b[f][5];
      for (int q = 0; q < 6; ++q) {
        s.v[q].assign(s.size(), T(0)); s.h[q].assign(s.size(), T(0));
        s.m[q].assign(s.size(), T(0)); s.t[q].assign(s.size(), T(0));
      }
    }
    return true;
  }

  // -------------------------------------------------------------------------
  // One-sided operators, mod_macdrp.h:69-103 (DRP/opt), :230-248 (2-4), :250-268 (2-2).
  // F(f)(i) = MCA_1 f(i-1)+MCA0 f(i)+MCA1 f(i+1)+MCA2 f(i+2)+MCA3 f(i+3)
  // B(f)(i) = -MCA3 f(i-3)-MCA2 f(i-2)-MCA1 f(i-1)-MCA0 f(i)-MCA_1 f(i+1)
  // -------------------------------------------------------------------------
  static T opF(const T* p, ptrdiff_t s) {
    return C::MCA_1 * p[-s] + C::MCA0 * p[0] + C::MCA1 * p[s] + C::MCA2 * p[2 * s] + C::MCA3 * p[3 * s];
  }
  static T opB(const T* p, ptrdiff_t s) {
    return -C::MCA3 * p[-3 * s] - C::MCA2 * p[-2 * s] - C::MCA1 * p[-s] - C::MCA0 * p[0] - C::MCA_1 * p[s];
  }
  static T op(bool fwd, const T* p, ptrdiff_t s) { return fwd ? opF(p, s) : opB(p, s); }
  static T op22(bool fwd, const T* p, ptrdiff_t s) {
    return fwd ? (C::A22_0 * p[0] + C::A22_1 * p[s]) : (-C::A22_1 * p[-s] - C::A22_0 * p[0]);
  }
  static T op24(bool fwd, const T* p, ptrdiff_t s) {
    return fwd ? (C::A24_0() * p[0] + C::A24_1() * p[s] + C::A24_2() * p[2 * s])
               : (-C::A24_2() * p[-2 * s] - C::A24_1() * p[-s] - C::A24_0() * p[0]);
  }

  // macdrp_syn (mod_macdrp.F90:268-288) and abs_syn (mod_abs_npml.F90:641-736)
  void syn() {
#pragma omp parallel for schedule(static)
    for (int k = nk1; k <= nk2; ++k)
      for (int j = nj1; j <= nj2; ++j)
        for (int i = ni1; i <= ni2; ++i) {
          size_t p = id(i, j, k);
          for (int f = 0; f < NF; ++f) M[f][p] = W[f][p];
        }
    for (int s = 0; s < 6; ++s)
      if (slab[s].on)
        for (int q = 0; q < 6; ++q) slab[s].m[q] = slab[s].v[q];
  }

  // free_timg (mod_macdrp.F90:3414-3436)
  void free_timg() {
    if (!freenode) return;
    for (int m = 1; m <= 3; ++m)
      for (int j = nj1; j <= nj2; ++j)
        for (int i = ni1; i <= ni2; ++i) {
          size_t q = id2(i, j);
          W[TZZ][id(i, j, nk2 + m)] = T(2) * TzSrc[q] - W[TZZ][id(i, j, nk2 - m)];
          W[TXZ][id(i, j, nk2 + m)] = T(2) * TxSrc[q] - W[TXZ][id(i, j, nk2 - m)];
          W[TYZ][id(i, j, nk2 + m)] = T(2) * TySrc[q] - W[TYZ][id(i, j, nk2 - m)];
        }
    for (int j = nj1; j <= nj2; ++j)
      for (int i = ni1; i <= ni2; ++i) {
        size_t q = id2(i, j);
        W[TZZ][id(i, j, nk2)] = TzSrc[q];
        W[TXZ][id(i, j, nk2)] = TxSrc[q];
        W[TYZ][id(i, j, nk2)] = TySrc[q];
      }
  }

  // L<X> stencil kernels (mod_macdrp.F90:790-962 and the seven mirrored copies; the
  // eight differ only in the F/B choice per axis).  On one domain the interior box plus
  // the six boundary boxes of the wrapper (mod_macdrp.F90:425-469) tile
  // ni1:ni2 x nj1:nj2 x nk1:nk2, so a single loop covers them.
  void stencil(bool fx, bool fy, bool fz) {
    const ptrdiff_t sx = 1, sy = nx, sz = ptrdiff_t(nx) * ny;
#pragma omp parallel for schedule(static)
    for (int k = nk1; k <= nk2; ++k)
      for (int j = nj1; j <= nj2; ++j)
        for (int i = ni1; i <= ni2; ++i) {
          size_t p = id(i, j, k);
          T lam_ = lam[p], miu = mu[p];
          T lam2mu = lam_ + T(2) * miu;
          T rrho = T(1) / rho[p];
          const T xi = xi_x[i], et = eta_y[j], ze = zeta_z[k];
          T DxTxx = op(fx, &W[TXX][p], sx) * xi;
          T DxTxy = op(fx, &W[TXY][p], sx) * xi;
          T DxTxz = op(fx, &W[TXZ][p], sx) * xi;
          T DxVx = op(fx, &W[VX][p], sx) * xi;
          T DxVy = op(fx, &W[VY][p], sx) * xi;
          T DxVz = op(fx, &W[VZ][p], sx) * xi;
          T DyTyy = op(fy, &W[TYY][p], sy) * et;
          T DyTxy = op(fy, &W[TXY][p], sy) * et;
          T DyTyz = op(fy, &W[TYZ][p], sy) * et;
          T DyVx = op(fy, &W[VX][p], sy) * et;
          T DyVy = op(fy, &W[VY][p], sy) * et;
          T DyVz = op(fy, &W[VZ][p], sy) * et;
          T DzTzz = op(fz, &W[TZZ][p], sz) * ze;
          T DzTxz = op(fz, &W[TXZ][p], sz) * ze;
          T DzTyz = op(fz, &W[TYZ][p], sz) * ze;
          T DzVx, DzVy, DzVz;
          if (freenode && k == nk2 - 1) {  // CondFreeVLOW, mod_macdrp.F90:872-915
            DzVx = op22(fz, &W[VX][p], sz) * ze;
            DzVy = op22(fz, &W[VY][p], sz) * ze;
            DzVz = op22(fz, &W[VZ][p], sz) * ze;
          } else if (freenode && k == nk2 - 2) {
            DzVx = op24(fz, &W[VX][p], sz) * ze;
            DzVy = op24(fz, &W[VY][p], sz) * ze;
            DzVz = op24(fz, &W[VZ][p], sz) * ze;
          } else {
            DzVx = op(fz, &W[VX][p], sz) * ze;
            DzVy = op(fz, &W[VY][p], sz) * ze;
            DzVz = op(fz, &W[VZ][p], sz) * ze;
          }
          if (miu <= T(1.0e-20f)) {  // WATER, mod_macdrp.F90:917-926
            DxTxy = T(0); DxTxz = T(0); DyTxy = T(0); DyTyz = T(0); DzTxz = T(0); DzTyz = T(0);
          }
          const T r = z[k], s = xsin[i], c = xcot[i];
          const T Txx = W[TXX][p], Tyy = W[TYY][p], Tzz = W[TZZ][p];
          const T Txy = W[TXY][p], Txz = W[TXZ][p], Tyz = W[TYZ][p];
          const T Vx = W[VX][p], Vy = W[VY][p], Vz = W[VZ][p];
          // mod_macdrp.F90:928-933
          H[VX][p] = rrho * (DxTxx / r + DyTxy / r / s + DzTxz + (T(3) * Txz + Txx * c - Tyy * c) / r);
          H[VY][p] = rrho * (DxTxy / r + DyTyy / r / s + DzTyz + (T(2) * Txy * c + T(3) * Tyz) / r);
          H[VZ][p] = rrho * (DxTxz / r + DyTyz / r / s + DzTzz + (T(2) * Tzz - Txx - Tyy + Txz * c) / r);
          // mod_macdrp.F90:935-941
          T E11 = (DxVx + Vz) / r;
          T E22 = (Vx * c + DyVy / s + Vz) / r;
          T E12 = (DxVy + DyVx / s - Vy * c) / r / T(2);
          T E33 = DzVz;
          T E13 = (DxVz / r + DzVx - Vx / r) / T(2);
          T E23 = (DyVz / r / s + DzVy - Vy / r) / T(2);
          if (freenode && k == nk2) {  // mod_macdrp.F90:944-948
            size_t q = id2(i, j);
            E33 = -(lam_ / lam2mu * (E11 + E22)) + VzSrc[q] / lam2mu;
            E13 = VxSrc[q] / miu / T(2);
            E23 = VySrc[q] / miu / T(2);
          }
          // mod_macdrp.F90:952-957
          H[TXX][p] = lam2mu * E11 + lam_ * (E22 + E33);
          H[TYY][p] = lam2mu * E22 + lam_ * (E11 + E33);
          H[TZZ][p] = lam2mu * E33 + lam_ * (E11 + E22);
          H[TXY][p] = T(2) * miu * E12;
          H[TXZ][p] = T(2) * miu * E13;
          H[TYZ][p] = T(2) * miu * E23;
        }
  }

  // abs_vsymm (mod_abs_npml.F90:9014-9067): antisymmetric velocity ghosts above the
  // free surface inside the x/y PML columns.  No stencil reads these ghosts under the
  // free surface, but they are part of the state.
  void abs_vsymm() {
    if (!freenode) return;
    for (int s = 0; s < 4; ++s) {
      if (!slab[s].on) continue;
      const Slab& sl = slab[s];
      for (int j = sl.j1; j <= sl.j2; ++j)
        for (int i = sl.i1; i <= sl.i2; ++i)
          for (int m = 1; m <= LenFD; ++m)
            for (int f = VX; f <= VZ; ++f)
              W[f][id(i, j, nk2 + m)] = T(2) * W[f][id(i, j, nk2)] - W[f][id(i, j, nk2 - m)];
    }
  }

  // abs_L<X> (mod_abs_npml.F90:1149-2123 and mirrored copies), isotropic branch.
  void abs_stencil(bool fx, bool fy, bool fz) {
    abs_vsymm();
    const ptrdiff_t sx = 1, sy = nx, sz = ptrdiff_t(nx) * ny;
    for (int sidx = 0; sidx < 6; ++sidx) {
      Slab& sl = slab[sidx];
      if (!sl.on) continue;
      const int axis = sidx / 2;
#pragma omp parallel for schedule(static)
      for (int k = sl.k1; k <= sl.k2; ++k)
        for (int j = sl.j1; j <= sl.j2; ++j)
          for (int i = sl.i1; i <= sl.i2; ++i) {
            size_t p = id(i, j, k);
            size_t a = sl.id(i, j, k);
            T rrho = T(1) / rho[p];
            T Bv = axis == 0 ? Bx[i] : axis == 1 ? By[j] : Bz[k];
            T Av = axis == 0 ? Ax[i] : axis == 1 ? Ay[j] : Az[k];
            T Dv = axis == 0 ? Dx[i] : axis == 1 ? Dy[j] : Dz[k];
            T b1 = T(1) / Bv;
            T b1_1 = b1 - T(1);
            T ad = Av + Dv;
            const T r = topo_on ? t_r[p] : z[k], s = xsin[i], c = xcot[i];
            const T Txx = W[TXX][p], Tyy = W[TYY][p], Tzz = W[TZZ][p];
            const T Txy = W[TXY][p], Txz = W[TXZ][p], Tyz = W[TYZ][p];
            const T Vx = W[VX][p], Vy = W[VY][p], Vz = W[VZ][p];
            // isotropic stiffness (mod_abs_npml.F90:1230-1240)
            T tc13 = lam[p], tc66 = mu[p];
            T tc11 = tc13 + T(2) * tc66;
            T tc12 = tc13, tc22 = tc11, tc23 = tc13, tc33 = tc11, tc44 = tc66, tc55 = tc66;
            T d0, d1, d2, d3, d4, d5;  // stress derivs for hVx,hVy,hVz; velocity derivs Vx,Vy,Vz
            if (axis == 0) {
              const T xi = xi_x[i];
              d0 = op(fx, &W[TXX][p], sx) * xi; d0 = (d0 + T(2) * Txz) / r;
              d1 = op(fx, &W[TXY][p], sx) * xi; d1 = (d1 + Tyz) / r;
              d2 = op(fx, &W[TXZ][p], sx) * xi; d2 = (d2 - Txx + Tzz) / r;
              d3 = op(fx, &W[VX][p], sx) * xi; d3 = (d3 + Vz) / r;
              d4 = op(fx, &W[VY][p], sx) * xi; d4 = d4 / r;
              d5 = op(fx, &W[VZ][p], sx) * xi; d5 = (d5 - Vx) / r;
            } else if (axis == 1) {
              const T et = eta_y[j];
              d0 = op(fy, &W[TXY][p], sy) * et; d0 = (d0 / s + (Txx - Tyy) * c + Txz) / r;
              d1 = op(fy, &W[TYY][p], sy) * et; d1 = (d1 / s + T(2) * Txy * c + T(2) * Tyz) / r;
              d2 = op(fy, &W[TYZ][p], sy) * et; d2 = (d2 / s + Txz * c + (Tzz - Tyy)) / r;
              d3 = op(fy, &W[VX][p], sy) * et; d3 = (d3 / s - Vy * c) / r;
              d4 = op(fy, &W[VY][p], sy) * et; d4 = (d4 / s + Vx * c + Vz) / r;
              d5 = op(fy, &W[VZ][p], sy) * et; d5 = (d5 / s - Vy) / r;
            } else {
              const T ze = topo_on ? t_az[p] : zeta_z[k];
              d0 = op(fz, &W[TXZ][p], sz) * ze;
              d1 = op(fz, &W[TYZ][p], sz) * ze;
              d2 = op(fz, &W[TZZ][p], sz) * ze;
              d3 = op(fz, &W[VX][p], sz) * ze;
              d4 = op(fz, &W[VY][p], sz) * ze;
              d5 = op(fz, &W[VZ][p], sz) * ze;
            }
            // velocity equations: aux 0..2
            H[VX][p] = H[VX][p] + (b1_1 * d0 - b1 * sl.v[0][a]) * rrho;
            sl.h[0][a] = Dv * d0 - ad * sl.v[0][a];
            H[VY][p] = H[VY][p] + (b1_1 * d1 - b1 * sl.v[1][a]) * rrho;
            sl.h[1][a] = Dv * d1 - ad * sl.v[1][a];
            H[VZ][p] = H[VZ][p] + (b1_1 * d2 - b1 * sl.v[2][a]) * rrho;
            sl.h[2][a] = Dv * d2 - ad * sl.v[2][a];
            const T av3 = sl.v[3][a], av4 = sl.v[4][a], av5 = sl.v[5][a];
            if (axis == 0) {
              H[TXX][p] = H[TXX][p] + b1_1 * tc11 * d3 - b1 * tc11 * av3;
              H[TYY][p] = H[TYY][p] + b1_1 * tc12 * d3 - b1 * tc12 * av3;
              H[TZZ][p] = H[TZZ][p] + b1_1 * tc13 * d3 - b1 * tc13 * av3;
              sl.h[3][a] = Dv * d3 - ad * av3;
              H[TXY][p] = H[TXY][p] + b1_1 * tc66 * d4 - b1 * tc66 * av4;
              sl.h[4][a] = Dv * d4 - ad * av4;
              H[TXZ][p] = H[TXZ][p] + b1_1 * tc55 * d5 - b1 * tc55 * av5;
              sl.h[5][a] = Dv * d5 - ad * av5;
              if (freenode && k == nk2) {  // mod_abs_npml.F90:1303-1333
                H[TXX][p] = H[TXX][p] - b1_1 * tc13 * tc13 / tc33 * d3 + b1 * tc13 * tc13 / tc33 * av3;
                H[TYY][p] = H[TYY][p] - b1_1 * tc23 * tc13 / tc33 * d3 + b1 * tc23 * tc13 / tc33 * av3;
              }
            } else if (axis == 1) {
              H[TXY][p] = H[TXY][p] + b1_1 * tc66 * d3 - b1 * tc66 * av3;
              sl.h[3][a] = Dv * d3 - ad * av3;
              H[TXX][p] = H[TXX][p] + b1_1 * tc12 * d4 - b1 * tc12 * av4;
              H[TYY][p] = H[TYY][p] + b1_1 * tc22 * d4 - b1 * tc22 * av4;
              H[TZZ][p] = H[TZZ][p] + b1_1 * tc23 * d4 - b1 * tc23 * av4;
              sl.h[4][a] = Dv * d4 - ad * av4;
              H[TYZ][p] = H[TYZ][p] + b1_1 * tc44 * d5 - b1 * tc44 * av5;
              sl.h[5][a] = Dv * d5 - ad * av5;
              if (freenode && k == nk2) {  // mod_abs_npml.F90:1647-1677
                H[TXX][p] = H[TXX][p] - b1_1 * tc13 * tc23 / tc33 * d4 + b1 * tc13 * tc23 / tc33 * av4;
                H[TYY][p] = H[TYY][p] - b1_1 * tc23 * tc23 / tc33 * d4 + b1 * tc23 * tc23 / tc33 * av4;
              }
            } else {
              H[TXZ][p] = H[TXZ][p] + b1_1 * tc55 * d3 - b1 * tc55 * av3;
              sl.h[3][a] = Dv * d3 - ad * av3;
              H[TYZ][p] = H[TYZ][p] + b1_1 * tc44 * d4 - b1 * tc44 * av4;
              sl.h[4][a] = Dv * d4 - ad * av4;
              H[TXX][p] = H[TXX][p] + b1_1 * tc13 * d5 - b1 * tc13 * av5;
              H[TYY][p] = H[TYY][p] + b1_1 * tc23 * d5 - b1 * tc23 * av5;
              H[TZZ][p] = H[TZZ][p] + b1_1 * tc33 * d5 - b1 * tc33 * av5;
              sl.h[5][a] = Dv * d5 - ad * av5;
            }
          }
    }
  }

  // src_surface (mod_src.F90:373-414)
  bool src_surface(T tinc) {
    if (!freenode || num_force <= 0) return true;
    T t = (T(ntime) + tinc) * stept;
    for (int n = 0; n < num_force; ++n) {
      int i = force_indx[3 * n], j = force_indx[3 * n + 1], k = force_indx[3 * n + 2];
      for (int m = 0; m < ntwin_force; ++m) {
        T disp, rate;
        if (!src_stf<T>(t - force_t0[n], frcstf_time[m], frcstf_freq[m], frcstf_id, ntime, stept, &disp) ||
            !src_svf<T>(t - force_t0[n], frcstf_time[m], frcstf_freq[m], frcstf_id, ntime, stept, &rate)) {
          err = "unknown force stf id"; return false;
        }
        T fx0 = ForceX[m + ntwin_force * n], fy0 = ForceY[m + ntwin_force * n], fz0 = ForceZ[m + ntwin_force * n];
        if (i <= ni2 && i >= ni1 && j <= nj2 && j >= nj1 && k == nk2) {
          T S = (x[i + 1] - x[i - 1]) * (y[j + 1] - y[j - 1]) / T(4) * (z[k] * z[k]) * xsin[i];
          size_t q = id2(i, j);
          TxSrc[q] = fx0 / S * disp; TySrc[q] = fy0 / S * disp; TzSrc[q] = fz0 / S * disp;
          VxSrc[q] = fx0 / S * rate; VySrc[q] = fy0 / S * rate; VzSrc[q] = fz0 / S * rate;
        }
      }
    }
    return true;
  }

  // smoothing weights of one source, including the free-surface renormalisation
  // (mod_src.F90:230-236 / 298-304)
  bool norm_delt(T* normd, int sk, T x0, T y0, T z0) {
    if (!cal_norm_delt<T>(normd, x0, y0, z0, T(1.5f), T(1.5f), T(1.5f))) {
      err = "cal_norm_delt is zero"; return false;
    }
    if (freenode && sk + LenFD > nk2) {
      T s = T(0);
      for (int lk = -LenFD; lk <= nk2 - sk; ++lk)
        for (int lj = -LenFD; lj <= LenFD; ++lj)
          for (int li = -LenFD; li <= LenFD; ++li)
            s += normd[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))];
      for (int q = 0; q < 343; ++q) normd[q] = normd[q] / s;
    }
    return true;
  }

  // src_stress (mod_src.F90:207-273)
  bool src_stress(T tinc) {
    if (num_moment <= 0) return true;
    T t = (T(ntime) + tinc) * stept;
    T normd[343];
    for (int n = 0; n < num_moment; ++n) {
      int si = moment_indx[3 * n], sj = moment_indx[3 * n + 1], sk = moment_indx[3 * n + 2];
      if (!norm_delt(normd, sk, moment_shift[3 * n], moment_shift[3 * n + 1], moment_shift[3 * n + 2])) return false;
      for (int m = 0; m < ntwin_moment; ++m) {
        T rate;
        if (!src_svf<T>(t - moment_t0[n], momstf_time[m], momstf_freq[m], momstf_id, ntime, stept, &rate)) {
          err = "unknown moment stf id"; return false;
        }
        size_t w = m + size_t(ntwin_moment) * n;
        T Mxx = MomTxx[w], Myy = MomTyy[w], Mzz = MomTzz[w], Mxy = MomTxy[w], Mxz = MomTxz[w], Myz = MomTyz[w];
        for (int lk = -LenFD; lk <= LenFD; ++lk)
          for (int lj = -LenFD; lj <= LenFD; ++lj)
            for (int li = -LenFD; li <= LenFD; ++li) {
              int i = li + si, j = lj + sj, k = lk + sk;
              T d = normd[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))];
              if (i <= ni2 && i >= ni1 && j <= nj2 && j >= nj1 && k <= nk2 && k >= nk1) {
                T V = (x[i + 1] - x[i - 1]) * (y[j + 1] - y[j - 1]) * (z[k + 1] - z[k - 1]) / T(8) * (z[k] * z[k]) * xsin[i];
                V = d * rate / V;
                size_t p = id(i, j, k);
                H[TXX][p] = H[TXX][p] - Mxx * V; H[TYY][p] = H[TYY][p] - Myy * V;
                H[TZZ][p] = H[TZZ][p] - Mzz * V; H[TXY][p] = H[TXY][p] - Mxy * V;
                H[TXZ][p] = H[TXZ][p] - Mxz * V; H[TYZ][p] = H[TYZ][p] - Myz * V;
              }
            }
      }
    }
    return true;
  }

  // src_force (mod_src.F90:275-345)
  bool src_force(T tinc) {
    if (num_force <= 0) return true;
    T t = (T(ntime) + tinc) * stept;
    T normd[343];
    for (int n = 0; n < num_force; ++n) {
      int si = force_indx[3 * n], sj = force_indx[3 * n + 1], sk = force_indx[3 * n + 2];
      if (!norm_delt(normd, sk, force_shift[3 * n], force_shift[3 * n + 1], force_shift[3 * n + 2])) return false;
      for (int m = 0; m < ntwin_force; ++m) {
        T disp;
        if (!src_stf<T>(t - force_t0[n], frcstf_time[m], frcstf_freq[m], frcstf_id, ntime, stept, &disp)) {
          err = "unknown force stf id"; return false;
        }
        size_t w = m + size_t(ntwin_force) * n;
        T fx0 = ForceX[w] * disp, fy0 = ForceY[w] * disp, fz0 = ForceZ[w] * disp;
        for (int lk = -LenFD; lk <= LenFD; ++lk)
          for (int lj = -LenFD; lj <= LenFD; ++lj)
            for (int li = -LenFD; li <= LenFD; ++li) {
              int i = li + si, j = lj + sj, k = lk + sk;
              T d = normd[(li + 3) + 7 * ((lj + 3) + 7 * (lk + 3))];
              if (i <= ni2 && i >= ni1 && j <= nj2 && j >= nj1 && k <= nk2 && k >= nk1) {
                size_t p = id(i, j, k);
                T V = (x[i + 1] - x[i - 1]) * (y[j + 1] - y[j - 1]) * (z[k + 1] - z[k - 1]) / T(8) * (z[k] * z[k]) * xsin[i];
                V = T(1) / (V * rho[p]) * d;
                T fx = fx0 * V, fy = fy0 * V, fz = fz0 * V;
                if (freenode && k == nk2) {
                  if (srcsurface) continue;
                  fx = T(2) * fx; fy = T(2) * fy; fz = T(2) * fz;
                }
                H[VX][p] = H[VX][p] + fx; H[VY][p] = H[VY][p] + fy; H[VZ][p] = H[VZ][p] + fz;
              }
            }
      }
    }
    return true;
  }

  // macdrp_RK_beg/inn/fin (mod_macdrp.F90:291-393) and abs_RK_* (mod_abs_npml.F90:738-1105)
  void rk(int stage) {
    const T a = C::rka(stage) * stept;  // a = rka*stept (formed in SP)
    const T b = C::rkb(stage) * stept;
#pragma omp parallel for schedule(static)
    for (int k = nk1; k <= nk2; ++k)
      for (int j = nj1; j <= nj2; ++j)
        for (int i = ni1; i <= ni2; ++i) {
          size_t p = id(i, j, k);
          for (int f = 0; f < NF; ++f) {
            if (stage == 0) {
              W[f][p] = M[f][p] + a * H[f][p];
              R[f][p] = M[f][p] + b * H[f][p];
            } else if (stage < 3) {
              W[f][p] = M[f][p] + a * H[f][p];
              R[f][p] = R[f][p] + b * H[f][p];
            } else {
              W[f][p] = R[f][p] + b * H[f][p];
            }
          }
        }
    for (int s = 0; s < 6; ++s) {
      Slab& sl = slab[s];
      if (!sl.on) continue;
      size_t n = sl.size();
      for (int q = 0; q < 6; ++q)
        for (size_t p = 0; p < n; ++p) {
          if (stage == 0) {
            sl.v[q][p] = sl.m[q][p] + a * sl.h[q][p];
            sl.t[q][p] = sl.m[q][p] + b * sl.h[q][p];
          } else if (stage < 3) {
            sl.v[q][p] = sl.m[q][p] + a * sl.h[q][p];
            sl.t[q][p] = sl.t[q][p] + b * sl.h[q][p];
          } else {
            sl.v[q][p] = sl.t[q][p] + b * sl.h[q][p];
          }
        }
    }
  }

  // io_seismo_put (mod_io.F90:461-497): sample after the step counter increments.
  void seismo_put() {
    if (num_pt <= 0) return;
    if (ntime % pt_tinv != 0) return;
    int m = ntime / pt_tinv;  // 1-based sample index
    if (m > nsamp_cap) {
      int cap = std::max(2 * nsamp_cap, m + 64);
      std::vector<T> s2(size_t(NF) * cap * num_pt, T(0));
      for (int v = 0; v < NF; ++v)
        for (int q = 0; q < nsamp_cap; ++q)
          for (int n = 0; n < num_pt; ++n)
            s2[(size_t(v) * cap + q) * num_pt + n] = seismo[(size_t(v) * nsamp_cap + q) * num_pt + n];
      seismo.swap(s2);
      nsamp_cap = cap;
    }
    for (int n = 0; n < num_pt; ++n) {
      size_t p = id(pt_indx[3 * n], pt_indx[3 * n + 1], pt_indx[3 * n + 2]);
      for (int v = 0; v < NF; ++v) seismo[(size_t(v) * nsamp_cap + (m - 1)) * num_pt + n] = W[v][p];
    }
    nsamp = std::max(nsamp, m);
  }

  // ---- Gaussian-hill extension -----------------------------------------------------
  // Derivative along one index of a coordinate-like array, as seis3d_metric forms x_xi
  // (seis3d_metric.F90:83-112): the mean of the backward and forward DRP/opt operators,
  // in double; indices outside [lo, hi] take the value at the nearest of them.
  static double dmetric(const std::vector<double>& f, ptrdiff_t stride, ptrdiff_t base, int i, int lo, int hi) {
    static const double cF[5] = {-0.30874, -0.6326, 1.2330, -0.3334, 0.04168};
    static const double cB[5] = {-0.04168, 0.3334, -1.2330, 0.6326, 0.30874};
    const int ii = i < lo ? lo : (i > hi ? hi : i);
    double sb = 0.0, sf = 0.0;
    for (int q = 0; q < 5; ++q) {
      sb = sb + f[base + (ii - 3 + q) * stride] * cB[q];
      sf = sf + f[base + (ii - 1 + q) * stride] * cF[q];
    }
    return (sb + sf) * 0.5;
  }

  // Metric of the terrain-following grid, in double from the coordinates, the 1-D metric
  // and the heights, rounded once to T:
  //   r       = z(k) + h s(k)
  //   zeta_r  = zeta_z(k) * z_zeta(k) / r_zeta(i,j,k)    (1 where h = 0)
  //   zeta_theta / r          = -r_xi  xi_x  zeta_r / r
  //   zeta_phi / (r sin theta) = -r_eta eta_y zeta_r / (r sin theta)
  // with r_xi = h_xi s(k), r_eta = h_eta s(k) and r_zeta the metric derivative of r along k.
  void set_topography(const double* h) {
    const size_t n2 = size_t(nx) * ny, n3 = n2 * nz;
    topo_h.assign(h, h + n2);
    topo_hx.assign(n2, 0.0); topo_hy.assign(n2, 0.0);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        topo_hx[id2(i, j)] = dmetric(topo_h, 1, ptrdiff_t(nx) * (j - 1) - 1, i, ni1, ni2);
        topo_hy[id2(i, j)] = dmetric(topo_h, nx, ptrdiff_t(i) - 1 - nx, j, nj1, nj2);
      }
    std::vector<double> zd(nz), sk(nz), rzf(nz);
    for (int k = 1; k <= nz; ++k) zd[k - 1] = double(z[k]);
    for (int k = 1; k <= nz; ++k) {
      sk[k - 1] = (zd[k - 1] - zd[0]) / (zd[nk2 - 1] - zd[0]);
      rzf[k - 1] = dmetric(zd, 1, -1, k, nk1, nk2);
    }
    t_r.assign(n3, T(0)); t_az.assign(n3, T(0)); t_bx.assign(n3, T(0)); t_by.assign(n3, T(0));
    std::vector<double> col(nz);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t q = id2(i, j);
        const double hh = topo_h[q], hx = topo_hx[q], hy = topo_hy[q];
        for (int k = 1; k <= nz; ++k) col[k - 1] = zd[k - 1] + hh * sk[k - 1];
        for (int k = 1; k <= nz; ++k) {
          const double r = col[k - 1];
          const double rz = dmetric(col, 1, -1, k, nk1, nk2);
          const double az = double(zeta_z[k]) * (rzf[k - 1] / rz);
          const double bx = -((hx * sk[k - 1]) * double(xi_x[i])) * az / r;
          const double by = -((hy * sk[k - 1]) * double(eta_y[j])) * az / (r * double(xsin[i]));
          const size_t p = id(i, j, k);
          t_r[p] = T(r); t_az[p] = T(az); t_bx[p] = T(bx); t_by[p] = T(by);
        }
      }
    topo_on = true;
    topo_bc_dirty = true;
  }

  // Surface arrays of the extension (they need the medium): the normal m = (m1, m2, 1) of
  // the surface k = nk2 (grad zeta scaled to a unit radial part) and the inverse of the
  // 3x3 map from the velocity's zeta-derivatives to the traction rate on that surface,
  // both in double, rounded to T.
  void topo_surface() {
    const size_t n2 = size_t(nx) * ny;
    t_m1.assign(n2, T(0)); t_m2.assign(n2, T(0)); t_minv.assign(9 * n2, T(0)); t_slope.assign(n2, 0);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t q = id2(i, j), p = id(i, j, nk2);
        const double az = double(t_az[p]), bx = double(t_bx[p]), by = double(t_by[p]);
        const double m1 = bx / az, m2 = by / az;
        t_m1[q] = T(m1); t_m2[q] = T(m2);
        t_slope[q] = (t_m1[q] != T(0) || t_m2[q] != T(0)) ? 1 : 0;  // zero slope: the flat path
        const double la = double(lam[p]), mu_ = double(mu[p]), l2 = la + 2.0 * mu_;
        double M[3][3];
        M[0][0] = l2 * bx * m1 + mu_ * by * m2 + mu_ * az;
        M[1][0] = mu_ * by * m1 + la * bx * m2;
        M[2][0] = mu_ * az * m1 + la * bx;
        M[0][1] = la * by * m1 + mu_ * bx * m2;
        M[1][1] = mu_ * bx * m1 + l2 * by * m2 + mu_ * az;
        M[2][1] = mu_ * az * m2 + la * by;
        M[0][2] = la * az * m1 + mu_ * bx;
        M[1][2] = la * az * m2 + mu_ * by;
        M[2][2] = mu_ * bx * m1 + mu_ * by * m2 + l2 * az;
        const double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
        const double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
        const double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
        const double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
        const double inv[9] = {c00 / det, (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det,
                               (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det,
                               c01 / det, (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det,
                               (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det,
                               c02 / det, (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det,
                               (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det};
        for (int e = 0; e < 9; ++e) t_minv[9 * q + e] = T(inv[e]);
      }
    topo_bc_dirty = false;
  }

  // Traction image of the extension (free_timg generalised): in a column whose surface
  // slopes, the images above k = nk2 hold the traction combination G = sigma . m with the
  // column's surface normal, antisymmetric about the surface around the source traction
  // (G(nk2+q) = 2 T*Src - G(nk2-q)), in the slots of Txz, Tyz, Tzz (G_x, G_y, G_z; the
  // Txx, Tyy, Txy ghosts stay zero), and the surface values of Txz, Tyz, Tzz are set so
  // that sigma . m = T*Src there.  Flat columns take free_timg's values.
  void free_timg_topo() {
    if (!freenode) return;
    for (int j = nj1; j <= nj2; ++j)
      for (int i = ni1; i <= ni2; ++i) {
        const size_t q = id2(i, j);
        if (!t_slope[q]) {
          for (int m = 1; m <= 3; ++m) {
            W[TZZ][id(i, j, nk2 + m)] = T(2) * TzSrc[q] - W[TZZ][id(i, j, nk2 - m)];
            W[TXZ][id(i, j, nk2 + m)] = T(2) * TxSrc[q] - W[TXZ][id(i, j, nk2 - m)];
            W[TYZ][id(i, j, nk2 + m)] = T(2) * TySrc[q] - W[TYZ][id(i, j, nk2 - m)];
          }
          W[TZZ][id(i, j, nk2)] = TzSrc[q];
          W[TXZ][id(i, j, nk2)] = TxSrc[q];
          W[TYZ][id(i, j, nk2)] = TySrc[q];
          continue;
        }
        const T m1 = t_m1[q], m2 = t_m2[q];
        for (int m = 1; m <= 3; ++m) {
          const size_t pm = id(i, j, nk2 - m);
          const T gx = W[TXZ][pm] + m1 * W[TXX][pm] + m2 * W[TXY][pm];
          const T gy = W[TYZ][pm] + m1 * W[TXY][pm] + m2 * W[TYY][pm];
          const T gz = W[TZZ][pm] + m1 * W[TXZ][pm] + m2 * W[TYZ][pm];
          const size_t pu = id(i, j, nk2 + m);
          W[TXZ][pu] = T(2) * TxSrc[q] - gx;
          W[TYZ][pu] = T(2) * TySrc[q] - gy;
          W[TZZ][pu] = T(2) * TzSrc[q] - gz;
        }
        const size_t p = id(i, j, nk2);
        const T sxz = TxSrc[q] - m1 * W[TXX][p] - m2 * W[TXY][p];
        const T syz = TySrc[q] - m1 * W[TXY][p] - m2 * W[TYY][p];
        W[TXZ][p] = sxz;
        W[TYZ][p] = syz;
        W[TZZ][p] = TzSrc[q] - m1 * sxz - m2 * syz;
      }
  }

  // The stencil on the terrain-following grid.  Every theta and phi derivative gains its
  // zeta part (cross terms zeta_theta d/dzeta, zeta_phi d/dzeta); in the top three planes
  // of a sloping column the stress cross terms use the column's surface normal, so that
  // with the traction images they form d(sigma . m)/dzeta.  On a sloping free surface the
  // velocity's zeta-derivatives come from the traction condition sigma . m = T*Src (the
  // 3x3 inverse of topo_surface), generalising mod_macdrp.F90:944-948.
  void stencil_topo(bool fx, bool fy, bool fz) {
    const ptrdiff_t sx = 1, sy = nx, sz = ptrdiff_t(nx) * ny;
#pragma omp parallel for schedule(static)
    for (int k = nk1; k <= nk2; ++k)
      for (int j = nj1; j <= nj2; ++j)
        for (int i = ni1; i <= ni2; ++i) {
          const size_t p = id(i, j, k), q2 = id2(i, j);
          const T lam_ = lam[p], miu = mu[p];
          const T lam2mu = lam_ + T(2) * miu;
          const T rrho = T(1) / rho[p];
          const T r = t_r[p], az = t_az[p], s = xsin[i], c = xcot[i];
          const bool slope = t_slope[q2] != 0;
          const bool top3 = freenode && slope && k >= nk2 - 2;
          const T bxv = t_bx[p], byv = t_by[p];                          // strain cross terms
          const T bxm = top3 ? az * t_m1[q2] : bxv, bym = top3 ? az * t_m2[q2] : byv;  // momentum
          const T ax = xi_x[i] / r, ay = eta_y[j] / r / s;
          auto D = [&](int f, bool fw, ptrdiff_t st) { return op(fw, &W[f][p], st); };
          auto Dz = [&](int f) { return op(fz, &W[f][p], sz); };
          auto DzV = [&](int f) {
            if (freenode && k == nk2 - 1) return op22(fz, &W[f][p], sz);
            if (freenode && k == nk2 - 2) return op24(fz, &W[f][p], sz);
            return op(fz, &W[f][p], sz);
          };
          const bool water = miu <= T(1.0e-20f);
          const T w = water ? T(0) : T(1);
          // stress derivatives: theta (x), phi (y), r (z) parts
          const T xTxx = D(TXX, fx, sx) * ax + Dz(TXX) * bxm;
          const T xTxy = w * (D(TXY, fx, sx) * ax + Dz(TXY) * bxm);
          const T xTxz = w * (D(TXZ, fx, sx) * ax + Dz(TXZ) * bxm);
          const T yTyy = D(TYY, fy, sy) * ay + Dz(TYY) * bym;
          const T yTxy = w * (D(TXY, fy, sy) * ay + Dz(TXY) * bym);
          const T yTyz = w * (D(TYZ, fy, sy) * ay + Dz(TYZ) * bym);
          const T zTzz = Dz(TZZ) * az, zTxz = w * (Dz(TXZ) * az), zTyz = w * (Dz(TYZ) * az);
          const T Txx = W[TXX][p], Tyy = W[TYY][p], Tzz = W[TZZ][p];
          const T Txy = W[TXY][p], Txz = W[TXZ][p], Tyz = W[TYZ][p];
          const T Vx = W[VX][p], Vy = W[VY][p], Vz = W[VZ][p];
          H[VX][p] = rrho * (xTxx + yTxy + zTxz + (T(3) * Txz + Txx * c - Tyy * c) / r);
          H[VY][p] = rrho * (xTxy + yTyy + zTyz + (T(2) * Txy * c + T(3) * Tyz) / r);
          H[VZ][p] = rrho * (xTxz + yTyz + zTzz + (T(2) * Tzz - Txx - Tyy + Txz * c) / r);
          // velocity derivatives without their zeta parts, then the zeta parts
          const T gxVx = D(VX, fx, sx) * ax, gxVy = D(VY, fx, sx) * ax, gxVz = D(VZ, fx, sx) * ax;
          const T gyVx = D(VX, fy, sy) * ay, gyVy = D(VY, fy, sy) * ay, gyVz = D(VZ, fy, sy) * ay;
          T E11 = gxVx + Vz / r;
          T E22 = (Vx * c + Vz) / r + gyVy;
          T E12 = (gxVy + gyVx - Vy * c / r) / T(2);
          T E33 = T(0);
          T E13 = (gxVz - Vx / r) / T(2);
          T E23 = (gyVz - Vy / r) / T(2);
          T ux, uy, uz;  // d(Vx, Vy, Vz)/dzeta
          if (freenode && k == nk2 && slope) {
            const T S11 = lam2mu * E11 + lam_ * E22, S22 = lam2mu * E22 + lam_ * E11, S33 = lam_ * (E11 + E22);
            const T S12 = T(2) * miu * E12, S13 = T(2) * miu * E13, S23 = T(2) * miu * E23;
            const T m1 = t_m1[q2], m2 = t_m2[q2];
            const T r0 = VxSrc[q2] - (S11 * m1 + S12 * m2 + S13);
            const T r1 = VySrc[q2] - (S12 * m1 + S22 * m2 + S23);
            const T r2 = VzSrc[q2] - (S13 * m1 + S23 * m2 + S33);
            const T* mi = &t_minv[9 * q2];
            ux = mi[0] * r0 + mi[1] * r1 + mi[2] * r2;
            uy = mi[3] * r0 + mi[4] * r1 + mi[5] * r2;
            uz = mi[6] * r0 + mi[7] * r1 + mi[8] * r2;
          } else {
            ux = DzV(VX); uy = DzV(VY); uz = DzV(VZ);
          }
          E11 = E11 + bxv * ux;
          E22 = E22 + byv * uy;
          E12 = E12 + (bxv * uy + byv * ux) / T(2);
          E33 = az * uz;
          E13 = E13 + (bxv * uz + az * ux) / T(2);
          E23 = E23 + (byv * uz + az * uy) / T(2);
          if (freenode && k == nk2 && !slope) {  // mod_macdrp.F90:944-948
            E33 = -(lam_ / lam2mu * (E11 + E22)) + VzSrc[q2] / lam2mu;
            E13 = VxSrc[q2] / miu / T(2);
            E23 = VySrc[q2] / miu / T(2);
          }
          H[TXX][p] = lam2mu * E11 + lam_ * (E22 + E33);
          H[TYY][p] = lam2mu * E22 + lam_ * (E11 + E33);
          H[TZZ][p] = lam2mu * E33 + lam_ * (E11 + E22);
          H[TXY][p] = T(2) * miu * E12;
          H[TXZ][p] = T(2) * miu * E13;
          H[TYZ][p] = T(2) * miu * E23;
        }
  }

  // The 8-step cycle of seis3d_wave_8op_p3.F90:82-591: stage-1/3 operator per step
  // (bit 2 = x, bit 1 = y, bit 0 = z; 1 = forward); stages 2/4 use the mirror.
  static int cycle_variant(int pos) {
    static const int v[8] = {0b000 /*BBB*/, 0b110 /*FFB*/, 0b111 /*FFF*/, 0b001 /*BBF*/,
                             0b010 /*BFB*/, 0b100 /*FBB*/, 0b101 /*FBF*/, 0b011 /*BFF*/};
    return v[pos & 7];
  }

  bool step() {
    const int X = cycle_variant(cycle_pos);
    syn();
    for (int s = 0; s < 4; ++s) {
      const T incr = s == 0 ? T(0) : C::rka(s - 1);  // set_cur_time(ntime, firRKa(s))
      if (srcsurface && !src_surface(incr)) return false;
      const int v = (s % 2 == 0) ? X : (~X & 7);
      const bool fx = (v >> 2) & 1, fy = (v >> 1) & 1, fz = v & 1;
      if (topo_on) {
        if (topo_bc_dirty) topo_surface();
        free_timg_topo();
        stencil_topo(fx, fy, fz);
      } else {
        free_timg();
        stencil(fx, fy, fz);
      }
      abs_stencil(fx, fy, fz);
      if (!src_stress(incr)) return false;
      if (!src_force(incr)) return false;
      rk(s);
    }
    ntime += 1;
    cycle_pos = (cycle_pos + 1) & 7;
    seismo_put();
    return true;
  }
};

// The same metric formula evaluated in double from the SP coordinates and rounded
// once: the FP64 precomputation the GPU path performs.
template <class O>
static void metric_dp(int nx, int ny, int nz, const float* x, const float* y, const float* z,
                      O* xsin, O* xcot, O* xi_x, O* eta_y, O* zeta_z) {
  const double coeF[5] = {-0.30874, -0.6326, 1.2330, -0.3334, 0.04168};
  const double coeB[5] = {-0.04168, 0.3334, -1.2330, 0.6326, 0.30874};
  for (int i = 0; i < nx; ++i) {
    xsin[i] = O(std::sin(double(x[i])));
    xcot[i] = O(1.0 / std::tan(double(x[i])));
  }
  auto one = [&](int n, const float* g, O* out) {
    const int lo = LenFD, hi = n - 1 - LenFD;
    for (int i = 0; i < n; ++i) {
      const int ii = i < lo ? lo : (i > hi ? hi : i);
      double sb = 0.0, sf = 0.0;
      for (int q = 0; q < 5; ++q) {
        sb += double(g[ii - 3 + q]) * coeB[q];
        sf += double(g[ii - 1 + q]) * coeF[q];
      }
      out[i] = O(1.0 / ((sb + sf) * 0.5));
    }
  };
  one(nx, x, xi_x);
  one(ny, y, eta_y);
  one(nz, z, zeta_z);
}

// seis3d_metric (seis3d_metric.F90:83-112): SP coordinates, DP sin/tan, SP metric.
static void metric_sp(int nx, int ny, int nz, const float* x, const float* y, const float* z,
                      float* xsin, float* xcot, float* xi_x, float* eta_y, float* zeta_z) {
  const int vecF[5] = {-1, 0, 1, 2, 3};
  const float coeF[5] = {-0.30874f, -0.6326f, 1.2330f, -0.3334f, 0.04168f};
  const int vecB[5] = {-3, -2, -1, 0, 1};
  const float coeB[5] = {-0.04168f, 0.3334f, -1.2330f, 0.6326f, 0.30874f};
  for (int i = 0; i < nx; ++i) {
    xsin[i] = float(std::sin(double(x[i])));
    xcot[i] = float(1.0 / std::tan(double(x[i])));
  }
  auto one = [&](int n, const float* g, float* out) {
    const int lo = LenFD, hi = n - 1 - LenFD;  // 0-based interior bounds
    for (int i = lo; i <= hi; ++i) {
      float sb = 0.0f, sf = 0.0f;
      for (int q = 0; q < 5; ++q) sb += g[i + vecB[q]] * coeB[q];
      for (int q = 0; q < 5; ++q) sf += g[i + vecF[q]] * coeF[q];
      float d = (sb + sf) * 0.5f;
      out[i] = 1.0f / d;
    }
    for (int q = 1; q <= LenFD; ++q) { out[lo - q] = out[lo]; out[hi + q] = out[hi]; }
  };
  one(nx, x, xi_x);
  one(ny, y, eta_y);
  one(nz, z, zeta_z);
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C interface for the test harness (ctypes).  All real-valued arrays cross the
// boundary as double so one entry point serves the float and double solvers without
// loss (float -> double -> float is exact).
// ---------------------------------------------------------------------------
struct OrcHandle {
  int dbl;
  orc::Solver<float>* f = nullptr;
  orc::Solver<double>* d = nullptr;
};

#define DISPATCH(h, ...) (h->dbl ? [&](auto& S) { __VA_ARGS__; }(*h->d) : [&](auto& S) { __VA_ARGS__; }(*h->f))

template <class T> static void cpy(std::vector<T>& dst, const double* src, size_t n, size_t off) {
  for (size_t q = 0; q < n; ++q) dst[q + off] = T(src[q]);
}

extern "C" {

void* orc_create(int ni, int nj, int nk, double stept, int freenode, int dbl) {
  OrcHandle* h = new OrcHandle;
  h->dbl = dbl;
  if (dbl) h->d = new orc::Solver<double>(ni, nj, nk, stept, freenode != 0);
  else h->f = new orc::Solver<float>(ni, nj, nk, float(stept), freenode != 0);
  return h;
}

void orc_destroy(void* hv) {
  OrcHandle* h = (OrcHandle*)hv;
  delete h->f; delete h->d; delete h;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n; return 1;
#endif
}

void orc_set_coord(void* hv, const double* x, const double* y, const double* z) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, { cpy(S.x, x, S.nx, 1); cpy(S.y, y, S.ny, 1); cpy(S.z, z, S.nz, 1); });
}

void orc_set_metric(void* hv, const double* xsin, const double* xcot, const double* xi_x,
                    const double* eta_y, const double* zeta_z) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, {
    cpy(S.xsin, xsin, S.nx, 1); cpy(S.xcot, xcot, S.nx, 1); cpy(S.xi_x, xi_x, S.nx, 1);
    cpy(S.eta_y, eta_y, S.ny, 1); cpy(S.zeta_z, zeta_z, S.nz, 1);
  });
}

void orc_set_media(void* hv, const double* lam, const double* mu, const double* rho) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, {
    size_t n = size_t(S.nx) * S.ny * S.nz;
    cpy(S.lam, lam, n, 0); cpy(S.mu, mu, n, 0); cpy(S.rho, rho, n, 0);
    S.topo_bc_dirty = true;
  });
}

// Gaussian-hill extension: heights h (nx*ny, i fastest, m) of the terrain-following
// radius; set after the coordinates and the metric.
void orc_set_topography(void* hv, const double* h) {
  OrcHandle* hd = (OrcHandle*)hv;
  DISPATCH(hd, { S.set_topography(h); });
}

// Metric arrays of the extension as T values in double: which 0 r, 1 zeta_r,
// 2 zeta_theta / r, 3 zeta_phi / (r sin theta) (nx*ny*nz); 4 m1, 5 m2 (nx*ny); 6 the 3x3
// inverses (9*nx*ny) (computed on demand).
void orc_topography_array(void* hv, int which, double* out) {
  OrcHandle* hd = (OrcHandle*)hv;
  DISPATCH(hd, {
    if (which >= 4 && S.topo_bc_dirty) S.topo_surface();
    const auto& v = which == 0 ? S.t_r : which == 1 ? S.t_az : which == 2 ? S.t_bx : which == 3 ? S.t_by
                  : which == 4 ? S.t_m1 : which == 5 ? S.t_m2 : S.t_minv;
    for (size_t q = 0; q < v.size(); ++q) out[q] = double(v[q]);
  });
}

int orc_set_pml(void* hv, const int* number, const double* vel, const double* bmax, const double* amax) {
  OrcHandle* h = (OrcHandle*)hv;
  return DISPATCH(h, { return S.set_pml(number, vel, bmax, amax) ? 0 : 1; });
}

void orc_set_srcsurface(void* hv, int on) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, { S.srcsurface = on != 0; });
}

// indx: 1-based Fortran indices (3 per source); Fx etc. are (ntwin, num) column-major.
void orc_set_forces(void* hv, int num, int ntwin, const int* indx, const double* shift,
                    const double* t0, const double* stf_time, const double* stf_freq,
                    const double* fx, const double* fy, const double* fz, int stf_id) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, {
    using T = typename std::remove_reference<decltype(S.stept)>::type;
    S.num_force = num; S.ntwin_force = ntwin; S.frcstf_id = stf_id;
    S.force_indx.assign(indx, indx + 3 * num);
    S.force_shift.assign(3 * num, T(0)); cpy(S.force_shift, shift, 3 * num, 0);
    S.force_t0.assign(num, T(0)); cpy(S.force_t0, t0, num, 0);
    S.frcstf_time.assign(ntwin, T(0)); cpy(S.frcstf_time, stf_time, ntwin, 0);
    S.frcstf_freq.assign(ntwin, T(0)); cpy(S.frcstf_freq, stf_freq, ntwin, 0);
    S.ForceX.assign(ntwin * num, T(0)); cpy(S.ForceX, fx, ntwin * num, 0);
    S.ForceY.assign(ntwin * num, T(0)); cpy(S.ForceY, fy, ntwin * num, 0);
    S.ForceZ.assign(ntwin * num, T(0)); cpy(S.ForceZ, fz, ntwin * num, 0);
  });
}

// mom: 6 arrays (Mxx Myy Mzz Mxy Mxz Myz) each (ntwin, num) column-major, concatenated.
void orc_set_moments(void* hv, int num, int ntwin, const int* indx, const double* shift,
                     const double* t0, const double* stf_time, const double* stf_freq,
                     const double* mom, int stf_id) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, {
    using T = typename std::remove_reference<decltype(S.stept)>::type;
    S.num_moment = num; S.ntwin_moment = ntwin; S.momstf_id = stf_id;
    S.moment_indx.assign(indx, indx + 3 * num);
    S.moment_shift.assign(3 * num, T(0)); cpy(S.moment_shift, shift, 3 * num, 0);
    S.moment_t0.assign(num, T(0)); cpy(S.moment_t0, t0, num, 0);
    S.momstf_time.assign(ntwin, T(0)); cpy(S.momstf_time, stf_time, ntwin, 0);
    S.momstf_freq.assign(ntwin, T(0)); cpy(S.momstf_freq, stf_freq, ntwin, 0);
    size_t n = size_t(ntwin) * num;
    std::vector<T>* dst[6] = {&S.MomTxx, &S.MomTyy, &S.MomTzz, &S.MomTxy, &S.MomTxz, &S.MomTyz};
    for (int c = 0; c < 6; ++c) { dst[c]->assign(n, T(0)); cpy(*dst[c], mom + c * n, n, 0); }
  });
}

void orc_set_receivers(void* hv, int num, const int* indx, int tinv) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, {
    S.num_pt = num; S.pt_tinv = tinv > 0 ? tinv : 1;
    S.pt_indx.assign(indx, indx + 3 * num);
    S.nsamp = 0; S.nsamp_cap = 0; S.seismo.clear();
  });
}

int orc_run(void* hv, int nsteps) {
  OrcHandle* h = (OrcHandle*)hv;
  return DISPATCH(h, {
    for (int q = 0; q < nsteps; ++q)
      if (!S.step()) return 1;
    return 0;
  });
}

int orc_ntime(void* hv) {
  OrcHandle* h = (OrcHandle*)hv;
  return DISPATCH(h, { return S.ntime; });
}

int orc_freenode(void* hv) {
  OrcHandle* h = (OrcHandle*)hv;
  return DISPATCH(h, { return S.freenode ? 1 : 0; });
}

// field f in receiver order (Vx..Tyz); writes nx*ny*nz values incl. ghosts
void orc_get_field(void* hv, int f, double* out) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, {
    size_t n = S.W[f].size();
    for (size_t q = 0; q < n; ++q) out[q] = double(S.W[f][q]);
  });
}

void orc_set_field(void* hv, int f, const double* in) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, { cpy(S.W[f], in, S.W[f].size(), 0); });
}

// PML profiles A, B, D (D already divided by B) for axis 0,1,2
void orc_get_pml_profile(void* hv, int axis, double* A, double* B, double* D) {
  OrcHandle* h = (OrcHandle*)hv;
  DISPATCH(h, {
    auto& a = axis == 0 ? S.Ax : axis == 1 ? S.Ay : S.Az;
    auto& b = axis == 0 ? S.Bx : axis == 1 ? S.By : S.Bz;
    auto& d = axis == 0 ? S.Dx : axis == 1 ? S.Dy : S.Dz;
    for (size_t q = 1; q < a.size(); ++q) { A[q - 1] = a[q]; B[q - 1] = b[q]; D[q - 1] = d[q]; }
  });
}

// returns number of samples; out is [9][nsamp][num_pt]
int orc_get_seismo(void* hv, double* out, int maxsamp) {
  OrcHandle* h = (OrcHandle*)hv;
  return DISPATCH(h, {
    int ns = std::min(S.nsamp, maxsamp);
    for (int v = 0; v < orc::NF; ++v)
      for (int q = 0; q < ns; ++q)
        for (int n = 0; n < S.num_pt; ++n)
          out[(size_t(v) * ns + q) * S.num_pt + n] = double(S.seismo[(size_t(v) * S.nsamp_cap + q) * S.num_pt + n]);
    return ns;
  });
}

const char* orc_last_error(void* hv) {
  OrcHandle* h = (OrcHandle*)hv;
  return h->dbl ? h->d->err.c_str() : h->f->err.c_str();
}

// --- primitives for known-answer tests -------------------------------------
double orc_stf(int which, int id, double t, double t0, double f0, int ntime, double stept, int dbl) {
  if (dbl) {
    double v = 0;
    bool ok = which == 0 ? orc::src_stf<double>(t, t0, f0, id, ntime, stept, &v)
                         : orc::src_svf<double>(t, t0, f0, id, ntime, stept, &v);
    return ok ? v : NAN;
  }
  float v = 0;
  bool ok = which == 0 ? orc::src_stf<float>(float(t), float(t0), float(f0), id, ntime, float(stept), &v)
                       : orc::src_svf<float>(float(t), float(t0), float(f0), id, ntime, float(stept), &v);
  return ok ? double(v) : NAN;
}

int orc_norm_delt(double x0, double y0, double z0, double* out) {
  float d[343];
  if (!orc::cal_norm_delt<float>(d, float(x0), float(y0), float(z0), 1.5f, 1.5f, 1.5f)) return 1;
  for (int q = 0; q < 343; ++q) out[q] = d[q];
  return 0;
}

double orc_pml_R(int n) { return double(orc::cal_pml_R<float>(n)); }

void orc_metric(int nx, int ny, int nz, const float* x, const float* y, const float* z, float* xsin,
                float* xcot, float* xi_x, float* eta_y, float* zeta_z) {
  orc::metric_sp(nx, ny, nz, x, y, z, xsin, xcot, xi_x, eta_y, zeta_z);
}

void orc_metric_dp(int nx, int ny, int nz, const float* x, const float* y, const float* z, float* xsin,
                   float* xcot, float* xi_x, float* eta_y, float* zeta_z) {
  orc::metric_dp(nx, ny, nz, x, y, z, xsin, xcot, xi_x, eta_y, zeta_z);
}

// The FP64 metric without rounding to FP32 (the metric of the double-precision run).
void orc_metric_dd(int nx, int ny, int nz, const float* x, const float* y, const float* z, double* xsin,
                   double* xcot, double* xi_x, double* eta_y, double* zeta_z) {
  orc::metric_dp(nx, ny, nz, x, y, z, xsin, xcot, xi_x, eta_y, zeta_z);
}

// One-sided operator applied to a 1-D array at 0-based index i (known-answer tests).
double orc_op(int kind, int fwd, const double* f, int i) {
  using S = orc::Solver<double>;
  const double* p = f + i;
  switch (kind) {
    case 0: return S::op(fwd != 0, p, 1);
    case 1: return S::op24(fwd != 0, p, 1);
    default: return S::op22(fwd != 0, p, 1);
  }
}

}  // extern "C"
