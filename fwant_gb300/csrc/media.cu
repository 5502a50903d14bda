// The medium preprocessor on the GPU (code/srcF/seis3d_media.F90): effective-medium
// evaluation (effmedia_eval :854-1249), ghost extension (media_extend / extend_equal
// :1264-1299) and the time-step check (media_stept_check :1544-1611), with the model
// look-ups of the six background kinds and two perturbation kinds and the helpers
// indx_locate_1d (:1315-1344), eval_poly (:1251-1262), dist_point2plane (:1301-1313) and
// interp_2d / interp_3d (code/srcF/mod_math.F90:128-208).
//
// One thread per grid point evaluates its (2 N)^3 sub-cell samples in the reference's
// order and writes lambda, mu, rho; the model arrays are small and read through L1/L2.
// Arithmetic is single precision where the reference declares SP and double where it
// declares DP, every product and sum rounded separately (this file is compiled with
// -fmad=false), divisions and square roots IEEE-rounded, so the results equal a sequential
// CPU evaluation bit for bit except where powf enters (composite and verpoly models: the
// device powf is within 2 ulp).  The time-step check takes the cosines and sines of the
// grid angles from host-computed tables, so its double-precision distances are exact
// functions of the same inputs too, and its minimum is reduced over (value, point index)
// pairs, which gives the reference's first-minimum-in-loop-order answer independent of
// the launch shape.
//
// Roofline: not memory-bound.  Each point writes 12 bytes (plus 12 per ghost point) and
// reads model data that stays in cache; the work is the per-sample look-ups (bisections,
// two-point Lagrange weights with IEEE divisions), issue-bound on the FP32 and integer
// pipes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/fwant_media.h"

namespace {

constexpr float SEIS_ZERO = 1.0e-20f;
constexpr double PI_D = 3.141592653589793;
constexpr int LENFD = 3;
constexpr int MD_THREADS = 256;
constexpr int MAX_HALF = 16;
constexpr int ST_BLOCKS = 1216;  // partial minima of the time-step check

struct DCart {
  int nk;
  const float *d, *vp, *vs, *dp;
};
struct DLayers {
  int ni, nj, nk;
  const float *x, *y, *z, *h, *vp, *vs, *dp, *vpd, *vsd, *dpd;
};
struct DVol {
  int ni, nj, nk;
  float rz0;
  const float *x, *y, *rz, *vp, *vs, *dp;
};
struct DPoly {
  int ni, nj, nk, np;
  float rz0;
  const float *x, *y, *rz, *vpc, *vsc, *dpc, *vpd, *vsd, *dpd;
};

struct Args {
  int ni, nj, nk, nx, ny, nz;
  int ng[3];
  float ztopo;
  const float *x, *y, *z;
  int bkind, pkind;
  DCart c;
  DLayers L;
  DVol bv, pv;
  DPoly bp, pp;
  float *lam, *mu, *rho;
  int* err;  // 1: a sample below the lowest layer's bottom of a layered / composite model
};

// indx_locate_1d: bracketing pair (1-based i1, i1 + 1) and the clamped coordinate
__device__ void locate(float x0, const float* x, int n, int& i1, float& x1) {
  int lo = 1, hi = n;
  x1 = x0;
  if (x0 <= x[0]) {
    x1 = x[0];
    lo = 1;
  } else if (x0 >= x[hi - 1]) {
    x1 = x[hi - 1];
    lo = hi - 1;
  } else {
    while (hi - lo > 1) {
      const int mid = (hi - lo) / 2 + lo;
      const float xm = x[mid - 1];
      if (xm == x0) {
        lo = mid;
        break;
      } else if (xm > x0) {
        hi = mid;
      } else {
        lo = mid;
      }
    }
  }
  i1 = lo;
}

// the two nonzero Lagrange weights of a two-point interp_2d / interp_3d axis
__device__ __forceinline__ void lweights(float xa, float xb, float xi, float& l1, float& l2) {
  l1 = (xi - xb) / (xa - xb);
  l2 = (xi - xa) / (xb - xa);
}

// interp_2d on corners c00, c10, c01, c11 (i fastest), summed j-major as the reference
__device__ __forceinline__ float bilin(float lx1, float lx2, float ly1, float ly2, float c00, float c10, float c01,
                                       float c11) {
  float z = 0.0f;
  z = z + lx1 * ly1 * c00;
  z = z + lx2 * ly1 * c10;
  z = z + lx1 * ly2 * c01;
  z = z + lx2 * ly2 * c11;
  return z;
}

struct Cell2 {  // a located horizontal cell of a model grid
  int i1, j1;
  float lx1, lx2, ly1, ly2;
};

__device__ Cell2 cell2(const float* xs, int ni, const float* ys, int nj, float x0, float y0) {
  Cell2 c;
  float x1, y1;
  locate(x0, xs, ni, c.i1, x1);
  locate(y0, ys, nj, c.j1, y1);
  lweights(xs[c.i1 - 1], xs[c.i1], x1, c.lx1, c.lx2);
  lweights(ys[c.j1 - 1], ys[c.j1], y1, c.ly1, c.ly2);
  return c;
}

// interp_2d of layer `plane` of f (ni, nj, ...) at a located cell
__device__ __forceinline__ float at2(const Cell2& c, const float* f, int ni, size_t plane) {
  const float* p = f + plane + size_t(c.j1 - 1) * ni + (c.i1 - 1);
  return bilin(c.lx1, c.lx2, c.ly1, c.ly2, p[0], p[1], p[ni], p[ni + 1]);
}

// interp_2d of slot s (0, 1) of a (2, ni, nj, nk) composite field in layer n (1-based)
__device__ __forceinline__ float at2c(const Cell2& c, const float* f, int ni, int nj, int s, int n) {
  const size_t b = size_t(2) * ((size_t(n - 1) * nj + (c.j1 - 1)) * ni + (c.i1 - 1)) + s;
  const size_t r = size_t(2) * ni;
  return bilin(c.lx1, c.lx2, c.ly1, c.ly2, f[b], f[b + 2], f[b + r], f[b + r + 2]);
}

struct Cell3 {
  int i1, j1, k1;
  float lx[2], ly[2], lz[2];
};

__device__ Cell3 cell3(const DVol& V, float x0, float y0, float z0) {
  Cell3 c;
  float x1, y1, z1;
  locate(x0, V.x, V.ni, c.i1, x1);
  locate(y0, V.y, V.nj, c.j1, y1);
  locate(V.rz0 - z0, V.rz, V.nk, c.k1, z1);
  lweights(V.x[c.i1 - 1], V.x[c.i1], x1, c.lx[0], c.lx[1]);
  lweights(V.y[c.j1 - 1], V.y[c.j1], y1, c.ly[0], c.ly[1]);
  lweights(V.rz[c.k1 - 1], V.rz[c.k1], z1, c.lz[0], c.lz[1]);
  return c;
}

__device__ float at3(const Cell3& c, const DVol& V, const float* f) {
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int i = 0; i < 2; ++i)
        s = s + c.lx[i] * c.ly[j] * c.lz[k] * f[(size_t(c.k1 - 1 + k) * V.nj + (c.j1 - 1 + j)) * V.ni + (c.i1 - 1 + i)];
  return s;
}

__device__ float eval_poly(const float* c, size_t stride, const float* d, int n, float x) {
  float f = 0.0f;
  for (int q = 0; q < n; ++q) f = f + c[q * stride] * powf(x, d[q]);
  return f;
}

__device__ int minloc_abs(const float* a, size_t stride, int n, float v) {
  int best = 1;
  float bv = fabsf(a[0] - v);
  for (int q = 1; q < n; ++q) {
    const float t = fabsf(a[q * stride] - v);
    if (t < bv) {
      bv = t;
      best = q + 1;
    }
  }
  return best;
}

// verpoly look-up (:1143-1171 and :1192-1220): values at the two sides of a piece boundary
// or the same value twice
__device__ void verpoly(const DPoly& P, float x0, float y0, float z0, float dz2, float* vp, float* vs, float* dp) {
  const int wi = minloc_abs(P.x, 1, P.ni, x0), wj = minloc_abs(P.y, 1, P.nj, y0);
  const size_t plane = size_t(P.ni) * P.nj, col = size_t(wj - 1) * P.ni + (wi - 1);
  const float* rz = P.rz + col;
  const float depth = P.rz0 - z0;
  int wk = minloc_abs(rz, plane, P.nk, depth);
  const size_t cs = plane * P.nk;
  if (fabsf(rz[plane * (wk - 1)] - depth) <= dz2 / 5.0f || depth < rz[0]) {
    const int k1 = max(1, wk - 1), k2 = wk;
    const float z1 = rz[plane * (k2 - 1)] - rz[plane * (k1 - 1)], z2 = 0.0f;
    const size_t o1 = col + plane * (k1 - 1), o2 = col + plane * (k2 - 1);
    vp[0] = eval_poly(P.vpc + o1, cs, P.vpd, P.np, z1);
    vp[1] = eval_poly(P.vpc + o2, cs, P.vpd, P.np, z2);
    vs[0] = eval_poly(P.vsc + o1, cs, P.vsd, P.np, z1);
    vs[1] = eval_poly(P.vsc + o2, cs, P.vsd, P.np, z2);
    dp[0] = eval_poly(P.dpc + o1, cs, P.dpd, P.np, z1);
    dp[1] = eval_poly(P.dpc + o2, cs, P.dpd, P.np, z2);
  } else {
    if (depth < rz[plane * (wk - 1)]) wk = wk - 1;
    const float z1 = depth - rz[plane * (wk - 1)];
    const size_t o = col + plane * (wk - 1);
    vp[0] = vp[1] = eval_poly(P.vpc + o, cs, P.vpd, P.np, z1);
    vs[0] = vs[1] = eval_poly(P.vsc + o, cs, P.vsd, P.np, z1);
    dp[0] = dp[1] = eval_poly(P.dpc + o, cs, P.dpd, P.np, z1);
  }
}

// cart1d look-up of one depth (:916-966)
__device__ __forceinline__ void cart1d_lookup(const DCart& c, float d0, float* Vp, float* Vs, float* Dp) {
  auto set1 = [&](float p, float s, float r) {
    Vp[0] = Vp[1] = p;
    Vs[0] = Vs[1] = s;
    Dp[0] = Dp[1] = r;
  };
  const float* d = c.d;
  auto V = [&](int q, int s) {
    Vp[s] = c.vp[q - 1];
    Vs[s] = c.vs[q - 1];
    Dp[s] = c.dp[q - 1];
  };
  int k1 = 1, k2 = c.nk;
  if (fabsf(d[k1 - 1] - d0) < SEIS_ZERO || d0 < d[k1 - 1]) {
    V(k1, 0);
    V(k1, 1);
  } else if (fabsf(d[k2 - 1] - d0) < SEIS_ZERO) {
    if (fabsf(d[k2 - 2] - d[k2 - 1]) < SEIS_ZERO) {
      V(k2 - 1, 0);
      V(k2, 1);
    } else {
      V(k2, 0);
      V(k2, 1);
    }
  } else if (d[k2 - 1] < d0) {
    V(k2, 0);
    V(k2, 1);
  } else {
    while (k2 - k1 > 1) {
      const int k0 = (k2 - k1) / 2 + k1;
      if (fabsf(d[k0 - 1] - d0) < SEIS_ZERO) {
        k1 = k0;
        k2 = k0;
        break;
      } else if (d[k0 - 1] > d0) {
        k2 = k0;
      } else {
        k1 = k0;
      }
    }
    if (k1 == k2) {
      if (fabsf(d[k1 - 2] - d[k1 - 1]) < SEIS_ZERO) {
        V(k1 - 1, 0);
        V(k1, 1);
      } else if (fabsf(d[k1] - d[k1 - 1]) < SEIS_ZERO) {
        V(k1, 0);
        V(k1 + 1, 1);
      } else {
        V(k1, 0);
        V(k1, 1);
      }
    } else {
      const float dd = d[k2 - 1], h = d[k2 - 1] - d[k1 - 1];
      const float L1 = (dd - d0) / h, L2 = 1.0f - L1;
      set1(c.vp[k1 - 1] * L1 + c.vp[k2 - 1] * L2, c.vs[k1 - 1] * L1 + c.vs[k2 - 1] * L2,
           c.dp[k1 - 1] * L1 + c.dp[k2 - 1] * L2);
    }
  }
}

// background look-up of one sample (:870-1171); false on the lowest-layer error
__device__ __forceinline__ bool bg_sample(const Args& a, float x0, float y0, float z0, float d0, float dz2, float* Vp,
                                          float* Vs, float* Dp) {
  auto set1 = [&](float p, float s, float r) {
    Vp[0] = Vp[1] = p;
    Vs[0] = Vs[1] = s;
    Dp[0] = Dp[1] = r;
  };
  if (a.bkind == FWANT_MEDIA_CART1D) {
    cart1d_lookup(a.c, d0, Vp, Vs, Dp);
  } else if (a.bkind == FWANT_MEDIA_INTERFACE) {  // :968-1054
    const DLayers& L = a.L;
    const Cell2 c = cell2(L.x, L.ni, L.y, L.nj, x0, y0);
    const size_t plane = size_t(L.ni) * L.nj;
    auto pick = [&](int n1, int k1, int n2, int k2) {
      const int p1 = (n1 - 1) + 2 * (k1 - 1), p2 = (n2 - 1) + 2 * (k2 - 1);
      Vp[0] = L.vp[p1];
      Vp[1] = L.vp[p2];
      Vs[0] = L.vs[p1];
      Vs[1] = L.vs[p2];
      Dp[0] = L.dp[p1];
      Dp[1] = L.dp[p2];
    };
    int n1 = 2, k1 = L.nk, n2 = 2, k2 = L.nk;
    for (int n = L.nk; n >= 1; --n) {
      const float z1 = at2(c, L.z, L.ni, plane * (n - 1));
      const float h = n == L.nk ? 1.0e3f : at2(c, L.h, L.ni, plane * (n - 1));
      if (h <= SEIS_ZERO && n > 1) continue;
      if (h <= SEIS_ZERO && n == 1) {
        if (L.vp[2 * (n - 1)] > SEIS_ZERO) n1 = k1 = n2 = k2 = 1;
        pick(n1, k1, n2, k2);
        break;
      }
      if (fabsf(z1 - z0) <= dz2 / 5.0f) {
        k2 = n;
        n2 = 2;
        if (n == 1) {
          k1 = n;
          n1 = L.vp[2 * (n - 1)] > SEIS_ZERO ? 1 : 2;
        }
        for (int mm = n - 1; mm >= 1; --mm) {
          if (at2(c, L.h, L.ni, plane * (mm - 1)) > SEIS_ZERO) {
            k1 = mm + 1;
            n1 = 1;
            break;
          } else if (mm == 1) {
            if (L.vp[2 * (mm - 1)] > SEIS_ZERO) {
              k1 = mm;
              n1 = 1;
            } else {
              k1 = n;
              n1 = 2;
            }
          }
        }
        pick(n1, k1, n2, k2);
        break;
      }
      if (z0 < z1) {
        const int q2 = 1 + 2 * (n - 1);
        if (n == L.nk) {
          set1(L.vp[q2], L.vs[q2], L.dp[q2]);
        } else {
          const int q1 = 2 * n;  // (1, n + 1)
          const float L2 = (z1 - z0) / h, L1 = 1.0f - L2;
          set1(L.vp[q2] * L1 + L.vp[q1] * L2, L.vs[q2] * L1 + L.vs[q1] * L2, L.dp[q2] * L1 + L.dp[q1] * L2);
        }
        break;
      }
      k1 = n;
      k2 = n;
      n1 = 2;
      n2 = 2;
      if (n == 1) {
        if (L.vp[2 * (n - 1)] > SEIS_ZERO) n1 = k1 = n2 = k2 = 1;
        pick(n1, k1, n2, k2);
        break;
      }
    }
  } else if (a.bkind == FWANT_MEDIA_LAYERED || a.bkind == FWANT_MEDIA_COMPOSITE) {  // :1055-1130
    const DLayers& L = a.L;
    const bool comp = a.bkind == FWANT_MEDIA_COMPOSITE;
    const Cell2 c = cell2(L.x, L.ni, L.y, L.nj, x0, y0);
    const size_t plane = size_t(L.ni) * L.nj;
    float d = 0.0f;
    for (int n = 1; n <= L.nk; ++n) {
      const float h = at2(c, L.h, L.ni, plane * (n - 1));
      if (h <= SEIS_ZERO) continue;
      d = d + h;
      if (fabsf(d - d0) <= dz2 / 5.0f) {
        if (n == L.nk) return false;
        const int n1 = n;
        int n2 = L.nk;
        for (int mm = n + 1; mm <= L.nk; ++mm)
          if (at2(c, L.h, L.ni, plane * (mm - 1)) > SEIS_ZERO) {
            n2 = mm;
            break;
          }
        if (!comp) {
          Vp[0] = L.vp[1 + 2 * (n1 - 1)];
          Vp[1] = L.vp[2 * (n2 - 1)];
          Vs[0] = L.vs[1 + 2 * (n1 - 1)];
          Vs[1] = L.vs[2 * (n2 - 1)];
          Dp[0] = L.dp[1 + 2 * (n1 - 1)];
          Dp[1] = L.dp[2 * (n2 - 1)];
        } else {
          Vp[0] = at2c(c, L.vp, L.ni, L.nj, 1, n1);
          Vs[0] = at2c(c, L.vs, L.ni, L.nj, 1, n1);
          Dp[0] = at2c(c, L.dp, L.ni, L.nj, 1, n1);
          Vp[1] = at2c(c, L.vp, L.ni, L.nj, 0, n2);
          Vs[1] = at2c(c, L.vs, L.ni, L.nj, 0, n2);
          Dp[1] = at2c(c, L.dp, L.ni, L.nj, 0, n2);
        }
        break;
      } else if (d > d0) {
        if (!comp) {
          const float L1 = (d - d0) / h, L2 = 1.0f - L1;
          const int q = 2 * (n - 1);
          set1(L.vp[q] * L1 + L.vp[q + 1] * L2, L.vs[q] * L1 + L.vs[q + 1] * L2, L.dp[q] * L1 + L.dp[q + 1] * L2);
        } else {
          const float p1 = at2c(c, L.vp, L.ni, L.nj, 0, n), s1 = at2c(c, L.vs, L.ni, L.nj, 0, n);
          const float r1 = at2c(c, L.dp, L.ni, L.nj, 0, n), p2 = at2c(c, L.vp, L.ni, L.nj, 1, n);
          const float s2 = at2c(c, L.vs, L.ni, L.nj, 1, n), r2 = at2c(c, L.dp, L.ni, L.nj, 1, n);
          const float t = d0 - (d - h);
          const float ep = L.vpd[n - 1], es = L.vsd[n - 1], er = L.dpd[n - 1];
          set1(p1 + (p2 - p1) / powf(h, ep) * powf(t, ep), s1 + (s2 - s1) / powf(h, es) * powf(t, es),
               r1 + (r2 - r1) / powf(h, er) * powf(t, er));
        }
        break;
      } else if (n == L.nk) {
        return false;
      }
    }
  } else if (a.bkind == FWANT_MEDIA_VOLUME) {  // :1131-1142
    const Cell3 c = cell3(a.bv, x0, y0, z0);
    set1(at3(c, a.bv, a.bv.vp), at3(c, a.bv, a.bv.vs), at3(c, a.bv, a.bv.dp));
  } else if (a.bkind == FWANT_MEDIA_VERPOLY) {  // :1143-1171
    verpoly(a.bp, x0, y0, z0, dz2, Vp, Vs, Dp);
  }
  return true;
}

// perturbation of one sample (:1173-1220)
__device__ __forceinline__ void pt_sample(const Args& a, float x0, float y0, float z0, float dz2, float* Vp, float* Vs,
                                          float* Dp) {
  if (a.pkind == FWANT_MEDIA_VOLUME) {  // :1175-1190
    const Cell3 c = cell3(a.pv, x0, y0, z0);
    const float dVp = at3(c, a.pv, a.pv.vp), dVs = at3(c, a.pv, a.pv.vs), dDp = at3(c, a.pv, a.pv.dp);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      Vp[s] = Vp[s] * (1.0f + dVp);
      Vs[s] = Vs[s] * (1.0f + dVs);
      Dp[s] = Dp[s] * (1.0f + dDp);
    }
  } else if (a.pkind == FWANT_MEDIA_VERPOLY) {  // :1192-1220
    float dVp[2], dVs[2], dDp[2];
    verpoly(a.pp, x0, y0, z0, dz2, dVp, dVs, dDp);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      Vp[s] = Vp[s] * (1.0f + dVp[s]);
      Vs[s] = Vs[s] * (1.0f + dVs[s]);
      Dp[s] = Dp[s] * (1.0f + dDp[s]);
    }
  }
}

// Lame parameters of one sample, arithmetic rho and harmonic lambda, mu (:1222-1235)
__device__ __forceinline__ void accumulate(const float* Vp, const float* Vs, const float* Dp, float& rho0, float& mu0,
                                           float& lam0, bool& flag_water, int& nwater) {
  float miu[2], la[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    miu[s] = Dp[s] * Vs[s] * Vs[s];
    la[s] = Vp[s] * Vp[s] * Dp[s] - 2.0f * miu[s];
  }
  rho0 = rho0 + 0.5f * (Dp[0] + Dp[1]);
  if (miu[0] <= SEIS_ZERO || miu[1] <= SEIS_ZERO) {
    flag_water = true;
    nwater = nwater + 1;
  } else {
    mu0 = mu0 + 0.5f * (1.0f / miu[0] + 1.0f / miu[1]);
  }
  lam0 = lam0 + 0.5f * (1.0f / la[0] + 1.0f / la[1]);
}

// effmedia_eval at one interior point (0-based array indices), any half_sample_point;
// false on the lowest-layer error
__device__ bool eval_point(const Args& a, int i, int j, int k, float& lam_out, float& mu_out, float& rho_out) {
  const int NX = a.ng[0], NY = a.ng[1], NZ = a.ng[2];
  const int nsamp = max(2 * NX, 1) * max(2 * NY, 1) * max(2 * NZ, 1);
  const float* x = a.x;
  const float* y = a.y;
  const float* z = a.z;
  const float dx1 = (x[i] - x[i - 1]) / 2.0f / float(NX + 1), dx2 = (x[i + 1] - x[i]) / 2.0f / float(NX + 1);
  const float dy1 = (y[j] - y[j - 1]) / 2.0f / float(NY + 1), dy2 = (y[j + 1] - y[j]) / 2.0f / float(NY + 1);
  const float dz1 = (z[k] - z[k - 1]) / 2.0f / float(NZ + 1), dz2 = (z[k + 1] - z[k]) / 2.0f / float(NZ + 1);
  float rho0 = 0.0f, mu0 = 0.0f, lam0 = 0.0f;
  bool flag_water = false;
  int nwater = 0;
  float Vp[2] = {0.0f, 0.0f}, Vs[2] = {0.0f, 0.0f}, Dp[2] = {0.0f, 0.0f};
  for (int mk = -NZ; mk <= NZ; ++mk) {
    if (NZ != 0 && mk == 0) continue;
    const float z0 = mk < 0 ? float(mk) * dz1 + z[k] : mk > 0 ? float(mk) * dz2 + z[k] : z[k];
    const float d0 = fmaxf(a.ztopo - z0, 0.0f);
    for (int mj = -NY; mj <= NY; ++mj) {
      if (NY != 0 && mj == 0) continue;
      const float y0 = mj < 0 ? float(mj) * dy1 + y[j] : mj > 0 ? float(mj) * dy2 + y[j] : y[j];
      for (int mi = -NX; mi <= NX; ++mi) {
        if (NX != 0 && mi == 0) continue;
        const float x0 = mi < 0 ? float(mi) * dx1 + x[i] : mi > 0 ? float(mi) * dx2 + x[i] : x[i];
        if (!bg_sample(a, x0, y0, z0, d0, dz2, Vp, Vs, Dp)) return false;
        pt_sample(a, x0, y0, z0, dz2, Vp, Vs, Dp);
        accumulate(Vp, Vs, Dp, rho0, mu0, lam0, flag_water, nwater);
      }
    }
  }
  rho_out = rho0 / float(nsamp);
  if (flag_water) mu_out = nwater >= nsamp / 2 ? 0.0f : float(nsamp - nwater) / mu0;
  else mu_out = float(nsamp) / mu0;
  lam_out = float(nsamp) / lam0;
  return true;
}

// A located model axis of a volume: bracketing index and the two Lagrange weights.
struct VolAxis {
  int i1;
  float l1, l2;
};

__device__ __forceinline__ VolAxis vaxis(const float* g, int n, float v) {
  VolAxis r;
  float v1;
  locate(v, g, n, r.i1, v1);
  lweights(g[r.i1 - 1], g[r.i1], v1, r.l1, r.l2);
  return r;
}

// interp_3d at axes located separately (the same products and sums as at3)
__device__ __forceinline__ float at3h(const VolAxis& cx, const VolAxis& cy, const VolAxis& cz, const DVol& V,
                                      const float* f) {
  const float lx[2] = {cx.l1, cx.l2}, ly[2] = {cy.l1, cy.l2}, lz[2] = {cz.l1, cz.l2};
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int i = 0; i < 2; ++i)
        s = s + lx[i] * ly[j] * lz[k] * f[(size_t(cz.i1 - 1 + k) * V.nj + (cy.i1 - 1 + j)) * V.ni + (cx.i1 - 1 + i)];
  return s;
}

// eval_point for half_sample_point 0 or 1 on each axis (SX, SY, SZ = samples per axis, 1
// or 2).  The look-ups that depend on one coordinate only are hoisted out of the sample
// loops: a cart1d background depends on the depth alone, and a volume's bisections and
// weights are separable by axis.  Every value is formed by the same operations as in
// eval_point, so both paths give identical results.
template <int SX, int SY, int SZ>
__device__ bool eval_fast(const Args& a, int i, int j, int k, float& lam_out, float& mu_out, float& rho_out) {
  constexpr int nsamp = SX * SY * SZ;
  const float* x = a.x;
  const float* y = a.y;
  const float* z = a.z;
  float xs[SX], ys[SY], zs[SZ], ds[SZ];
  if constexpr (SX == 2) {
    xs[0] = -1.0f * ((x[i] - x[i - 1]) / 2.0f / 2.0f) + x[i];
    xs[1] = 1.0f * ((x[i + 1] - x[i]) / 2.0f / 2.0f) + x[i];
  } else {
    xs[0] = x[i];
  }
  if constexpr (SY == 2) {
    ys[0] = -1.0f * ((y[j] - y[j - 1]) / 2.0f / 2.0f) + y[j];
    ys[1] = 1.0f * ((y[j + 1] - y[j]) / 2.0f / 2.0f) + y[j];
  } else {
    ys[0] = y[j];
  }
  const float dz2 = (z[k + 1] - z[k]) / 2.0f / float(SZ);
  if constexpr (SZ == 2) {
    zs[0] = -1.0f * ((z[k] - z[k - 1]) / 2.0f / 2.0f) + z[k];
    zs[1] = 1.0f * dz2 + z[k];
  } else {
    zs[0] = z[k];
  }
#pragma unroll
  for (int q = 0; q < SZ; ++q) ds[q] = fmaxf(a.ztopo - zs[q], 0.0f);
  const bool cart = a.bkind == FWANT_MEDIA_CART1D, bvol = a.bkind == FWANT_MEDIA_VOLUME;
  const bool pvol = a.pkind == FWANT_MEDIA_VOLUME;
  float cVp[SZ][2], cVs[SZ][2], cDp[SZ][2];
  if (cart) {
#pragma unroll
    for (int q = 0; q < SZ; ++q) cart1d_lookup(a.c, ds[q], cVp[q], cVs[q], cDp[q]);
  }
  VolAxis bx[SX], by[SY], bz[SZ], px[SX], py[SY], pz[SZ];
  if (bvol) {
#pragma unroll
    for (int q = 0; q < SX; ++q) bx[q] = vaxis(a.bv.x, a.bv.ni, xs[q]);
#pragma unroll
    for (int q = 0; q < SY; ++q) by[q] = vaxis(a.bv.y, a.bv.nj, ys[q]);
#pragma unroll
    for (int q = 0; q < SZ; ++q) bz[q] = vaxis(a.bv.rz, a.bv.nk, a.bv.rz0 - zs[q]);
  }
  if (pvol) {
#pragma unroll
    for (int q = 0; q < SX; ++q) px[q] = vaxis(a.pv.x, a.pv.ni, xs[q]);
#pragma unroll
    for (int q = 0; q < SY; ++q) py[q] = vaxis(a.pv.y, a.pv.nj, ys[q]);
#pragma unroll
    for (int q = 0; q < SZ; ++q) pz[q] = vaxis(a.pv.rz, a.pv.nk, a.pv.rz0 - zs[q]);
  }
  float rho0 = 0.0f, mu0 = 0.0f, lam0 = 0.0f;
  bool flag_water = false;
  int nwater = 0;
  float Vp[2] = {0.0f, 0.0f}, Vs[2] = {0.0f, 0.0f}, Dp[2] = {0.0f, 0.0f};
#pragma unroll
  for (int mk = 0; mk < SZ; ++mk)
#pragma unroll
    for (int mj = 0; mj < SY; ++mj)
#pragma unroll
      for (int mi = 0; mi < SX; ++mi) {
        if (cart) {
          Vp[0] = cVp[mk][0]; Vp[1] = cVp[mk][1];
          Vs[0] = cVs[mk][0]; Vs[1] = cVs[mk][1];
          Dp[0] = cDp[mk][0]; Dp[1] = cDp[mk][1];
        } else if (bvol) {
          Vp[0] = Vp[1] = at3h(bx[mi], by[mj], bz[mk], a.bv, a.bv.vp);
          Vs[0] = Vs[1] = at3h(bx[mi], by[mj], bz[mk], a.bv, a.bv.vs);
          Dp[0] = Dp[1] = at3h(bx[mi], by[mj], bz[mk], a.bv, a.bv.dp);
        } else if (!bg_sample(a, xs[mi], ys[mj], zs[mk], ds[mk], dz2, Vp, Vs, Dp)) {
          return false;
        }
        if (pvol) {
          const float dVp = at3h(px[mi], py[mj], pz[mk], a.pv, a.pv.vp);
          const float dVs = at3h(px[mi], py[mj], pz[mk], a.pv, a.pv.vs);
          const float dDp = at3h(px[mi], py[mj], pz[mk], a.pv, a.pv.dp);
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            Vp[s] = Vp[s] * (1.0f + dVp);
            Vs[s] = Vs[s] * (1.0f + dVs);
            Dp[s] = Dp[s] * (1.0f + dDp);
          }
        } else {
          pt_sample(a, xs[mi], ys[mj], zs[mk], dz2, Vp, Vs, Dp);
        }
        accumulate(Vp, Vs, Dp, rho0, mu0, lam0, flag_water, nwater);
      }
  rho_out = rho0 / float(nsamp);
  if (flag_water) mu_out = nwater >= nsamp / 2 ? 0.0f : float(nsamp - nwater) / mu0;
  else mu_out = float(nsamp) / mu0;
  lam_out = float(nsamp) / lam0;
  return true;
}

// SX = 0: any half_sample_point (eval_point); else the hoisted form for 0 / 1 per axis
template <int SX, int SY, int SZ>
__global__ void __launch_bounds__(MD_THREADS, SX == 0 ? 2 : 3) effmedia_kernel(const Args a) {
  const long long n = (long long)a.ni * a.nj * a.nk;
  for (long long p = (long long)blockIdx.x * MD_THREADS + threadIdx.x; p < n; p += (long long)gridDim.x * MD_THREADS) {
    const int i = int(p % a.ni) + LENFD;
    const int j = int((p / a.ni) % a.nj) + LENFD;
    const int k = int(p / ((long long)a.ni * a.nj)) + LENFD;
    float l, m, r;
    bool ok;
    if constexpr (SX == 0) ok = eval_point(a, i, j, k, l, m, r);
    else ok = eval_fast<SX, SY, SZ>(a, i, j, k, l, m, r);
    if (!ok) {
      atomicExch(a.err, 1);
      l = m = r = 0.0f;
    }
    const size_t q = (size_t(k) * a.ny + j) * a.nx + i;
    a.lam[q] = l;
    a.mu[q] = m;
    a.rho[q] = r;
  }
}

void launch_effmedia(const Args& a, int grid, cudaStream_t st) {
  const int s0 = a.ng[0] + 1, s1 = a.ng[1] + 1, s2 = a.ng[2] + 1;
  const int key = (s0 <= 2 && s1 <= 2 && s2 <= 2) ? (s0 - 1) * 4 + (s1 - 1) * 2 + (s2 - 1) : -1;
  switch (key) {
    case 0: effmedia_kernel<1, 1, 1><<<grid, MD_THREADS, 0, st>>>(a); break;
    case 1: effmedia_kernel<1, 1, 2><<<grid, MD_THREADS, 0, st>>>(a); break;
    case 2: effmedia_kernel<1, 2, 1><<<grid, MD_THREADS, 0, st>>>(a); break;
    case 3: effmedia_kernel<1, 2, 2><<<grid, MD_THREADS, 0, st>>>(a); break;
    case 4: effmedia_kernel<2, 1, 1><<<grid, MD_THREADS, 0, st>>>(a); break;
    case 5: effmedia_kernel<2, 1, 2><<<grid, MD_THREADS, 0, st>>>(a); break;
    case 6: effmedia_kernel<2, 2, 1><<<grid, MD_THREADS, 0, st>>>(a); break;
    case 7: effmedia_kernel<2, 2, 2><<<grid, MD_THREADS, 0, st>>>(a); break;
    default: effmedia_kernel<0, 0, 0><<<grid, MD_THREADS, 0, st>>>(a); break;
  }
}

// extend_equal: every ghost point takes the value of the nearest interior point (the
// reference's x, y and z passes leave exactly that)
__global__ void __launch_bounds__(MD_THREADS) extend_kernel(const Args a) {
  const long long n = (long long)a.nx * a.ny * a.nz;
  for (long long p = (long long)blockIdx.x * MD_THREADS + threadIdx.x; p < n; p += (long long)gridDim.x * MD_THREADS) {
    const int i = int(p % a.nx), j = int((p / a.nx) % a.ny), k = int(p / ((long long)a.nx * a.ny));
    const int ci = min(max(i, LENFD), LENFD + a.ni - 1), cj = min(max(j, LENFD), LENFD + a.nj - 1);
    const int ck = min(max(k, LENFD), LENFD + a.nk - 1);
    if (ci == i && cj == j && ck == k) continue;
    const size_t s = (size_t(ck) * a.ny + cj) * a.nx + ci;
    a.lam[p] = a.lam[s];
    a.mu[p] = a.mu[s];
    a.rho[p] = a.rho[s];
  }
}

struct StArgs {
  int ni, nj, nk, nx, ny;
  const float *z, *lam, *mu, *rho;
  const double *ca, *sa, *cb, *sb;  // cos / sin of x - pi/2 and of y, per grid index
  // FP32 screen: the same cos / sin and their differences to the next and previous grid
  // index (formed in double on the host), and the z differences
  const float *fca, *fsa, *dcap, *dcam, *dsap, *dsam;   // [nx]
  const float *fcb, *fsb, *dcbp, *dcbm, *dsbp, *dsbm;   // [ny]
  const float *dzp, *dzm;                               // [nz]
  const unsigned* screen_min;  // bits of the screen's minimum (pass 2)
};

__device__ __forceinline__ void gpoint(const StArgs& s, int i, int j, int k, double* g) {
  const double zz = double(s.z[k]);
  g[0] = zz * s.ca[i] * s.cb[j];
  g[1] = zz * s.ca[i] * s.sb[j];
  g[2] = zz * s.sa[i];
}

// dist_point2plane (:1301-1313)
__device__ double plane_dist(const double* P, const double* A, const double* B, const double* C) {
  double AB[3], AC[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    AB[q] = B[q] - A[q];
    AC[q] = C[q] - A[q];
  }
  const double p0 = AB[1] * AC[2] - AB[2] * AC[1];
  const double p1 = AB[2] * AC[0] - AB[0] * AC[2];
  const double p2 = AB[0] * AC[1] - AB[1] * AC[0];
  const double d = -(p0 * A[0] + p1 * A[1] + p2 * A[2]);
  return fabs((p0 * P[0] + p1 * P[1] + p2 * P[2] + d) / sqrt(p0 * p0 + p1 * p1 + p2 * p2));
}

// 1.3 / Vp * dL at an interior point (:1564-1600); dL the distance to the nearest of the
// eight planes through one neighbour along each axis
__device__ float point_dt(const StArgs& s, int i, int j, int k, float& vp, float& dl) {
  const size_t p = (size_t(k) * s.ny + j) * s.nx + i;
  vp = sqrtf((s.lam[p] + 2.0f * s.mu[p]) / s.rho[p]);
  double P[3], A[3], B[3], C[3];
  gpoint(s, i, j, k, P);
  double dmin = 0.0;
#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    gpoint(s, (q & 1) ? i + 1 : i - 1, j, k, A);
    gpoint(s, i, (q & 2) ? j + 1 : j - 1, k, B);
    gpoint(s, i, j, (q & 4) ? k + 1 : k - 1, C);
    const double dd = plane_dist(P, A, B, C);
    dmin = q == 0 ? dd : fmin(dmin, dd);
  }
  dl = float(dmin);
  return 1.3f / vp * dl;
}

// The same quantity in FP32 from neighbour offsets relative to the point (each a product of
// a few accurately rounded factors, so no large coordinates cancel): within about 1e-6 of
// the exact value, used only to find the points that can hold the minimum.
__device__ float point_dt32(const StArgs& s, int i, int j, int k) {
  const size_t p = (size_t(k) * s.ny + j) * s.nx + i;
  const float vp = sqrtf((s.lam[p] + 2.0f * s.mu[p]) / s.rho[p]);
  const float zk = s.z[k], ca = s.fca[i], sa = s.fsa[i], cb = s.fcb[j], sb = s.fsb[j];
  float ax[2][3], by[2][3], cz[2][3];
  const float dca[2] = {s.dcam[i], s.dcap[i]}, dsa[2] = {s.dsam[i], s.dsap[i]};
  const float dcb[2] = {s.dcbm[j], s.dcbp[j]}, dsb[2] = {s.dsbm[j], s.dsbp[j]};
  const float dz[2] = {s.dzm[k], s.dzp[k]};
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    ax[q][0] = zk * dca[q] * cb;
    ax[q][1] = zk * dca[q] * sb;
    ax[q][2] = zk * dsa[q];
    by[q][0] = zk * ca * dcb[q];
    by[q][1] = zk * ca * dsb[q];
    by[q][2] = 0.0f;
    cz[q][0] = dz[q] * ca * cb;
    cz[q][1] = dz[q] * ca * sb;
    cz[q][2] = dz[q] * sa;
  }
  float dmin = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float* a = ax[q & 1];
    const float* b = by[(q >> 1) & 1];
    const float* c = cz[(q >> 2) & 1];
    const float u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
    const float v0 = c[0] - a[0], v1 = c[1] - a[1], v2 = c[2] - a[2];
    const float p0 = u1 * v2 - u2 * v1, p1 = u2 * v0 - u0 * v2, p2 = u0 * v1 - u1 * v0;
    const float d = fabsf(p0 * a[0] + p1 * a[1] + p2 * a[2]) / sqrtf(p0 * p0 + p1 * p1 + p2 * p2);
    dmin = q == 0 ? d : fminf(dmin, d);
  }
  return 1.3f / vp * dmin;
}

// pass 1: the screen's minimum over interior points (NaN excluded) as float bits
__global__ void __launch_bounds__(MD_THREADS) stept_screen_kernel(const StArgs s, unsigned* out) {
  const long long n = (long long)s.ni * s.nj * s.nk;
  float best = INFINITY;
  for (long long p = (long long)blockIdx.x * MD_THREADS + threadIdx.x; p < n; p += (long long)gridDim.x * MD_THREADS) {
    const int i = int(p % s.ni) + LENFD, j = int((p / s.ni) % s.nj) + LENFD, k = int(p / ((long long)s.ni * s.nj)) + LENFD;
    const float v = point_dt32(s, i, j, k);
    if (v < best) best = v;
  }
  for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_down_sync(0xffffffffu, best, o));
  // non-negative floats order like their bit patterns
  if ((threadIdx.x & 31) == 0 && best < INFINITY) atomicMin(out, __float_as_uint(fmaxf(best, 0.0f)));
}

// a point can hold the exact minimum only if its screen value is within this factor of the
// screen's minimum (the screen's error is about 1e-6 relative)
constexpr float SCREEN_MARGIN = 1.0e-3f;

// (value, interior point number) minimum; NaN counts as no candidate, as `dtlocal < dtmax`
// is false for it in the reference
__device__ __forceinline__ bool better(float v, long long p, float bv, long long bp) {
  return v < bv || (v == bv && p < bp);
}

__global__ void __launch_bounds__(MD_THREADS) stept_kernel(const StArgs s, float* pv, long long* pp) {
  __shared__ float sv[MD_THREADS / 32];
  __shared__ long long sp[MD_THREADS / 32];
  const long long n = (long long)s.ni * s.nj * s.nk;
  float bv = 1.0e10f;
  long long bp = n;  // none
  const unsigned sm = *s.screen_min;
  const float thr = sm == 0xffffffffu ? INFINITY : __uint_as_float(sm) * (1.0f + SCREEN_MARGIN);
  for (long long p = (long long)blockIdx.x * MD_THREADS + threadIdx.x; p < n; p += (long long)gridDim.x * MD_THREADS) {
    const int i = int(p % s.ni) + LENFD, j = int((p / s.ni) % s.nj) + LENFD, k = int(p / ((long long)s.ni * s.nj)) + LENFD;
    if (!(point_dt32(s, i, j, k) <= thr)) continue;  // cannot hold the minimum
    float vp, dl;
    const float v = point_dt(s, i, j, k, vp, dl);
    if (better(v, p, bv, bp)) {
      bv = v;
      bp = p;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_down_sync(0xffffffffu, bv, o);
    const long long op = __shfl_down_sync(0xffffffffu, bp, o);
    if (better(ov, op, bv, bp)) {
      bv = ov;
      bp = op;
    }
  }
  if ((threadIdx.x & 31) == 0) {
    sv[threadIdx.x >> 5] = bv;
    sp[threadIdx.x >> 5] = bp;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < MD_THREADS / 32; ++w)
      if (better(sv[w], sp[w], bv, bp)) {
        bv = sv[w];
        bp = sp[w];
      }
    pv[blockIdx.x] = bv;
    pp[blockIdx.x] = bp;
  }
}

// result[0] = dtmax, [1] = Vp, [2] = dL; *ip = interior point number (n if none)
__global__ void stept_final_kernel(const StArgs s, const float* pv, const long long* pp, int np, float* result,
                                   long long* ip) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const long long n = (long long)s.ni * s.nj * s.nk;
  float bv = 1.0e10f;
  long long bp = n;
  for (int q = 0; q < np; ++q)
    if (better(pv[q], pp[q], bv, bp)) {
      bv = pv[q];
      bp = pp[q];
    }
  result[0] = bv;
  result[1] = result[2] = 0.0f;
  *ip = bp;
  if (bp < n) {
    const int i = int(bp % s.ni) + LENFD, j = int((bp / s.ni) % s.nj) + LENFD, k = int(bp / ((long long)s.ni * s.nj)) + LENFD;
    float vp, dl;
    point_dt(s, i, j, k, vp, dl);
    result[1] = vp;
    result[2] = dl;
  }
}

// volume_read / verpoly_read column selection: [a, b] (1-based) from the largest model
// coordinate <= max(grid first, model first) to the smallest >= min(grid last, model last)
void model_range(const float* g, int n, float lo, float hi, int& a, int& b) {
  const float tlo = std::max(lo, g[0]), thi = std::min(hi, g[n - 1]);
  a = 1;
  b = n;
  bool fa = false, fb = false;
  float av = 0.0f, bv = 0.0f;
  for (int q = 0; q < n; ++q) {
    if (g[q] <= tlo && (!fa || g[q] > av)) {
      av = g[q];
      a = q + 1;
      fa = true;
    }
    if (g[q] >= thi && (!fb || g[q] < bv)) {
      bv = g[q];
      b = q + 1;
      fb = true;
    }
  }
}

}  // namespace

struct fwant_media {
  int device = 0;
  int ni = 0, nj = 0, nk = 0, nx = 0, ny = 0, nz = 0;
  int ng[3] = {0, 0, 0};
  float ztopo = 0.0f;
  std::vector<float> hx, hy, hz;  // grid on the host (model selection)
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<void*> model_bufs[2];  // device arrays of the background (0) and perturbation (1)
  int slot = 0;                      // the model being uploaded
  float *x = nullptr, *y = nullptr, *z = nullptr;
  float *lam = nullptr, *mu = nullptr, *rho = nullptr;
  double* trig = nullptr;  // ca[nx], sa[nx], cb[ny], sb[ny]
  float* screen = nullptr;  // FP32 screen tables: 6 x nx, 6 x ny, 2 x nz
  unsigned* smin = nullptr;
  int* err = nullptr;
  float* pv = nullptr;
  long long* pp = nullptr;
  float* res = nullptr;
  long long* ip = nullptr;
  Args a{};
  bool evaluated = false;
  double last_ms = 0.0;
  std::string msg;

  ~fwant_media() {
    cudaSetDevice(device);
    free_models();
    for (void* p : {(void*)x, (void*)y, (void*)z, (void*)lam, (void*)mu, (void*)rho, (void*)trig, (void*)screen,
                    (void*)smin, (void*)err,
                    (void*)pv, (void*)pp, (void*)res, (void*)ip})
      cudaFree(p);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (st) cudaStreamDestroy(st);
  }
  void free_models() {
    for (auto& v : model_bufs) {
      for (void* p : v) cudaFree(p);
      v.clear();
    }
  }
  // A new background (s = 0) or perturbation (s = 1) replaces the previous one: its arrays
  // are freed and the kind cleared until the new model is complete.
  void begin_model(int s) {
    for (void* p : model_bufs[s]) cudaFree(p);
    model_bufs[s].clear();
    if (s == 0) a.bkind = 0;
    else a.pkind = 0;
    slot = s;
  }
  fwant_status fail(fwant_status c, const std::string& m) {
    msg = m;
    return c;
  }
  // upload n floats; nullptr on failure (msg set)
  const float* up(const float* h, size_t n, const char* what) {
    void* d = nullptr;
    if (cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      msg = std::string("out of device memory: ") + what;
      return nullptr;
    }
    model_bufs[slot].push_back(d);
    if (cudaMemcpy(d, h, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      msg = std::string("copy failed: ") + what;
      return nullptr;
    }
    return static_cast<const float*>(d);
  }
};

extern "C" {

fwant_status fwant_media_create(int ni, int nj, int nk, const float* x, const float* y, const float* z, float ztopo,
                                const int half_sample[3], int device, fwant_media** out) {
  if (!out) return FWANT_ERR_INVALID_ARG;
  *out = nullptr;
  if (ni < 1 || nj < 1 || nk < 1 || !x || !y || !z || !half_sample) return FWANT_ERR_INVALID_ARG;
  for (int q = 0; q < 3; ++q)
    if (half_sample[q] < 0 || half_sample[q] > MAX_HALF) return FWANT_ERR_INVALID_ARG;
  const long long npts = (long long)(ni + 2 * LENFD) * (nj + 2 * LENFD) * (nk + 2 * LENFD);
  if (npts > (1LL << 40)) return FWANT_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return FWANT_ERR_CUDA;
  }
  auto* m = new fwant_media();
  m->device = device;
  m->ni = ni;
  m->nj = nj;
  m->nk = nk;
  m->nx = ni + 2 * LENFD;
  m->ny = nj + 2 * LENFD;
  m->nz = nk + 2 * LENFD;
  for (int q = 0; q < 3; ++q) m->ng[q] = half_sample[q];
  m->ztopo = ztopo;
  m->hx.assign(x, x + m->nx);
  m->hy.assign(y, y + m->ny);
  m->hz.assign(z, z + m->nz);
  // cos / sin of the grid angles for the time-step check (media_stept_check :1551-1559)
  std::vector<double> trig(size_t(2) * (m->nx + m->ny));
  for (int i = 0; i < m->nx; ++i) {
    const double ang = double(x[i]) - PI_D / 2;
    trig[i] = std::cos(ang);
    trig[m->nx + i] = std::sin(ang);
  }
  for (int j = 0; j < m->ny; ++j) {
    const double ang = double(y[j]);
    trig[2 * m->nx + j] = std::cos(ang);
    trig[2 * m->nx + m->ny + j] = std::sin(ang);
  }
  // FP32 screen of the time-step check: cos / sin and their differences to the next and
  // previous index (differences formed in double), z differences
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  std::vector<float> scr(size_t(6) * nx + size_t(6) * ny + size_t(2) * nz, 0.0f);
  {
    float* f = scr.data();
    const double* ca = trig.data();
    const double* sa = ca + nx;
    const double* cb = sa + nx;
    const double* sb = cb + ny;
    for (int i = 0; i < nx; ++i) {
      f[i] = float(ca[i]);
      f[nx + i] = float(sa[i]);
      f[2 * nx + i] = i + 1 < nx ? float(ca[i + 1] - ca[i]) : 0.0f;
      f[3 * nx + i] = i > 0 ? float(ca[i - 1] - ca[i]) : 0.0f;
      f[4 * nx + i] = i + 1 < nx ? float(sa[i + 1] - sa[i]) : 0.0f;
      f[5 * nx + i] = i > 0 ? float(sa[i - 1] - sa[i]) : 0.0f;
    }
    float* g = f + 6 * nx;
    for (int j = 0; j < ny; ++j) {
      g[j] = float(cb[j]);
      g[ny + j] = float(sb[j]);
      g[2 * ny + j] = j + 1 < ny ? float(cb[j + 1] - cb[j]) : 0.0f;
      g[3 * ny + j] = j > 0 ? float(cb[j - 1] - cb[j]) : 0.0f;
      g[4 * ny + j] = j + 1 < ny ? float(sb[j + 1] - sb[j]) : 0.0f;
      g[5 * ny + j] = j > 0 ? float(sb[j - 1] - sb[j]) : 0.0f;
    }
    float* h = g + 6 * ny;
    for (int k = 0; k < nz; ++k) {
      h[k] = k + 1 < nz ? float(double(z[k + 1]) - double(z[k])) : 0.0f;
      h[nz + k] = k > 0 ? float(double(z[k - 1]) - double(z[k])) : 0.0f;
    }
  }
  const size_t n3 = size_t(npts);
  cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&m->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&m->ev1);
  if (e == cudaSuccess) e = cudaMalloc(&m->x, m->nx * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->y, m->ny * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->z, m->nz * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->trig, trig.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&m->screen, scr.size() * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->smin, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&m->lam, n3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->mu, n3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->rho, n3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&m->pv, ST_BLOCKS * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->pp, ST_BLOCKS * sizeof(long long));
  if (e == cudaSuccess) e = cudaMalloc(&m->res, 4 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->ip, sizeof(long long));
  if (e == cudaSuccess) e = cudaMemcpy(m->x, x, m->nx * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->y, y, m->ny * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->z, z, m->nz * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->trig, trig.data(), trig.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->screen, scr.data(), scr.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    const fwant_status rc = e == cudaErrorMemoryAllocation ? FWANT_ERR_OOM : FWANT_ERR_CUDA;
    cudaGetLastError();
    delete m;
    return rc;
  }
  Args& a = m->a;
  a.ni = ni;
  a.nj = nj;
  a.nk = nk;
  a.nx = m->nx;
  a.ny = m->ny;
  a.nz = m->nz;
  for (int q = 0; q < 3; ++q) a.ng[q] = half_sample[q];
  a.ztopo = ztopo;
  a.x = m->x;
  a.y = m->y;
  a.z = m->z;
  a.lam = m->lam;
  a.mu = m->mu;
  a.rho = m->rho;
  a.err = m->err;
  *out = m;
  return FWANT_OK;
}

void fwant_media_destroy(fwant_media* m) { delete m; }

const char* fwant_media_last_error(fwant_media* m) { return m ? m->msg.c_str() : "null handle"; }

fwant_status fwant_media_set_cart1d(fwant_media* m, int nk, const float* depth, const float* vp, const float* vs,
                                    const float* rho) {
  if (!m) return FWANT_ERR_INVALID_ARG;
  if (nk < 2 || !depth || !vp || !vs || !rho)
    return m->fail(FWANT_ERR_INVALID_ARG, "media_set_cart1d: nk >= 2 samples and all arrays required");
  for (int k = 1; k < nk; ++k)
    if (!(depth[k] >= depth[k - 1])) return m->fail(FWANT_ERR_INVALID_ARG, "media_set_cart1d: depths must ascend");
  cudaSetDevice(m->device);
  m->begin_model(0);
  DCart c;
  c.nk = nk;
  if (!(c.d = m->up(depth, nk, "cart1d")) || !(c.vp = m->up(vp, nk, "cart1d")) || !(c.vs = m->up(vs, nk, "cart1d")) ||
      !(c.dp = m->up(rho, nk, "cart1d")))
    return FWANT_ERR_OOM;
  m->a.c = c;
  m->a.bkind = FWANT_MEDIA_CART1D;
  return FWANT_OK;
}

fwant_status fwant_media_set_layers(fwant_media* m, int kind, int ni, int nj, int nk, const float* x, const float* y,
                                    const float* z, const float* h, const float* vp, const float* vs, const float* rho,
                                    const float* vp_exp, const float* vs_exp, const float* rho_exp) {
  if (!m) return FWANT_ERR_INVALID_ARG;
  if (kind != FWANT_MEDIA_INTERFACE && kind != FWANT_MEDIA_LAYERED && kind != FWANT_MEDIA_COMPOSITE)
    return m->fail(FWANT_ERR_INVALID_ARG, "media_set_layers: kind must be interface, layered or composite");
  if (ni < 2 || nj < 2 || nk < 1 || !x || !y || !h || !vp || !vs || !rho)
    return m->fail(FWANT_ERR_INVALID_ARG, "media_set_layers: ni, nj >= 2, nk >= 1 and all arrays required");
  if (kind == FWANT_MEDIA_INTERFACE && !z) return m->fail(FWANT_ERR_INVALID_ARG, "media_set_layers: interface needs z");
  if (kind == FWANT_MEDIA_COMPOSITE && (!vp_exp || !vs_exp || !rho_exp))
    return m->fail(FWANT_ERR_INVALID_ARG, "media_set_layers: composite needs the exponents");
  cudaSetDevice(m->device);
  m->begin_model(0);
  const size_t n3 = size_t(ni) * nj * nk, nv = kind == FWANT_MEDIA_COMPOSITE ? 2 * n3 : size_t(2) * nk;
  DLayers L{};
  L.ni = ni;
  L.nj = nj;
  L.nk = nk;
  if (!(L.x = m->up(x, ni, "layers")) || !(L.y = m->up(y, nj, "layers")) || !(L.h = m->up(h, n3, "layers")) ||
      !(L.vp = m->up(vp, nv, "layers")) || !(L.vs = m->up(vs, nv, "layers")) || !(L.dp = m->up(rho, nv, "layers")))
    return FWANT_ERR_OOM;
  if (kind == FWANT_MEDIA_INTERFACE && !(L.z = m->up(z, n3, "layers"))) return FWANT_ERR_OOM;
  if (kind == FWANT_MEDIA_COMPOSITE && (!(L.vpd = m->up(vp_exp, nk, "layers")) || !(L.vsd = m->up(vs_exp, nk, "layers")) ||
                                        !(L.dpd = m->up(rho_exp, nk, "layers"))))
    return FWANT_ERR_OOM;
  m->a.L = L;
  m->a.bkind = kind;
  return FWANT_OK;
}

fwant_status fwant_media_set_volume(fwant_media* m, int perturbed, int ni, int nj, int nk, const float* x,
                                    const float* y, const float* rz, float rz0, const float* vp, const float* vs,
                                    const float* rho) {
  if (!m) return FWANT_ERR_INVALID_ARG;
  if (ni < 2 || nj < 2 || nk < 2 || !x || !y || !rz || !vp || !vs || !rho)
    return m->fail(FWANT_ERR_INVALID_ARG, "media_set_volume: ni, nj, nk >= 2 and all arrays required");
  cudaSetDevice(m->device);
  int i1, i2, j1, j2;
  model_range(x, ni, m->hx.front(), m->hx.back(), i1, i2);
  model_range(y, nj, m->hy.front(), m->hy.back(), j1, j2);
  if (i2 - i1 < 1 || j2 - j1 < 1)
    return m->fail(FWANT_ERR_INVALID_ARG, "media_set_volume: the model covers fewer than two columns of the grid");
  const int vi = i2 - i1 + 1, vj = j2 - j1 + 1;
  std::vector<float> f[3];
  const float* src[3] = {vp, vs, rho};
  for (int q = 0; q < 3; ++q) {
    f[q].resize(size_t(vi) * vj * nk);
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < vj; ++j)
        for (int i = 0; i < vi; ++i)
          f[q][(size_t(k) * vj + j) * vi + i] = src[q][(size_t(k) * nj + (j1 - 1 + j)) * ni + (i1 - 1 + i)];
  }
  m->begin_model(perturbed ? 1 : 0);
  DVol V{};
  V.ni = vi;
  V.nj = vj;
  V.nk = nk;
  V.rz0 = rz0;
  if (!(V.x = m->up(x + i1 - 1, vi, "volume")) || !(V.y = m->up(y + j1 - 1, vj, "volume")) ||
      !(V.rz = m->up(rz, nk, "volume")) || !(V.vp = m->up(f[0].data(), f[0].size(), "volume")) ||
      !(V.vs = m->up(f[1].data(), f[1].size(), "volume")) || !(V.dp = m->up(f[2].data(), f[2].size(), "volume")))
    return FWANT_ERR_OOM;
  if (perturbed) {
    m->a.pv = V;
    m->a.pkind = FWANT_MEDIA_VOLUME;
  } else {
    m->a.bv = V;
    m->a.bkind = FWANT_MEDIA_VOLUME;
  }
  return FWANT_OK;
}

fwant_status fwant_media_set_verpoly(fwant_media* m, int perturbed, int ni, int nj, int nk, int npoly,
                                     const float* x, const float* y, const float* rz, float rz0, const float* vp_c,
                                     const float* vs_c, const float* rho_c, const float* vp_exp, const float* vs_exp,
                                     const float* rho_exp) {
  if (!m) return FWANT_ERR_INVALID_ARG;
  if (ni < 1 || nj < 1 || nk < 1 || npoly < 1 || !x || !y || !rz || !vp_c || !vs_c || !rho_c || !vp_exp || !vs_exp ||
      !rho_exp)
    return m->fail(FWANT_ERR_INVALID_ARG, "media_set_verpoly: positive sizes and all arrays required");
  cudaSetDevice(m->device);
  int i1, i2, j1, j2;
  model_range(x, ni, m->hx.front(), m->hx.back(), i1, i2);
  model_range(y, nj, m->hy.front(), m->hy.back(), j1, j2);
  if (i2 < i1 || j2 < j1) return m->fail(FWANT_ERR_INVALID_ARG, "media_set_verpoly: empty model range");
  const int vi = i2 - i1 + 1, vj = j2 - j1 + 1;
  const size_t n3 = size_t(vi) * vj * nk;
  std::vector<float> r(n3), c[3];
  const float* src[3] = {vp_c, vs_c, rho_c};
  for (int q = 0; q < 3; ++q) c[q].resize(n3 * npoly);
  for (int p = 0; p < npoly; ++p)
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < vj; ++j)
        for (int i = 0; i < vi; ++i) {
          const size_t s = ((size_t(p) * nk + k) * nj + (j1 - 1 + j)) * ni + (i1 - 1 + i);
          const size_t d = ((size_t(p) * nk + k) * vj + j) * vi + i;
          if (p == 0) r[d] = rz[s];
          for (int q = 0; q < 3; ++q) c[q][d] = src[q][s];
        }
  m->begin_model(perturbed ? 1 : 0);
  DPoly P{};
  P.ni = vi;
  P.nj = vj;
  P.nk = nk;
  P.np = npoly;
  P.rz0 = rz0;
  if (!(P.x = m->up(x + i1 - 1, vi, "verpoly")) || !(P.y = m->up(y + j1 - 1, vj, "verpoly")) ||
      !(P.rz = m->up(r.data(), n3, "verpoly")) || !(P.vpc = m->up(c[0].data(), c[0].size(), "verpoly")) ||
      !(P.vsc = m->up(c[1].data(), c[1].size(), "verpoly")) || !(P.dpc = m->up(c[2].data(), c[2].size(), "verpoly")) ||
      !(P.vpd = m->up(vp_exp, npoly, "verpoly")) || !(P.vsd = m->up(vs_exp, npoly, "verpoly")) ||
      !(P.dpd = m->up(rho_exp, npoly, "verpoly")))
    return FWANT_ERR_OOM;
  if (perturbed) {
    m->a.pp = P;
    m->a.pkind = FWANT_MEDIA_VERPOLY;
  } else {
    m->a.bp = P;
    m->a.bkind = FWANT_MEDIA_VERPOLY;
  }
  return FWANT_OK;
}

fwant_status fwant_media_eval(fwant_media* m, float* lambda, float* mu, float* rho) {
  if (!m) return FWANT_ERR_INVALID_ARG;
  if (m->a.bkind == 0) return m->fail(FWANT_ERR_STATE, "media_eval: no background model set");
  cudaSetDevice(m->device);
  m->evaluated = false;
  cudaError_t e = cudaMemsetAsync(m->err, 0, sizeof(int), m->st);
  if (e != cudaSuccess) return m->fail(FWANT_ERR_CUDA, std::string("media_eval: ") + cudaGetErrorString(e));
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
  const long long ni3 = (long long)m->ni * m->nj * m->nk, nx3 = (long long)m->nx * m->ny * m->nz;
  const int g1 = int(std::min<long long>((ni3 + MD_THREADS - 1) / MD_THREADS, (long long)sms * 64));
  const int g2 = int(std::min<long long>((nx3 + MD_THREADS - 1) / MD_THREADS, (long long)sms * 32));
  cudaEventRecord(m->ev0, m->st);
  launch_effmedia(m->a, g1, m->st);
  extend_kernel<<<g2, MD_THREADS, 0, m->st>>>(m->a);
  cudaEventRecord(m->ev1, m->st);
  int herr = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
  if (e != cudaSuccess) return m->fail(FWANT_ERR_CUDA, std::string("media_eval: ") + cudaGetErrorString(e));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, m->ev0, m->ev1);
  m->last_ms = ms;
  if (herr) return m->fail(FWANT_ERR_INVALID_ARG, "media_eval: please increase the thickness of the lowest layer");
  const size_t bytes = size_t(nx3) * sizeof(float);
  if (lambda) e = cudaMemcpy(lambda, m->lam, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && mu) e = cudaMemcpy(mu, m->mu, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rho) e = cudaMemcpy(rho, m->rho, bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return m->fail(FWANT_ERR_CUDA, std::string("media_eval copy: ") + cudaGetErrorString(e));
  m->evaluated = true;
  return FWANT_OK;
}

fwant_status fwant_media_stept_check(fwant_media* m, float* dtmax, int ijk[3], float* vp, float* dl) {
  if (!m || !dtmax) return FWANT_ERR_INVALID_ARG;
  if (!m->evaluated) return m->fail(FWANT_ERR_STATE, "media_stept_check: no evaluated medium");
  cudaSetDevice(m->device);
  StArgs s;
  s.ni = m->ni;
  s.nj = m->nj;
  s.nk = m->nk;
  s.nx = m->nx;
  s.ny = m->ny;
  s.z = m->z;
  s.lam = m->lam;
  s.mu = m->mu;
  s.rho = m->rho;
  s.ca = m->trig;
  s.sa = m->trig + m->nx;
  s.cb = m->trig + 2 * m->nx;
  s.sb = m->trig + 2 * m->nx + m->ny;
  {
    const float* f = m->screen;
    const int nx = m->nx, ny = m->ny;
    s.fca = f; s.fsa = f + nx; s.dcap = f + 2 * nx; s.dcam = f + 3 * nx; s.dsap = f + 4 * nx; s.dsam = f + 5 * nx;
    const float* g = f + 6 * nx;
    s.fcb = g; s.fsb = g + ny; s.dcbp = g + 2 * ny; s.dcbm = g + 3 * ny; s.dsbp = g + 4 * ny; s.dsbm = g + 5 * ny;
    s.dzp = g + 6 * ny;
    s.dzm = g + 6 * ny + m->nz;
    s.screen_min = m->smin;
  }
  // pass 1: FP32 screen for the minimum; pass 2: the exact FP64 check on the points that can
  // hold it, reduced over (value, point number)
  cudaMemsetAsync(m->smin, 0xff, sizeof(unsigned), m->st);
  stept_screen_kernel<<<ST_BLOCKS, MD_THREADS, 0, m->st>>>(s, m->smin);
  stept_kernel<<<ST_BLOCKS, MD_THREADS, 0, m->st>>>(s, m->pv, m->pp);
  stept_final_kernel<<<1, 32, 0, m->st>>>(s, m->pv, m->pp, ST_BLOCKS, m->res, m->ip);
  float r[3];
  long long ip = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(r, m->res, 3 * sizeof(float), cudaMemcpyDeviceToHost, m->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&ip, m->ip, sizeof(long long), cudaMemcpyDeviceToHost, m->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
  if (e != cudaSuccess) return m->fail(FWANT_ERR_CUDA, std::string("media_stept_check: ") + cudaGetErrorString(e));
  *dtmax = r[0];
  const long long n = (long long)m->ni * m->nj * m->nk;
  if (ijk) {
    if (ip < n) {
      ijk[0] = int(ip % m->ni) + LENFD + 1;
      ijk[1] = int((ip / m->ni) % m->nj) + LENFD + 1;
      ijk[2] = int(ip / ((long long)m->ni * m->nj)) + LENFD + 1;
    } else {
      ijk[0] = ijk[1] = ijk[2] = 0;
    }
  }
  if (vp) *vp = r[1];
  if (dl) *dl = r[2];
  return FWANT_OK;
}

fwant_status fwant_media_device_arrays(fwant_media* m, const float** lambda, const float** mu, const float** rho) {
  if (!m || !lambda || !mu || !rho) return FWANT_ERR_INVALID_ARG;
  if (!m->evaluated) return m->fail(FWANT_ERR_STATE, "media_device_arrays: no evaluated medium");
  *lambda = m->lam;
  *mu = m->mu;
  *rho = m->rho;
  return FWANT_OK;
}

fwant_status fwant_media_last_eval_ms(fwant_media* m, double* ms) {
  if (!m || !ms) return FWANT_ERR_INVALID_ARG;
  *ms = m->last_ms;
  return FWANT_OK;
}

}  // extern "C"
