// Fused LDDRK4 stage kernel for sm_103a.
//
// One launch performs, for every interior point, what the reference does in five
// separate sweeps of one Runge-Kutta stage:
//   free_timg        traction image above the free surface   mod_macdrp.F90:3414-3436
//   L<X>             18 one-sided derivatives, spherical RHS  mod_macdrp.F90:790-962
//   abs_L<X>         CFS-PML memory-variable corrections      mod_abs_npml.F90:1149-2123
//   src_stress/force source injection with 7^3 smoothing      mod_src.F90:207-345
//   RK_beg/inn/fin   register update of W, t (and PML aux)    mod_macdrp.F90:291-393
// The right-hand side h never goes to memory.  The image values above the surface are
// substituted while loading instead of being written (the stored stress on k = nk2 keeps
// its RK value, exactly as in the reference where RK overwrites the imaged value).
//
// Arithmetic follows the reference's operand order; this file is compiled with
// -fmad=false so that every product and sum rounds exactly like the reference's FP32
// source expression.
#include <cuda_runtime.h>
#include "kernels.h"

namespace fw {

#define MCA_1 (-0.30874f)
#define MCA0 (-0.6326f)
#define MCA1 (1.233f)
#define MCA2 (-0.3334f)
#define MCA3 (0.04168f)

// DRP/opt MacCormack operators (mod_macdrp.h:69-103); v[0..6] hold offsets -3..+3.
template <int F>
__device__ __forceinline__ float dop(const float* v) {
  if (F)
    return MCA_1 * v[2] + MCA0 * v[3] + MCA1 * v[4] + MCA2 * v[5] + MCA3 * v[6];
  else
    return -MCA3 * v[0] - MCA2 * v[1] - MCA1 * v[2] - MCA0 * v[3] - MCA_1 * v[4];
}

// Same operator reading memory along stride s around c.
template <int F>
__device__ __forceinline__ float dopm(const float* __restrict__ c, long long s) {
  if (F)
    return MCA_1 * __ldg(c - s) + MCA0 * __ldg(c) + MCA1 * __ldg(c + s) + MCA2 * __ldg(c + 2 * s) +
           MCA3 * __ldg(c + 3 * s);
  else
    return -MCA3 * __ldg(c - 3 * s) - MCA2 * __ldg(c - 2 * s) - MCA1 * __ldg(c - s) - MCA0 * __ldg(c) -
           MCA_1 * __ldg(c + s);
}

// 2-2 and 2-4 MacCormack operators used by CondFreeVLOW (mod_macdrp.h:230-268).
template <int F>
__device__ __forceinline__ float dop22(const float* __restrict__ c, long long s) {
  if (F) return -1.0f * __ldg(c) + 1.0f * __ldg(c + s);
  else return -1.0f * __ldg(c - s) - -1.0f * __ldg(c);
}
template <int F>
__device__ __forceinline__ float dop24(const float* __restrict__ c, long long s) {
  const float A0 = -7.0f / 6.0f, A1 = 8.0f / 6.0f, A2 = -1.0f / 6.0f;
  if (F) return A0 * __ldg(c) + A1 * __ldg(c + s) + A2 * __ldg(c + 2 * s);
  else return -A2 * __ldg(c - 2 * s) - A1 * __ldg(c - s) - A0 * __ldg(c);
}

// T*Src of component comp (0 = x for Txz, 1 = y for Tyz, 2 = z for Tzz) at interior
// column (i, j) and global stage gst: src_surface (mod_src.F90:373-414), last entry wins.
__device__ __forceinline__ float tsrc(const Sources& S, int gst, int comp, int i, int j) {
  float v = 0.0f;
  for (int e = 0; e < S.nsurf; ++e)
    if (S.surf_ij[2 * e] == i && S.surf_ij[2 * e + 1] == j)
      v = S.surf_q[3 * e + comp] * S.disp[(long long)gst * S.nw_f + S.surf_w[e]];
  return v;
}
__device__ __forceinline__ float vsrc(const Sources& S, int gst, int comp, int i, int j) {
  float v = 0.0f;
  for (int e = 0; e < S.nsurf; ++e)
    if (S.surf_ij[2 * e] == i && S.surf_ij[2 * e + 1] == j)
      v = S.surf_q[3 * e + comp] * S.rate[(long long)gst * S.nw_f + S.surf_w[e]];
  return v;
}

// Value of an imaged stress component (Tzz, Txz, Tyz) on plane kk >= k2 of an interior
// column: free_timg (mod_macdrp.F90:3414-3436).
__device__ __forceinline__ float imaged(const float* __restrict__ col, long long plane, int k2, int kk,
                                        float ts) {
  if (kk == k2) return ts;
  return 2.0f * ts - __ldg(col + (long long)(2 * k2 - kk) * plane);
}

template <int F>
__device__ __forceinline__ void zvals_img(float* v, const float* __restrict__ col, long long plane, int k,
                                          int k2, float ts) {
  const int lo = F ? -1 : -3, hi = F ? 3 : 1;
#pragma unroll
  for (int d = lo; d <= hi; ++d) {
    const int kk = k + d;
    v[d + 3] = (kk < k2) ? __ldg(col + (long long)kk * plane) : imaged(col, plane, k2, kk, ts);
  }
}

template <int F>
__device__ __forceinline__ void hvals_surf(float* v, const float* __restrict__ c, long long s, const Sources& S,
                                           int gst, int comp, int i, int j, int di, int dj, const Geom& g) {
  const int lo = F ? -1 : -3, hi = F ? 3 : 1;
#pragma unroll
  for (int d = lo; d <= hi; ++d) {
    const int ii = i + d * di, jj = j + d * dj;
    const bool inside = ii >= g.i1 && ii <= g.i2 && jj >= g.j1 && jj <= g.j2;
    v[d + 3] = inside ? tsrc(S, gst, comp, ii, jj) : __ldg(c + d * s);
  }
}

template <int FX, int FY, int FZ, int RK, bool NEAR>
__device__ __forceinline__ void stage_point(const StageArgs<float>& A, int i, int j, int k) {
  const Geom& g = A.g;
  const long long plane = g.plane, fs = g.fstride;
  const long long col = (long long)(i + PADL) + (long long)g.px * j;
  const long long p = col + plane * k;
  const float* __restrict__ W = A.win;
  const int gst = __ldg(A.ntime) * 4 + A.stage;

  const float lam = __ldg(A.lam + p), miu = __ldg(A.mu + p);
  const float lam2mu = lam + 2.0f * miu;
  const float rrho = 1.0f / __ldg(A.rho + p);
  const float xi = __ldg(A.xi_x + i), et = __ldg(A.eta_y + j), ze = __ldg(A.zeta_z + k);
  const float r = __ldg(A.zc + k), s = __ldg(A.xsin + i), c = __ldg(A.xcot + i);

  const float* __restrict__ cVx = W + VX * fs + p;
  const float* __restrict__ cVy = W + VY * fs + p;
  const float* __restrict__ cVz = W + VZ * fs + p;
  const float* __restrict__ cTxx = W + TXX * fs + p;
  const float* __restrict__ cTyy = W + TYY * fs + p;
  const float* __restrict__ cTzz = W + TZZ * fs + p;
  const float* __restrict__ cTxy = W + TXY * fs + p;
  const float* __restrict__ cTxz = W + TXZ * fs + p;
  const float* __restrict__ cTyz = W + TYZ * fs + p;

  const bool surf = NEAR && k == g.k2;
  float tsx = 0.0f, tsy = 0.0f, tsz = 0.0f;
  if (NEAR) {
    tsx = tsrc(A.src, gst, 0, i, j);
    tsy = tsrc(A.src, gst, 1, i, j);
    tsz = tsrc(A.src, gst, 2, i, j);
  }

  // centre values (the imaged components read T*Src on the surface)
  const float Vx = __ldg(cVx), Vy = __ldg(cVy), Vz = __ldg(cVz);
  const float Txx = __ldg(cTxx), Tyy = __ldg(cTyy), Txy = __ldg(cTxy);
  const float Tzz = surf ? tsz : __ldg(cTzz);
  const float Txz = surf ? tsx : __ldg(cTxz);
  const float Tyz = surf ? tsy : __ldg(cTyz);

  // ---- x derivatives
  float DxTxx = dopm<FX>(cTxx, 1) * xi;
  float DxTxy = dopm<FX>(cTxy, 1) * xi;
  float DxTxz;
  if (surf) {
    float v[7];
    hvals_surf<FX>(v, cTxz, 1, A.src, gst, 0, i, j, 1, 0, g);
    DxTxz = dop<FX>(v) * xi;
  } else {
    DxTxz = dopm<FX>(cTxz, 1) * xi;
  }
  const float DxVx = dopm<FX>(cVx, 1) * xi;
  const float DxVy = dopm<FX>(cVy, 1) * xi;
  const float DxVz = dopm<FX>(cVz, 1) * xi;
  // ---- y derivatives
  const long long py = g.px;
  float DyTyy = dopm<FY>(cTyy, py) * et;
  float DyTxy = dopm<FY>(cTxy, py) * et;
  float DyTyz;
  if (surf) {
    float v[7];
    hvals_surf<FY>(v, cTyz, py, A.src, gst, 1, i, j, 0, 1, g);
    DyTyz = dop<FY>(v) * et;
  } else {
    DyTyz = dopm<FY>(cTyz, py) * et;
  }
  const float DyVx = dopm<FY>(cVx, py) * et;
  const float DyVy = dopm<FY>(cVy, py) * et;
  const float DyVz = dopm<FY>(cVz, py) * et;
  // ---- z derivatives
  float DzTzz, DzTxz, DzTyz;
  if (NEAR) {
    float v[7];
    zvals_img<FZ>(v, W + TZZ * fs + col, plane, k, g.k2, tsz);
    DzTzz = dop<FZ>(v) * ze;
    zvals_img<FZ>(v, W + TXZ * fs + col, plane, k, g.k2, tsx);
    DzTxz = dop<FZ>(v) * ze;
    zvals_img<FZ>(v, W + TYZ * fs + col, plane, k, g.k2, tsy);
    DzTyz = dop<FZ>(v) * ze;
  } else {
    DzTzz = dopm<FZ>(cTzz, plane) * ze;
    DzTxz = dopm<FZ>(cTxz, plane) * ze;
    DzTyz = dopm<FZ>(cTyz, plane) * ze;
  }
  float DzVx = 0.0f, DzVy = 0.0f, DzVz = 0.0f;
  if (NEAR && k == g.k2 - 1) {
    DzVx = dop22<FZ>(cVx, plane) * ze;
    DzVy = dop22<FZ>(cVy, plane) * ze;
    DzVz = dop22<FZ>(cVz, plane) * ze;
  } else if (NEAR && k == g.k2 - 2) {
    DzVx = dop24<FZ>(cVx, plane) * ze;
    DzVy = dop24<FZ>(cVy, plane) * ze;
    DzVz = dop24<FZ>(cVz, plane) * ze;
  } else if (!surf) {  // on the surface these three are replaced by the traction condition
    DzVx = dopm<FZ>(cVx, plane) * ze;
    DzVy = dopm<FZ>(cVy, plane) * ze;
    DzVz = dopm<FZ>(cVz, plane) * ze;
  }

  // ---- WATER (mod_macdrp.F90:917-926) acts on the main equations only
  float wDxTxy = DxTxy, wDxTxz = DxTxz, wDyTxy = DyTxy, wDyTyz = DyTyz, wDzTxz = DzTxz, wDzTyz = DzTyz;
  if (miu <= 1.0e-20f) {
    wDxTxy = 0.0f; wDxTxz = 0.0f; wDyTxy = 0.0f; wDyTyz = 0.0f; wDzTxz = 0.0f; wDzTyz = 0.0f;
  }

  // ---- momentum (mod_macdrp.F90:928-933)
  float hVx = rrho * (DxTxx / r + wDyTxy / r / s + wDzTxz + (3.0f * Txz + Txx * c - Tyy * c) / r);
  float hVy = rrho * (wDxTxy / r + DyTyy / r / s + wDzTyz + (2.0f * Txy * c + 3.0f * Tyz) / r);
  float hVz = rrho * (wDxTxz / r + wDyTyz / r / s + DzTzz + (2.0f * Tzz - Txx - Tyy + Txz * c) / r);
  // ---- strain rates (mod_macdrp.F90:935-948)
  const float E11 = (DxVx + Vz) / r;
  const float E22 = (Vx * c + DyVy / s + Vz) / r;
  const float E12 = (DxVy + DyVx / s - Vy * c) / r / 2.0f;
  float E33 = DzVz;
  float E13 = (DxVz / r + DzVx - Vx / r) / 2.0f;
  float E23 = (DyVz / r / s + DzVy - Vy / r) / 2.0f;
  if (surf) {
    E33 = -(lam / lam2mu * (E11 + E22)) + vsrc(A.src, gst, 2, i, j) / lam2mu;
    E13 = vsrc(A.src, gst, 0, i, j) / miu / 2.0f;
    E23 = vsrc(A.src, gst, 1, i, j) / miu / 2.0f;
  }
  // ---- Hooke (mod_macdrp.F90:952-957)
  float hTxx = lam2mu * E11 + lam * (E22 + E33);
  float hTyy = lam2mu * E22 + lam * (E11 + E33);
  float hTzz = lam2mu * E33 + lam * (E11 + E22);
  float hTxy = 2.0f * miu * E12;
  float hTxz = 2.0f * miu * E13;
  float hTyz = 2.0f * miu * E23;

  // ---- CFS-PML (mod_abs_npml.F90:1149-2123), slabs in the reference's order
  const float tc13 = lam, tc66 = miu;
  const float tc11 = tc13 + 2.0f * tc66;
  const float tc12 = tc13, tc22 = tc11, tc23 = tc13, tc33 = tc11, tc44 = tc66, tc55 = tc66;
#pragma unroll 1
  for (int sidx = 0; sidx < 6; ++sidx) {
    const Slab& sl = A.slab[sidx];
    if (!sl.on) continue;
    if (i < sl.i1 || i > sl.i2 || j < sl.j1 || j > sl.j2 || k < sl.k1 || k > sl.k2) continue;
    const int axis = sidx >> 1;
    const int ia = axis == 0 ? i : axis == 1 ? j : k;
    const float Bv = __ldg(A.pB[axis] + ia), Av = __ldg(A.pA[axis] + ia), Dv = __ldg(A.pD[axis] + ia);
    const float b1 = 1.0f / Bv;
    const float b1_1 = b1 - 1.0f;
    const float ad = Av + Dv;
    const long long q = (long long)(i - sl.i1) + (long long)sl.sx * ((long long)(j - sl.j1) + (long long)sl.sy * (k - sl.k1));
    const long long vs = sl.vstride;
    const float* __restrict__ ai = A.ain[sidx] + q;
    float d0, d1, d2, d3, d4, d5;
    if (axis == 0) {
      d0 = (DxTxx + 2.0f * Txz) / r;
      d1 = (DxTxy + Tyz) / r;
      d2 = (DxTxz - Txx + Tzz) / r;
      d3 = (DxVx + Vz) / r;
      d4 = DxVy / r;
      d5 = (DxVz - Vx) / r;
    } else if (axis == 1) {
      d0 = (DyTxy / s + (Txx - Tyy) * c + Txz) / r;
      d1 = (DyTyy / s + 2.0f * Txy * c + 2.0f * Tyz) / r;
      d2 = (DyTyz / s + Txz * c + (Tzz - Tyy)) / r;
      d3 = (DyVx / s - Vy * c) / r;
      d4 = (DyVy / s + Vx * c + Vz) / r;
      d5 = (DyVz / s - Vy) / r;
    } else {
      d0 = DzTxz; d1 = DzTyz; d2 = DzTzz;
      d3 = DzVx; d4 = DzVy; d5 = DzVz;
    }
    const float a0 = __ldg(ai), a1 = __ldg(ai + vs), a2 = __ldg(ai + 2 * vs);
    const float a3 = __ldg(ai + 3 * vs), a4 = __ldg(ai + 4 * vs), a5 = __ldg(ai + 5 * vs);
    float h[6];
    hVx = hVx + (b1_1 * d0 - b1 * a0) * rrho; h[0] = Dv * d0 - ad * a0;
    hVy = hVy + (b1_1 * d1 - b1 * a1) * rrho; h[1] = Dv * d1 - ad * a1;
    hVz = hVz + (b1_1 * d2 - b1 * a2) * rrho; h[2] = Dv * d2 - ad * a2;
    if (axis == 0) {
      hTxx = hTxx + b1_1 * tc11 * d3 - b1 * tc11 * a3;
      hTyy = hTyy + b1_1 * tc12 * d3 - b1 * tc12 * a3;
      hTzz = hTzz + b1_1 * tc13 * d3 - b1 * tc13 * a3;
      h[3] = Dv * d3 - ad * a3;
      hTxy = hTxy + b1_1 * tc66 * d4 - b1 * tc66 * a4;
      h[4] = Dv * d4 - ad * a4;
      hTxz = hTxz + b1_1 * tc55 * d5 - b1 * tc55 * a5;
      h[5] = Dv * d5 - ad * a5;
      if (surf) {
        hTxx = hTxx - b1_1 * tc13 * tc13 / tc33 * d3 + b1 * tc13 * tc13 / tc33 * a3;
        hTyy = hTyy - b1_1 * tc23 * tc13 / tc33 * d3 + b1 * tc23 * tc13 / tc33 * a3;
      }
    } else if (axis == 1) {
      hTxy = hTxy + b1_1 * tc66 * d3 - b1 * tc66 * a3;
      h[3] = Dv * d3 - ad * a3;
      hTxx = hTxx + b1_1 * tc12 * d4 - b1 * tc12 * a4;
      hTyy = hTyy + b1_1 * tc22 * d4 - b1 * tc22 * a4;
      hTzz = hTzz + b1_1 * tc23 * d4 - b1 * tc23 * a4;
      h[4] = Dv * d4 - ad * a4;
      hTyz = hTyz + b1_1 * tc44 * d5 - b1 * tc44 * a5;
      h[5] = Dv * d5 - ad * a5;
      if (surf) {
        hTxx = hTxx - b1_1 * tc13 * tc23 / tc33 * d4 + b1 * tc13 * tc23 / tc33 * a4;
        hTyy = hTyy - b1_1 * tc23 * tc23 / tc33 * d4 + b1 * tc23 * tc23 / tc33 * a4;
      }
    } else {
      hTxz = hTxz + b1_1 * tc55 * d3 - b1 * tc55 * a3;
      h[3] = Dv * d3 - ad * a3;
      hTyz = hTyz + b1_1 * tc44 * d4 - b1 * tc44 * a4;
      h[4] = Dv * d4 - ad * a4;
      hTxx = hTxx + b1_1 * tc13 * d5 - b1 * tc13 * a5;
      hTyy = hTyy + b1_1 * tc23 * d5 - b1 * tc23 * a5;
      hTzz = hTzz + b1_1 * tc33 * d5 - b1 * tc33 * a5;
      h[5] = Dv * d5 - ad * a5;
    }
    // RK update of the memory variables (abs_RK_*, mod_abs_npml.F90:738-1105)
    const float av[6] = {a0, a1, a2, a3, a4, a5};
    float* __restrict__ ao = A.aout[sidx] + q;
#pragma unroll
    for (int v = 0; v < 6; ++v) {
      if (RK == 0) {
        ao[v * vs] = av[v] + A.a * h[v];
        A.at[sidx][q + v * vs] = av[v] + A.b * h[v];
      } else if (RK == 1) {
        ao[v * vs] = __ldg(A.am[sidx] + q + v * vs) + A.a * h[v];
        float* tp = A.at[sidx] + q + v * vs;
        *tp = *tp + A.b * h[v];
      } else {
        float* tp = A.at[sidx] + q + v * vs;
        *tp = *tp + A.b * h[v];
      }
    }
  }

  // ---- moment tensors (src_stress, mod_src.F90:207-273)
  const Sources& S = A.src;
#pragma unroll 1
  for (int n = 0; n < S.nmom; ++n) {
    const int li = i - S.mom_c[3 * n], lj = j - S.mom_c[3 * n + 1], lk = k - S.mom_c[3 * n + 2];
    if (li < -3 || li > 3 || lj < -3 || lj > 3 || lk < -3 || lk > 3) continue;
    const int e = n * 343 + (li + 3) + 7 * ((lj + 3) + 7 * (lk + 3));
    if (!S.mom_on[e]) continue;
    const float d = S.mom_d[e], vol = S.mom_vol[e];
    for (int m = 0; m < S.ntwin_m; ++m) {
      const float rate = S.mrate[(long long)gst * S.nw_m + n * S.ntwin_m + m];
      const float V = d * rate / vol;
      const float* M = S.mom_M + 6 * (n * S.ntwin_m + m);
      hTxx = hTxx - M[0] * V; hTyy = hTyy - M[1] * V; hTzz = hTzz - M[2] * V;
      hTxy = hTxy - M[3] * V; hTxz = hTxz - M[4] * V; hTyz = hTyz - M[5] * V;
    }
  }
  // ---- body forces (src_force, mod_src.F90:275-345)
#pragma unroll 1
  for (int n = 0; n < S.nforce; ++n) {
    const int li = i - S.force_c[3 * n], lj = j - S.force_c[3 * n + 1], lk = k - S.force_c[3 * n + 2];
    if (li < -3 || li > 3 || lj < -3 || lj > 3 || lk < -3 || lk > 3) continue;
    const int e = n * 343 + (li + 3) + 7 * ((lj + 3) + 7 * (lk + 3));
    if (!S.force_on[e]) continue;
    const float V = S.force_wt[e];
    for (int m = 0; m < S.ntwin_f; ++m) {
      const float disp = S.disp[(long long)gst * S.nw_f + n * S.ntwin_f + m];
      const float* F = S.force_F + 3 * (n * S.ntwin_f + m);
      const float fx0 = F[0] * disp, fy0 = F[1] * disp, fz0 = F[2] * disp;
      hVx = hVx + fx0 * V; hVy = hVy + fy0 * V; hVz = hVz + fz0 * V;
    }
  }

  // ---- RK update of the nine components (mod_macdrp.F90:291-393)
  const float hh[9] = {hVx, hVy, hVz, hTxx, hTyy, hTzz, hTxy, hTxz, hTyz};
#pragma unroll
  for (int f = 0; f < 9; ++f) {
    const long long o = f * fs + p;
    if (RK == 0) {
      const float m = __ldg(A.win + o);
      A.wout[o] = m + A.a * hh[f];
      A.wt[o] = m + A.b * hh[f];
    } else if (RK == 1) {
      A.wout[o] = __ldg(A.wm + o) + A.a * hh[f];
      A.wt[o] = A.wt[o] + A.b * hh[f];
    } else {
      A.wt[o] = A.wt[o] + A.b * hh[f];
    }
  }
}

template <int FX, int FY, int FZ, int RK>
__global__ void __launch_bounds__(128) stage_kernel(const __grid_constant__ StageArgs<float> A) {
  const int i = A.g.i1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = A.g.j1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = A.g.k1 + blockIdx.z;
  if (i > A.g.i2 || j > A.g.j2) return;
  if (A.g.freesurf && k >= A.g.k2 - 3)
    stage_point<FX, FY, FZ, RK, true>(A, i, j, k);
  else
    stage_point<FX, FY, FZ, RK, false>(A, i, j, k);
}

template <int V, int RK>
static void launch_v(const StageArgs<float>& a, cudaStream_t st) {
  dim3 block(32, 4, 1);
  dim3 grid((a.g.ni + 31) / 32, (a.g.nj + 3) / 4, a.g.nk);
  stage_kernel<(V >> 2) & 1, (V >> 1) & 1, V & 1, RK><<<grid, block, 0, st>>>(a);
}

template <int RK>
static void launch_rk(const StageArgs<float>& a, int variant, cudaStream_t st) {
  switch (variant) {
    case 0: launch_v<0, RK>(a, st); break;
    case 1: launch_v<1, RK>(a, st); break;
    case 2: launch_v<2, RK>(a, st); break;
    case 3: launch_v<3, RK>(a, st); break;
    case 4: launch_v<4, RK>(a, st); break;
    case 5: launch_v<5, RK>(a, st); break;
    case 6: launch_v<6, RK>(a, st); break;
    default: launch_v<7, RK>(a, st); break;
  }
}

void launch_stage_f32(const StageArgs<float>& a, int variant, int rk, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (rk == 0) launch_rk<0>(a, variant, st);
  else if (rk == 1) launch_rk<1>(a, variant, st);
  else launch_rk<2>(a, variant, st);
}

}  // namespace fw
