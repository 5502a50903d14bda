// Fused LDDRK4 stage kernel for sm_103a (included by the stage_*.cu instantiation units).
//
// One launch performs, for every interior point, what the reference does in five
// separate sweeps of one Runge-Kutta stage:
//   free_timg        traction image above the free surface   mod_macdrp.F90:3414-3436
//   L<X>             18 one-sided derivatives, spherical RHS  mod_macdrp.F90:790-962
//   abs_L<X>         CFS-PML memory-variable corrections      mod_abs_npml.F90:1149-2123
//   src_stress/force source injection with 7^3 smoothing      mod_src.F90:207-345
//   RK_beg/inn/fin   register update of W, t (and PML aux)    mod_macdrp.F90:291-393
// The right-hand side h never goes to memory.  Image values above the free surface are
// substituted while loading instead of being written: the stored stress on k = nk2 keeps
// its RK value, as in the reference where the RK update overwrites the imaged value.
//
// Blocking (2.5-D): a CTA owns a 32 x 8 (i, j) tile and marches along k over kc planes.
// Each thread keeps its column of the six z-differentiated components (Vx Vy Vz Tzz Txz
// Tyz) in a five-plane register queue; the eight x/y-differentiated components of the
// current plane sit in a double-buffered shared-memory tile with a 3-cell halo, so every
// plane of every component is read from DRAM about once per stage.
#pragma once
#include <cuda_runtime.h>

#include "kernels.h"

namespace fw {

constexpr int TX = STAGE_TX, TY = STAGE_TY, HALO = 3;
constexpr int SW = TX + 2 * HALO;  // shared tile row length
constexpr int SH = TY + 2 * HALO;  // shared tile rows
constexpr int NSF = 8;             // shared fields
enum { S_VX = 0, S_VY, S_VZ, S_TXX, S_TYY, S_TXY, S_TXZ, S_TYZ };
enum { Q_VX = 0, Q_VY, Q_VZ, Q_TZZ, Q_TXZ, Q_TYZ };
// component of queue entry qf
__device__ __forceinline__ int qfield(int qf) { return qf < 3 ? qf : (qf == Q_TZZ ? TZZ : (qf == Q_TXZ ? TXZ : TYZ)); }
// component of shared field sf
__device__ __forceinline__ int sfield(int sf) {
  return sf < 3 ? sf : (sf == S_TXX ? TXX : (sf == S_TYY ? TYY : (sf == S_TXY ? TXY : (sf == S_TXZ ? TXZ : TYZ))));
}
// e-th shared field with an x halo (Vx Vy Vz Txx Txy Txz) / a y halo (Vx Vy Vz Tyy Txy Tyz)
__device__ __forceinline__ int xh_field(int e) { return e < 3 ? e : (e == 3 ? S_TXX : (e == 4 ? S_TXY : S_TXZ)); }
__device__ __forceinline__ int yh_field(int e) { return e < 3 ? e : (e == 3 ? S_TYY : (e == 4 ? S_TXY : S_TYZ)); }

#define MCA_1 (-0.30874f)
#define MCA0 (-0.6326f)
#define MCA1 (1.233f)
#define MCA2 (-0.3334f)
#define MCA3 (0.04168f)

// DRP/opt MacCormack operators (mod_macdrp.h:69-103) on values at offsets -3..+3 of c.
template <int F>
__device__ __forceinline__ float dop(const float* c, int s) {
  if (F)
    return MCA_1 * c[-s] + MCA0 * c[0] + MCA1 * c[s] + MCA2 * c[2 * s] + MCA3 * c[3 * s];
  else
    return -MCA3 * c[-3 * s] - MCA2 * c[-2 * s] - MCA1 * c[-s] - MCA0 * c[0] - MCA_1 * c[s];
}
// Same operator on a five-entry z queue (F: planes -1..+3, B: planes -3..+1).
template <int F>
__device__ __forceinline__ float dopq(const float* q) {
  if (F)
    return MCA_1 * q[0] + MCA0 * q[1] + MCA1 * q[2] + MCA2 * q[3] + MCA3 * q[4];
  else
    return -MCA3 * q[0] - MCA2 * q[1] - MCA1 * q[2] - MCA0 * q[3] - MCA_1 * q[4];
}
// 2-2 and 2-4 MacCormack operators of CondFreeVLOW (mod_macdrp.h:230-268) on the queue.
template <int F>
__device__ __forceinline__ float dop22q(const float* q) {
  if (F) return -1.0f * q[1] + 1.0f * q[2];  // centre at q[1]
  else return -1.0f * q[2] - -1.0f * q[3];   // centre at q[3]
}
template <int F>
__device__ __forceinline__ float dop24q(const float* q) {
  const float A0 = -7.0f / 6.0f, A1 = 8.0f / 6.0f, A2 = -1.0f / 6.0f;
  if (F) return A0 * q[1] + A1 * q[2] + A2 * q[3];
  else return -A2 * q[1] - A1 * q[2] - A0 * q[3];
}

// T*Src / V*Src (comp 0 x, 1 y, 2 z) at an interior column for global stage gst:
// src_surface (mod_src.F90:373-414), the last window of the last force wins.
__device__ __forceinline__ float surf_val(const Sources& S, const float* tab, int gst, int comp, int i, int j) {
  float v = 0.0f;
  for (int e = 0; e < S.nsurf; ++e)
    if (S.surf_ij[2 * e] == i && S.surf_ij[2 * e + 1] == j)
      v = S.surf_q[3 * e + comp] * tab[(long long)gst * S.nw_f + S.surf_w[e]];
  return v;
}

template <bool EXACT, int FX, int FY, int FZ, int RK>
__global__ void __launch_bounds__(TX* TY, 2) stage_kernel(const __grid_constant__ StageArgs<float> A) {
  __shared__ float sm[2][NSF][SH][SW];
  const Geom& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = g.i1 + blockIdx.x * TX, j0 = g.j1 + blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool act = i <= g.i2 && j <= g.j2;  // interior point owned by this thread
  const bool inarr = i < g.nx && j < g.ny;  // column inside the array (ghosts included)
  const int kb = g.k1 + blockIdx.z * A.kc;
  if (kb > g.k2) return;
  const int ke = min(kb + A.kc - 1, g.k2);
  const int px = g.px, plane = int(g.plane);
  const long long fs = g.fstride;
  const int col = (i + PADL) + px * j;
  const float* __restrict__ W = A.win;
  const int gst = __ldg(A.ntime) * 4 + A.stage;
  const bool fsurf = g.freesurf != 0;
  const Sources& S = A.src;

  constexpr int LEAD = FZ ? 3 : 1;   // planes ahead of k in the z operator
  constexpr int TRAIL = FZ ? 1 : 3;  // planes behind k

  // T*Src of this column (only read on the top planes)
  float tsx = 0.0f, tsy = 0.0f, tsz = 0.0f;
  if (fsurf && act && ke >= g.k2 - 3) {
    tsx = surf_val(S, S.disp, gst, 0, i, j);
    tsy = surf_val(S, S.disp, gst, 1, i, j);
    tsz = surf_val(S, S.disp, gst, 2, i, j);
  }

  // Load plane kk of queue field qf for this column, with the free-surface image.
  auto zload = [&](int qf, int kk) -> float {
    if (!inarr) return 0.0f;
    const float* base = W + qfield(qf) * fs + col;
    if (qf >= Q_TZZ && fsurf && act && kk >= g.k2) {
      const float ts = qf == Q_TZZ ? tsz : (qf == Q_TXZ ? tsx : tsy);
      if (kk == g.k2) return ts;
      return 2.0f * ts - __ldg(base + (2 * g.k2 - kk) * plane);
    }
    return __ldg(base + kk * plane);
  };

  float q[6][5];
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    q[f][0] = 0.0f;
#pragma unroll
    for (int d = 1; d < 5; ++d) q[f][d] = zload(f, kb - TRAIL + d - 1);
  }

  // halo assignment of this thread (fixed for all planes)
  //   tid < 6*TX: y halo, row r = tid / TX (-3,-2,-1,TY,TY+1,TY+2), column tid % TX
  //   6*TX <= tid < 6*TX + 6*TY: x halo, row e / 6, column (-3,-2,-1,TX,TX+1,TX+2)
  int hrow = -100, hcol = -100, hkind = 0;
  if (tid < 6 * TX) {
    const int r = tid / TX;
    hrow = r < 3 ? r - 3 : TY + r - 3;
    hcol = tid % TX;
    hkind = 1;
  } else if (tid < 6 * TX + 6 * TY) {
    const int e = tid - 6 * TX;
    const int c = e % 6;
    hrow = e / 6;
    hcol = c < 3 ? c - 3 : TX + c - 3;
    hkind = 2;
  }
  const int hi = i0 + hcol, hj = j0 + hrow;
  const bool hin = hkind != 0 && hi < g.nx && hj < g.ny;
  const bool hinterior = hi >= g.i1 && hi <= g.i2 && hj >= g.j1 && hj <= g.j2;
  const int hcolof = (hi + PADL) + px * hj;

  const float xi = __ldg(A.xi_x + min(i, g.nx - 1));
  const float et = __ldg(A.eta_y + min(j, g.ny - 1));
  const float xs = __ldg(A.xsin + min(i, g.nx - 1));
  const float c = __ldg(A.xcot + min(i, g.nx - 1));
  const float rs = __ldg(A.rsinv + min(i, g.nx - 1));

  int buf = 0;
  for (int k = kb; k <= ke; ++k) {
    // advance the z queue
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      q[f][0] = q[f][1]; q[f][1] = q[f][2]; q[f][2] = q[f][3]; q[f][3] = q[f][4];
      q[f][4] = zload(f, k + LEAD);
    }
    const bool top = fsurf && k == g.k2;
    // fill the shared tile of plane k
    float(*s)[SH][SW] = sm[buf];
    {
      const int r = ty + HALO, cc = tx + HALO;
      s[S_VX][r][cc] = q[Q_VX][TRAIL];
      s[S_VY][r][cc] = q[Q_VY][TRAIL];
      s[S_VZ][r][cc] = q[Q_VZ][TRAIL];
      s[S_TXZ][r][cc] = q[Q_TXZ][TRAIL];
      s[S_TYZ][r][cc] = q[Q_TYZ][TRAIL];
      const int o = col + k * plane;
      s[S_TXX][r][cc] = inarr ? __ldg(W + TXX * fs + o) : 0.0f;
      s[S_TYY][r][cc] = inarr ? __ldg(W + TYY * fs + o) : 0.0f;
      s[S_TXY][r][cc] = inarr ? __ldg(W + TXY * fs + o) : 0.0f;
    }
    if (hkind != 0) {
      const int r = hrow + HALO, cc = hcol + HALO;
      const int o = hcolof + k * plane;
#pragma unroll
      for (int e = 0; e < 6; ++e) {
        const int sf = hkind == 1 ? yh_field(e) : xh_field(e);
        float v = hin ? __ldg(W + sfield(sf) * fs + o) : 0.0f;
        if (top && hinterior && (sf == S_TXZ || sf == S_TYZ))
          v = surf_val(S, S.disp, gst, sf == S_TXZ ? 0 : 1, hi, hj);
        s[sf][r][cc] = v;
      }
    }
    __syncthreads();
    buf ^= 1;
    if (!act) continue;

    const int p = col + k * plane;
    const float lam = __ldg(A.lam + p), miu = __ldg(A.mu + p), rhov = __ldg(A.rho + p);
    const float ze = __ldg(A.zeta_z + k);
    const int r0 = ty + HALO, c0 = tx + HALO;
    // stencil sums along x (shared rows), y (shared columns), z (queue)
    const float sxTxx = dop<FX>(&s[S_TXX][r0][c0], 1);
    const float sxTxy = dop<FX>(&s[S_TXY][r0][c0], 1);
    const float sxTxz = dop<FX>(&s[S_TXZ][r0][c0], 1);
    const float sxVx = dop<FX>(&s[S_VX][r0][c0], 1);
    const float sxVy = dop<FX>(&s[S_VY][r0][c0], 1);
    const float sxVz = dop<FX>(&s[S_VZ][r0][c0], 1);
    const float syTyy = dop<FY>(&s[S_TYY][r0][c0], SW);
    const float syTxy = dop<FY>(&s[S_TXY][r0][c0], SW);
    const float syTyz = dop<FY>(&s[S_TYZ][r0][c0], SW);
    const float syVx = dop<FY>(&s[S_VX][r0][c0], SW);
    const float syVy = dop<FY>(&s[S_VY][r0][c0], SW);
    const float syVz = dop<FY>(&s[S_VZ][r0][c0], SW);
    const float szTzz = dopq<FZ>(q[Q_TZZ]);
    const float szTxz = dopq<FZ>(q[Q_TXZ]);
    const float szTyz = dopq<FZ>(q[Q_TYZ]);
    float szVx, szVy, szVz;
    if (fsurf && k == g.k2 - 1) {
      szVx = dop22q<FZ>(q[Q_VX]); szVy = dop22q<FZ>(q[Q_VY]); szVz = dop22q<FZ>(q[Q_VZ]);
    } else if (fsurf && k == g.k2 - 2) {
      szVx = dop24q<FZ>(q[Q_VX]); szVy = dop24q<FZ>(q[Q_VY]); szVz = dop24q<FZ>(q[Q_VZ]);
    } else {
      szVx = dopq<FZ>(q[Q_VX]); szVy = dopq<FZ>(q[Q_VY]); szVz = dopq<FZ>(q[Q_VZ]);
    }
    const float Vx = q[Q_VX][TRAIL], Vy = q[Q_VY][TRAIL], Vz = q[Q_VZ][TRAIL];
    const float Tzz = q[Q_TZZ][TRAIL], Txz = q[Q_TXZ][TRAIL], Tyz = q[Q_TYZ][TRAIL];
    const float Txx = s[S_TXX][r0][c0], Tyy = s[S_TYY][r0][c0], Txy = s[S_TXY][r0][c0];
    const bool water = miu <= 1.0e-20f;

    float hVx, hVy, hVz, hTxx, hTyy, hTzz, hTxy, hTxz, hTyz;
    // PML derivative terms per axis: d[0..2] stress terms of hVx,hVy,hVz; d[3..5] Vx,Vy,Vz
    float dx_[6], dy_[6], dz_[6];
    const float lam2mu = lam + 2.0f * miu;
    float rrho, rr = 0.0f;
    if constexpr (EXACT) {
      // reference operand order, IEEE division (mod_macdrp.F90:928-957)
      const float r = __ldg(A.zc + k);
      rrho = 1.0f / rhov;
      const float DxTxx = sxTxx * xi, DxTxy = sxTxy * xi, DxTxz = sxTxz * xi;
      const float DxVx = sxVx * xi, DxVy = sxVy * xi, DxVz = sxVz * xi;
      const float DyTyy = syTyy * et, DyTxy = syTxy * et, DyTyz = syTyz * et;
      const float DyVx = syVx * et, DyVy = syVy * et, DyVz = syVz * et;
      const float DzTzz = szTzz * ze, DzTxz = szTxz * ze, DzTyz = szTyz * ze;
      const float DzVx = szVx * ze, DzVy = szVy * ze, DzVz = szVz * ze;
      const float wDxTxy = water ? 0.0f : DxTxy, wDxTxz = water ? 0.0f : DxTxz;
      const float wDyTxy = water ? 0.0f : DyTxy, wDyTyz = water ? 0.0f : DyTyz;
      const float wDzTxz = water ? 0.0f : DzTxz, wDzTyz = water ? 0.0f : DzTyz;
      hVx = rrho * (DxTxx / r + wDyTxy / r / xs + wDzTxz + (3.0f * Txz + Txx * c - Tyy * c) / r);
      hVy = rrho * (wDxTxy / r + DyTyy / r / xs + wDzTyz + (2.0f * Txy * c + 3.0f * Tyz) / r);
      hVz = rrho * (wDxTxz / r + wDyTyz / r / xs + DzTzz + (2.0f * Tzz - Txx - Tyy + Txz * c) / r);
      const float E11 = (DxVx + Vz) / r;
      const float E22 = (Vx * c + DyVy / xs + Vz) / r;
      const float E12 = (DxVy + DyVx / xs - Vy * c) / r / 2.0f;
      float E33 = DzVz;
      float E13 = (DxVz / r + DzVx - Vx / r) / 2.0f;
      float E23 = (DyVz / r / xs + DzVy - Vy / r) / 2.0f;
      if (top) {
        E33 = -(lam / lam2mu * (E11 + E22)) + surf_val(S, S.rate, gst, 2, i, j) / lam2mu;
        E13 = surf_val(S, S.rate, gst, 0, i, j) / miu / 2.0f;
        E23 = surf_val(S, S.rate, gst, 1, i, j) / miu / 2.0f;
      }
      hTxx = lam2mu * E11 + lam * (E22 + E33);
      hTyy = lam2mu * E22 + lam * (E11 + E33);
      hTzz = lam2mu * E33 + lam * (E11 + E22);
      hTxy = 2.0f * miu * E12;
      hTxz = 2.0f * miu * E13;
      hTyz = 2.0f * miu * E23;
      // PML terms (mod_abs_npml.F90:1179-1301, 1523-1645, 1867-1983)
      dx_[0] = (DxTxx + 2.0f * Txz) / r; dx_[1] = (DxTxy + Tyz) / r; dx_[2] = (DxTxz - Txx + Tzz) / r;
      dx_[3] = (DxVx + Vz) / r; dx_[4] = DxVy / r; dx_[5] = (DxVz - Vx) / r;
      dy_[0] = (DyTxy / xs + (Txx - Tyy) * c + Txz) / r;
      dy_[1] = (DyTyy / xs + 2.0f * Txy * c + 2.0f * Tyz) / r;
      dy_[2] = (DyTyz / xs + Txz * c + (Tzz - Tyy)) / r;
      dy_[3] = (DyVx / xs - Vy * c) / r; dy_[4] = (DyVy / xs + Vx * c + Vz) / r; dy_[5] = (DyVz / xs - Vy) / r;
      dz_[0] = DzTxz; dz_[1] = DzTyz; dz_[2] = DzTzz; dz_[3] = DzVx; dz_[4] = DzVy; dz_[5] = DzVz;
    } else {
      // same equations with the metric folded into one factor per axis
      rr = __ldg(A.rzinv + k);
      rrho = __frcp_rn(rhov);
      const float ax = xi * rr, ay = et * rr * rs;
      const float gxTxx = sxTxx * ax, gxTxy = sxTxy * ax, gxTxz = sxTxz * ax;
      const float gxVx = sxVx * ax, gxVy = sxVy * ax, gxVz = sxVz * ax;
      const float gyTyy = syTyy * ay, gyTxy = syTxy * ay, gyTyz = syTyz * ay;
      const float gyVx = syVx * ay, gyVy = syVy * ay, gyVz = syVz * ay;
      const float gzTzz = szTzz * ze, gzTxz = szTxz * ze, gzTyz = szTyz * ze;
      const float gzVx = szVx * ze, gzVy = szVy * ze, gzVz = szVz * ze;
      const float wxTxy = water ? 0.0f : gxTxy, wxTxz = water ? 0.0f : gxTxz;
      const float wyTxy = water ? 0.0f : gyTxy, wyTyz = water ? 0.0f : gyTyz;
      const float wzTxz = water ? 0.0f : gzTxz, wzTyz = water ? 0.0f : gzTyz;
      hVx = rrho * (gxTxx + wyTxy + wzTxz + (3.0f * Txz + (Txx - Tyy) * c) * rr);
      hVy = rrho * (wxTxy + gyTyy + wzTyz + (2.0f * Txy * c + 3.0f * Tyz) * rr);
      hVz = rrho * (wxTxz + wyTyz + gzTzz + (2.0f * Tzz - Txx - Tyy + Txz * c) * rr);
      const float E11 = gxVx + Vz * rr;
      const float E22 = (Vx * c + Vz) * rr + gyVy;
      const float E12 = 0.5f * (gxVy + gyVx - Vy * c * rr);
      float E33 = gzVz;
      float E13 = 0.5f * (gxVz + gzVx - Vx * rr);
      float E23 = 0.5f * (gyVz + gzVy - Vy * rr);
      if (top) {
        E33 = (surf_val(S, S.rate, gst, 2, i, j) - lam * (E11 + E22)) / lam2mu;
        E13 = 0.5f * surf_val(S, S.rate, gst, 0, i, j) / miu;
        E23 = 0.5f * surf_val(S, S.rate, gst, 1, i, j) / miu;
      }
      hTxx = lam2mu * E11 + lam * (E22 + E33);
      hTyy = lam2mu * E22 + lam * (E11 + E33);
      hTzz = lam2mu * E33 + lam * (E11 + E22);
      hTxy = 2.0f * miu * E12;
      hTxz = 2.0f * miu * E13;
      hTyz = 2.0f * miu * E23;
      dx_[0] = gxTxx + 2.0f * Txz * rr; dx_[1] = gxTxy + Tyz * rr; dx_[2] = gxTxz + (Tzz - Txx) * rr;
      dx_[3] = gxVx + Vz * rr; dx_[4] = gxVy; dx_[5] = gxVz - Vx * rr;
      dy_[0] = gyTxy + ((Txx - Tyy) * c + Txz) * rr;
      dy_[1] = gyTyy + (2.0f * Txy * c + 2.0f * Tyz) * rr;
      dy_[2] = gyTyz + (Txz * c + (Tzz - Tyy)) * rr;
      dy_[3] = gyVx - Vy * c * rr; dy_[4] = gyVy + (Vx * c + Vz) * rr; dy_[5] = gyVz - Vy * rr;
      dz_[0] = gzTxz; dz_[1] = gzTyz; dz_[2] = gzTzz; dz_[3] = gzVx; dz_[4] = gzVy; dz_[5] = gzVz;
    }

    // ---- CFS-PML slabs in the reference's order x1 x2 y1 y2 z1 z2 (additive at corners)
    const float tc13 = lam, tc66 = miu;
    const float tc11 = tc13 + 2.0f * tc66;
    const float tc12 = tc13, tc22 = tc11, tc23 = tc13, tc33 = tc11, tc44 = tc66, tc55 = tc66;
#pragma unroll 1
    for (int sidx = 0; sidx < 6; ++sidx) {
      const Slab& sl = A.slab[sidx];
      if (!sl.on || i < sl.i1 || i > sl.i2 || j < sl.j1 || j > sl.j2 || k < sl.k1 || k > sl.k2) continue;
      const int axis = sidx >> 1;
      const int ia = axis == 0 ? i : (axis == 1 ? j : k);
      const float b1 = __ldg(A.pb1[axis] + ia), b1_1 = __ldg(A.pb11[axis] + ia);
      const float ad = __ldg(A.pad[axis] + ia), Dv = __ldg(A.pD[axis] + ia);
      float d[6];
#pragma unroll
      for (int v = 0; v < 6; ++v) d[v] = axis == 0 ? dx_[v] : (axis == 1 ? dy_[v] : dz_[v]);
      const long long qa = (long long)(i - sl.i1) + (long long)sl.sx * ((long long)(j - sl.j1) + (long long)sl.sy * (k - sl.k1));
      const long long vs = sl.vstride;
      const float* __restrict__ ai = A.ain[sidx] + qa;
      float av[6], h[6];
#pragma unroll
      for (int v = 0; v < 6; ++v) av[v] = __ldg(ai + v * vs);
      hVx = hVx + (b1_1 * d[0] - b1 * av[0]) * rrho; h[0] = Dv * d[0] - ad * av[0];
      hVy = hVy + (b1_1 * d[1] - b1 * av[1]) * rrho; h[1] = Dv * d[1] - ad * av[1];
      hVz = hVz + (b1_1 * d[2] - b1 * av[2]) * rrho; h[2] = Dv * d[2] - ad * av[2];
      if (axis == 0) {
        hTxx = hTxx + b1_1 * tc11 * d[3] - b1 * tc11 * av[3];
        hTyy = hTyy + b1_1 * tc12 * d[3] - b1 * tc12 * av[3];
        hTzz = hTzz + b1_1 * tc13 * d[3] - b1 * tc13 * av[3];
        h[3] = Dv * d[3] - ad * av[3];
        hTxy = hTxy + b1_1 * tc66 * d[4] - b1 * tc66 * av[4];
        h[4] = Dv * d[4] - ad * av[4];
        hTxz = hTxz + b1_1 * tc55 * d[5] - b1 * tc55 * av[5];
        h[5] = Dv * d[5] - ad * av[5];
        if (top) {  // mod_abs_npml.F90:1303-1333
          hTxx = hTxx - b1_1 * tc13 * tc13 / tc33 * d[3] + b1 * tc13 * tc13 / tc33 * av[3];
          hTyy = hTyy - b1_1 * tc23 * tc13 / tc33 * d[3] + b1 * tc23 * tc13 / tc33 * av[3];
        }
      } else if (axis == 1) {
        hTxy = hTxy + b1_1 * tc66 * d[3] - b1 * tc66 * av[3];
        h[3] = Dv * d[3] - ad * av[3];
        hTxx = hTxx + b1_1 * tc12 * d[4] - b1 * tc12 * av[4];
        hTyy = hTyy + b1_1 * tc22 * d[4] - b1 * tc22 * av[4];
        hTzz = hTzz + b1_1 * tc23 * d[4] - b1 * tc23 * av[4];
        h[4] = Dv * d[4] - ad * av[4];
        hTyz = hTyz + b1_1 * tc44 * d[5] - b1 * tc44 * av[5];
        h[5] = Dv * d[5] - ad * av[5];
        if (top) {  // mod_abs_npml.F90:1647-1677
          hTxx = hTxx - b1_1 * tc13 * tc23 / tc33 * d[4] + b1 * tc13 * tc23 / tc33 * av[4];
          hTyy = hTyy - b1_1 * tc23 * tc23 / tc33 * d[4] + b1 * tc23 * tc23 / tc33 * av[4];
        }
      } else {
        hTxz = hTxz + b1_1 * tc55 * d[3] - b1 * tc55 * av[3];
        h[3] = Dv * d[3] - ad * av[3];
        hTyz = hTyz + b1_1 * tc44 * d[4] - b1 * tc44 * av[4];
        h[4] = Dv * d[4] - ad * av[4];
        hTxx = hTxx + b1_1 * tc13 * d[5] - b1 * tc13 * av[5];
        hTyy = hTyy + b1_1 * tc23 * d[5] - b1 * tc23 * av[5];
        hTzz = hTzz + b1_1 * tc33 * d[5] - b1 * tc33 * av[5];
        h[5] = Dv * d[5] - ad * av[5];
      }
      // abs_RK_* (mod_abs_npml.F90:738-1105)
      float* __restrict__ ao = A.aout[sidx] + qa;
      float* __restrict__ at = A.at[sidx] + qa;
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        if (RK == 0) {
          ao[v * vs] = av[v] + A.a * h[v];
          at[v * vs] = av[v] + A.b * h[v];
        } else if (RK == 1) {
          ao[v * vs] = __ldg(A.am[sidx] + qa + v * vs) + A.a * h[v];
          at[v * vs] = at[v * vs] + A.b * h[v];
        } else {
          at[v * vs] = at[v * vs] + A.b * h[v];
        }
      }
    }

    // ---- moment tensors (src_stress, mod_src.F90:207-273)
#pragma unroll 1
    for (int n = 0; n < S.nmom; ++n) {
      const int li = i - S.mom_c[3 * n], lj = j - S.mom_c[3 * n + 1], lk = k - S.mom_c[3 * n + 2];
      if (li < -3 || li > 3 || lj < -3 || lj > 3 || lk < -3 || lk > 3) continue;
      const int e = n * 343 + (li + 3) + 7 * ((lj + 3) + 7 * (lk + 3));
      if (!S.mom_on[e]) continue;
      const float dd = S.mom_d[e], vol = S.mom_vol[e];
      for (int m = 0; m < S.ntwin_m; ++m) {
        const float rate = S.mrate[(long long)gst * S.nw_m + n * S.ntwin_m + m];
        const float V = dd * rate / vol;
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

    // ---- RK update (mod_macdrp.F90:291-393); m of stage 1 is the stored input value
    const float hh[9] = {hVx, hVy, hVz, hTxx, hTyy, hTzz, hTxy, hTxz, hTyz};
#pragma unroll
    for (int f = 0; f < 9; ++f) {
      const long long o = f * fs + p;
      if (RK == 0) {
        const float m = __ldg(W + o);
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
}

template <bool EXACT, int RK>
static void launch_rk_variant(const StageArgs<float>& a, int variant, cudaStream_t st) {
  const dim3 block(TX, TY, 1);
  const dim3 grid((a.g.ni + TX - 1) / TX, (a.g.nj + TY - 1) / TY, (a.g.nk + a.kc - 1) / a.kc);
  switch (variant) {
    case 0: stage_kernel<EXACT, 0, 0, 0, RK><<<grid, block, 0, st>>>(a); break;
    case 1: stage_kernel<EXACT, 0, 0, 1, RK><<<grid, block, 0, st>>>(a); break;
    case 2: stage_kernel<EXACT, 0, 1, 0, RK><<<grid, block, 0, st>>>(a); break;
    case 3: stage_kernel<EXACT, 0, 1, 1, RK><<<grid, block, 0, st>>>(a); break;
    case 4: stage_kernel<EXACT, 1, 0, 0, RK><<<grid, block, 0, st>>>(a); break;
    case 5: stage_kernel<EXACT, 1, 0, 1, RK><<<grid, block, 0, st>>>(a); break;
    case 6: stage_kernel<EXACT, 1, 1, 0, RK><<<grid, block, 0, st>>>(a); break;
    default: stage_kernel<EXACT, 1, 1, 1, RK><<<grid, block, 0, st>>>(a); break;
  }
}

}  // namespace fw
