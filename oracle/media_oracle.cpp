// TEST INFRASTRUCTURE ONLY (the oracle).  CPU restatement of the reference's medium
// preprocessor, code/srcF/seis3d_media.F90:
//   effmedia_eval :854-1249 (sub-cell sampling and harmonic averaging over the six
//   background and two perturbation model kinds), eval_poly :1251-1262, extend_equal
//   :1269-1299, dist_point2plane :1301-1313, indx_locate_1d :1315-1344, media_stept_check
//   :1544-1611, and the sub-volume selection of volume_read :761-779 / verpoly_read
//   :829-850; with interp_2d / interp_3d of code/srcF/mod_math.F90:128-208.
// Single precision where the reference declares real(SP), double where it declares DP;
// sequential, every expression in the reference's evaluation order, compiled without
// contraction.  Used by the tests and the benchmark's CPU baseline to check and time the
// GPU preprocessor; never by the product.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr float SEIS_ZERO = 1.0e-20f;
constexpr double PI = 3.141592653589793;
constexpr int LENFD = 3;

// indx_locate_1d (1-based i1, i2 out; x has n >= 2 entries)
void locate(float x0, const float* x, int n, int& i1, int& i2, float& x1) {
  i1 = 1;
  i2 = n;
  x1 = x0;
  if (x0 <= x[0]) {
    x1 = x[0];
    i1 = 1;
    i2 = 2;
  } else if (x0 >= x[i2 - 1]) {
    x1 = x[i2 - 1];
    i1 = i2 - 1;
  } else {
    while (i2 - i1 > 1) {
      const int i0 = (i2 - i1) / 2 + i1;
      if (x[i0 - 1] == x0) {
        i1 = i0;
        i2 = i0 + 1;
        break;
      } else if (x[i0 - 1] > x0) {
        i2 = i0;
      } else {
        i1 = i0;
      }
    }
  }
}

// two-point Lagrange weights of interp_2d / interp_3d: L(1) = (xi - x2) / (x1 - x2),
// L(2) = (xi - x1) / (x2 - x1) (the other factors of the product are exactly 1)
void weights(float xa, float xb, float xi, float& l1, float& l2) {
  l1 = (xi - xb) / (xa - xb);
  l2 = (xi - xa) / (xb - xa);
}

// interp_2d on the 2 x 2 cell (i1, j1) of f (ni x nj, i fastest; 1-based corners)
float interp2(const float* xs, const float* ys, const float* f, int ni, int i1, int j1, float xi, float yi) {
  float lx1, lx2, ly1, ly2;
  weights(xs[i1 - 1], xs[i1], xi, lx1, lx2);
  weights(ys[j1 - 1], ys[j1], yi, ly1, ly2);
  const float* c = f + (size_t(j1 - 1) * ni + (i1 - 1));
  float z = 0.0f;
  z = z + lx1 * ly1 * c[0];
  z = z + lx2 * ly1 * c[1];
  z = z + lx1 * ly2 * c[ni];
  z = z + lx2 * ly2 * c[ni + 1];
  return z;
}

float interp3(const float* xs, const float* ys, const float* zs, const float* f, int ni, int nj, int i1, int j1,
              int k1, float xi, float yi, float zi) {
  float lx[2], ly[2], lz[2];
  weights(xs[i1 - 1], xs[i1], xi, lx[0], lx[1]);
  weights(ys[j1 - 1], ys[j1], yi, ly[0], ly[1]);
  weights(zs[k1 - 1], zs[k1], zi, lz[0], lz[1]);
  float s = 0.0f;
  for (int k = 0; k < 2; ++k)
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i)
        s = s + lx[i] * ly[j] * lz[k] * f[(size_t(k1 - 1 + k) * nj + (j1 - 1 + j)) * ni + (i1 - 1 + i)];
  return s;
}

float eval_poly(const float* c, size_t cstride, const float* d, int n, float x) {
  float f = 0.0f;
  for (int q = 0; q < n; ++q) f = f + c[q * cstride] * std::pow(x, d[q]);
  return f;
}

// first index (1-based) of the minimum of |a[q * stride] - v|, q < n (minloc)
int minloc_abs(const float* a, size_t stride, int n, float v) {
  int best = 1;
  float bv = std::fabs(a[0] - v);
  for (int q = 1; q < n; ++q) {
    const float t = std::fabs(a[q * stride] - v);
    if (t < bv) {
      bv = t;
      best = q + 1;
    }
  }
  return best;
}

struct Volume {  // volume model (x, y, rz and fields (ni, nj, nk), i fastest) after volume_read
  int ni = 0, nj = 0, nk = 0;
  float rz0 = 0.0f;
  std::vector<float> x, y, rz, vp, vs, dp;
};

struct Verpoly {  // verpoly model after verpoly_read: rz (ni,nj,nk), coefficients (ni,nj,nk,np)
  int ni = 0, nj = 0, nk = 0, np = 0;
  float rz0 = 0.0f;
  std::vector<float> x, y, rz, vpc, vsc, dpc, vpd, vsd, dpd;
};

struct Layers {  // interface / layered / composite models
  int ni = 0, nj = 0, nk = 0;
  std::vector<float> x, y, z, h;         // z: interfaces (interface kind); h: thicknesses
  std::vector<float> vp, vs, dp;         // (2, nk) or (2, ni, nj, nk) for composite
  std::vector<float> vpd, vsd, dpd;      // composite exponents (nk)
};

}  // namespace

struct orc_media {
  int ni, nj, nk, nx, ny, nz;
  int ng[3];
  float ztopo;
  std::vector<float> x, y, z;
  int bkind = 0, pkind = 0;  // 1 cart1d, 2 interface, 3 layered, 4 composite, 5 volume, 6 verpoly
  std::vector<float> c_d, c_vp, c_vs, c_dp;
  Layers L;
  Volume bv, pv;
  Verpoly bp, pp;
  std::vector<float> lam, mu, rho;  // (nx, ny, nz)
  std::string err;
};

namespace {

// volume_read / verpoly_read: the model columns between the grid's first and last
// coordinates (maxloc of gx <= max(x(nx1), gx(1)), minloc of gx >= min(x(nx2), gx(end)))
void select_range(const float* g, int n, float lo, float hi, int& a, int& b) {
  const float tlo = std::max(lo, g[0]), thi = std::min(hi, g[n - 1]);
  a = 0;
  float av = -INFINITY;
  bool found = false;
  for (int q = 0; q < n; ++q)
    if (g[q] <= tlo && (!found || g[q] > av)) {
      av = g[q];
      a = q + 1;
      found = true;
    }
  a = std::max(a, 1);
  b = 0;
  float bv = INFINITY;
  found = false;
  for (int q = 0; q < n; ++q)
    if (g[q] >= thi && (!found || g[q] < bv)) {
      bv = g[q];
      b = q + 1;
      found = true;
    }
}

// effmedia_eval for one interior point (0-based array indices i, j, k)
bool point(orc_media* m, int i, int j, int k, float* lam_out, float* mu_out, float* rho_out) {
  const int NX = m->ng[0], NY = m->ng[1], NZ = m->ng[2];
  const int nsamp = std::max(2 * NX, 1) * std::max(2 * NY, 1) * std::max(2 * NZ, 1);
  const float* x = m->x.data();
  const float* y = m->y.data();
  const float* z = m->z.data();
  std::vector<float> xvec(2 * NX + 1), yvec(2 * NY + 1), zvec(2 * NZ + 1);
  float rho0 = 0.0f, mu0 = 0.0f, lam0 = 0.0f;
  bool flag_water = false;
  int nwater = 0;
  xvec[NX] = x[i];
  yvec[NY] = y[j];
  zvec[NZ] = z[k];
  const float dx1 = (x[i] - x[i - 1]) / 2.0f / float(NX + 1), dx2 = (x[i + 1] - x[i]) / 2.0f / float(NX + 1);
  for (int q = -NX; q <= -1; ++q) xvec[NX + q] = float(q) * dx1 + x[i];
  for (int q = 1; q <= NX; ++q) xvec[NX + q] = float(q) * dx2 + x[i];
  const float dy1 = (y[j] - y[j - 1]) / 2.0f / float(NY + 1), dy2 = (y[j + 1] - y[j]) / 2.0f / float(NY + 1);
  for (int q = -NY; q <= -1; ++q) yvec[NY + q] = float(q) * dy1 + y[j];
  for (int q = 1; q <= NY; ++q) yvec[NY + q] = float(q) * dy2 + y[j];
  const float dz1 = (z[k] - z[k - 1]) / 2.0f / float(NZ + 1), dz2 = (z[k + 1] - z[k]) / 2.0f / float(NZ + 1);
  for (int q = -NZ; q <= -1; ++q) zvec[NZ + q] = float(q) * dz1 + z[k];
  for (int q = 1; q <= NZ; ++q) zvec[NZ + q] = float(q) * dz2 + z[k];
  (void)dz1;
  float Vp[2] = {0, 0}, Vs[2] = {0, 0}, Dp[2] = {0, 0};
  for (int mk = -NZ; mk <= NZ; ++mk) {
    if (NZ != 0 && mk == 0) continue;
    for (int mj = -NY; mj <= NY; ++mj) {
      if (NY != 0 && mj == 0) continue;
      for (int mi = -NX; mi <= NX; ++mi) {
        if (NX != 0 && mi == 0) continue;
        const float x0 = xvec[NX + mi], y0 = yvec[NY + mj], z0 = zvec[NZ + mk];
        const float d0 = std::max(m->ztopo - z0, 0.0f);
        auto set1 = [&](float p, float s, float d) {
          Vp[0] = Vp[1] = p;
          Vs[0] = Vs[1] = s;
          Dp[0] = Dp[1] = d;
        };
        // ---- background ----
        if (m->bkind == 1) {  // cart1d :916-966 (1-based d(k))
          const float* d = m->c_d.data();
          const int nk = int(m->c_d.size());
          auto V = [&](int q, int slot) {
            Vp[slot] = m->c_vp[q - 1];
            Vs[slot] = m->c_vs[q - 1];
            Dp[slot] = m->c_dp[q - 1];
          };
          int k1 = 1, k2 = nk;
          if (std::fabs(d[k1 - 1] - d0) < SEIS_ZERO || d0 < d[k1 - 1]) {
            V(k1, 0);
            V(k1, 1);
          } else if (std::fabs(d[k2 - 1] - d0) < SEIS_ZERO) {
            if (std::fabs(d[k2 - 2] - d[k2 - 1]) < SEIS_ZERO) {
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
              if (std::fabs(d[k0 - 1] - d0) < SEIS_ZERO) {
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
              if (std::fabs(d[k1 - 2] - d[k1 - 1]) < SEIS_ZERO) {
                V(k1 - 1, 0);
                V(k1, 1);
              } else if (std::fabs(d[k1] - d[k1 - 1]) < SEIS_ZERO) {
                V(k1, 0);
                V(k1 + 1, 1);
              } else {
                V(k1, 0);
                V(k1, 1);
              }
            } else {
              const float dd = d[k2 - 1];
              const float h = d[k2 - 1] - d[k1 - 1];
              const float L1 = (dd - d0) / h, L2 = 1.0f - L1;
              set1(m->c_vp[k1 - 1] * L1 + m->c_vp[k2 - 1] * L2, m->c_vs[k1 - 1] * L1 + m->c_vs[k2 - 1] * L2,
                   m->c_dp[k1 - 1] * L1 + m->c_dp[k2 - 1] * L2);
            }
          }
        } else if (m->bkind == 2) {  // interface :968-1054
          const Layers& L = m->L;
          int i1, i2, j1, j2;
          float x1, y1;
          locate(x0, L.x.data(), L.ni, i1, i2, x1);
          locate(y0, L.y.data(), L.nj, j1, j2, y1);
          const size_t plane = size_t(L.ni) * L.nj;
          auto I2 = [&](const float* f) { return interp2(L.x.data(), L.y.data(), f, L.ni, i1, j1, x1, y1); };
          auto VA = [&](int n, int kk) { return std::make_pair((n - 1) + 2 * (kk - 1), 0); };
          auto pick = [&](int n1, int k1, int n2, int k2) {
            Vp[0] = L.vp[VA(n1, k1).first];
            Vp[1] = L.vp[VA(n2, k2).first];
            Vs[0] = L.vs[VA(n1, k1).first];
            Vs[1] = L.vs[VA(n2, k2).first];
            Dp[0] = L.dp[VA(n1, k1).first];
            Dp[1] = L.dp[VA(n2, k2).first];
          };
          int n1 = 2, k1 = L.nk, n2 = 2, k2 = L.nk;
          for (int n = L.nk; n >= 1; --n) {
            const float z1 = I2(L.z.data() + plane * (n - 1));
            const float h = n == L.nk ? 1.0e3f : I2(L.h.data() + plane * (n - 1));
            if (h <= SEIS_ZERO && n > 1) continue;
            if (h <= SEIS_ZERO && n == 1) {
              if (L.vp[VA(1, n).first] > SEIS_ZERO) n1 = k1 = n2 = k2 = 1;
              pick(n1, k1, n2, k2);
              break;
            }
            if (std::fabs(z1 - z0) <= dz2 / 5.0f) {
              k2 = n;
              n2 = 2;
              if (n == 1) {
                if (L.vp[VA(1, n).first] > SEIS_ZERO) {
                  k1 = n;
                  n1 = 1;
                } else {
                  k1 = n;
                  n1 = 2;
                }
              }
              for (int mm = n - 1; mm >= 1; --mm) {
                const float hh = I2(L.h.data() + plane * (mm - 1));
                if (hh > SEIS_ZERO) {
                  k1 = mm + 1;
                  n1 = 1;
                  break;
                } else if (mm == 1) {
                  if (L.vp[VA(1, mm).first] > SEIS_ZERO) {
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
              if (n == L.nk) {
                set1(L.vp[VA(2, n).first], L.vs[VA(2, n).first], L.dp[VA(2, n).first]);
              } else {
                const float L2 = (z1 - z0) / h, L1 = 1.0f - L2;
                set1(L.vp[VA(2, n).first] * L1 + L.vp[VA(1, n + 1).first] * L2,
                     L.vs[VA(2, n).first] * L1 + L.vs[VA(1, n + 1).first] * L2,
                     L.dp[VA(2, n).first] * L1 + L.dp[VA(1, n + 1).first] * L2);
              }
              break;
            }
            k1 = n;
            k2 = n;
            n1 = 2;
            n2 = 2;
            if (n == 1) {
              if (L.vp[VA(1, n).first] > SEIS_ZERO) n1 = k1 = n2 = k2 = 1;
              pick(n1, k1, n2, k2);
              break;
            }
          }
        } else if (m->bkind == 3 || m->bkind == 4) {  // layered :1055-1084, composite :1085-1130
          const Layers& L = m->L;
          const bool comp = m->bkind == 4;
          int i1, i2, j1, j2;
          float x1, y1;
          locate(x0, L.x.data(), L.ni, i1, i2, x1);
          locate(y0, L.y.data(), L.nj, j1, j2, y1);
          const size_t plane = size_t(L.ni) * L.nj;
          auto I2 = [&](const float* f) { return interp2(L.x.data(), L.y.data(), f, L.ni, i1, j1, x1, y1); };
          // composite value (slot s = 1, 2) of layer n interpolated to the sample
          auto CI = [&](const std::vector<float>& v, int s, int n) {
            // v is (2, ni, nj, nk): slot fastest; gather the 2 x 2 corners of slot s
            float c[4];
            for (int jj = 0; jj < 2; ++jj)
              for (int ii = 0; ii < 2; ++ii)
                c[jj * 2 + ii] = v[(s - 1) + 2 * ((size_t(n - 1) * L.nj + (j1 - 1 + jj)) * L.ni + (i1 - 1 + ii))];
            float lx1, lx2, ly1, ly2;
            weights(L.x[i1 - 1], L.x[i1], x1, lx1, lx2);
            weights(L.y[j1 - 1], L.y[j1], y1, ly1, ly2);
            float zz = 0.0f;
            zz = zz + lx1 * ly1 * c[0];
            zz = zz + lx2 * ly1 * c[1];
            zz = zz + lx1 * ly2 * c[2];
            zz = zz + lx2 * ly2 * c[3];
            return zz;
          };
          float d = 0.0f;
          for (int n = 1; n <= L.nk; ++n) {
            const float h = I2(L.h.data() + plane * (n - 1));
            if (h <= SEIS_ZERO) continue;
            d = d + h;
            if (std::fabs(d - d0) <= dz2 / 5.0f) {
              if (n == L.nk) return false;
              const int n1 = n;
              int n2 = L.nk;
              for (int mm = n + 1; mm <= L.nk; ++mm) {
                if (I2(L.h.data() + plane * (mm - 1)) > SEIS_ZERO) {
                  n2 = mm;
                  break;
                }
              }
              if (!comp) {
                Vp[0] = L.vp[1 + 2 * (n1 - 1)];
                Vp[1] = L.vp[0 + 2 * (n2 - 1)];
                Vs[0] = L.vs[1 + 2 * (n1 - 1)];
                Vs[1] = L.vs[0 + 2 * (n2 - 1)];
                Dp[0] = L.dp[1 + 2 * (n1 - 1)];
                Dp[1] = L.dp[0 + 2 * (n2 - 1)];
              } else {
                Vp[0] = CI(L.vp, 2, n1);
                Vs[0] = CI(L.vs, 2, n1);
                Dp[0] = CI(L.dp, 2, n1);
                Vp[1] = CI(L.vp, 1, n2);
                Vs[1] = CI(L.vs, 1, n2);
                Dp[1] = CI(L.dp, 1, n2);
              }
              break;
            } else if (d > d0) {
              if (!comp) {
                const float L1 = (d - d0) / h, L2 = 1.0f - L1;
                set1(L.vp[2 * (n - 1)] * L1 + L.vp[1 + 2 * (n - 1)] * L2,
                     L.vs[2 * (n - 1)] * L1 + L.vs[1 + 2 * (n - 1)] * L2,
                     L.dp[2 * (n - 1)] * L1 + L.dp[1 + 2 * (n - 1)] * L2);
              } else {
                const float p1 = CI(L.vp, 1, n), s1 = CI(L.vs, 1, n), r1 = CI(L.dp, 1, n);
                const float p2 = CI(L.vp, 2, n), s2 = CI(L.vs, 2, n), r2 = CI(L.dp, 2, n);
                const float t = d0 - (d - h);
                const float ep = L.vpd[n - 1], es = L.vsd[n - 1], er = L.dpd[n - 1];
                set1(p1 + (p2 - p1) / std::pow(h, ep) * std::pow(t, ep), s1 + (s2 - s1) / std::pow(h, es) * std::pow(t, es),
                     r1 + (r2 - r1) / std::pow(h, er) * std::pow(t, er));
              }
              break;
            } else if (n == L.nk) {
              return false;
            }
          }
        } else if (m->bkind == 5) {  // volume :1131-1142
          const Volume& V = m->bv;
          int i1, i2, j1, j2, k1, k2;
          float x1, y1, zz1;
          locate(x0, V.x.data(), V.ni, i1, i2, x1);
          locate(y0, V.y.data(), V.nj, j1, j2, y1);
          locate(V.rz0 - z0, V.rz.data(), V.nk, k1, k2, zz1);
          set1(interp3(V.x.data(), V.y.data(), V.rz.data(), V.vp.data(), V.ni, V.nj, i1, j1, k1, x1, y1, zz1),
               interp3(V.x.data(), V.y.data(), V.rz.data(), V.vs.data(), V.ni, V.nj, i1, j1, k1, x1, y1, zz1),
               interp3(V.x.data(), V.y.data(), V.rz.data(), V.dp.data(), V.ni, V.nj, i1, j1, k1, x1, y1, zz1));
        } else if (m->bkind == 6) {  // verpoly :1143-1171
          const Verpoly& P = m->bp;
          const int wi = minloc_abs(P.x.data(), 1, P.ni, x0), wj = minloc_abs(P.y.data(), 1, P.nj, y0);
          const size_t plane = size_t(P.ni) * P.nj, col = size_t(wj - 1) * P.ni + (wi - 1);
          const float* rz = P.rz.data() + col;
          const float depth = P.rz0 - z0;
          int wk = minloc_abs(rz, plane, P.nk, depth);
          const size_t cs = plane * P.nk;  // stride between coefficients
          auto C = [&](const std::vector<float>& c, int kk) { return c.data() + col + plane * (kk - 1); };
          if (std::fabs(rz[plane * (wk - 1)] - depth) <= dz2 / 5.0f || depth < rz[0]) {
            const int k1 = std::max(1, wk - 1), k2 = wk;
            const float z1 = rz[plane * (k2 - 1)] - rz[plane * (k1 - 1)], z2 = 0.0f;
            Vp[0] = eval_poly(C(P.vpc, k1), cs, P.vpd.data(), P.np, z1);
            Vp[1] = eval_poly(C(P.vpc, k2), cs, P.vpd.data(), P.np, z2);
            Vs[0] = eval_poly(C(P.vsc, k1), cs, P.vsd.data(), P.np, z1);
            Vs[1] = eval_poly(C(P.vsc, k2), cs, P.vsd.data(), P.np, z2);
            Dp[0] = eval_poly(C(P.dpc, k1), cs, P.dpd.data(), P.np, z1);
            Dp[1] = eval_poly(C(P.dpc, k2), cs, P.dpd.data(), P.np, z2);
          } else {
            if (depth < rz[plane * (wk - 1)]) wk = wk - 1;
            const float z1 = depth - rz[plane * (wk - 1)];
            set1(eval_poly(C(P.vpc, wk), cs, P.vpd.data(), P.np, z1), eval_poly(C(P.vsc, wk), cs, P.vsd.data(), P.np, z1),
                 eval_poly(C(P.dpc, wk), cs, P.dpd.data(), P.np, z1));
          }
        }
        // ---- perturbation ----
        if (m->pkind == 5) {  // volume :1175-1190
          const Volume& V = m->pv;
          int i1, i2, j1, j2, k1, k2;
          float x1, y1, zz1;
          locate(x0, V.x.data(), V.ni, i1, i2, x1);
          locate(y0, V.y.data(), V.nj, j1, j2, y1);
          locate(V.rz0 - z0, V.rz.data(), V.nk, k1, k2, zz1);
          const float dVp = interp3(V.x.data(), V.y.data(), V.rz.data(), V.vp.data(), V.ni, V.nj, i1, j1, k1, x1, y1, zz1);
          const float dVs = interp3(V.x.data(), V.y.data(), V.rz.data(), V.vs.data(), V.ni, V.nj, i1, j1, k1, x1, y1, zz1);
          const float dDp = interp3(V.x.data(), V.y.data(), V.rz.data(), V.dp.data(), V.ni, V.nj, i1, j1, k1, x1, y1, zz1);
          for (int s = 0; s < 2; ++s) {
            Vp[s] = Vp[s] * (1.0f + dVp);
            Vs[s] = Vs[s] * (1.0f + dVs);
            Dp[s] = Dp[s] * (1.0f + dDp);
          }
        } else if (m->pkind == 6) {  // verpoly :1192-1220
          const Verpoly& P = m->pp;
          const int wi = minloc_abs(P.x.data(), 1, P.ni, x0), wj = minloc_abs(P.y.data(), 1, P.nj, y0);
          const size_t plane = size_t(P.ni) * P.nj, col = size_t(wj - 1) * P.ni + (wi - 1);
          const float* rz = P.rz.data() + col;
          const float depth = P.rz0 - z0;
          int wk = minloc_abs(rz, plane, P.nk, depth);
          const size_t cs = plane * P.nk;
          auto C = [&](const std::vector<float>& c, int kk) { return c.data() + col + plane * (kk - 1); };
          float dVp[2], dVs[2], dDp[2];
          if (std::fabs(rz[plane * (wk - 1)] - depth) <= dz2 / 5.0f || depth < rz[0]) {
            const int k1 = std::max(1, wk - 1), k2 = wk;
            const float z1 = rz[plane * (k2 - 1)] - rz[plane * (k1 - 1)], z2 = 0.0f;
            dVp[0] = eval_poly(C(P.vpc, k1), cs, P.vpd.data(), P.np, z1);
            dVp[1] = eval_poly(C(P.vpc, k2), cs, P.vpd.data(), P.np, z2);
            dVs[0] = eval_poly(C(P.vsc, k1), cs, P.vsd.data(), P.np, z1);
            dVs[1] = eval_poly(C(P.vsc, k2), cs, P.vsd.data(), P.np, z2);
            dDp[0] = eval_poly(C(P.dpc, k1), cs, P.dpd.data(), P.np, z1);
            dDp[1] = eval_poly(C(P.dpc, k2), cs, P.dpd.data(), P.np, z2);
          } else {
            if (depth < rz[plane * (wk - 1)]) wk = wk - 1;
            const float z1 = depth - rz[plane * (wk - 1)];
            dVp[0] = dVp[1] = eval_poly(C(P.vpc, wk), cs, P.vpd.data(), P.np, z1);
            dVs[0] = dVs[1] = eval_poly(C(P.vsc, wk), cs, P.vsd.data(), P.np, z1);
            dDp[0] = dDp[1] = eval_poly(C(P.dpc, wk), cs, P.dpd.data(), P.np, z1);
          }
          for (int s = 0; s < 2; ++s) {
            Vp[s] = Vp[s] * (1.0f + dVp[s]);
            Vs[s] = Vs[s] * (1.0f + dVs[s]);
            Dp[s] = Dp[s] * (1.0f + dDp[s]);
          }
        }
        // ---- Lame parameters and the harmonic accumulation :1222-1235 ----
        float miu[2], la[2];
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
    }
  }
  *rho_out = rho0 / float(nsamp);
  if (flag_water) {
    *mu_out = nwater >= nsamp / 2 ? 0.0f : float(nsamp - nwater) / mu0;
  } else {
    *mu_out = float(nsamp) / mu0;
  }
  *lam_out = float(nsamp) / lam0;
  return true;
}

double plane_dist(const double* P, const double* A, const double* B, const double* Cc) {
  double AB[3], AC[3], p[3];
  for (int q = 0; q < 3; ++q) {
    AB[q] = B[q] - A[q];
    AC[q] = Cc[q] - A[q];
  }
  p[0] = AB[1] * AC[2] - AB[2] * AC[1];
  p[1] = AB[2] * AC[0] - AB[0] * AC[2];
  p[2] = AB[0] * AC[1] - AB[1] * AC[0];
  const double d = -(p[0] * A[0] + p[1] * A[1] + p[2] * A[2]);
  return std::fabs((p[0] * P[0] + p[1] * P[1] + p[2] * P[2] + d) / std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]));
}

}  // namespace

extern "C" {

// grid with ghosts: x[ni+6], y[nj+6], z[nk+6]; ng = half_sample_point
orc_media* orc_media_create(int ni, int nj, int nk, const float* x, const float* y, const float* z, float ztopo,
                            const int* ng) {
  auto* m = new orc_media();
  m->ni = ni;
  m->nj = nj;
  m->nk = nk;
  m->nx = ni + 2 * LENFD;
  m->ny = nj + 2 * LENFD;
  m->nz = nk + 2 * LENFD;
  for (int q = 0; q < 3; ++q) m->ng[q] = ng[q];
  m->ztopo = ztopo;
  m->x.assign(x, x + m->nx);
  m->y.assign(y, y + m->ny);
  m->z.assign(z, z + m->nz);
  return m;
}

void orc_media_destroy(orc_media* m) { delete m; }
const char* orc_media_last_error(orc_media* m) { return m->err.c_str(); }

void orc_media_set_cart1d(orc_media* m, int nk, const float* d, const float* vp, const float* vs, const float* dp) {
  m->bkind = 1;
  m->c_d.assign(d, d + nk);
  m->c_vp.assign(vp, vp + nk);
  m->c_vs.assign(vs, vs + nk);
  m->c_dp.assign(dp, dp + nk);
}

// kind 2 interface (z and h (ni,nj,nk) with h's last layer unused), 3 layered (h), 4
// composite (h; values (2,ni,nj,nk); exponents (nk)); values (2,nk) for kinds 2 and 3
void orc_media_set_layers(orc_media* m, int kind, int ni, int nj, int nk, const float* x, const float* y,
                          const float* z, const float* h, const float* vp, const float* vs, const float* dp,
                          const float* vpd, const float* vsd, const float* dpd) {
  m->bkind = kind;
  Layers& L = m->L;
  L.ni = ni;
  L.nj = nj;
  L.nk = nk;
  const size_t n3 = size_t(ni) * nj * nk, nv = kind == 4 ? 2 * n3 : size_t(2) * nk;
  L.x.assign(x, x + ni);
  L.y.assign(y, y + nj);
  if (z) L.z.assign(z, z + n3);
  L.h.assign(h, h + n3);
  L.vp.assign(vp, vp + nv);
  L.vs.assign(vs, vs + nv);
  L.dp.assign(dp, dp + nv);
  if (kind == 4) {
    L.vpd.assign(vpd, vpd + nk);
    L.vsd.assign(vsd, vsd + nk);
    L.dpd.assign(dpd, dpd + nk);
  }
}

// full model arrays as read from the file; the sub-volume of volume_read is taken here
void orc_media_set_volume(orc_media* m, int perturbed, int ni, int nj, int nk, const float* gx, const float* gy,
                          const float* grz, float rz0, const float* vp, const float* vs, const float* dp) {
  Volume& V = perturbed ? m->pv : m->bv;
  if (perturbed) m->pkind = 5;
  else m->bkind = 5;
  int i1, i2, j1, j2;
  select_range(gx, ni, m->x[0], m->x[m->nx - 1], i1, i2);
  select_range(gy, nj, m->y[0], m->y[m->ny - 1], j1, j2);
  V.ni = i2 - i1 + 1;
  V.nj = j2 - j1 + 1;
  V.nk = nk;
  V.rz0 = rz0;
  V.x.assign(gx + i1 - 1, gx + i2);
  V.y.assign(gy + j1 - 1, gy + j2);
  V.rz.assign(grz, grz + nk);
  const size_t n = size_t(V.ni) * V.nj * V.nk;
  for (std::vector<float>* f : {&V.vp, &V.vs, &V.dp}) f->assign(n, 0.0f);
  for (int k = 0; k < nk; ++k)
    for (int j = 0; j < V.nj; ++j)
      for (int i = 0; i < V.ni; ++i) {
        const size_t src = (size_t(k) * nj + (j1 - 1 + j)) * ni + (i1 - 1 + i);
        const size_t dst = (size_t(k) * V.nj + j) * V.ni + i;
        V.vp[dst] = vp[src];
        V.vs[dst] = vs[src];
        V.dp[dst] = dp[src];
      }
}

// rz (ni,nj,nk), coefficients (ni,nj,nk,np), exponents (np); full arrays
void orc_media_set_verpoly(orc_media* m, int perturbed, int ni, int nj, int nk, int np, const float* gx,
                           const float* gy, const float* rz, float rz0, const float* vpc, const float* vsc,
                           const float* dpc, const float* vpd, const float* vsd, const float* dpd) {
  Verpoly& P = perturbed ? m->pp : m->bp;
  if (perturbed) m->pkind = 6;
  else m->bkind = 6;
  int i1, i2, j1, j2;
  select_range(gx, ni, m->x[0], m->x[m->nx - 1], i1, i2);
  select_range(gy, nj, m->y[0], m->y[m->ny - 1], j1, j2);
  P.ni = i2 - i1 + 1;
  P.nj = j2 - j1 + 1;
  P.nk = nk;
  P.np = np;
  P.rz0 = rz0;
  P.x.assign(gx + i1 - 1, gx + i2);
  P.y.assign(gy + j1 - 1, gy + j2);
  const size_t n3 = size_t(P.ni) * P.nj * nk;
  P.rz.assign(n3, 0.0f);
  for (std::vector<float>* f : {&P.vpc, &P.vsc, &P.dpc}) f->assign(n3 * np, 0.0f);
  for (int q = 0; q < np; ++q)
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < P.nj; ++j)
        for (int i = 0; i < P.ni; ++i) {
          const size_t src = ((size_t(q) * nk + k) * nj + (j1 - 1 + j)) * ni + (i1 - 1 + i);
          const size_t dst = ((size_t(q) * nk + k) * P.nj + j) * P.ni + i;
          if (q == 0) P.rz[dst] = rz[src];
          P.vpc[dst] = vpc[src];
          P.vsc[dst] = vsc[src];
          P.dpc[dst] = dpc[src];
        }
  P.vpd.assign(vpd, vpd + np);
  P.vsd.assign(vsd, vsd + np);
  P.dpd.assign(dpd, dpd + np);
}

// effmedia_eval + media_extend; out arrays (nx, ny, nz), i fastest.  0 on success.
int orc_media_eval(orc_media* m, float* lam, float* mu, float* rho) {
  const int nx = m->nx, ny = m->ny;
  int bad = 0;
  // points are independent: planes in parallel (OpenMP), each point's samples in order
#pragma omp parallel for schedule(dynamic) reduction(| : bad)
  for (int k = LENFD; k < LENFD + m->nk; ++k)
    for (int j = LENFD; j < LENFD + m->nj; ++j)
      for (int i = LENFD; i < LENFD + m->ni; ++i) {
        const size_t p = (size_t(k) * ny + j) * nx + i;
        if (!point(m, i, j, k, &lam[p], &mu[p], &rho[p])) bad = 1;
      }
  if (bad) {
    m->err = "please increase the thickness of the lowest layer";
    return 1;
  }
  // extend_equal: each ghost takes the value of the nearest interior point (x, then y,
  // then z, as the reference's three passes leave it)
  for (float* w : {lam, mu, rho})
    for (int k = 0; k < m->nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const int ci = std::min(std::max(i, LENFD), LENFD + m->ni - 1);
          const int cj = std::min(std::max(j, LENFD), LENFD + m->nj - 1);
          const int ck = std::min(std::max(k, LENFD), LENFD + m->nk - 1);
          w[(size_t(k) * ny + j) * nx + i] = w[(size_t(ck) * ny + cj) * nx + ci];
        }
  return 0;
}

// media_stept_check on media (nx, ny, nz): dtmax, its 1-based local index (ghosts
// included, interior from 4) and the Vp and dL there
void orc_media_stept_check(orc_media* m, const float* lam, const float* mu, const float* rho, float* dtmax,
                           int* ijk, float* vp_out, float* dl_out) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  std::vector<double> g(size_t(nx) * ny * nz * 3);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double* q = &g[((size_t(k) * ny + j) * nx + i) * 3];
        const double a = double(m->x[i]) - PI / 2, b = double(m->y[j]);
        q[0] = double(m->z[k]) * std::cos(a) * std::cos(b);
        q[1] = double(m->z[k]) * std::cos(a) * std::sin(b);
        q[2] = double(m->z[k]) * std::sin(a);
      }
  auto G = [&](int i, int j, int k) { return &g[((size_t(k) * ny + j) * nx + i) * 3]; };
  float best = 1.0e10f;
  for (int k = LENFD; k < LENFD + m->nk; ++k)
    for (int j = LENFD; j < LENFD + m->nj; ++j)
      for (int i = LENFD; i < LENFD + m->ni; ++i) {
        const size_t p = (size_t(k) * ny + j) * nx + i;
        const float Vp = std::sqrt((lam[p] + 2.0f * mu[p]) / rho[p]);
        double dmin = 0.0;
        for (int s = 0; s < 8; ++s) {
          const int a = (s & 1) ? i + 1 : i - 1, b = (s & 2) ? j + 1 : j - 1, c = (s & 4) ? k + 1 : k - 1;
          const double dd = plane_dist(G(i, j, k), G(a, j, k), G(i, b, k), G(i, j, c));
          dmin = s == 0 ? dd : std::min(dmin, dd);
        }
        const float dtLe = float(dmin);
        const float dtlocal = 1.3f / Vp * dtLe;
        if (dtlocal < best) {
          best = dtlocal;
          ijk[0] = i + 1;
          ijk[1] = j + 1;
          ijk[2] = k + 1;
          *vp_out = Vp;
          *dl_out = dtLe;
        }
      }
  *dtmax = best;
}

}  // extern "C"
