// Gaussian-hill extension (no counterpart in the reference, whose grid is orthogonal
// spherical with a flat top): the FP64 metric of the terrain-following radius
// r(i,j,k) = z(k) + h(i,j) s(k), s(k) = (z(k) - z(0)) / (z(nk2) - z(0)).
//
// Derivatives along an index use the stencil of seis3d_metric (seis3d_metric.F90:83-112):
// the mean of the backward and forward DRP/opt operators, ends clamped to the interior.
// Every double operation is an explicit round-to-nearest intrinsic in a fixed order (no
// contraction), so the arrays equal those of a CPU evaluation of the same expressions.
#include <cuda_runtime.h>

#include "kernels.h"

namespace fw {

__constant__ double kMetF[5] = {-0.30874, -0.6326, 1.2330, -0.3334, 0.04168};
__constant__ double kMetB[5] = {-0.04168, 0.3334, -1.2330, 0.6326, 0.30874};

// metric derivative of f (values f(n) = get(n)) at index i, ends clamped to [lo, hi]
template <class Get>
__device__ __forceinline__ double dmetric(Get get, int i, int lo, int hi) {
  const int ii = i < lo ? lo : (i > hi ? hi : i);
  double sb = 0.0, sf = 0.0;
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    sb = __dadd_rn(sb, __dmul_rn(get(ii - 3 + q), kMetB[q]));
    sf = __dadd_rn(sf, __dmul_rn(get(ii - 1 + q), kMetF[q]));
  }
  return __dmul_rn(__dadd_rn(sb, sf), 0.5);
}

__global__ void topo_slopes_kernel(const Geom g, const float* __restrict__ h, double* __restrict__ hxi,
                                   double* __restrict__ heta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= g.nx || j >= g.ny) return;
  hxi[i + (long long)g.nx * j] = dmetric([&](int n) { return double(h[n + (long long)g.nx * j]); }, i, g.i1, g.i2);
  heta[i + (long long)g.nx * j] = dmetric([&](int n) { return double(h[i + (long long)g.nx * n]); }, j, g.j1, g.j2);
}

// One thread per column (i, j): for every k the radius, its metric derivative along k and
// the four stored terms: r, zeta_r =
// zeta_z(k) z_zeta(k) / r_zeta, zeta_theta / r = -(h_xi s xi_x) zeta_r / r and
// zeta_phi / (r sin theta) = -(h_eta s eta_y) zeta_r / (r sin theta).
__global__ void topo_metric_kernel(const TopoMetricArgs a) {
  const Geom& g = a.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= g.nx || j >= g.ny) return;
  const long long c2 = i + (long long)g.nx * j;
  const double hh = double(a.h[c2]), hx = a.hxi[c2], hy = a.heta[c2];
  auto rad = [&](int k) { return __dadd_rn(double(a.z[k]), __dmul_rn(hh, a.sk[k])); };
  const double xi = double(a.xi_x[i]), et = double(a.eta_y[j]), xs = double(a.xsin[i]);
  for (int k = 0; k < g.nz; ++k) {
    const double r = rad(k);
    const double rz = dmetric(rad, k, g.k1, g.k2);
    const double az = __dmul_rn(double(a.zeta_z[k]), __ddiv_rn(a.rzf[k], rz));
    const double bx = __ddiv_rn(__dmul_rn(-__dmul_rn(__dmul_rn(hx, a.sk[k]), xi), az), r);
    const double by = __ddiv_rn(__dmul_rn(-__dmul_rn(__dmul_rn(hy, a.sk[k]), et), az), __dmul_rn(r, xs));
    const long long p = (long long)(i + PADL) + (long long)g.px * ((long long)j + (long long)g.ny * k);
    a.out[p] = float(r);
    a.out[g.fstride + p] = float(az);
    a.out[2 * g.fstride + p] = float(bx);
    a.out[3 * g.fstride + p] = float(by);
  }
}

// Surface arrays per column: the normal m = (bx / az, by / az, 1) of k = nk2 and the
// inverse of the 3x3 map M from the velocity's zeta-derivatives u to the traction rate
// (S(u) . m) there; column q of M is S(L(e_q)) . m with L the strain of a unit
// zeta-derivative.  Out: 11 planes (m1, m2, inverse row-major), g.plane apart.
__global__ void topo_surface_kernel(const Geom g, const float* __restrict__ met, const float* __restrict__ lam,
                                    const float* __restrict__ mu, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= g.nx || j >= g.ny) return;
  const long long col = (long long)(i + PADL) + (long long)g.px * j;
  const long long p = col + g.plane * g.k2;
  const double az = double(met[g.fstride + p]), bx = double(met[2 * g.fstride + p]),
               by = double(met[3 * g.fstride + p]);
  const double m1 = __ddiv_rn(bx, az), m2 = __ddiv_rn(by, az);
  const double la = double(lam[p]), mv = double(mu[p]);
  const double l2 = __dadd_rn(la, __dmul_rn(2.0, mv));
  auto mul = [](double a, double b) { return __dmul_rn(a, b); };
  auto add = [](double a, double b) { return __dadd_rn(a, b); };
  auto sub = [](double a, double b) { return __dsub_rn(a, b); };
  double M[3][3];
  M[0][0] = add(add(mul(mul(l2, bx), m1), mul(mul(mv, by), m2)), mul(mv, az));
  M[1][0] = add(mul(mul(mv, by), m1), mul(mul(la, bx), m2));
  M[2][0] = add(mul(mul(mv, az), m1), mul(la, bx));
  M[0][1] = add(mul(mul(la, by), m1), mul(mul(mv, bx), m2));
  M[1][1] = add(add(mul(mul(mv, bx), m1), mul(mul(l2, by), m2)), mul(mv, az));
  M[2][1] = add(mul(mul(mv, az), m2), mul(la, by));
  M[0][2] = add(mul(mul(la, az), m1), mul(mv, bx));
  M[1][2] = add(mul(mul(la, az), m2), mul(mv, by));
  M[2][2] = add(add(mul(mul(mv, bx), m1), mul(mul(mv, by), m2)), mul(l2, az));
  const double c00 = sub(mul(M[1][1], M[2][2]), mul(M[1][2], M[2][1]));
  const double c01 = sub(mul(M[1][2], M[2][0]), mul(M[1][0], M[2][2]));
  const double c02 = sub(mul(M[1][0], M[2][1]), mul(M[1][1], M[2][0]));
  const double det = add(add(mul(M[0][0], c00), mul(M[0][1], c01)), mul(M[0][2], c02));
  const double inv[9] = {__ddiv_rn(c00, det),
                         __ddiv_rn(sub(mul(M[0][2], M[2][1]), mul(M[0][1], M[2][2])), det),
                         __ddiv_rn(sub(mul(M[0][1], M[1][2]), mul(M[0][2], M[1][1])), det),
                         __ddiv_rn(c01, det),
                         __ddiv_rn(sub(mul(M[0][0], M[2][2]), mul(M[0][2], M[2][0])), det),
                         __ddiv_rn(sub(mul(M[0][2], M[1][0]), mul(M[0][0], M[1][2])), det),
                         __ddiv_rn(c02, det),
                         __ddiv_rn(sub(mul(M[0][1], M[2][0]), mul(M[0][0], M[2][1])), det),
                         __ddiv_rn(sub(mul(M[0][0], M[1][1]), mul(M[0][1], M[1][0])), det)};
  out[col] = float(m1);
  out[g.plane + col] = float(m2);
#pragma unroll
  for (int e = 0; e < 9; ++e) out[(2 + e) * g.plane + col] = float(inv[e]);
}

void launch_topo_slopes(const Geom& g, const float* h, double* hxi, double* heta, void* stream) {
  topo_slopes_kernel<<<dim3((g.nx + 127) / 128, g.ny), 128, 0, (cudaStream_t)stream>>>(g, h, hxi, heta);
}

void launch_topo_metric(const TopoMetricArgs& a, void* stream) {
  topo_metric_kernel<<<dim3((a.g.nx + 127) / 128, a.g.ny), 128, 0, (cudaStream_t)stream>>>(a);
}

void launch_topo_surface(const Geom& g, const float* metric, const float* lam, const float* mu, float* out,
                         void* stream) {
  topo_surface_kernel<<<dim3((g.nx + 127) / 128, g.ny), 128, 0, (cudaStream_t)stream>>>(g, metric, lam, mu, out);
}

}  // namespace fw
