/* fwant_gb300 — the medium preprocessor on the GPU (the stage before the solver).
 *
 * Replaces the computation of the reference's seis3d_media program
 * (code/srcF/seis3d_media.F90): the effective-medium evaluation effmedia_eval (:854-1249),
 * which samples the background and perturbation models at (2 N)^3 sub-cell points around
 * every grid point (N = half_sample_point) and averages rho arithmetically and lambda, mu
 * harmonically; the ghost extension media_extend / extend_equal (:1264-1299); and the
 * time-step check media_stept_check (:1544-1611).  Model files are read by the caller (the
 * fwant_media program reads the reference's formats); these entry points take the arrays
 * as the reference's readers leave them: coordinates in radians (theta, phi) and metres,
 * velocities in m/s, densities in kg/m^3.
 *
 * Arrays are Fortran order (first index fastest).  The grid (x, y, z) includes the three
 * ghost points on each side: x[ni+6], y[nj+6], z[nk+6]; outputs are (ni+6, nj+6, nk+6).
 */
#ifndef FWANT_MEDIA_H
#define FWANT_MEDIA_H

#include "fwant_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fwant_media fwant_media;

/* background model kinds (init_media :281-315) */
enum {
  FWANT_MEDIA_CART1D = 1,
  FWANT_MEDIA_INTERFACE = 2,
  FWANT_MEDIA_LAYERED = 3,
  FWANT_MEDIA_COMPOSITE = 4,
  FWANT_MEDIA_VOLUME = 5,
  FWANT_MEDIA_VERPOLY = 6
};

/* Grid and sampling (seis3d_media :156-190): ztopo is the radius of the free surface,
 * z(nk2) of the top subdomain; half_sample[3] = half_sample_point (NGRIDX, NGRIDY,
 * NGRIDZ), each 0..16. */
fwant_status fwant_media_create(int ni, int nj, int nk, const float* x, const float* y, const float* z, float ztopo,
                                const int half_sample[3], int device, fwant_media** out);
void fwant_media_destroy(fwant_media* m);
const char* fwant_media_last_error(fwant_media* m);

/* cart1d background (layer1d_read :341-430): nk >= 2 samples of depth (m, ascending),
 * vp, vs (m/s) and rho (kg/m^3). */
fwant_status fwant_media_set_cart1d(fwant_media* m, int nk, const float* depth, const float* vp, const float* vs,
                                    const float* rho);

/* interface, layered or composite background (interface_read :433-532, layered_read
 * :535-643, composite_read :646-702): horizontal sampling x[ni], y[nj] (radians,
 * ascending, ni, nj >= 2), nk layers or interfaces.
 *   interface: z (ni,nj,nk) interface radii; h (ni,nj,nk) with h(:,:,n) = z(:,:,n) -
 *              z(:,:,n+1) as interface_read forms it (the last layer is not read);
 *              vp, vs, rho (2, nk).
 *   layered:   h (ni,nj,nk) layer thicknesses; vp, vs, rho (2, nk); z may be NULL.
 *   composite: h (ni,nj,nk); vp, vs, rho (2, ni, nj, nk); vp_exp, vs_exp, rho_exp (nk) the
 *              polynomial exponents (Vp_poly_d ...); z may be NULL.
 * Exponents are NULL except for composite. */
fwant_status fwant_media_set_layers(fwant_media* m, int kind, int ni, int nj, int nk, const float* x, const float* y,
                                    const float* z, const float* h, const float* vp, const float* vs, const float* rho,
                                    const float* vp_exp, const float* vs_exp, const float* rho_exp);

/* volume model as background (perturbed 0) or relative perturbation (perturbed 1)
 * (volume_init :705-729, volume_read :759-779): the whole file's theta x[ni], phi y[nj]
 * (radians), depth2sealevel rz[nk] (ascending), sealevel rz0, and vp, vs, rho (ni,nj,nk);
 * the sub-volume covering the grid is selected as volume_read does. */
fwant_status fwant_media_set_volume(fwant_media* m, int perturbed, int ni, int nj, int nk, const float* x,
                                    const float* y, const float* rz, float rz0, const float* vp, const float* vs,
                                    const float* rho);

/* verpoly model (verpoly_init :782-806, verpoly_read :829-850): x[ni], y[nj] (radians),
 * rz (ni,nj,nk) depth to sealevel of each polynomial piece, rz0, coefficients
 * vp_c, vs_c, rho_c (ni,nj,nk,npoly) and exponents (npoly). */
fwant_status fwant_media_set_verpoly(fwant_media* m, int perturbed, int ni, int nj, int nk, int npoly,
                                     const float* x, const float* y, const float* rz, float rz0, const float* vp_c,
                                     const float* vs_c, const float* rho_c, const float* vp_exp, const float* vs_exp,
                                     const float* rho_exp);

/* effmedia_eval + media_extend: lambda, mu, rho (ni+6, nj+6, nk+6) on the host (each may
 * be NULL to leave it on the device only).  A background must be set.  A sample at the
 * depth of the bottom of the lowest layer of a layered or composite model fails with
 * FWANT_ERR_INVALID_ARG ("please increase the thickness of the lowest layer"), as the
 * reference stops there. */
fwant_status fwant_media_eval(fwant_media* m, float* lambda, float* mu, float* rho);

/* media_stept_check on the last evaluated medium: the largest stable time step dtmax =
 * min over interior points of 1.3 / Vp * dL (dL the smallest distance from the point to the
 * eight planes through its neighbours), its 1-based local index ijk[3] (ghosts included:
 * the interior starts at 4; the first point in i-fastest order on ties), and Vp and dL
 * there. */
fwant_status fwant_media_stept_check(fwant_media* m, float* dtmax, int ijk[3], float* vp, float* dl);

/* Device addresses of the last evaluated lambda, mu and rho ((ni+6, nj+6, nk+6) floats each,
 * Fortran order), valid until the next fwant_media_eval or fwant_media_destroy; hand them
 * to fwant_set_media_device of a solver on the same GPU. */
fwant_status fwant_media_device_arrays(fwant_media* m, const float** lambda, const float** mu, const float** rho);

/* device time (ms) of the last fwant_media_eval's kernels */
fwant_status fwant_media_last_eval_ms(fwant_media* m, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* FWANT_MEDIA_H */
