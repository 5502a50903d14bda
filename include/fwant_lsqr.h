/* fwant_gb300 — LSQR least-squares solver on the GPU (the inversion stage after the
 * sensitivity kernels).
 *
 * Replaces the LSQR package of the reference's inversion (inv.LSQR/mod_LSQR.f90): the
 * row-stored sparse system of lsqr_init + lldrow (:44-135), the Paige-Saunders iteration
 * slsqr (:137-268) and the solution / standard-error extraction lgtsol (:270-285).  The
 * matrix is given at once in compressed rows; the device keeps it in compressed rows and
 * in compressed columns, so A v and A^T u are both gathers summed in a fixed order and the
 * results do not depend on the launch shape.  All arithmetic is FP64, as in the reference.
 */
#ifndef FWANT_LSQR_H
#define FWANT_LSQR_H

#include "fwant_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fwant_lsqr fwant_lsqr;

/* A is nrow x ncol with row_ptr[nrow+1] 0-based offsets into col[] (0-based column
 * indices, repeats allowed: they add) and val[]; rhs[nrow] is b.  Rows without entries are
 * allowed (the reference's lldrow skips them before they reach the matrix).  Copies
 * everything to the device.  ncol < 2^31. */
fwant_status fwant_lsqr_create(long long nrow, long long ncol, const long long* row_ptr, const int* col,
                               const double* val, const double* rhs, int device, fwant_lsqr** out);
void fwant_lsqr_destroy(fwant_lsqr* l);
const char* fwant_lsqr_last_error(fwant_lsqr* l);

/* slsqr: iterate from x = 0 until test1 = phibar / (|A|_F |x|) <= atol, or test2 =
 * alpha |c| / |A|_F <= btol, or maxit iterations (the reference: 1e-7, 1e-7, 30000);
 * *itct (may be NULL) receives the iteration count.  A zero rho (an exactly solved or
 * zero system) ends the iteration without updating the residual norm, as the reference
 * returns early. */
fwant_status fwant_lsqr_solve(fwant_lsqr* l, double atol, double btol, long long maxit, long long* itct);

/* lgtsol for the first nvar unknowns: x and the standard errors
 * sqrt(res2 / max(nrow - nvar, 1) * sig). */
fwant_status fwant_lsqr_solution(fwant_lsqr* l, long long nvar, double* x, double* serr);

/* info[6] = |A|_F, res2 (final phibar), test1, test2, phibar, |x| of the last iteration. */
fwant_status fwant_lsqr_info(fwant_lsqr* l, double* info);

/* y[nrow] = A x[ncol] (for residual evaluation). */
fwant_status fwant_lsqr_multiply(fwant_lsqr* l, const double* x, double* y);

/* Device time of the last fwant_lsqr_solve (ms) and the iterations per CUDA-graph replay. */
fwant_status fwant_lsqr_last_solve_ms(fwant_lsqr* l, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* FWANT_LSQR_H */
