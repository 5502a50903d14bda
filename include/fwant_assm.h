/* fwant_gb300 — kernel assembly onto inversion blocks on the GPU (the stage between the
 * sensitivity kernels and the inversion).
 *
 * Replaces the computation of the reference's SI_ker2assm / SI_ker_kamu2assm programs
 * (code/srcF.kernel/SI_ker2assm.F90, SI_ker_kamu2assm.F90): for every pick, each kernel
 * volume K (phase Vp and Vs, or kappa and mu) is projected onto the inversion blocks,
 * B(n) = sum over the pixels m of block n of K(i,j,k) * volume(m,n) in the order of the
 * block file (:306-323), and |B(n)| is added to the running sums S(n) that the reference
 * writes as inv_G_sum.  The caller scales B by the C factors and writes the compact rows
 * (export_G_compact :545-571), as the fwant_assm program does.
 *
 * Arrays are Fortran order (first index fastest).  Sums are single precision in the
 * reference's order (each product rounded, then added), so the blocks equal the
 * reference's values bit for bit.
 */
#ifndef FWANT_ASSM_H
#define FWANT_ASSM_H

#include "fwant_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fwant_assm fwant_assm;

/* The inversion blocks of init_inv_block (SI_ker2assm.F90:466-485) over a kernel volume of
 * ki x kj x kk points (the snapshot's subc): num_blk blocks of at most max_pix pixels;
 * volume (max_pix, num_blk), num_of_pix (num_blk), indx_of_pix (3, max_pix, num_blk) with
 * 1-based (i, j, k) in the kernel volume.  Every used pixel index must lie inside the volume
 * (FWANT_ERR_INVALID_ARG otherwise: the reference would read outside its array). */
fwant_status fwant_assm_create(int ki, int kj, int kk, int num_blk, int max_pix, const float* volume,
                               const int* num_of_pix, const int* indx_of_pix, int device, fwant_assm** out);
void fwant_assm_destroy(fwant_assm* a);
const char* fwant_assm_last_error(fwant_assm* a);

/* One pick: nq (1..4) kernel volumes of ki*kj*kk floats each on the host; blocks
 * (num_blk, nq) receives B for each volume, and |B| is added to the sums of slots 0..nq-1. */
fwant_status fwant_assm_project(fwant_assm* a, int nq, const float* const* kernels, float* blocks);

/* The same with the kernel volumes already in device memory of the handle's GPU (a
 * caller's own device arrays, ki*kj*kk floats each, Fortran order): no upload.  Pointers
 * that are not device memory of that GPU are refused before any access. */
fwant_status fwant_assm_project_device(fwant_assm* a, int nq, const float* const* d_kernels, float* blocks);

/* The running sums of |B| (num_blk, 4), slots beyond the largest nq used are zero. */
fwant_status fwant_assm_sums(fwant_assm* a, float* sums);

/* device time (ms) of the last projection's kernel */
fwant_status fwant_assm_last_ms(fwant_assm* a, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* FWANT_ASSM_H */
