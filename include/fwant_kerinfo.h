/* fwant_gb300 — sensitivity-kernel statistics on the GPU (the kernel-distribution pass run
 * over the kernel files of all picks).
 *
 * Replaces the computation of the reference's SI_ker2info program
 * (code/srcF.kernel/SI_ker2info.F90): for every pick of every event of every station, the
 * four kernel volumes K (phase_Vp, amplitude_Vp, phase_Vs, amplitude_Vs, slots q = ap, aq,
 * bp, bq) are read and, point by point (:271-289),
 *   S_q += |K_q|                 (single precision, in pick order, never reset)
 *   M_q += 1 if |K_q| > K0_q     (reset at the start of every event with picks, :227)
 * and at the end of such an event (:294-334), at every point,
 *   if M_ap >= 1: N_ap += 1 and record N_ap gets (station, event, M_ap) for slot ap;
 *   for q in aq, bp, bq: if M_q >= 1: N_q += 1 and record N_ap (not N_q: the reference
 *   indexes all four record variables by N_ap) gets (station, event, M_q) for slot q,
 *   unless N_ap is still 0, where the reference's write is refused by the NetCDF library
 *   and nothing is stored.
 * A name longer than its record field (8 characters for stations, 20 for events) is
 * likewise refused by the library, so that slot keeps the name it had; the caller passes
 * tag 0 for such a name (and for an empty one).
 *
 * Arrays are Fortran order (first index fastest), npts points per volume; per-slot arrays
 * are (4, npts) with the slot slowest.  Sums equal the reference's single-precision values
 * bit for bit.
 */
#ifndef FWANT_KERINFO_H
#define FWANT_KERINFO_H

#include "fwant_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fwant_kerinfo fwant_kerinfo;

/* npts kernel points (the snapshot's I x J x K, SI_ker2info.F90:147-150) and the
 * thresholds kap0 kaq0 kbp0 kbq0 read from standard input (:118). */
fwant_status fwant_kerinfo_create(long long npts, const float thresholds[4], int device, fwant_kerinfo** out);
void fwant_kerinfo_destroy(fwant_kerinfo* k);
const char* fwant_kerinfo_last_error(fwant_kerinfo* k);

/* One pick (:268-289): the four kernel volumes in host memory, npts floats each. */
fwant_status fwant_kerinfo_add_pick(fwant_kerinfo* k, const float* const kernels[4]);

/* Closes an event that had picks (:294-334): the counts N and the records as above, then M
 * is reset.  station_tag and event_tag (>= 1) are the caller's names for KSTNM and KEVNM;
 * 0 stores no name (the slot keeps its earlier one). */
fwant_status fwant_kerinfo_end_event(fwant_kerinfo* k, int station_tag, int event_tag);

/* Number of records (the largest N_ap over the points). */
fwant_status fwant_kerinfo_records(fwant_kerinfo* k, int* nrec);

/* The sums S (4, npts) and the counts N (4, npts) (:344-353). */
fwant_status fwant_kerinfo_totals(fwant_kerinfo* k, float* sums, int* counts);

/* Record r (0 .. nrec-1, the reference's N index r + 1): M, station and event tags, each
 * (4, npts); 0 where nothing was stored. */
fwant_status fwant_kerinfo_record(fwant_kerinfo* k, int r, int* m, int* station, int* event);

/* device time (ms) of the kernels of the last fwant_kerinfo_add_pick */
fwant_status fwant_kerinfo_last_ms(fwant_kerinfo* k, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* FWANT_KERINFO_H */
