/*
 * fwant_gb300 — C ABI of the GB300 forward solver for FWANT (seis3d_wave).
 *
 * The reference solver is the Fortran program `seis3d_wave_mpi`
 * (code/srcF/seis3d_wave_8op_p3.F90).  It has no library API: its modules read
 * per-rank NetCDF inputs into module globals and run the time loop.  Each entry point
 * below replaces one of those import/run/export steps, named on its line as
 * file:line of the reference (paths relative to the reference project root).
 *
 * Conventions
 *  - Every call returns fwant_status; fwant_last_error() gives the message.  No
 *    call aborts the process (the reference stops or calls MPI_ABORT instead).
 *  - Arrays are plain host pointers.  Each call copies what it needs; the handle
 *    keeps no caller pointer after it returns.
 *  - 3-D arrays are Fortran-ordered (i fastest, then j, then k) and include the
 *    LenFD = 3 ghost cells on every side: nx = ni+6, ny = nj+6, nz = nk+6
 *    (code/srcF/mod_para.F90:79-82).  1-D coordinate and metric arrays have
 *    nx, ny or nz entries.
 *  - Grid indices (sources, receivers, snapshots) are the reference's 1-based
 *    Fortran indices including ghosts: the first interior point is 4.
 *  - Wavefield components are numbered in the receiver output order of
 *    io_seismo_put (code/srcF/mod_io.F90:461-497):
 *      0 Vx, 1 Vy, 2 Vz, 3 Txx, 4 Tyy, 5 Tzz, 6 Txy, 7 Txz, 8 Tyz.
 *  - One host thread per handle.  Handles are independent and may live on
 *    different devices.
 */
#ifndef FWANT_GB300_H
#define FWANT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fwant_status {
  FWANT_OK = 0,
  FWANT_ERR_INVALID_ARG = 1,
  FWANT_ERR_OOM = 2,
  FWANT_ERR_CUDA = 3,
  FWANT_ERR_NUMERIC_OVERFLOW = 4, /* macdrp_check found Inf/NaN/huge (mod_macdrp.F90:228-264) */
  FWANT_ERR_TIMEOUT = 5,
  FWANT_ERR_STATE = 6 /* call made in the wrong order (e.g. run before set_media) */
} fwant_status;

/* Storage kind of the wavefield registers (W and the RK registers m, t).  Arithmetic is
 * FP32 for all three; the PML memory variables and the medium stay FP32.  BF16/FP16 store
 * value * scale (fwant_set_storage_scale) and round to nearest even on every store.
 * FP64 is reserved: the solver rejects it (FWANT_ERR_INVALID_ARG); the double-precision
 * run used as the precision reference is the CPU restatement compiled for double. */
typedef enum fwant_storage {
  FWANT_STORAGE_FP32 = 0,
  FWANT_STORAGE_BF16 = 1,
  FWANT_STORAGE_FP16 = 2,
  FWANT_STORAGE_FP64 = 3
} fwant_storage;

/* Source time function ids of src_stf/src_svf (code/srcF/mod_src.F90:48-57). */
enum {
  FWANT_SVF_BELL = 100,
  FWANT_SVF_TRIANGLE = 110,
  FWANT_SVF_GAUSS = 120,
  FWANT_STF_RICKER = 200,
  FWANT_STF_GAUSS = 220,
  FWANT_STF_BELL = 230,
  FWANT_STF_STEP = 240,
  FWANT_STF_DELTA = 250
};

typedef struct fwant_config {
  int ni, nj, nk;      /* interior size: keys ni nj nk (code/srcF/mod_para.F90:75-77) */
  double stept;        /* time step in s: key stept (code/srcF/mod_para.F90:84) */
  int free_surface;    /* 1: top face k=nk2 is the traction-free surface (freenode) */
  int src_surface;     /* 1: forces on the surface act as traction (-DSrcSurface) */
  int storage;         /* fwant_storage */
  int device;          /* CUDA device ordinal */
  int exact_arith;     /* 1: the reference's FP32 operand order, IEEE division, no FMA
                          (reproduces an FP32 CPU run of the same expressions bit for bit);
                          0: fast form (FMA, precomputed reciprocals) */
} fwant_config;

/* One value of the source time function (which = 0: src_stf, the displacement/moment
 * history, code/srcF/mod_src.F90:464-487) or of its rate (which = 1: src_svf,
 * :438-463) at time t for window start t0 and frequency or rise time f0; ntime and stept
 * feed the delta function (:617-622).  These are the values the solver tabulates per RK
 * stage.  Host-only: needs no GPU.  FWANT_ERR_INVALID_ARG for an id the function does
 * not define (the reference stops there). */
fwant_status fwant_source_time_function(int which, int stf_id, float t, float t0, float f0, int ntime, float stept,
                                        float* out);


typedef struct fwant_solver fwant_solver;

/* Library version string. */
const char* fwant_version(void);

/* Allocate a solver: replaces para_init + macdrp_init
 * (code/srcF/mod_para.F90:70-88, code/srcF/mod_macdrp.F90:124-218). */
fwant_status fwant_create(const fwant_config* cfg, fwant_solver** out);

/* Release every device and host resource of the handle (macdrp_destroy,
 * code/srcF/mod_macdrp.F90:219-227).  Accepts NULL. */
void fwant_destroy(fwant_solver* s);

/* Message of the last failing call on this handle ("" if none). */
const char* fwant_last_error(const fwant_solver* s);

/* Coordinates x=theta (rad), y=phi (rad), z=r (m), nx/ny/nz entries including the
 * ghost cells: grid_coord_import (code/srcF/mod_grid.F90:85-94). */
fwant_status fwant_set_coord(fwant_solver* s, const float* x, const float* y, const float* z);

/* Metric arrays as stored in metric_mpi*.nc: grid_metric_import
 * (code/srcF/mod_grid.F90:95-114).  xsin, xcot, xi_x have nx entries; eta_y ny; zeta_z nz. */
fwant_status fwant_set_metric(fwant_solver* s, const float* xsin, const float* xcot,
                              const float* xi_x, const float* eta_y, const float* zeta_z);

/* Compute the metric from the coordinates on the device in FP64 and round to FP32:
 * replaces the seis3d_metric preprocessor (code/srcF/seis3d_metric.F90:83-112). */
fwant_status fwant_compute_metric(fwant_solver* s);

/* Terrain-following grid (the Gaussian-hill extension of the workload).  No counterpart in
 * the reference: its grid is orthogonal spherical with a flat top at k = nk2
 * (code/srcF/mod_grid.F90:36-38, code/srcF/seis3d_metric.F90:83-112, the radial term of
 * code/srcF/mod_macdrp.F90:928-957) and cannot represent topography.
 *
 * h: nx*ny heights in m (i fastest, ghosts included).  The radius becomes
 * r(i,j,k) = z(k) + h(i,j) s(k) with s(k) = (z(k) - z(1)) / (z(nk2) - z(1)), so the free
 * surface follows h and the bottom stays flat.  Every theta and phi derivative gains its
 * zeta part (metric terms zeta_theta, zeta_phi; zeta_r becomes three-dimensional), computed
 * in FP64 on the device.  On a sloping free surface the stress images are the traction
 * combination sigma . m (m the surface normal) and the velocity's zeta-derivatives solve the
 * traction condition sigma . m = T*Src; columns with zero slope run the reference's flat
 * formulas, so h = 0 reproduces the flat solver bit for bit.  Surface-force areas and
 * body-force cell volumes keep the flat grid's values; the cross-metric terms are not
 * damped by the PML, so the slopes must vanish inside the PML slabs.  Needs FP32 storage
 * (either arithmetic form); call after the coordinates and the metric (setting either again
 * recomputes the terrain metric).  A solver with topography steps alone (not in a batch). */
fwant_status fwant_set_topography(fwant_solver* s, const float* h);

/* The terrain metric as stored (FP32): which 0..3 give nx*ny*nz values (r, zeta_r,
 * zeta_theta / r, zeta_phi / (r sin theta)); 4 and 5 the surface normal's m1, m2 and 6..14
 * the row-major inverse of the traction condition, nx*ny values each (i fastest). */
fwant_status fwant_get_topography_array(fwant_solver* s, int which, float* out);

/* The metric of a grid without a solver: the seis3d_metric program
 * (code/srcF/seis3d_metric.F90:83-112; the fwant_prep program's metric stage) on the device in
 * FP64, rounded to FP32, the same values as fwant_compute_metric.  x[ni+6], y[nj+6], z[nk+6]
 * include the ghosts; xsin, xcot, xi_x have ni+6 entries, eta_y nj+6, zeta_z nk+6. */
fwant_status fwant_metric_arrays(int ni, int nj, int nk, const float* x, const float* y, const float* z,
                                 int device, float* xsin, float* xcot, float* xi_x, float* eta_y,
                                 float* zeta_z);

/* Copy the metric currently in use back to the host (same shapes as fwant_set_metric). */
fwant_status fwant_get_metric(fwant_solver* s, float* xsin, float* xcot, float* xi_x,
                              float* eta_y, float* zeta_z);

/* Lame parameters and density, (nx,ny,nz) each: media_import
 * (code/srcF/mod_media.F90:76-96). */
fwant_status fwant_set_media(fwant_solver* s, const float* lambda, const float* mu,
                             const float* rho);
/* fwant_set_media from arrays already in device memory on the solver's GPU (the same
 * (nx,ny,nz) Fortran-ordered float arrays), e.g. fwant_media_device_arrays of the medium
 * preprocessor: the medium goes from preprocessing to the solver without a round trip
 * through the host.  No counterpart in the reference (its stages exchange files). */
fwant_status fwant_set_media_device(fwant_solver* s, const float* d_lambda, const float* d_mu,
                                    const float* d_rho);

/* CFS-PML on the faces x1 x2 y1 y2 z1 z2 (6 entries each): keys abs_number,
 * abs_velocity, CFS_bmax, CFS_amax of abs_init (code/srcF/mod_abs_npml.F90:135-616).
 * number[f] <= 0 disables face f.  A PML on z2 turns the free surface off
 * (code/srcF/mod_abs_npml.F90:182-184).  Call after fwant_set_coord. */
fwant_status fwant_set_pml(fwant_solver* s, const int number[6], const float velocity[6],
                           const float bmax[6], const float amax[6]);

/* Force sources as stored in source_mpi*.nc: src_import (code/srcF/mod_src.F90:148-202).
 * indx, shift: 3 x num (column-major); start_time: num; stf_time, stf_freq: ntwin;
 * fx, fy, fz: ntwin x num (column-major); stf_id: one of the FWANT_STF_* ids. */
fwant_status fwant_set_forces(fwant_solver* s, int num, int ntwin, const int* indx,
                              const float* shift, const float* start_time,
                              const float* stf_time, const float* stf_freq, const float* fx,
                              const float* fy, const float* fz, int stf_id);

/* Moment-tensor sources: src_import (code/srcF/mod_src.F90:155-173).
 * mom holds Mxx Myy Mzz Mxy Mxz Myz, each ntwin x num, one after the other. */
fwant_status fwant_set_moments(fwant_solver* s, int num, int ntwin, const int* indx,
                               const float* shift, const float* start_time,
                               const float* stf_time, const float* stf_freq, const float* mom,
                               int stf_id);

/* Receivers at grid nodes, sampled every tinv steps: io_pt_import
 * (code/srcF/mod_io.F90:160-176); indx is 3 x num (1-based). */
fwant_status fwant_set_receivers(fwant_solver* s, int num, const int* indx, int tinv);

/* Advance nsteps time steps of the 8-step F/B LDDRK4 cycle
 * (code/srcF/seis3d_wave_8op_p3.F90:92-594).  Asynchronous device work is finished
 * before the call returns. */
fwant_status fwant_run(fwant_solver* s, int nsteps);

/* Number of steps the reference executes for a configured nt: the exit test runs only
 * at the start of each 8-step block (code/srcF/seis3d_wave_8op_p3.F90:92-95). */
int fwant_reference_steps(int nt);

/* Completed time steps (the reference's ntime). */
fwant_status fwant_get_ntime(fwant_solver* s, int* ntime);

/* Receiver seismograms recorded so far: out is [9][nsamp][num] (component, sample,
 * receiver), i.e. per component the (num_pt, time) layout of seismo_mpi*.nc
 * (code/srcF/mod_nfseis.F90:81-126).  Writes at most max_samples samples; *nsamp gets
 * the number written. */
fwant_status fwant_get_seismo(fwant_solver* s, float* out, int max_samples, int* nsamp);

/* Whole component including ghosts, (nx,ny,nz): the data of a restart file
 * (io_rest_export, code/srcF/mod_io.F90:342-405). */
fwant_status fwant_get_field(fwant_solver* s, int component, float* out);

/* Overwrite a component, (nx,ny,nz): io_rest_import (code/srcF/mod_io.F90:406-427).
 * Only the interior is taken; ghosts stay zero. */
fwant_status fwant_set_field(fwant_solver* s, int component, const float* in);

/* Checkpoint of the complete time-stepping state to a file: the wavefield, the CFS-PML
 * memory variables (which the reference's restart files leave out, so its restarts are
 * inexact inside the PML: io_rest_export, code/srcF/mod_io.F90:342-405), the step
 * counters, the recorded seismograms and SGT frames; with a checksum.  The model
 * (coordinates, metric, media, PML profile, sources, receivers) is not stored: load into a
 * solver set up with the same inputs (io_rest_import, code/srcF/mod_io.F90:406-427).
 * Loading checks the file (FWANT_ERR_INVALID_ARG: unreadable, truncated or corrupt) and
 * the configuration (FWANT_ERR_STATE: another grid, storage, PML, receiver or SGT setup);
 * a resumed run then gives the results of the uninterrupted run bit for bit. */
fwant_status fwant_save_checkpoint(fwant_solver* s, const char* path);
fwant_status fwant_load_checkpoint(fwant_solver* s, const char* path);

/* Strided sub-volume of the current wavefield: the data one frame of the vel_/sgt_
 * snapshot files holds (io_wave_export, code/srcF/mod_io.F90:505-645).  subs: first point
 * (1-based Fortran indices with ghosts; the interior starts at 4), subc: points per axis,
 * subt: stride per axis (snap_NNN subs/subc/subt, code/srcF/mod_io.F90:180-205; the
 * sub-volume must lie in the interior).  comps: ncomp component ids (0..8, receiver order;
 * the reference writes Vx Vy Vz or Txx Tyy Tzz Txy Txz Tyz).  out receives
 * [ncomp][subc[2]][subc[1]][subc[0]] floats, i fastest: per component the (I,J,K) layout of
 * one NetCDF snapshot frame (code/srcF/mod_nfseis.F90:131-203). */
fwant_status fwant_get_snapshot(fwant_solver* s, const int subs[3], const int subc[3], const int subt[3],
                                int ncomp, const int* comps, float* out);

/* fwant_get_snapshot without any device allocation.  No counterpart in the reference.
 *
 * For callers that must not allocate device memory at this point: monitoring or output
 * hooks that run in the middle of a long solve on a GPU whose memory is fully committed to
 * the wavefield registers (an allocation could fail with out-of-memory partway through a
 * run), and host programs that route every device allocation through their own budgeted
 * pool and forbid hidden library allocations.
 *
 * Same arguments and output as fwant_get_snapshot.  The values are staged in a fixed
 * device array of 4,194,304 floats (16 MiB) that the library holds on every GPU it is
 * loaded on until the process exits; a request for more values (ncomp * subc[0] *
 * subc[1] * subc[2]) is rejected with FWANT_ERR_INVALID_ARG, so large volumes are read in
 * pieces (e.g. k-ranges).  Every call looks up that array's device address, which
 * allocates nothing; the first call on a device may load the library's device code there,
 * so make it before any stream capture.  All calls on one device share the array:
 * each call overwrites every value it returns, but calls that overlap on the GPU (other
 * threads or handles on the same device) race with each other. */
fwant_status fwant_get_snapshot_noalloc(fwant_solver* s, const int subs[3], const int subc[3], const int subt[3],
                                        int ncomp, const int* comps, float* out);

/* Record the strain Green's tensor on the device: the six stresses (Txx Tyy Tzz Txy Txz
 * Tyz) of a strided sub-volume after every step whose counter is a multiple of tinv, i.e.
 * the frames of the sgt_ snapshot files (io_wave_export, code/srcF/mod_io.F90:505-560,
 * snap_NNN with a "T" variable list, :180-205), kept in device memory instead of files.
 * subs/subc/subt as in fwant_get_snapshot; frame f (0-based) is taken at ntime =
 * (f+1)*tinv; at most max_frames frames are kept.  Set before the first time step. */
fwant_status fwant_set_sgt_record(fwant_solver* s, const int subs[3], const int subc[3], const int subt[3], int tinv,
                                  int max_frames);

/* Recorded SGT frames: out is [6][nframes][subc[2]][subc[1]][subc[0]] (component, frame,
 * point with i fastest): per component the (I,J,K,time) layout of one sgt_ file variable.
 * Copies at most max_frames frames; *nframes gets the number copied. */
fwant_status fwant_get_sgt(fwant_solver* s, float* out, int max_frames, int* nframes);

/* ---- Sensitivity-kernel accumulation (code/srcF.kernel/SI_ker_sta.F90) ----
 * One fwant_sgtker holds one block of npts kernel points: the strain Green's tensors of
 * the receiver station's three force simulations (which = 0 X, 1 Y, 2 Z) and of the
 * source station (which = 3), each as knt frames of the six stresses
 * ([6][knt][npts], Txx Tyy Tzz Txy Txz Tyz), frame n at time n*kdt
 * (kdt = sub_gtinv*stept, SI_ker_sta.F90:274), and lambda, mu at the points.
 * Strains are formed in FP32 exactly as stress2strain (SI_ker_sta.F90:1185-1211); the
 * convolutions and window integrals accumulate in FP64 on the device. */
typedef struct fwant_sgtker fwant_sgtker;
fwant_status fwant_sgtker_create(long long npts, int knt, double kdt, int device, fwant_sgtker** out);
void fwant_sgtker_destroy(fwant_sgtker* k);
const char* fwant_sgtker_last_error(fwant_sgtker* k);
/* lambda, mu at the npts kernel points (the media file read with the block's
 * bsubs/bsubc/bsubt); mu must be > 0 everywhere (stress2strain divides by it). */
fwant_status fwant_sgtker_set_media(fwant_sgtker* k, const float* lam, const float* mu);
/* SGT of one simulation from host memory ([6][knt][npts] FP32 stresses). */
fwant_status fwant_sgtker_set_sgt(fwant_sgtker* k, int which, const float* stress);
/* SGT of one simulation from a solver's device record (fwant_set_sgt_record with npts
 * points and at least knt recorded frames; device-to-device copy of the first knt). */
fwant_status fwant_sgtker_take_sgt(fwant_sgtker* k, int which, fwant_solver* s);
/* sgt2scatter3 (SI_ker_sta.F90:1257-1337) for the force components in flags (bit 0 X,
 * bit 1 Y, bit 2 Z; the reference's flag_udx/y/z), outputs n = nt1..nt2 (1-based):
 *   x1(n) = dt sum_{m=1}^{n-1} tr E_R(m) tr E_S(n-m)
 *   x2(n) = dt sum_{m=1}^{n-1} E_R(m) : E_S(n-m)   (shear terms doubled)
 *   Ka(n) = x1 * 2 (lambda + 2 mu),  Kb(n) = (x2 - x1) * 4 mu
 * into the series slots of the reference's in-place outputs: X -> (0 Exx, 3 Exy),
 * Y -> (1 Eyy, 5 Eyz), Z -> (2 Ezz, 4 Exz).  Slots of components not computed hold 0. */
fwant_status fwant_sgtker_scatter(fwant_sgtker* k, int flags, int nt1, int nt2);
/* Kernel parameterisation of later fwant_sgtker_scatter calls: 0 (the default) the Vp/Vs
 * kernels above (SI_ker_sta.F90:1297-1298); 1 the lambda/mu kernels of SI_ker_sta_lamu
 * (SI_ker_sta_lamu.F90:1299-1300): Ka(n) = x1 * lambda, Kb(n) = 2 x2 * mu. */
fwant_status fwant_sgtker_set_param(fwant_sgtker* k, int param);
/* One series slot (0..5: Exx Eyy Ezz Exy Exz Eyz positions), [knt][npts] FP64. */
fwant_status fwant_sgtker_get_scatter(fwant_sgtker* k, int slot, double* out);
/* scatter2kernel (SI_ker_sta.F90:1375-1431) for component ncmp (1 X, 2 Y, 3 Z: the
 * reference's ncmp 1..3, no rotation): trapezoid integrals over frames nt1..nt2 of
 * V(n) Ka(n), U(n) Ka(n), V(n) Kb(n), U(n) Kb(n), each divided by the trapezoid integral
 * of V^2 (or U^2) times sgt_m0.  v, u: [knt] receiver velocity and displacement
 * (already filtered); outputs [npts] FP64: phase_Vp, amplitude_Vp, phase_Vs,
 * amplitude_Vs of the kernel file. */
fwant_status fwant_sgtker_kernel(fwant_sgtker* k, int ncmp, const float* v, const float* u, int nt1, int nt2,
                                 double sgt_m0, double* kap, double* kaq, double* kbp, double* kbq);
/* scatter_rotate + syn_rotate (SI_ker_sta.F90:1339-1373, used for the reference's ncmp 4-6):
 * replace the series of the three force components by their rotation, for Ka (slots 0 1 2)
 * and Kb (slots 3 5 4): new_c = sum_d old_d rot(d,c), rot column-major 3x3 (rot_mat).
 * Needs the scatter of all three components; rotate the synthetics the same way before
 * passing them to fwant_sgtker_kernel. */
fwant_status fwant_sgtker_rotate(fwant_sgtker* k, const double rot[9]);
/* fwant_sgtker_kernel with the pick's band filter applied first (SI_ker_sta.F90:756-773):
 * mode 0 none, 1 one-pass IIR (scatter_filter / syn_filter, zero padding in front), 2
 * zero-phase forward-backward IIR (scatter_filtfilt / syn_filtfilt, 3(nod1-1) samples
 * reflected about each end); b[nod1], a[nod1] the coefficients of the filter file
 * (nod1 <= 16).  The series are filtered on the device in FP64, V and U on the host. */
fwant_status fwant_sgtker_kernel_filtered(fwant_sgtker* k, int ncmp, const float* v, const float* u, int nt1,
                                          int nt2, double sgt_m0, int mode, int nod1, const double* b,
                                          const double* a, double* kap, double* kaq, double* kbp, double* kbq);
/* Kernel parameter conversion of the kernel-file programs, in place over the block's npts
 * points with the lambda, mu of fwant_sgtker_set_media (FP32, the reference's operand
 * order): kap/kbp the phase kernels of the two parameters, kaq/kbq the amplitude kernels.
 *   mode 1 lambda/mu -> kappa/mu  SI_ker_lamu2kamu (code/srcF.kernel/SI_ker_lamu2kamu.F90:823-830)
 *   mode 2 lambda/mu -> Vp/Vs     SI_ker_lamu2vpvs (code/srcF.kernel/SI_ker_lamu2vpvs.F90:823-830)
 *   mode 3 Vp/Vs -> kappa/mu      SI_ker_vpvs2kamu (code/srcF.kernel/SI_ker_vpvs2kamu.F90:823-831) */
fwant_status fwant_sgtker_convert(fwant_sgtker* k, int mode, float* kap, float* kaq, float* kbp, float* kbq);
/* SI_ker_pair (code/srcF.kernel/SI_ker_pair.F90), the single source-receiver pair: the
 * scattering series of the receiver SGT (fwant_sgtker_set_sgt slot 0) against the source
 * SGT (slot 3) over all knt frames, stress2strain and sgt2scatter (:710-780) in single
 * precision with every operation rounded in the reference's order (Sa = x1 2 (lam + 2 mu),
 * Sb = 2 (x2 - x1) 2 mu).  Replaces the series of fwant_sgtker_scatter. */
fwant_status fwant_sgtker_scatter_pair(fwant_sgtker* k);
/* The pair's window kernel (scatter2kernel :782-838, FP32) over frames nt1..nt2 (1-based)
 * with the synthetics v, u (knt values), after the pair program's filter of the band (mode
 * 0 none, 1 one pass, 2 forward-backward with zero padding, :840-932; nod1 coefficients b,
 * a in FP64) applied to the series and the synthetics; kap kaq kbp kbq receive npts
 * values each. */
fwant_status fwant_sgtker_kernel_pair(fwant_sgtker* k, const float* v, const float* u, int nt1, int nt2, float sgt_m0,
                                      int mode, int nod1, const double* b, const double* a, float* kap, float* kaq,
                                      float* kbp, float* kbq);
/* Device time of the last fwant_sgtker_scatter in milliseconds.  No counterpart in the
 * reference. */
fwant_status fwant_sgtker_last_scatter_ms(fwant_sgtker* k, double* ms);

/* Scale factors of 2-byte storage: velocities are stored as v * velocity_scale and stresses
 * as t * stress_scale, and divided back on every load, so that FP16's range (6.1e-5 to
 * 65504 normal) can be centred on the field's magnitudes.  Both must be powers of two
 * (scaling is then exact) and set before the first time step; default 1, 1.  Ignored
 * for FP32 storage.  No counterpart in the reference (it stores FP32 only). */
fwant_status fwant_set_storage_scale(fwant_solver* s, float velocity_scale, float stress_scale);

/* Largest |value| of each of the nine components over the whole register set, in receiver
 * order (Vx Vy Vz Txx Tyy Tzz Txy Txz Tyz), physical units; NaN propagates.  The reduction
 * macdrp_check (code/srcF/mod_macdrp.F90:228-264) makes, reported per component. */
fwant_status fwant_max_abs(fwant_solver* s, float out[9]);

/* Overflow check of the nine components: macdrp_check (code/srcF/mod_macdrp.F90:228-264).
 * Returns FWANT_ERR_NUMERIC_OVERFLOW when a value is NaN, Inf or >= huge(1.0). */
fwant_status fwant_check(fwant_solver* s);

/* Advance nsteps steps with one CUDA event pair around every launch (no graph) and
 * report the average device time of each of the four stage launches (stage_ms[4],
 * stage order inside the step) and of the step-end receiver/counter kernel.  Same
 * results as fwant_run; used for per-kernel timing. */
fwant_status fwant_profile_stages(fwant_solver* s, int nsteps, double* stage_ms, double* other_ms);

/* Device time of the last fwant_run call in milliseconds (CUDA events). */
fwant_status fwant_last_run_ms(fwant_solver* s, double* ms);

/* Planes along k that one CTA of the stage kernel marches through (default chosen from
 * the grid size; a tuning knob of the autotuner).  No counterpart in the reference. */
fwant_status fwant_set_planes_per_cta(fwant_solver* s, int planes);
fwant_status fwant_get_planes_per_cta(fwant_solver* s, int* planes);
/* Rows of the stage kernel's 32-column tile: 8 (the default; every storage and form) or 16
 * (FP32 storage without topography; 512-thread CTAs, one per SM).  Same results as the
 * default in the reference-order form; a tuning knob of the autotuners.  Batch members
 * must share it.  No counterpart in the reference. */
fwant_status fwant_set_tile_rows(fwant_solver* s, int rows);
fwant_status fwant_get_tile_rows(fwant_solver* s, int* rows);
/* Which RK stages split their work items into an interior-only launch and a full launch
 * (bit 0: stage 1, bit 1: stages 2 and 3, bit 2: stage 4; default 5, or 7 where the RK
 * stages run without t, fwant_set_rk_scheme); 0 runs every stage as one full launch.
 * No counterpart in the reference (a tuning knob of the stage kernel, set by
 * fwant_batch_autotune). */
fwant_status fwant_set_lean_stages(fwant_solver* s, int mask);
/* Deadline check of the stage kernel's bounded waits, without a fault: a one-thread kernel
 * waits on a barrier phase that nothing completes, gives up after `spins` polls (1 ..
 * 2^20) and reports through the solver's device error word, so the call returns
 * FWANT_ERR_TIMEOUT and the solver stays usable.  No counterpart in the reference. */
fwant_status fwant_check_wait_timeout(fwant_solver* s, int spins);
fwant_status fwant_get_lean_stages(fwant_solver* s, int* mask);
/* RK4 step form of the fast arithmetic: 1 (the default) runs stages 1-3 without the
 * accumulator t, which stage 3 then forms from the stage values, t = m + ((W2 - m) +
 * 2 (W3 - m) + a3 h3) / 3 (algebraically the reference's m + b1 h1 + b2 h2 + b3 h3,
 * mod_macdrp.F90:291-393;
 * the same results up to FP32 rounding, 129 instead of 156 floats moved per point and
 * step); 0 carries t as the reference does.  Applies to the fast form (every storage, flat
 * or terrain-following grid); the reference-order form always carries t
 * (fwant_get_rk_scheme then reads 0).  May change between steps.  No counterpart in the
 * reference. */
fwant_status fwant_set_rk_scheme(fwant_solver* s, int scheme);
fwant_status fwant_get_rk_scheme(fwant_solver* s, int* scheme);

/* Autotuner: times every tile shape (32 x 8, and 32 x 16 where fwant_set_tile_rows allows
 * it) with every planes-per-CTA candidate (4 ... 128, up to nk) over trial_steps eager
 * steps with CUDA events, keeps the fastest pair (fwant_get_tile_rows reads the shape) and
 * returns the planes in *planes (may be NULL).
 * Call before the first time step: the trial steps run from the initial state, which is
 * restored afterwards (wavefield, memory variables, receiver and SGT records).  Results
 * are cached per process by problem shape.  No counterpart in the reference. */
fwant_status fwant_autotune(fwant_solver* s, int trial_steps, int* planes);

/* ---- Batches: many simulations stepped together ----
 * No counterpart in the reference, which runs one virtual source per job.  A batch steps
 * n solvers (same device, storage and arithmetic form; sizes, media, sources and
 * receivers may all differ) in lockstep: each RK stage of up to 16 members is one launch
 * whose CTAs walk the work items (tiles x k-chunks) of every member, and whole 8-step
 * blocks replay a CUDA graph.  Results are those of fwant_run on each member: bit for bit
 * with exact_arith, to FP32 rounding in the fast form (multiply-add contraction may differ
 * between the batched and the single-simulation kernels).
 * Members must be at the same time step when fwant_batch_run is called and must not run
 * on their own while the batch runs; they stay usable on their own (fwant_get_seismo,
 * fwant_run, ...) between batch runs.  n <= 64; the batch does not own the solvers. */
typedef struct fwant_batch fwant_batch;
fwant_status fwant_batch_create(fwant_solver* const* sims, int n, fwant_batch** out);
void fwant_batch_destroy(fwant_batch* b);
const char* fwant_batch_last_error(fwant_batch* b);
/* CTAs per stage launch: 0 (default) = one CTA per work item; a smaller count makes the
 * launch persistent, each CTA walking items ctas apart. */
fwant_status fwant_batch_set_ctas(fwant_batch* b, int ctas);
fwant_status fwant_batch_run(fwant_batch* b, int nsteps);
fwant_status fwant_batch_last_run_ms(fwant_batch* b, double* ms);
/* Autotune the batch as it runs: one planes-per-CTA value for every member (4 ... 32,
 * timed on the batched launches), then the CTA schedule (one CTA per work item, or
 * persistent grids of 1, 2 or 4 CTAs per SM), then which stages split off an interior-only
 * launch; the chosen CTA count (0 = one per work item) goes to *ctas (may be NULL).
 * Before the first step; the members' states are restored. */
fwant_status fwant_batch_autotune(fwant_batch* b, int trial_steps, int* ctas);
/* fwant_profile_stages for a batch: eager steps with events around each stage's launches
 * (stage_ms[4]: all members' launches of that stage) and the step-end kernels. */
fwant_status fwant_batch_profile_stages(fwant_batch* b, int nsteps, double* stage_ms, double* other_ms);
/* Kernels one step of the batch launches (stage launches of the interior-only and full
 * forms, step-end kernels), as counted by the last step enqueued; 0 before the first. */
fwant_status fwant_batch_launches_per_step(fwant_batch* b, int* n);

#ifdef __cplusplus
}
#endif

#endif /* FWANT_GB300_H */
