/*
 * ekgpu.h -- C ABI of the GB300 RK3 duct substep (RK_DUCT + REM_DIV_CURV).
 *
 * Drop-in boundary for the Fortran driver of ekman_bl.  The reference path
 * has no argument lists: RK_DUCT (src/duct.F90:237-2469) and REM_DIV_CURV
 * (src/duct.F90:2472-2818) read and write module globals declared in
 * src/modules.F90:95-316.  Each entry point below replaces one of those
 * subroutine calls plus the module state it touches; the comment on each
 * declaration names the reference routine (file:line).  Plain C types only:
 * every array is a host pointer in the reference's own Fortran layout
 * (column-major, first index fastest, complex*16 stored as interleaved
 * (re,im) doubles), so a Fortran caller passes its module arrays through
 * ISO_C_BINDING with no copy or transpose.
 *
 * Layouts (NX, NY, NZ as in grid_def; one MPI rank, so NXP = NX+1,
 * NX2P = NX/2, NZV = NZ+2):
 *   spectral field  CU1X(0:NX/2, 0:NZ+1, 0:NY+1) complex*16  -> 2*(NX/2+1)*(NZ+2)*(NY+2) doubles
 *   physical field  U1X (0:NX+1, 0:NZ+1, 0:NY+1) real*8      -> (NX+2)*(NZ+2)*(NY+2) doubles
 *   2-D metric      INT_JACOB(0:NZ+2, 0:NY+2)                 -> (NZ+3)*(NY+3) doubles
 *   face metric     GMAT_11(0:NZ+2, 0:NY+2, 2)                -> 2*(NZ+3)*(NY+3) doubles
 *   grid points     xpoint(0:NZ+1, 0:NY+1)                    -> (NZ+2)*(NY+2) doubles
 *
 * Ownership: the caller owns every host buffer and the library only reads or
 * writes it during the call.  The library owns device memory, which stays
 * resident between calls (state never leaves HBM between substeps).
 * Errors: every entry point returns an ek_status; none calls exit().  A
 * failed call leaves a message readable through ekgpu_last_error().
 * Threading: one context per host thread; calls on one context are
 * serialised on the context's stream.
 */
#ifndef EKGPU_H
#define EKGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ek_status {
  EK_OK = 0,
  EK_ERR_ARG = 1,            /* bad or unsupported argument                     */
  EK_ERR_CUDA = 2,           /* a CUDA call failed                              */
  EK_ERR_NOT_CONVERGED = 3,  /* multigrid hit its cycle cap; phi still returned */
  EK_ERR_NAN = 4,            /* divergence is NaN (reference: STOP 'DIV is a NaN', duct.F90:2811) */
  EK_ERR_TIMEOUT = 5,        /* a tensor-core convolution of the U-Net gave up its
                                bounded wait for its MMAs (ekgpu_unet_forward,
                                _train_step, _gradient); no other kernel waits  */
  EK_ERR_STATE = 6,          /* call order violated (e.g. step before metrics)  */
  EK_ERR_IO = 7,             /* restart file missing, unreadable or malformed  */
  EK_ERR_DT = 8              /* DELTA_T below 1.0E-4 after a projection (reference:
                                STOP 'DELTA_T is zero', duct.F90:2812; the bound is
                                the REAL*4 literal, 9.99999974737875e-05).  The
                                substep is complete; its CP update, which the
                                reference would not reach, is included.        */
} ek_status;

/* Boundary-wall index into the *_bc arrays, in input.dat order
 * (diablo.F90:260-284): LOWER=YMIN, UPPER=YMAX, LEFT=ZMIN, RIGHT=ZMAX. */
enum { EK_YMIN = 0, EK_YMAX = 1, EK_ZMIN = 2, EK_ZMAX = 3 };

/* Multigrid stopping rule. */
enum {
  EK_MG_STOP_RELCHANGE = 0,  /* MUDPACK rule: max|phi_k - phi_{k-1}| / max|phi_k| <= tol (mud2cr.f:301-326) */
  EK_MG_STOP_RESIDUAL = 1    /* ||b - A phi||_2 / ||b||_2 <= tol, per real 2-D problem.  A problem with
                                kx^2 = 0 (singular: periodic x, Neumann y, A 1 = 0) is made well
                                posed first -- not a reference behaviour, whose MUDPACK iterate for
                                that mode is whatever 6 cycles leave: b loses its component along the
                                left null vector z of the operator (A^T z = 0, computed once per
                                metric set), b' = b - (z.b / z.z) z, the tolerance applies to
                                ||b' - A phi|| / ||b'||, and phi is shifted to zero mean over the
                                (NZ+2)(NY+2) points.  The part z.b of the divergence is the one no
                                pressure can remove; it stays in the divergence check.             */
};

/* Run parameters: the values the Fortran driver reads from input.dat and
 * grid_def (diablo.F90:242-337, grid_def:7-50).  Fill with
 * ekgpu_default_params() and override. */
typedef struct ek_params {
  int nx, ny, nz;            /* NX (spanwise, Fourier), NY, NZ interior counts          */
  double lx;                 /* LX, spanwise period: KX(i) = 2*pi*i/LX                 */
  double nu;                 /* NU                                                      */
  double delta_t;            /* DELTA_T; with variable_dt = 1 COURANT_CURV_MPI resets it
                                (read it back with ekgpu_get_time)                      */
  double f0;                 /* F_0, Coriolis parameter                                 */
  double wbulk0;             /* WBULK0 (geostrophic wind of the Coriolis term)          */
  int f_type;                /* F_TYPE: 1 constant PX0, 2 oscillatory                   */
  double px0, omega0, amp_omega0, time;  /* mean-pressure forcing (duct.F90:411-455)  */
  int n_th;                  /* N_TH: 0 or 1 scalar                                     */
  double pr;                 /* PR(1)                                                   */
  double ri_tau;             /* RI_TAU(1) (buoyancy coefficient)                        */
  int cont_strat;            /* CONTINUOUS stratification flag CONT_STRAT               */
  int ic_type;               /* IC_TYPE (only 7, the shipped value, is supported)       */
  int u_bc[4], v_bc[4], w_bc[4], th_bc[4];            /* BC codes per wall            */
  double u_bc_c1[4], v_bc_c1[4], w_bc_c1[4], th_bc_c1[4]; /* BC constants *_C1      */
  int mudpack_bc[4];         /* MUDPACK_BC nxa,nxb,nyc,nyd (only 0 0 2 2 supported)    */
  int mg_ixp, mg_jyq, mg_iex, mg_jey; /* grid_def iixp,jjyq,iiex,jjey; 0 = choose    */
  int mg_maxcy;              /* maxcy (reference 6)                                     */
  int mg_kcycle;             /* mgopt(1): 1 V, 2 W (reference 2)                        */
  int mg_iprer, mg_ipost;    /* mgopt(2),(3) (reference 2,1)                            */
  int mg_intpol;             /* mgopt(4): 1 linear, 3 cubic (reference 3)               */
  int mg_stop;               /* EK_MG_STOP_*                                            */
  double mg_tol;             /* tolmax: reference REAL*4 10.0**(-6) widened to REAL*8   */
  int quirk_phi_fp32;        /* Q1: CMPLX(P_TMP2,P_TMP) rounds phi to REAL*4 (duct.F90:2664) */
  int mg_fast;               /* 0: MUDPACK's own iteration (FP64, point smoother, the parity
                                default); 1: mixed precision -- float-float residual and update
                                around FP32 V-cycles with an alternating-direction line smoother,
                                same discrete operator, needs mg_stop = EK_MG_STOP_RESIDUAL;
                                mg_maxcy caps the corrections                                   */
  int sponge_type;           /* SPONGE_TYPE: 0 none, 1 parabolic, 2 exponential profiles;
                                sponge_th (duct.F90:3196-3362) runs when != 0 and N_TH >= 1 */
  int les;                   /* LES: dynamic-Smagorinsky subgrid terms of les_chan /
                                les_chan_th (les_chan.F90, les_chan_th.F90) in every substep
                                with TIME_STEP > 1 or create_new_flow = 0; needs
                                ekgpu_set_les_metrics                                   */
  int ny_s_t, nz_s_r, nz_s_l;/* grid_def NY_S_T, NZ_S_R, NZ_S_L: sponge extents         */
  int save_stats_int;        /* SAVE_STATS_INT (input.dat); sponge_th zeroes mode 0 of CU2X
                                when MOD(2*TIME_STEP, SAVE_STATS_INT) = 0 in its stratified,
                                z-periodic branch                                        */
  int time_step;             /* TIME_STEP of the step being taken; ekgpu_step adds 1 before
                                each step, as the driver's DO TIME_STEP loop does        */
  int variable_dt;           /* VARIABLE_DT: COURANT_CURV_MPI (duct.F90:3605-3674) after the
                                RK_STEP = 3 ADI when MOD(TIME_STEP, UPDATE_DT) = 0       */
  int update_dt;             /* UPDATE_DT                                               */
  double cfl;                /* CFL                                                     */
  double delta_t_set;        /* DELTA_T_SET: the cap of the CFL time step               */
  int fft_fp32;              /* x-transforms in FP32 arithmetic (fields stay FP64): 0 none,
                                1 the nonlinear product/flux transforms and the explicit
                                increment S = R - J phi_old that the ADI starts from (CR then
                                holds CR - J CU), 2 every transform */
  int ff_arith;              /* 1: the x-transforms fft_fp32 leaves in FP64 use float-float
                                arithmetic (~48 bits) on the FP32 pipe; with fft_fp32 = 1
                                (and no LES in the substep) the physical fields are then
                                float-float planes and the ADI runs in float-float too.
                                2 (fft_fp32 = 1): the state's inverse transforms and the ADI
                                run in FP32 on increments -- each sweep solves for the
                                change of its field, whose FP32 forward transform is added
                                to the FP64 spectral state (LES substeps as with 1).
                                The spectral fields stay FP64 in every mode.              */
  int les_model_type;        /* LES_MODEL_TYPE: only 2 (dynamic Smagorinsky, C_DYN from the
                                test filter every 5 steps) is supported                   */
  int les_model_type_th;     /* LES_MODEL_TYPE_TH: only 1 (KAPPA_T = NU_T/PR) is supported */
  int create_new_flow;       /* CREATE_NEW_FLOW (input.dat): 1 leaves the subgrid terms out of
                                the run's first step (TIME_STEP = 1)                     */
} ek_params;

/* Geometry and background fields of JACOBI_TRANS (diablo.F90:1088-1570);
 * host pointers in the layouts listed at the top of this file. */
typedef struct ek_metrics {
  const double *int_jacob;                  /* INT_JACOB(0:NZ+2,0:NY+2)       */
  const double *gmat_11, *gmat_12, *gmat_22; /* GMAT_**(0:NZ+2,0:NY+2,2)      */
  const double *cjob_11, *cjob_12, *cjob_21, *cjob_22; /* CJOB_**(...,2)     */
  const double *th_bar;                      /* TH_BAR(0:NZ+2,0:NY+2), may be NULL when n_th == 0 */
} ek_metrics;

/* Per-call multigrid report. */
typedef struct ek_mg_stats {
  int nprob;                 /* real 2-D problems solved                         */
  int min_cycles, max_cycles;/* cycles after FMG (mg_fast: FP32 corrections), over
                                problems; with mg_fast over the kx^2 != 0 problems
                                when there are any                              */
  int n_not_converged;       /* problems that hit maxcy                          */
  double max_relchange;      /* largest final relmax                             */
  double max_residual;       /* largest final ||b-A phi||/||b|| (residual rule)  */
} ek_mg_stats;

/* Plane statistics of SAVE_STATS_CURVI (flow_statistics.F90:2-1023).  Every
 * plane is a caller-owned (0:NZ+1, 0:NY+1) array, (NZ+2)*(NY+2) doubles in
 * the layout of the reference's URMS, UV, ... (K fastest); a NULL plane is
 * not copied.  Sums over x run over I = 0..NX-1; fluctuations are taken
 * about DBLE(C*X(0,K,J)), the x-mean.  Planes the reference leaves
 * unassigned (fresh allocations) are zero. */
typedef struct ek_stats {
  double ubulk, vbulk;       /* UBULK, VBULK: cell averages of mode-0 CU3X, CU1X (:80-95)    */
  double thbulk;             /* the scalar's cell average, printed as THBULK (:540-555)       */
  double urms_b, vrms_b, wrms_b; /* INT_JACOB-weighted cell averages of URMS.. (:851-879)   */
  double u3_probe, u1_probe; /* U3X(NXP,2,NY), U1X(NXP,2,NY) of the time_bulk.txt line (:403) */
  double *urms, *vrms, *wrms;          /* SQRT(SUM (u - <u>)**2 / NX), all K, J            */
  double *uv, *uw, *wv, *pu, *pv;      /* SUM u'v' / NX etc. on K = 1..NZ (:181-207);
                                          pu = <w'p'>, pv = <v'p'>, p' about P_MEAN      */
  double *tke;                         /* TKE: squared mode-0 velocities (:165-174)      */
  double *dudy, *dwdy, *dudz, *dwdz, *omega_x; /* mode-0 gradients (:216-325)            */
  double *thrms, *thv, *thw;           /* scalar rms and fluxes (n_th >= 1; :456-503)    */
  double *dthdy, *dthdz, *rig;         /* scalar gradients, gradient Richardson number   */
  double *mean_u1, *mean_u2, *mean_u3, *mean_p, *mean_th; /* DBLE(C*X(0,K,J)) after the
                                          transforms back, as plot_binary writes them   */
} ek_stats;

/* Field selectors for ekgpu_get_field / ekgpu_put_field. */
enum {
  EK_F_CU1 = 0, EK_F_CU2, EK_F_CU3, EK_F_CP, EK_F_CTH,   /* state (spectral)   */
  EK_F_CF1, EK_F_CF2, EK_F_CF3, EK_F_CFTH,              /* RK explicit terms  */
  EK_F_CR1,                                              /* phi after REM_DIV  */
  EK_F_NFIELDS
};

typedef struct ek_ctx ek_ctx;

/* Fill *p with the shipped rundir_unst/input.dat choices that the path
 * supports (input.dat:1-62), sizes from the caller. */
int ekgpu_default_params(ek_params *p);

/* Allocate a context and its device state.  Replaces allocate_var
 * (ALLOCATION.F90:1-217), INIT_FFT (diablo.F90:563, source missing from the
 * reference tree), the RKW3 constants (diablo.F90:568-576) and INIT_DUCT
 * (duct.F90:7-232).  Unsupported options give EK_ERR_ARG. */
int ekgpu_create(const ek_params *p, ek_ctx **ctx);

/* Free the context and its device memory. */
void ekgpu_destroy(ek_ctx *ctx);

/* Text of the last error on this context (never NULL).  With ctx == NULL:
 * the last error of a context-free call (ekgpu_fft_*) on this host thread. */
const char *ekgpu_last_error(const ek_ctx *ctx);

/* Bind the context to an existing CUDA stream (cudaStream_t passed as a
 * pointer; NULL returns to the context's own stream). */
int ekgpu_set_stream(ek_ctx *ctx, void *stream);

/* Upload the metric arrays built by JACOBI_TRANS (diablo.F90:1088-1570). */
int ekgpu_set_metrics(ek_ctx *ctx, const ek_metrics *m);

/* Host helper: JACOBI_TRANS restated (diablo.F90:1088-1570) from grid
 * points xpoint/ypoint(0:NZ+1,0:NY+1).  Writes the metric arrays into the
 * caller's buffers (sizes as in the layout table); th_bar gets the
 * CONT_STRAT profile -ypoint+ypoint(0,NY+1) when cont_strat != 0. */
int ekgpu_metrics_from_grid(const ek_params *p, const double *xpoint,
                            const double *ypoint, double *int_jacob,
                            double *gmat_11, double *gmat_12, double *gmat_22,
                            double *cjob_11, double *cjob_12, double *cjob_21,
                            double *cjob_22, double *th_bar);

/* Host helper: the sponge profiles of diablo.F90:1489-1556 from the grid
 * points: SPONGE_SIGMA(0:NY+1) (vertical, from NY_S_T up) and
 * SPONGE_SIGMA_OUT(0:NZ+1) (streamwise, K >= NZ_S_R and K <= NZ_S_L when
 * NZ_S_R < NZ+1), parabolic (SPONGE_TYPE 1) or exponential (2); zero for 0. */
int ekgpu_sponge_profiles(const ek_params *p, const double *xpoint, const double *ypoint,
                          double *sponge_sigma, double *sponge_sigma_out);

/* LES (ek_params.les = 1; les_chan.F90 with LES_MODEL_TYPE 2 and
 * les_chan_th.F90 with LES_MODEL_TYPE_TH 1, called from RK_DUCT at
 * duct.F90:641-654).
 * ekgpu_les_metrics_from_grid: host helper, the GMAT_*_y / GMAT_*_z arrays
 *   of JACOBI_TRANS's LES branch (diablo.F90:1379-1467) from the grid
 *   points, each (0:NZ+2,0:NY+2,2) like GMAT_11.
 * ekgpu_set_les_metrics: upload them (replaces allocation_les_var's arrays
 *   filled by JACOBI_TRANS); needed before the first substep with LES.
 * ekgpu_les_set_first_time: set FIRST_TIME (diablo.F90:88,157), which makes
 *   every substep recompute C_DYN.  It is 1 after ekgpu_create and after
 *   ekgpu_read_flow, and ekgpu_step clears it after each step; a driver that
 *   calls ekgpu_rk_substep itself clears it after its first step.
 * ekgpu_les_get: copy NU_T (physical layout) and C_DYN ((0:NZ+1,0:NY+1),
 *   (NZ+2)*(NY+2) doubles) out; either pointer may be NULL.
 * The subgrid terms act in every substep with TIME_STEP > 1, or in every
 * substep when create_new_flow = 0 (the IF of duct.F90:641).  NU_T and C_DYN
 * start at zero (diablo.F90:541-557). */
int ekgpu_les_metrics_from_grid(const ek_params *p, const double *xpoint, const double *ypoint,
                                double *gmat_11_y, double *gmat_12_y, double *gmat_22_y,
                                double *gmat_11_z, double *gmat_12_z, double *gmat_22_z);
int ekgpu_set_les_metrics(ek_ctx *ctx, const double *gmat_11_y, const double *gmat_12_y,
                          const double *gmat_22_y, const double *gmat_11_z, const double *gmat_12_z,
                          const double *gmat_22_z);
int ekgpu_les_set_first_time(ek_ctx *ctx, int first_time);
int ekgpu_les_get(ek_ctx *ctx, double *nu_t, double *c_dyn);

/* Upload SPONGE_SIGMA(0:NY+1) and SPONGE_SIGMA_OUT(0:NZ+1) (the module arrays
 * that sponge_th reads).  Both default to zero. */
int ekgpu_set_sponge(ek_ctx *ctx, const double *sponge_sigma, const double *sponge_sigma_out);

/* Set TIME and TIME_STEP for the next substep (a driver that calls
 * ekgpu_rk_substep itself keeps them in step with its own loop). */
int ekgpu_set_time(ek_ctx *ctx, double time, int time_step);

/* Read TIME, TIME_STEP and DELTA_T back (DELTA_T changes when VARIABLE_DT
 * runs COURANT_CURV_MPI). */
int ekgpu_get_time(ek_ctx *ctx, double *time, int *time_step, double *delta_t);

/* Copy the Fourier-space state CU1X, CU2X, CU3X, CPX, CTHX in (upload) or
 * out (download).  Replaces READ_FLOW's fill of the module arrays
 * (diablo.F90:918-1072) and SAVE_FLOW's read of them (diablo.F90:753-837).
 * cth may be NULL when n_th == 0.  Upload also zeroes CF*. */
int ekgpu_upload_state(ek_ctx *ctx, const double *cu1, const double *cu2,
                       const double *cu3, const double *cp, const double *cth);
int ekgpu_download_state(ek_ctx *ctx, double *cu1, double *cu2, double *cu3,
                         double *cp, double *cth);

/* Restart files.  ekgpu_save_flow replaces the file writes of SAVE_FLOW
 * (diablo.F90:753-837) and BACKUP_FLOW (diablo.F90:841-915); ekgpu_read_flow
 * the reads of READ_FLOW (diablo.F90:918-1072).  The caller composes the
 * file names (the reference's last_saved/diablo_001.saved, .res, backup/
 * diablo_001.saved_mmmm, diablo_th01_001.*), so the Fortran routines keep
 * their naming and directory logic and pass FNAME and FNAME_TH(N).
 *
 * Format: Fortran unformatted sequential, 4-byte record markers in host byte
 * order, records over 2^31 - 9 bytes split into subrecords (the ifort and
 * gfortran convention).  flow_path gets the records
 * [NX NY NZ TIME TIME_STEP] and [CU1X CU2X CU3X CPX]; th_path (may be NULL,
 * no scalar file) gets [NX NY NZ TIME TIME_STEP] and [CTHX(:,:,:,1)].  The
 * data stream from HBM through pinned staging with no full host copy.
 * The environment variable EKGPU_FORTRAN_SUBRECORD=<bytes> lowers the
 * subrecord limit (to exercise the split on small files).
 *
 * Read: flow_path's dimensions must equal the context's (reference: STOP
 * 'Error: old flowfield wrong dimensions.'; here EK_ERR_IO and the state is
 * unchanged); th_path NULL skips the scalar (NUM_READ_TH = 0), and is an
 * error when n_th == 0.  Both files are checked (markers, lengths,
 * dimensions) before device memory is written, so on any error the state is
 * left as it was.  TIME and TIME_STEP are taken from the last header read,
 * CF* are zeroed as by ekgpu_upload_state; IC_TYPE = 7 applies no boundary
 * conditions after the read (diablo.F90:1062-1069). */
int ekgpu_save_flow(ek_ctx *ctx, const char *flow_path, const char *th_path);
int ekgpu_read_flow(ek_ctx *ctx, const char *flow_path, const char *th_path);

/* SAVE_STATS_CURVI (flow_statistics.F90:2-1023) on the resident state:
 * fills *stats and, as the reference routine does, transforms CU1X, CU2X,
 * CU3X, CPX, CTHX to physical space and back (which zeroes modes above
 * NX/3) and zeroes CF1X, CF2X, CF3X (:956-963).  The file output
 * (plane_data/time_bulk.txt, plot_binary's .pln record) is the caller's;
 * the TKE budget, the plane dumps and the Tecplot writer are not part of it. */
int ekgpu_save_stats(ek_ctx *ctx, ek_stats *stats);

/* ---- Tile-shape autotuner of the mixed solver's line solves ----------------
 * (No counterpart in the reference.)  For every multigrid level l = 2..ngrid
 * above the coarse levels that run as one launch (ekgpu_mg_tail_levels)
 * and both line directions, time one zebra sweep in each valid layout -- 8,
 * 16 or 32 problems per block, line segments of 8 or 4 rows -- `reps` times
 * on the context's own work arrays, and use the fastest from then on.  Each
 * problem's arithmetic does not depend on the problems per block; the
 * segment length changes the order of the line elimination (results agree
 * to the solve tolerance, not bit for bit).  report (may be NULL) receives
 * the timings as JSON text.  Needs mg_fast = 1 and metrics. */
int ekgpu_mg_autotune(ek_ctx *ctx, int reps, char *report, int report_len);
/* Set one layout by hand (0 restores the default: lanes by line length,
 * seg 8; dir 0 y-lines, 1 x-lines), e.g. to replay a table tuned earlier. */
int ekgpu_mg_set_layout(ek_ctx *ctx, int level, int dir, int lanes, int seg);
/* The multigrid levels: ngrid and the sizes nx[l-1] x ny[l-1], l = 1..ngrid. */
int ekgpu_mg_levels(ek_ctx *ctx, int *ngrid, int *nx, int *ny, int cap);
/* The mixed solver runs its coarse levels 1..ltop as one launch per cycle,
 * each problem's levels in shared memory (ltop = 0: none).  Those levels have
 * no line-solve launches, so the autotuner times levels max(2, ltop+1)..ngrid
 * only and their layouts are not used. */
int ekgpu_mg_tail_levels(ek_ctx *ctx, int *ltop);

/* ---- Learned initial guess of the per-kx Poisson problems -------------------
 * (No counterpart in the reference: its solves always start from zero.)
 *
 * A U-Net (4 levels of two 3x3 convolutions + ReLU, `channels` channels at
 * every level, 2x2 average pooling, nearest upsampling, skip connections,
 * a final 3x3 convolution to one channel) with BF16 tensor-core kernels and
 * FP32 accumulation, trained on the GPU with Adam.  Images are h x w
 * (multiples of 8), cin input channels, FP32 NHWC on the device.  Parameter
 * layout: for each of the 15 convolutions in network order (encoder levels
 * 0..3, decoder levels 2, 1, 0, output), W[cout][9][cin] then b[cout]
 * (tap = 3*(dy+1) + (dx+1)).  The multigrid stays the solver and the judge
 * of convergence: the guess only sets the starting iterate, scaled by the
 * least-squares factor, and the tolerance is unchanged. */
typedef struct ek_unet ek_unet;
int ekgpu_unet_create(int cin, int channels, int max_batch, int h, int w, ek_unet **net);
void ekgpu_unet_destroy(ek_unet *net);
const char *ekgpu_unet_last_error(const ek_unet *net);
long ekgpu_unet_num_params(const ek_unet *net);
int ekgpu_unet_set_params(ek_unet *net, const float *params);   /* host; resets Adam */
int ekgpu_unet_get_params(ek_unet *net, float *params);         /* host               */
/* y[n][h][w] = net(x[n][h][w][cin]); device pointers; stream may be NULL */
int ekgpu_unet_forward(ek_unet *net, const float *x_dev, int n, float *y_dev, void *stream);
/* Forward convolutions with cin and cout multiples of 16 run on the tcgen05
 * tensor-core kernel (on by default); 0 puts every layer on the mma.sync
 * kernel.  No counterpart in the reference (method tuning). */
int ekgpu_unet_set_tcgen05(ek_unet *net, int on);
/* one Adam step (beta 0.9/0.999, eps 1e-8) on the mean-square error against
 * t[n][h][w] over the top-left hv x wv pixels of each image */
int ekgpu_unet_train_step(ek_unet *net, const float *x_dev, const float *t_dev, int n, int hv, int wv,
                          double lr, double *loss, void *stream);
/* forward and backward without an update: loss, prediction (y_dev may be
 * NULL) and the parameter gradient copied to grad_host (may be NULL) */
int ekgpu_unet_gradient(ek_unet *net, const float *x_dev, const float *t_dev, int n, int hv, int wv,
                        double *loss, float *y_dev, float *grad_host, void *stream);
/* Image geometry of the guess at averaging factor f: the finest multigrid
 * grid (NZ+2 across, NY+2 down) averaged over f x f blocks is hv x wv,
 * padded to h x w. */
int ekgpu_guess_geometry(ek_ctx *ctx, int factor, int *h, int *w, int *hv, int *wv);
/* Use net (cin = 2: scaled right-hand side, log(1 + kx^2 J)/8) as the
 * starting iterate of the kx^2 != 0 problems (mg_fast = 1); NULL turns it off.
 * The caller keeps the network alive while it is set. */
int ekgpu_set_poisson_guess(ek_ctx *ctx, ek_unet *net, int factor);
/* After each projection solve, append (input [h][w][2], target [h][w]) pairs
 * of the kx^2 != 0 problems to the caller's device buffers, at most capacity
 * pairs; NULL pointers stop collecting. */
int ekgpu_set_pair_sink(ek_ctx *ctx, float *x_dev, float *t_dev, int capacity, int factor);
int ekgpu_pair_count(ek_ctx *ctx, int *count);
/* Last mixed solve: mean of |b - A g|/|b| after the scaled guess (1 without
 * a guess) and mean number of corrections, over the kx^2 != 0 problems. */
int ekgpu_last_guess_stats(ek_ctx *ctx, double *mean_rho, double *mean_cycles);

/* Read or write one spectral field (EK_F_*) in the CU1X layout. */
int ekgpu_get_field(ek_ctx *ctx, int field, double *out);
int ekgpu_put_field(ek_ctx *ctx, int field, const double *in);

/* One RK substep rk_step in {1,2,3}: RK_DUCT (duct.F90:237-2469) including
 * REM_DIV_CURV and the pressure update (duct.F90:2455-2466).  Under
 * EK_MG_STOP_RESIDUAL, EK_ERR_NOT_CONVERGED when a projection problem reached
 * mg_maxcy above the tolerance: the substep is complete and its state valid.
 * Under EK_MG_STOP_RELCHANGE such problems are counted (ekgpu_last_mg_stats,
 * ekgpu_mg_counters) but the call returns EK_OK, as MULTIGRID_MUDPACK ignores
 * mud2cr's ierror (mg_solver2d.F90:195-199). */
int ekgpu_rk_substep(ek_ctx *ctx, int rk_step);

/* nsteps full RK3 steps: the driver loop DO RK_STEP=1,3; CALL RK_DUCT
 * (diablo.F90:152-154), repeated; advances params.time by DELTA_T per step.
 * A substep that returns EK_ERR_NOT_CONVERGED does not stop the loop; the
 * call returns it after the last step. */
int ekgpu_step(ek_ctx *ctx, int nsteps);

/* Whether ekgpu_step may run each RK3 step as one CUDA graph (default on).
 * No counterpart in the reference.  The graph path applies with mg_fast = 1,
 * a fixed time step, F_TYPE = 1, no learned guess or pair collection and the
 * per-kernel timer off; the first step after ekgpu_set_metrics, the autotuner
 * or a layout change runs eagerly, later steps replay a graph captured once
 * per variant (LES on/off, FIRST_TIME, C_DYN due, sponge reset), in which the
 * mixed solver's correction cycles repeat in conditional while-nodes until
 * its device-side check stops them.  Results are the same either way; the
 * statistics and the divergence check are read once per step instead of
 * once per substep. */
int ekgpu_set_step_graph(ek_ctx *ctx, int on);

/* An ensemble of independent runs, each with its own sizes, parameters and
 * metrics (one context per member), advanced by nsteps RK3 steps together
 * on one GPU.  The reference runs each member as its own MPI job.  Here,
 * when every member takes ekgpu_step's graph path and has stepped once
 * since its plan was set, each ensemble step is one CUDA graph launch on
 * member 0's stream (ordered after the work queued on every member's
 * stream): every member's three substeps form a branch of that graph, so
 * the members' kernels run side by side.  Otherwise every member steps on
 * its own stream, from its own host thread, so the members' kernels share
 * the GPU and one member's host waits overlap the others' work.  Results
 * are the same either way.  status[m] (optional, n entries)
 * receives member m's ekgpu_step result; the call returns EK_OK when every
 * member succeeded, else the first failing member's code (its message stays
 * in that member's ekgpu_last_error).  A member that fails leaves the others
 * running.  EK_ERR_ARG (no member touched) for n < 1, nsteps < 0, a null
 * member or the same context twice. */
int ekgpu_ensemble_step(ek_ctx *const *members, int n, int nsteps, int *status);

/* The projection alone: REM_DIV_CURV (duct.F90:2472-2818) on the current
 * state, leaving phi in CR1 (as the reference leaves it in CR1X).  Status as
 * for ekgpu_rk_substep. */
int ekgpu_rem_div(ek_ctx *ctx);

/* Batched per-kx Poisson: for each problem p, solve the 9-point operator of
 * dismd2cr (mud2cr.f:501-1270) with coefficients cofcr (duct.F90:3900-3934)
 * and ce = -kx2[p]*INT_JACOB, right-hand side rhs[p] on the MUDPACK grid
 * (0:NZ+1,0:NY+1) (what phi_bc, duct.F90:3867, hands to mud2cr), phi zero
 * initial guess, FMG + k-cycles as MULTIGRID_MUDPACK (mg_solver2d.F90:75-201).
 * rhs and phi are host arrays of nprob*(NZ+2)*(NY+2) doubles, problem
 * outermost.  Returns EK_ERR_NOT_CONVERGED (phi still written) when a
 * problem hits the cycle cap. */
int ekgpu_poisson_batch(ek_ctx *ctx, const double *rhs, double *phi,
                        const double *kx2, int nprob, ek_mg_stats *stats);

/* Same solve on device pointers (rhs, phi, kx2 in device memory, same
 * layout); no host copies.  For callers that keep data resident. */
int ekgpu_poisson_batch_device(ek_ctx *ctx, const double *rhs_dev,
                               double *phi_dev, const double *kx2_dev,
                               int nprob, ek_mg_stats *stats);

/* Mean |div| after the last projection (duct.F90:2790-2806, the value the
 * reference prints as "Divergence after the projection step"). */
int ekgpu_last_divergence(ek_ctx *ctx, double *div);

/* Stats of the last multigrid call made by a substep or poisson call. */
int ekgpu_last_mg_stats(ek_ctx *ctx, ek_mg_stats *stats);

/* Real 2-D Poisson problems solved since the context was created, and how
 * many of them stopped at the cycle cap before their rule was met (either
 * rule).  No counterpart in the reference, which ignores mud2cr's ierror. */
int ekgpu_mg_counters(ek_ctx *ctx, long long *solved, long long *not_converged);

/* Context-free batched x-transforms on device memory: the
 * FFT_X_TO_FOURIER_OP / FFT_X_TO_PHYSICAL_OP pair the reference calls
 * (duct.F90:700, mpi_duct.F90:290,308; fft.F90 itself is missing from the
 * reference tree, FFTW 2.1.5 underneath).  nlines lines, each NX reals with
 * stride NX+2 doubles (physical) or NX/2+1 complex (spectral).  Forward:
 * (1/NX) sum_n u_n exp(-2 pi i k n/NX) for k <= nkx, zero above.  Inverse:
 * the Hermitian sum over k <= nkx (imaginary part of k = 0 ignored), points
 * x = NX, NX+1 set to 0.  nx a power of two in [8, 1024], nkx < nx/2;
 * stream is a cudaStream_t or NULL.  The twiddle tables are device scratch
 * allocated once per (device, nx).  Asynchronous on the stream. */
int ekgpu_fft_x_to_fourier(int nx, int nkx, long nlines, const double *in_dev, double *out_dev, void *stream);
int ekgpu_fft_x_to_physical(int nx, int nkx, long nlines, const double *in_dev, double *out_dev, void *stream);

/* Number of (device, nx) twiddle tables the two transforms above have
 * allocated so far in this process (a diagnostic of their device memory; no
 * counterpart in the reference). */
int ekgpu_fft_table_count(void);

/* ekgpu_fft_x_to_fourier without any device allocation.  No counterpart in
 * the reference: it exists for callers that are not allowed to allocate
 * device memory themselves or through this library -- for example a host
 * application that reserved the GPU's memory up front for its own pool, or
 * a time-critical loop that cannot pay for cudaMalloc and for the device-wide
 * synchronisation of cudaFree.  Same arguments and results as
 * ekgpu_fft_x_to_fourier; the caller still owns in_dev and out_dev.
 * Limit: nx <= 1024 (larger nx returns EK_ERR_ARG, message via
 * ekgpu_last_error(NULL)).  Its scratch -- the twiddle table, at most 769
 * complex doubles (12.3 KB) -- lives in one fixed array in device memory
 * that every GPU loading this library holds until the process exits.  The
 * first call on each device looks up that array's device address (a one-
 * time set-up), so make the first call on a device before any stream
 * capture.  Every call rewrites the whole table before using it, so nothing
 * has to start at zero; but all calls share the one table, so calls that
 * overlap on the GPU (e.g. on two streams) race and must be ordered by the
 * caller.  The looked-up address is kept for the life of the process: do not
 * use this library across a cudaDeviceReset. */
int ekgpu_fft_x_to_fourier_noalloc(int nx, int nkx, long nlines, const double *in_dev, double *out_dev,
                                   void *stream);

/* Number of kernel launches this context issued since creation. */
long long ekgpu_launch_count(const ek_ctx *ctx);

/* Optional per-kernel-class timer (CUDA events around every launch on the
 * context's stream).  ekgpu_set_timing clears the totals; get_timing fills
 * up to n classes (milliseconds, launch counts and the algorithmic HBM bytes
 * those launches must move, for roofline fractions) and returns the number
 * of classes; ekgpu_timing_class_name names class k.  Profiling aid with no
 * counterpart in the reference (it only prints a wall clock,
 * diablo.F90:171-176). */
int ekgpu_set_timing(ek_ctx *ctx, int on);
int ekgpu_get_timing(ek_ctx *ctx, double *ms, long long *count, double *bytes, int n);
const char *ekgpu_timing_class_name(int k);

#ifdef __cplusplus
}
#endif

#endif
