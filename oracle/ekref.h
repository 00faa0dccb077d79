/*
 * ekref.h -- CPU oracle for the GB300 duct substep.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain FP64 C++ restatement of the reference Fortran (ekman_bl) hot path:
 * RK_DUCT (src/duct.F90:237-2469), REM_DIV_CURV (src/duct.F90:2472-2818),
 * the called MUDPACK subset (src/mud2cr.f, src/mudcom.f), the Thomas and
 * boundary-row routines (src/boundary.F90) and JACOBI_TRANS
 * (src/diablo.F90:1088-1570).  Loop orders and floating-point expression
 * order follow the Fortran so that it can serve as the checker.
 *
 * Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load this library.  It is never part of the product path.
 *
 * The reference cannot be compiled here (no Fortran compiler, no MPI, no
 * FFTW).  Its unmodified source is run instead through an interpreter of
 * the Fortran subset it uses (tests/golden/fortran_interp.py), and this
 * oracle is pinned against those runs: the MUDPACK solves bit for bit,
 * REM_DIV_CURV plus two RK3 steps of RK_DUCT to rounding level on five
 * cases (tests/test_golden_reference.py).  src/fft.F90 is missing from the
 * tree, so the x-FFT convention is pinned by known-answer tests of our
 * own: forward = (1/NX) sum_n u_n exp(-2 pi i k n/NX) for k = 0..NX/3
 * (higher modes zeroed), inverse = Hermitian sum over k = 0..NX/3
 * (imaginary part of k=0 ignored), KX = 2 pi k/LX.
 */
#ifndef EKREF_H
#define EKREF_H

#include "../include/ekgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ekref_ctx ekref_ctx;

int ekref_create(const ek_params *p, ekref_ctx **ctx);
void ekref_destroy(ekref_ctx *ctx);
const char *ekref_last_error(const ekref_ctx *ctx);
void ekref_set_threads(int nthreads);

int ekref_metrics_from_grid(const ek_params *p, const double *xpoint,
                            const double *ypoint, double *int_jacob,
                            double *gmat_11, double *gmat_12, double *gmat_22,
                            double *cjob_11, double *cjob_12, double *cjob_21,
                            double *cjob_22, double *th_bar);
int ekref_set_metrics(ekref_ctx *ctx, const ek_metrics *m);
/* SPONGE_SIGMA(0:NY+1), SPONGE_SIGMA_OUT(0:NZ+1) of diablo.F90:1489-1556. */
int ekref_sponge_profiles(const ek_params *p, const double *xpoint, const double *ypoint,
                          double *sponge_sigma, double *sponge_sigma_out);
int ekref_set_sponge(ekref_ctx *ctx, const double *sponge_sigma, const double *sponge_sigma_out);
int ekref_set_time(ekref_ctx *ctx, double time, int time_step);
int ekref_get_time(ekref_ctx *ctx, double *time, int *time_step, double *delta_t);
int ekref_upload_state(ekref_ctx *ctx, const double *cu1, const double *cu2,
                       const double *cu3, const double *cp, const double *cth);
int ekref_download_state(ekref_ctx *ctx, double *cu1, double *cu2, double *cu3,
                         double *cp, double *cth);
int ekref_get_field(ekref_ctx *ctx, int field, double *out);
int ekref_put_field(ekref_ctx *ctx, int field, const double *in);
int ekref_rk_substep(ekref_ctx *ctx, int rk_step);
int ekref_step(ekref_ctx *ctx, int nsteps);
int ekref_rem_div(ekref_ctx *ctx);
int ekref_poisson_batch(ekref_ctx *ctx, const double *rhs, double *phi,
                        const double *kx2, int nprob, ek_mg_stats *stats);
int ekref_last_divergence(ekref_ctx *ctx, double *div);
int ekref_last_mg_stats(ekref_ctx *ctx, ek_mg_stats *stats);
/* SAVE_STATS_CURVI (flow_statistics.F90:2-1023): statistics and state round trip. */
int ekref_save_stats(ekref_ctx *ctx, ek_stats *stats);

/* LES (les_chan.F90 LES_MODEL_TYPE 2, les_chan_th.F90 LES_MODEL_TYPE_TH 1):
 * the GMAT_*_y / GMAT_*_z metrics of JACOBI_TRANS (diablo.F90:1379-1467), in
 * the face-metric layout; the context's copy of them; FIRST_TIME; and the
 * NU_T (physical layout) and C_DYN ((0:NZ+1,0:NY+1)) arrays. */
int ekref_les_metrics_from_grid(const ek_params *p, const double *xpoint, const double *ypoint,
                                double *gmat_11_y, double *gmat_12_y, double *gmat_22_y,
                                double *gmat_11_z, double *gmat_12_z, double *gmat_22_z);
int ekref_set_les_metrics(ekref_ctx *ctx, const double *gmat_11_y, const double *gmat_12_y,
                          const double *gmat_22_y, const double *gmat_11_z, const double *gmat_12_z,
                          const double *gmat_22_z);
int ekref_les_set_first_time(ekref_ctx *ctx, int first_time);
int ekref_les_get(ekref_ctx *ctx, double *nu_t, double *c_dyn);

/* Building blocks exposed for unit tests. */
/* r2c along x of nlines lines of stride nx+2 doubles -> (nx/2+1) complex per
 * line, modes above nkx zeroed; c2r the inverse (x >= nx set to 0). */
void ekref_fft_r2c(int nx, int nkx, long nlines, const double *in, double *out);
void ekref_fft_c2r(int nx, int nkx, long nlines, const double *in, double *out);
/* THOMAS_REAL (boundary.F90:53-84) on nsys systems of rows 0..n, arrays
 * (0:nsys-1, 0:n) column-major; solution returned in g. */
void ekref_thomas_real(int nsys, int n, double *a, double *b, double *c, double *g);
/* Apply the finest-level 9-point operator of dismd2cr (with ce = -kx2*J)
 * to phi(0:NZ+1,0:NY+1): out = A phi on the MUDPACK grid. */
int ekref_mg_apply(ekref_ctx *ctx, double kx2, const double *phi, double *out);
/* Left null vector z of the finest kx = 0 operator (A^T z = 0, |z| = 1),
 * (NZ+2)*(NY+2) doubles in the MUDPACK grid layout. */
int ekref_mg_left_null(ekref_ctx *ctx, double *z);

#ifdef __cplusplus
}
#endif

#endif
