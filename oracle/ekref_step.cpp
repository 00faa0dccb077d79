// Oracle (test infrastructure): RK_DUCT + REM_DIV_CURV restated from the
// reference (src/duct.F90:237-2818) with the x-FFT glue of
// src/mpi_duct.F90:271-717 for one MPI rank, the Thomas solver and boundary
// rows of src/boundary.F90, and MULTIGRID_MUDPACK (src/mg_solver2d.F90).
// Lines outside the J/K ranges that the reference computes but never reads
// are skipped; every value that reaches the state is computed as in the
// reference.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ekref_ctx.h"

using namespace ekref_detail;

static int fail(ekref_ctx *c, int code, const std::string &m) {
  c->err = m;
  return code;
}

extern "C" void ekref_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

extern "C" const char *ekref_last_error(const ekref_ctx *c) { return c ? c->err.c_str() : "null context"; }

static bool pick_mg_shape(int n, int &p, int &e) {
  // n = p*2^(e-1)+1 with p >= 2; choose the smallest p >= 3 (else 2).
  const int m = n - 1;
  int best_p = -1, best_e = -1;
  for (int ee = 1; (1 << (ee - 1)) <= m; ++ee) {
    if (m % (1 << (ee - 1))) continue;
    const int pp = m >> (ee - 1);
    if (pp < 2) continue;
    if (pp >= 3 && (best_p < 3 || pp < best_p)) { best_p = pp; best_e = ee; }
    if (best_p < 0) { best_p = pp; best_e = ee; }
  }
  if (best_p < 0) return false;
  p = best_p;
  e = best_e;
  return true;
}

extern "C" int ekref_create(const ek_params *p, ekref_ctx **out) {
  *out = nullptr;
  auto c = std::make_unique<ekref_ctx>();
  c->p = *p;
  const int NX = p->nx, NY = p->ny, NZ = p->nz;
  if (NX < 4 || (NX & (NX - 1)) || NY < 4 || NZ < 4) return fail(c.get(), EK_ERR_ARG, "bad sizes"), *out = c.release(), EK_ERR_ARG;
  c->NX = NX; c->NY = NY; c->NZ = NZ;
  c->NKX = NX / 3; c->NX2P = NX / 2; c->NXP = NX + 1;
  c->LDX = NX + 2; c->LDC = NX / 2 + 1; c->NZ2 = NZ + 2; c->NY2 = NY + 2;
  // INIT_DUCT (duct.F90:7-232), IC_TYPE = 7 branches.
  const int *ub = p->u_bc, *wb = p->w_bc, *tb = p->th_bc;
  c->JSTART = (wb[EK_YMIN] == 0 || wb[EK_YMIN] == 1 || wb[EK_YMIN] == 6 || wb[EK_YMIN] == 7 || wb[EK_YMIN] == 3) ? 1 : 2;
  c->ZSTART = (ub[EK_ZMIN] == 1 || ub[EK_ZMIN] == 6) ? 1 : 2;
  c->JEND = (wb[EK_YMAX] == 0 || wb[EK_YMAX] == 1 || wb[EK_YMAX] == 6) ? NY : NY - 1;
  c->ZEND = (ub[EK_ZMAX] == 0) ? ((p->ic_type == 7) ? NZ : NZ - 1) : ((ub[EK_ZMAX] == 1 || ub[EK_ZMAX] == 6) ? NZ : NZ - 1);
  {
    const int t = tb[EK_YMIN];
    c->JSTART_TH = (t == 0 || t == 1 || t == 5 || t == 2 || t == 6 || t == 7 || t == 8) ? 1 : 2;
    const int z = tb[EK_ZMIN];
    c->ZSTART_TH = (z == 0) ? ((p->ic_type == 7) ? 1 : 2) : ((z == 1 || z == 6) ? 1 : 2);
    const int u = tb[EK_YMAX];
    c->JEND_TH = (u == 0) ? ((p->ic_type == 7) ? NY : NY - 1) : ((u == 1 || u == 6 || u == 5) ? NY : NY - 1);
    const int r = tb[EK_ZMAX];
    c->ZEND_TH = (r == 0) ? ((p->ic_type == 7) ? NZ : NZ - 1) : ((r == 1 || r == 5 || r == 6) ? NZ : NZ - 1);
  }
  // RKW3 constants (diablo.F90:568-576)
  const double dt = p->delta_t;
  c->H_BAR[1] = dt * (8.0 / 15.0); c->H_BAR[2] = dt * (2.0 / 15.0); c->H_BAR[3] = dt * (5.0 / 15.0);
  c->BETA_BAR[1] = 1.0; c->BETA_BAR[2] = 25.0 / 8.0; c->BETA_BAR[3] = 9.0 / 4.0;
  c->ZETA_BAR[1] = 0.0; c->ZETA_BAR[2] = -17.0 / 8.0; c->ZETA_BAR[3] = -5.0 / 4.0;
  // wavenumbers (the convention of the missing INIT_FFT)
  c->KXP.resize(c->NX2P + 1);
  c->KX2P.resize(c->NX2P + 1);
  for (int i = 0; i <= c->NX2P; ++i) {
    c->KXP[i] = i * (2.0 * M_PI) / p->lx;
    c->KX2P[i] = c->KXP[i] * c->KXP[i];
  }
  // MUDPACK shape (grid_def:45-47 or automatic)
  auto &m = c->mud;
  if (p->mg_ixp > 0) {
    m.ixp = p->mg_ixp; m.jyq = p->mg_jyq; m.iex = p->mg_iex; m.jey = p->mg_jey;
  } else {
    if (!pick_mg_shape(NZ + 2, m.ixp, m.iex) || !pick_mg_shape(NY + 2, m.jyq, m.jey))
      return fail(c.get(), EK_ERR_ARG, "NZ+2 and NY+2 must be p*2^k+1"), *out = c.release(), EK_ERR_ARG;
  }
  if (m.ixp * (1 << (m.iex - 1)) + 1 != NZ + 2 || m.jyq * (1 << (m.jey - 1)) + 1 != NY + 2)
    return fail(c.get(), EK_ERR_ARG, "Mudpack Multigrid Parameters are not Matching Grid Dimensions."), *out = c.release(), EK_ERR_ARG;
  m.kcycle = p->mg_kcycle; m.iprer = p->mg_iprer; m.ipost = p->mg_ipost; m.intpol = p->mg_intpol;
  m.maxcy = p->mg_maxcy; m.stop_rule = p->mg_stop; m.tol = p->mg_tol;
  // storage (zero-filled as a fresh allocation)
  const size_t np = (size_t)c->LDX * c->NZ2 * c->NY2, nc = (size_t)c->LDC * c->NZ2 * c->NY2;
  for (auto *v : {&c->CU1, &c->CU2, &c->CU3, &c->CP, &c->CTH, &c->CF1, &c->CF2, &c->CF3, &c->CFTH, &c->CR1, &c->CR2,
                  &c->CR3, &c->CRTH, &c->CS1, &c->CS2, &c->CU2b, &c->CU3b})
    v->assign(nc, cplx{0.0, 0.0});
  for (auto *v : {&c->U1, &c->U2, &c->U3, &c->TH, &c->R1, &c->R2, &c->R3, &c->RTH, &c->S1, &c->S2, &c->U2b, &c->U3b})
    v->assign(np, 0.0);
  c->sponge_sigma.assign(NY + 2, 0.0);
  c->sponge_sigma_out.assign(NZ + 2, 0.0);
  if (p->sponge_type != 0 && p->save_stats_int < 1)
    return fail(c.get(), EK_ERR_ARG, "SAVE_STATS_INT must be >= 1 with a sponge"), *out = c.release(), EK_ERR_ARG;
  if (p->les) {
    if (p->les_model_type != 2 || (p->n_th > 0 && p->les_model_type_th != 1))
      return fail(c.get(), EK_ERR_ARG, "LES: only LES_MODEL_TYPE 2 with LES_MODEL_TYPE_TH 1"), *out = c.release(), EK_ERR_ARG;
    if (wb[EK_YMIN] == 3)
      return fail(c.get(), EK_ERR_ARG, "LES: the wall model (W_BC_YMIN = 3) is not restated"), *out = c.release(), EK_ERR_ARG;
    les_alloc(c.get());
  }
  c->fft = std::make_unique<FFT>(NX);
  *out = c.release();
  return EK_OK;
}

extern "C" void ekref_destroy(ekref_ctx *c) { delete c; }

// SPONGE_SIGMA / SPONGE_SIGMA_OUT (diablo.F90:1489-1556).  b, co_b and xx are
// REAL*8; REAL(...) of a difference is default-kind REAL*4 (no -r8 in the
// Makefiles), so the spans are rounded to float before dividing.
extern "C" int ekref_sponge_profiles(const ek_params *p, const double *xpoint, const double *ypoint,
                                     double *SPONGE_SIGMA, double *SPONGE_SIGMA_OUT) {
  if (!p || !xpoint || !ypoint || !SPONGE_SIGMA || !SPONGE_SIGMA_OUT) return EK_ERR_ARG;
  const int NY = p->ny, NZ = p->nz, NZ_S_R = p->nz_s_r, NZ_S_L = p->nz_s_l, NY_S_T = p->ny_s_t;
  auto xpt = [&](int K, int J) { return xpoint[(size_t)J * (NZ + 2) + K]; };
  auto ypt = [&](int K, int J) { return ypoint[(size_t)J * (NZ + 2) + K]; };
  double b, co_b, xx;
  for (int K = 0; K <= NZ + 1; ++K) SPONGE_SIGMA_OUT[K] = 0.0;
  if (p->sponge_type == 1 && NZ_S_R < NZ + 1) {
    b = 1.0 / (double)(float)(xpt(NZ + 1, NY + 1) - xpt(NZ_S_R, NY + 1));
    for (int K = 0; K <= NZ + 1; ++K) {
      if (K >= NZ_S_R) {
        xx = (xpt(K, NY + 1) - xpt(NZ_S_R, NY + 1)) * b;
        SPONGE_SIGMA_OUT[K] = xx * xx;
      } else if (K <= NZ_S_L) {
        xx = (xpt(NZ_S_L, NY + 1) - xpt(K, NY + 1)) * b;
        SPONGE_SIGMA_OUT[K] = xx * xx;
      }
    }
  } else if (p->sponge_type == 2 && NZ_S_R < NZ + 1) {
    co_b = 25.0;
    b = std::log(co_b) / (double)(float)(NZ + 1 - NZ_S_R);
    for (int K = 0; K <= NZ + 1; ++K) {
      if (K >= NZ_S_R)
        SPONGE_SIGMA_OUT[K] = (std::exp(b * std::abs(K - NZ_S_R)) - 1.0) / (co_b - 1.0);
      else if (K <= NZ_S_L)
        SPONGE_SIGMA_OUT[K] = (std::exp(b * std::abs(NZ_S_L - K)) - 1.0) / (co_b - 1.0);
    }
  }
  for (int J = 0; J <= NY + 1; ++J) SPONGE_SIGMA[J] = 0.0;
  if (p->sponge_type == 1) {
    if (NY_S_T < 0 || NY_S_T > NY + 1) return EK_ERR_ARG;
    b = 1.0 / (double)(float)(ypt(NZ + 1, NY + 1) - ypt(NZ + 1, NY_S_T));
    for (int J = NY_S_T; J <= NY + 1; ++J) {
      xx = (ypt(NZ + 1, J) - ypt(NZ + 1, NY_S_T)) * b;
      SPONGE_SIGMA[J] = xx * xx;
    }
  } else if (p->sponge_type == 2) {
    if (NY_S_T < 0 || NY_S_T > NY + 1) return EK_ERR_ARG;
    co_b = 30.0;
    b = std::log(co_b) / (double)(float)(NY + 1 - NY_S_T);
    for (int J = NY_S_T; J <= NY + 1; ++J) SPONGE_SIGMA[J] = (std::exp(b * (J - NY_S_T)) - 1.0) / (co_b - 1.0);
  }
  return EK_OK;
}

extern "C" int ekref_set_sponge(ekref_ctx *c, const double *s, const double *so) {
  if (!s || !so) return fail(c, EK_ERR_ARG, "sponge profile is NULL");
  c->sponge_sigma.assign(s, s + c->NY + 2);
  c->sponge_sigma_out.assign(so, so + c->NZ + 2);
  return EK_OK;
}

extern "C" int ekref_set_time(ekref_ctx *c, double time, int time_step) {
  c->p.time = time;
  c->p.time_step = time_step;
  return EK_OK;
}

extern "C" int ekref_get_time(ekref_ctx *c, double *time, int *time_step, double *delta_t) {
  if (time) *time = c->p.time;
  if (time_step) *time_step = c->p.time_step;
  if (delta_t) *delta_t = c->p.delta_t;
  return EK_OK;
}

// sponge_th(N) (duct.F90:3196-3362), restated loop by loop.
static void sponge_th(ekref_ctx *c) {
  const ek_params &p = c->p;
  const int NX2P = c->NX2P, NY = c->NY, NZ = c->NZ;
  const int JSTART = c->JSTART, JEND = c->JEND, ZSTART = c->ZSTART, ZEND = c->ZEND;
  auto &CU1 = c->CU1, &CU2 = c->CU2, &CU3 = c->CU3, &CTH = c->CTH;
  auto &CF1 = c->CF1, &CF2 = c->CF2, &CF3 = c->CF3, &CFTH = c->CFTH;
  const std::vector<double> &SPONGE_SIGMA = c->sponge_sigma, &SPONGE_SIGMA_OUT = c->sponge_sigma_out;
  const double Sponge_Amp = 0.1 / p.delta_t;
  const double Dynamic_sponge_threshold = 0.001;
  // F - ((a * s) * (U - t)) * J, complex minus a real target
  auto term = [](cplx f, double as, cplx u, double t, double jac) {
    const cplx v{as * (u.re - t), as * u.im};
    return cplx{f.re - v.re * jac, f.im - v.im * jac};
  };
  int i = 0, j = 0, k = 0;
  // damp fluctuations: top and bottom
  for (j = JSTART; j <= JEND; ++j)
    for (k = ZSTART; k <= ZEND; ++k)
      for (i = 1; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        const double as = Sponge_Amp * SPONGE_SIGMA[j], J = c->JAC(k, j);
        CF1[q] = term(CF1[q], as, CU1[q], 0.0, J);
        CF2[q] = term(CF2[q], as, CU2[q], 0.0, J);
        CF3[q] = term(CF3[q], as, CU3[q], 0.0, J);
        CFTH[q] = term(CFTH[q], as, CTH[q], 0.0, J);
      }
  // inflow / outflow
  for (j = JSTART; j <= JEND; ++j)
    for (k = ZSTART; k <= ZEND; ++k)
      for (i = 1; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        const double as = Sponge_Amp * SPONGE_SIGMA_OUT[k], J = c->JAC(k, j);
        CF1[q] = term(CF1[q], as, CU1[q], 0.0, J);
        CF2[q] = term(CF2[q], as, CU2[q], 0.0, J);
        CF3[q] = term(CF3[q], as, CU3[q], 0.0, J);
        CFTH[q] = term(CFTH[q], as, CTH[q], 0.0, J);
      }
  const int NY_sponge = (p.ny_s_t > NY) ? (2 * NY) / 3 : p.ny_s_t;
  double CU3X_sponge = 0.0;
  for (j = NY_sponge; j <= JEND; ++j)
    for (k = ZSTART; k <= ZEND; ++k) CU3X_sponge = CU3X_sponge + CU3[c->ic(0, k, j)].re;
  CU3X_sponge = CU3X_sponge / (double)((ZEND - ZSTART + 1) * (JEND - NY_sponge + 1));
  const double CU1X_target = p.v_bc_c1[EK_YMAX], CU2X_target = p.u_bc_c1[EK_YMAX], CU3X_target = p.wbulk0;
  // damp the mean flow (RANK 0, DYNAMIC_SPONE = .TRUE.)
  if (std::fabs(CU3X_sponge - CU3X_target) > CU3X_target * Dynamic_sponge_threshold) {
    for (j = JSTART; j <= JEND; ++j)
      for (k = ZSTART; k <= ZEND; ++k) {
        const size_t q = c->ic(0, k, j);
        const double as = Sponge_Amp * SPONGE_SIGMA[j], J = c->JAC(k, j);
        CF1[q] = term(CF1[q], as, CU1[q], CU1X_target, J);
        CF2[q] = term(CF2[q], as, CU2[q], CU2X_target, J);
        CF3[q] = term(CF3[q], as, CU3[q], CU3X_target, J);
        CFTH[q] = term(CFTH[q], as, CTH[q], 0.0, J);
      }
  } else {
    for (j = JSTART; j <= JEND; ++j)
      for (k = ZSTART; k <= ZEND; ++k) {
        const size_t q = c->ic(0, k, j);
        const double as = Sponge_Amp * SPONGE_SIGMA[j], J = c->JAC(k, j);
        CF2[q] = term(CF2[q], as, CU2[q], CU2X_target, J);
        CF1[q] = term(CF1[q], as, CU1[q], CU1X_target, J);
      }
  }
  // j = JEND+1, k = ZEND+1 here, as after the Fortran DO loops
  if (p.v_bc[EK_ZMAX] == 6 && p.u_bc[EK_ZMAX] == 6 && p.w_bc[EK_ZMAX] == 6 && p.ri_tau != 0.0) {
    const double J = c->JAC(k, j);
    for (int jj = 0; jj <= NY + 1; ++jj)
      for (int kk = 0; kk <= NZ + 1; ++kk) {
        const size_t q = c->ic(0, kk, jj);
        CF2[q] = term(CF2[q], Sponge_Amp, CU2[q], CU2X_target, J);
      }
    if ((2 * p.time_step) % p.save_stats_int == 0)
      for (int jj = 0; jj <= NY + 1; ++jj)
        for (int kk = 0; kk <= NZ + 1; ++kk) CU2[c->ic(0, kk, jj)] = cplx{0.0, 0.0};
  }
  // inflow / outflow of the mean
  for (j = JSTART; j <= JEND; ++j)
    for (k = ZSTART; k <= ZEND; ++k) {
      const size_t q = c->ic(0, k, j);
      const double as = 2.0 * Sponge_Amp * SPONGE_SIGMA_OUT[k], J = c->JAC(k, j);
      CF1[q] = term(CF1[q], as, CU1[q], 0.0, J);
      CF2[q] = term(CF2[q], as, CU2[q], 0.0, J);
      CF3[q] = term(CF3[q], as, CU3[q], CU3X_target, J);
      CFTH[q] = term(CFTH[q], as, CTH[q], 0.0, J);
    }
}

extern "C" int ekref_set_metrics(ekref_ctx *c, const ek_metrics *m) {
  const size_t n2 = (size_t)(c->NZ + 3) * (c->NY + 3);
  auto cp2 = [&](std::vector<double> &d, const double *s, size_t n) {
    if (s) d.assign(s, s + n); else d.assign(n, 0.0);
  };
  if (!m->int_jacob || !m->gmat_11 || !m->gmat_12 || !m->gmat_22 || !m->cjob_11 || !m->cjob_12 || !m->cjob_21 || !m->cjob_22)
    return fail(c, EK_ERR_ARG, "metric pointer is NULL");
  cp2(c->int_jacob, m->int_jacob, n2);
  cp2(c->gmat_11, m->gmat_11, 2 * n2); cp2(c->gmat_12, m->gmat_12, 2 * n2); cp2(c->gmat_22, m->gmat_22, 2 * n2);
  cp2(c->cjob_11, m->cjob_11, 2 * n2); cp2(c->cjob_12, m->cjob_12, 2 * n2);
  cp2(c->cjob_21, m->cjob_21, 2 * n2); cp2(c->cjob_22, m->cjob_22, 2 * n2);
  cp2(c->th_bar, m->th_bar, n2);
  c->mg_z.clear();
  c->have_metrics = true;
  return EK_OK;
}

static std::vector<cplx> *field_ptr(ekref_ctx *c, int f) {
  switch (f) {
    case EK_F_CU1: return &c->CU1; case EK_F_CU2: return &c->CU2; case EK_F_CU3: return &c->CU3;
    case EK_F_CP: return &c->CP; case EK_F_CTH: return &c->CTH; case EK_F_CF1: return &c->CF1;
    case EK_F_CF2: return &c->CF2; case EK_F_CF3: return &c->CF3; case EK_F_CFTH: return &c->CFTH;
    case EK_F_CR1: return &c->CR1;
    default: return nullptr;
  }
}

extern "C" int ekref_get_field(ekref_ctx *c, int f, double *out) {
  auto *v = field_ptr(c, f);
  if (!v) return fail(c, EK_ERR_ARG, "bad field");
  std::memcpy(out, v->data(), v->size() * sizeof(cplx));
  return EK_OK;
}

extern "C" int ekref_put_field(ekref_ctx *c, int f, const double *in) {
  auto *v = field_ptr(c, f);
  if (!v) return fail(c, EK_ERR_ARG, "bad field");
  std::memcpy(v->data(), in, v->size() * sizeof(cplx));
  return EK_OK;
}

extern "C" int ekref_upload_state(ekref_ctx *c, const double *cu1, const double *cu2, const double *cu3,
                                  const double *cp, const double *cth) {
  ekref_put_field(c, EK_F_CU1, cu1); ekref_put_field(c, EK_F_CU2, cu2); ekref_put_field(c, EK_F_CU3, cu3);
  ekref_put_field(c, EK_F_CP, cp);
  if (cth) ekref_put_field(c, EK_F_CTH, cth);
  for (auto *v : {&c->CF1, &c->CF2, &c->CF3, &c->CFTH}) std::fill(v->begin(), v->end(), cplx{0.0, 0.0});
  return EK_OK;
}

extern "C" int ekref_download_state(ekref_ctx *c, double *cu1, double *cu2, double *cu3, double *cp, double *cth) {
  ekref_get_field(c, EK_F_CU1, cu1); ekref_get_field(c, EK_F_CU2, cu2); ekref_get_field(c, EK_F_CU3, cu3);
  ekref_get_field(c, EK_F_CP, cp);
  if (cth) ekref_get_field(c, EK_F_CTH, cth);
  return EK_OK;
}

// ---------------------------------------------------------------------------
// x-transforms (mpi_duct.F90:271-717 with NP = 1; MPI transposes are copies)
void to_fourier(ekref_ctx *c, const std::vector<double> &in, std::vector<cplx> &out, int j0, int j1, int k0, int k1) {
  const FFT &f = *c->fft;
#pragma omp parallel
  {
    std::vector<std::complex<double>> buf(c->NX);
#pragma omp for collapse(2) schedule(static)
    for (int j = j0; j <= j1; ++j)
      for (int k = k0; k <= k1; ++k) r2c_line(f, c->NKX, &in[c->ip(0, k, j)], &out[c->ic(0, k, j)], buf.data());
  }
}
void to_physical(ekref_ctx *c, const std::vector<cplx> &in, std::vector<double> &out, int j0, int j1, int k0, int k1) {
  const FFT &f = *c->fft;
#pragma omp parallel
  {
    std::vector<std::complex<double>> buf(c->NX);
#pragma omp for collapse(2) schedule(static)
    for (int j = j0; j <= j1; ++j)
      for (int k = k0; k <= k1; ++k) c2r_line(f, c->NKX, &in[c->ic(0, k, j)], &out[c->ip(0, k, j)], buf.data());
  }
}

static bool pow2(int n) { return n >= 2 && (n & (n - 1)) == 0; }

extern "C" void ekref_fft_r2c(int nx, int nkx, long nlines, const double *in, double *out) {
  if (!pow2(nx)) return;
  FFT f(nx);
  std::vector<std::complex<double>> buf(nx);
  for (long l = 0; l < nlines; ++l)
    r2c_line(f, nkx, in + l * (nx + 2), reinterpret_cast<cplx *>(out) + l * (nx / 2 + 1), buf.data());
}
extern "C" void ekref_fft_c2r(int nx, int nkx, long nlines, const double *in, double *out) {
  if (!pow2(nx)) return;
  FFT f(nx);
  std::vector<std::complex<double>> buf(nx);
  for (long l = 0; l < nlines; ++l)
    c2r_line(f, nkx, reinterpret_cast<const cplx *>(in) + l * (nx / 2 + 1), out + l * (nx + 2), buf.data());
}

// THOMAS_REAL (boundary.F90:53-84): arrays (0:NX,0:NY) column-major.
static void thomas_real(double *A, double *B, double *C, double *G, int NY, int NX) {
  const int ld = NX + 1;
  for (int j = 0; j <= NY - 1; ++j)
    for (int i = 0; i <= NX; ++i) {
      A[(j + 1) * ld + i] = -A[(j + 1) * ld + i] / B[j * ld + i];
      B[(j + 1) * ld + i] = B[(j + 1) * ld + i] + A[(j + 1) * ld + i] * C[j * ld + i];
      G[(j + 1) * ld + i] = G[(j + 1) * ld + i] + A[(j + 1) * ld + i] * G[j * ld + i];
    }
  for (int i = 0; i <= NX; ++i) G[NY * ld + i] = G[NY * ld + i] / B[NY * ld + i];
  for (int j = NY - 1; j >= 0; --j)
    for (int i = 0; i <= NX; ++i) G[j * ld + i] = (G[j * ld + i] - C[j * ld + i] * G[(j + 1) * ld + i]) / B[j * ld + i];
}

extern "C" void ekref_thomas_real(int nsys, int n, double *a, double *b, double *c, double *g) {
  thomas_real(a, b, c, g, n, nsys - 1);
}

// ---------------------------------------------------------------------------
// Boundary rows (boundary.F90:124-1763), IC_TYPE = 7 branches.  var: 0 TH,
// 1 U1, 2 U2, 3 U3.  The row arrays are (0:NXP, 0:N+1).
struct Rows {
  double *L, *D, *U, *V;
  int ld;
  void set(int row, int i, double l, double d, double u, double v) {
    L[row * ld + i] = l; D[row * ld + i] = d; U[row * ld + i] = u; V[row * ld + i] = v;
  }
};

static void bc_y(ekref_ctx *c, int var, int K, Rows &r, const std::vector<double> &phi) {
  const ek_params &p = c->p;
  const int NY = c->NY, NXP = c->NXP;
  const int lo = (var == 0) ? p.th_bc[EK_YMIN] : (var == 1) ? p.u_bc[EK_YMIN] : (var == 2) ? p.v_bc[EK_YMIN] : p.w_bc[EK_YMIN];
  const int hi = (var == 0) ? p.th_bc[EK_YMAX] : (var == 1) ? p.u_bc[EK_YMAX] : (var == 2) ? p.v_bc[EK_YMAX] : p.w_bc[EK_YMAX];
  const double clo = (var == 0) ? p.th_bc_c1[EK_YMIN] : (var == 1) ? p.u_bc_c1[EK_YMIN] : (var == 2) ? p.v_bc_c1[EK_YMIN] : p.w_bc_c1[EK_YMIN];
  const double chi = (var == 0) ? p.th_bc_c1[EK_YMAX] : (var == 1) ? p.u_bc_c1[EK_YMAX] : (var == 2) ? p.v_bc_c1[EK_YMAX] : p.w_bc_c1[EK_YMAX];
  for (int i = 0; i <= NXP; ++i) {
    // lower wall
    if (lo == 0) {
      r.set(0, i, 0., 1., 0., clo);
    } else if (lo == 1 || (var == 0 && lo == 5)) {
      if (var == 0)
        r.set(0, i, 0., -1., 1., clo / (0.5 * (c->M3(c->cjob_22, K, 1, 2) + c->M3(c->cjob_22, K + 1, 1, 1))) * c->JAC(K, 1));
      else if (var == 3)
        r.set(0, i, 0., -1., 1., clo);
      else
        r.set(1, i, 0., -1., 1., clo);
    } else if (lo == 6) {
      r.set(0, i, 0., 1., 0., phi[c->ip(i, K, NY)]);
    }
    // upper wall
    if (hi == 0) {
      r.set(NY + 1, i, 0., 1., 0., chi);
      if (var == 2 || var == 3) r.set(NY, i, 0., 1., 0., chi);
    } else if (hi == 1) {
      if (var == 0) {
        r.set(NY, i, -1., 1., 0., 0.5 * chi * (c->JAC(K, NY) + c->JAC(K, NY - 1)) / c->M3(c->cjob_22, K, NY - 1, 1));
        r.set(NY + 1, i, -1., 1., 0., 0.5 * chi * (c->JAC(K, NY + 1) + c->JAC(K, NY)) / c->M3(c->cjob_22, K, NY, 1));
      } else if (var == 2) {
        r.set(NY, i, -1., 1., 0., chi);
      } else {
        r.set(NY + 1, i, -1., 1., 0., chi);
      }
    } else if (hi == 6) {
      r.set(NY + 1, i, 0., 1., 0., phi[c->ip(i, K, 1)]);
    }
  }
}

static void bc_z(ekref_ctx *c, int var, int J, Rows &r, const std::vector<double> &phi) {
  const ek_params &p = c->p;
  const int NZ = c->NZ, NXP = c->NXP;
  const int lo = (var == 0) ? p.th_bc[EK_ZMIN] : (var == 1) ? p.u_bc[EK_ZMIN] : (var == 2) ? p.v_bc[EK_ZMIN] : p.w_bc[EK_ZMIN];
  const int hi = (var == 0) ? p.th_bc[EK_ZMAX] : (var == 1) ? p.u_bc[EK_ZMAX] : (var == 2) ? p.v_bc[EK_ZMAX] : p.w_bc[EK_ZMAX];
  const double clo = (var == 0) ? p.th_bc_c1[EK_ZMIN] : (var == 1) ? p.u_bc_c1[EK_ZMIN] : (var == 2) ? p.v_bc_c1[EK_ZMIN] : p.w_bc_c1[EK_ZMIN];
  const double chi = (var == 0) ? p.th_bc_c1[EK_ZMAX] : (var == 1) ? p.u_bc_c1[EK_ZMAX] : (var == 2) ? p.v_bc_c1[EK_ZMAX] : p.w_bc_c1[EK_ZMAX];
  for (int i = 0; i <= NXP; ++i) {
    if (lo == 0) {  // TH and U1 only (U2/U3 use background profiles; rejected at create)
      r.set(0, i, 0., 1., 0., (var == 0) ? 0.0 : clo);
      r.set(1, i, 0., 1., 0., clo);
    } else if (lo == 1) {
      r.set(0, i, 0., -1., 1., clo);
    } else if (lo == 6) {
      r.set(0, i, 0., 1., 0., phi[c->ip(i, NZ, J)]);
    }
    if (hi == 0) {
      r.set(NZ + 1, i, 0., 1., 0., (var == 3) ? chi : 0.0);
      r.set(NZ, i, 0., 1., 0., chi);
    } else if (hi == 1) {
      if (var == 1)
        r.set(NZ + 1, i, 0., 1., 0., 0.0);  // APPLY_BC_1_RIGHT overwrites the Neumann row
      else
        r.set(NZ + 1, i, -1., 1., 0., chi);
    } else if (hi == 6) {
      r.set(NZ + 1, i, 0., 1., 0., phi[c->ip(i, 1, J)]);
    }
  }
}

// One ADI-CN field update (e.g. U1: duct.F90:1640-1854).  coef = TEMP1 (or
// TEMP1/PR for TH).  phi is U1X/U2X/U3X/THX, R the matching R*X.
static void adi_field(ekref_ctx *c, int var, double coef, std::vector<double> &phi, std::vector<double> &R,
                      int js, int je, int zs, int ze, const LesAdi *les) {
  // half-sum of the eddy viscosity over a face, times TEMP2 (duct.F90:1667-1854)
  auto nuf = [&](int i, int k1, int j1, int k2, int j2) {
    return 0.5 * ((*les->nu)[c->ip(i, k1, j1)] + (*les->nu)[c->ip(i, k2, j2)]);
  };
  const int NXP = c->NXP, NY = c->NY, NZ = c->NZ;
  std::vector<double> &S = c->S1;
  // S = R - J*phi ; R = 0.5*S + J*phi + coef*d_zeta(G11 d_zeta phi)
#pragma omp parallel for schedule(static)
  for (int j = js; j <= je; ++j)
    for (int k = zs; k <= ze; ++k) {
      const double jac = c->JAC(k, j);
      const double g1 = c->M3(c->gmat_11, k + 1, j, 2), g0 = c->M3(c->gmat_11, k, j, 2);
      for (int i = 0; i <= NXP; ++i) {
        S[c->ip(i, k, j)] = R[c->ip(i, k, j)] - jac * phi[c->ip(i, k, j)];
      }
      for (int i = 0; i <= NXP; ++i) {
        R[c->ip(i, k, j)] = 0.5 * S[c->ip(i, k, j)] + jac * phi[c->ip(i, k, j)] +
                            coef * (g1 * (phi[c->ip(i, k + 1, j)] - phi[c->ip(i, k, j)]) -
                                    g0 * (phi[c->ip(i, k, j)] - phi[c->ip(i, k - 1, j)]));
      }
      if (les) {  // e.g. duct.F90:1667-1680
        const double l1 = c->M3(*les->g11, k + 1, j, 2), l0 = c->M3(*les->g11, k, j, 2);
        for (int i = 0; i <= NXP; ++i)
          R[c->ip(i, k, j)] = R[c->ip(i, k, j)] +
                              les->temp2 * (nuf(i, k + 1, j, k, j) * (l1 * (phi[c->ip(i, k + 1, j)] - phi[c->ip(i, k, j)])) -
                                            nuf(i, k, j, k - 1, j) * (l0 * (phi[c->ip(i, k, j)] - phi[c->ip(i, k - 1, j)])));
      }
    }
  // y-systems, one per K (THOMAS_REAL over I)
  const int ldy = NXP + 1;
#pragma omp parallel
  {
    std::vector<double> L((size_t)ldy * (NY + 2), 0.0), D((size_t)ldy * (NY + 2), 1.0), U((size_t)ldy * (NY + 2), 0.0),
        V((size_t)ldy * (NY + 2), 0.0);
    Rows rows{L.data(), D.data(), U.data(), V.data(), ldy};
#pragma omp for schedule(static)
    for (int k = zs; k <= ze; ++k) {
      for (int j = js; j <= je; ++j) {
        const double gl = c->M3(c->gmat_22, k, j, 1), gu = c->M3(c->gmat_22, k, j + 1, 1);
        const double dd = c->JAC(k, j) + coef * (gu + gl);
        for (int i = 0; i <= NXP; ++i) {
          L[j * ldy + i] = -coef * gl;
          D[j * ldy + i] = dd;
          U[j * ldy + i] = -coef * gu;
          V[j * ldy + i] = R[c->ip(i, k, j)];
        }
        if (les) {  // e.g. duct.F90:1720-1731
          const double ml = c->M3(*les->g22, k, j, 1), mu = c->M3(*les->g22, k, j + 1, 1);
          for (int i = 0; i <= NXP; ++i) {
            const double nl = les->temp2 * nuf(i, k, j, k, j - 1), nu = les->temp2 * nuf(i, k, j, k, j + 1);
            L[j * ldy + i] = L[j * ldy + i] - nl * ml;
            D[j * ldy + i] = D[j * ldy + i] + nu * mu + nl * ml;
            U[j * ldy + i] = U[j * ldy + i] - nu * mu;
          }
        }
      }
      bc_y(c, var, k, rows, phi);
      thomas_real(L.data(), D.data(), U.data(), V.data(), NY + 1, NXP);
      for (int j = 0; j <= NY + 1; ++j)
        for (int i = 0; i <= NXP; ++i) phi[c->ip(i, k, j)] = V[j * ldy + i];
    }
  }
  // R = 0.5*S + J*phi* + coef*d_eta(G22 d_eta phi*)
#pragma omp parallel for schedule(static)
  for (int j = js; j <= je; ++j)
    for (int k = zs; k <= ze; ++k) {
      const double jac = c->JAC(k, j);
      const double g1 = c->M3(c->gmat_22, k, j + 1, 1), g0 = c->M3(c->gmat_22, k, j, 1);
      for (int i = 0; i <= NXP; ++i)
        R[c->ip(i, k, j)] = 0.5 * S[c->ip(i, k, j)] + jac * phi[c->ip(i, k, j)] +
                            coef * (+g1 * (phi[c->ip(i, k, j + 1)] - phi[c->ip(i, k, j)]) -
                                    g0 * (phi[c->ip(i, k, j)] - phi[c->ip(i, k, j - 1)]));
      if (les) {  // e.g. duct.F90:1771-1784
        const double l1 = c->M3(*les->g22, k, j + 1, 1), l0 = c->M3(*les->g22, k, j, 1);
        for (int i = 0; i <= NXP; ++i)
          R[c->ip(i, k, j)] = R[c->ip(i, k, j)] +
                              les->temp2 * (nuf(i, k, j + 1, k, j) * (l1 * (phi[c->ip(i, k, j + 1)] - phi[c->ip(i, k, j)])) -
                                            nuf(i, k, j - 1, k, j) * (l0 * (phi[c->ip(i, k, j)] - phi[c->ip(i, k, j - 1)])));
      }
    }
  // z-systems, one per J
#pragma omp parallel
  {
    std::vector<double> L((size_t)ldy * (NZ + 2), 0.0), D((size_t)ldy * (NZ + 2), 1.0), U((size_t)ldy * (NZ + 2), 0.0),
        V((size_t)ldy * (NZ + 2), 0.0);
    Rows rows{L.data(), D.data(), U.data(), V.data(), ldy};
#pragma omp for schedule(static)
    for (int j = js; j <= je; ++j) {
      for (int k = zs; k <= ze; ++k) {
        const double gl = c->M3(c->gmat_11, k, j, 2), gu = c->M3(c->gmat_11, k + 1, j, 2);
        const double dd = c->JAC(k, j) + coef * (gu + gl);
        for (int i = 0; i <= NXP; ++i) {
          L[k * ldy + i] = -coef * gl;
          D[k * ldy + i] = dd;
          U[k * ldy + i] = -coef * gu;
          V[k * ldy + i] = R[c->ip(i, k, j)];
        }
        if (les) {  // e.g. duct.F90:1821-1832
          const double ml = c->M3(*les->g11, k, j, 2), mu = c->M3(*les->g11, k + 1, j, 2);
          for (int i = 0; i <= NXP; ++i) {
            const double nl = les->temp2 * nuf(i, k, j, k - 1, j), nu = les->temp2 * nuf(i, k + 1, j, k, j);
            L[k * ldy + i] = L[k * ldy + i] - nl * ml;
            D[k * ldy + i] = D[k * ldy + i] + nu * mu + nl * ml;
            U[k * ldy + i] = U[k * ldy + i] - nu * mu;
          }
        }
      }
      bc_z(c, var, j, rows, phi);
      thomas_real(L.data(), D.data(), U.data(), V.data(), NZ + 1, NXP);
      for (int k = 0; k <= NZ + 1; ++k)
        for (int i = 0; i <= NXP; ++i) phi[c->ip(i, k, j)] = V[k * ldy + i];
    }
  }
}

// ---------------------------------------------------------------------------
// MULTIGRID_MUDPACK over a batch of real problems (mg_solver2d.F90:75-201).
static ekref::CoefFn make_cofcr(const ekref_ctx *c, double kx2) {
  // cofcr (duct.F90:3900-3934)
  return [c, kx2](double x, double y, double &cxx, double &cxy, double &cyy, double &cx, double &cy, double &ce) {
    const int k = (int)x, j = (int)y;
    const auto &G11 = c->gmat_11, &G12 = c->gmat_12, &G22 = c->gmat_22;
    cxx = 0.25 * (c->M3(G11, k, j, 2) + c->M3(G11, k + 1, j, 2) + c->M3(G11, k, j, 1) + c->M3(G11, k, j + 1, 1));
    cxy = 0.5 * (c->M3(G12, k, j, 2) + c->M3(G12, k + 1, j, 2) + c->M3(G12, k, j, 1) + c->M3(G12, k, j + 1, 1));
    cyy = 0.25 * (c->M3(G22, k, j, 2) + c->M3(G22, k + 1, j, 2) + c->M3(G22, k, j, 1) + c->M3(G22, k, j + 1, 1));
    cx = c->M3(G11, k + 1, j, 2) - c->M3(G11, k, j, 2) + c->M3(G12, k, j + 1, 1) - c->M3(G12, k, j, 1);
    cy = c->M3(G22, k, j + 1, 1) - c->M3(G22, k, j, 1) + c->M3(G12, k + 1, j, 2) - c->M3(G12, k, j, 2);
    ce = -kx2 * c->JAC(k, j);
  };
}

// rhs/phi: nprob problems of (NZ+2)*(NY+2) doubles (MUDPACK grid, x = K fastest).
// The left null vector of the finest kx = 0 operator, built once per metric set.
static const double *mg_left_null(ekref_ctx *c) {
  if (c->mg_z.empty()) {
    ekref::Mud2cr mg(c->mud);
    mg.discretize(make_cofcr(c, 0.0));
    c->mg_z = mg.left_null();
  }
  return c->mg_z.data();
}

static int mg_batch(ekref_ctx *c, const double *rhs, double *phi, const double *kx2, int nprob, ek_mg_stats *st) {
  const size_t n = (size_t)(c->NZ + 2) * (c->NY + 2);
  std::vector<ekref::MudResult> res(nprob);
  const double *z = nullptr;
  if (c->mud.stop_rule == 1)
    for (int p = 0; p < nprob; ++p)
      if (kx2[p] == 0.0) z = mg_left_null(c);
#pragma omp parallel
  {
    ekref::Mud2cr mg(c->mud);
#pragma omp for schedule(dynamic, 1)
    for (int p = 0; p < nprob; ++p) {
      mg.discretize(make_cofcr(c, kx2[p]));
      std::fill(phi + p * n, phi + (p + 1) * n, 0.0);  // P_TMP = 0
      res[p] = mg.solve(rhs + p * n, phi + p * n, kx2[p] == 0.0, z);
    }
  }
  ek_mg_stats s{};
  s.nprob = nprob;
  s.min_cycles = nprob ? 1 << 30 : 0;
  for (int p = 0; p < nprob; ++p) {
    s.min_cycles = std::min(s.min_cycles, res[p].cycles);
    s.max_cycles = std::max(s.max_cycles, res[p].cycles);
    if (!res[p].converged) s.n_not_converged++;
    s.max_relchange = std::max(s.max_relchange, res[p].relmax);
    s.max_residual = std::max(s.max_residual, res[p].resid);
  }
  c->last_stats = s;
  if (st) *st = s;
  return s.n_not_converged ? EK_ERR_NOT_CONVERGED : EK_OK;
}

extern "C" int ekref_poisson_batch(ekref_ctx *c, const double *rhs, double *phi, const double *kx2, int nprob,
                                   ek_mg_stats *st) {
  if (!c->have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
  return mg_batch(c, rhs, phi, kx2, nprob, st);
}

extern "C" int ekref_mg_apply(ekref_ctx *c, double kx2, const double *phi, double *out) {
  if (!c->have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
  ekref::Mud2cr mg(c->mud);
  mg.discretize(make_cofcr(c, kx2));
  mg.apply_finest(phi, out);
  return EK_OK;
}

extern "C" int ekref_mg_left_null(ekref_ctx *c, double *z) {
  if (!c->have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
  const double *v = mg_left_null(c);
  std::copy(v, v + c->mg_z.size(), z);
  return EK_OK;
}

// ---------------------------------------------------------------------------
// REM_DIV_CURV (duct.F90:2472-2818)
extern "C" int ekref_rem_div(ekref_ctx *c) {
  if (!c->have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
  const int NX2P = c->NX2P, JS = c->JSTART, JE = c->JEND, ZS = c->ZSTART, ZE = c->ZEND;
  const int NY = c->NY, NZ = c->NZ;
  std::fill(c->CR1.begin(), c->CR1.end(), cplx{0, 0});
  std::fill(c->CS1.begin(), c->CS1.end(), cplx{0, 0});
  std::fill(c->CU2b.begin(), c->CU2b.end(), cplx{0, 0});
  std::fill(c->CU3b.begin(), c->CU3b.end(), cplx{0, 0});
  auto &CU1 = c->CU1, &CU2 = c->CU2, &CU3 = c->CU3, &CR1 = c->CR1, &CS1 = c->CS1, &CU2b = c->CU2b, &CU3b = c->CU3b;
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE + 1; ++j)
    for (int k = ZS; k <= ZE + 1; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        CU2b[c->ic(i, k, j)] = cadd(cscale(0.5 * c->M3(c->cjob_22, k, j, 1), cadd(CU2[c->ic(i, k, j)], CU2[c->ic(i, k, j - 1)])),
                                    cscale(0.5 * c->M3(c->cjob_21, k, j, 1), cadd(CU3[c->ic(i, k, j)], CU3[c->ic(i, k, j - 1)])));
        CU3b[c->ic(i, k, j)] = cadd(cscale(0.5 * c->M3(c->cjob_11, k, j, 2), cadd(CU3[c->ic(i, k, j)], CU3[c->ic(i, k - 1, j)])),
                                    cscale(0.5 * c->M3(c->cjob_12, k, j, 2), cadd(CU2[c->ic(i, k, j)], CU2[c->ic(i, k - 1, j)])));
      }
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS - 1; k <= ZE; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        const cplx ikj = cmul(cplx{0.0, c->KXP[i]}, cplx{c->JAC(k, j), 0.0});  // CIKXP(I)*INT_JACOB(K,J)
        CR1[c->ic(i, k, j)] = cadd(cadd(cmul(ikj, CU1[c->ic(i, k, j)]), csub(CU2b[c->ic(i, k, j + 1)], CU2b[c->ic(i, k, j)])),
                                   csub(CU3b[c->ic(i, k + 1, j)], CU3b[c->ic(i, k, j)]));
        CS1[c->ic(i, k, j)] = CR1[c->ic(i, k, j)];
      }
  // Per-kx solves, imaginary part then real part (duct.F90:2620-2669).
  // The first-call warm-up solve (duct.F90:2574-2614) leaves no state behind
  // and is not repeated here.
  const int nmode = NX2P + 1;
  const size_t n = (size_t)(NZ + 2) * (NY + 2);
  std::vector<double> rhs(2 * nmode * n, 0.0), phi(2 * nmode * n, 0.0), kx2(2 * nmode);
  for (int i = 0; i < nmode; ++i) {
    kx2[2 * i] = c->KX2P[i];
    kx2[2 * i + 1] = c->KX2P[i];
    for (int k = ZS; k <= ZE; ++k)
      for (int j = JS; j <= JE; ++j) {
        // RHS_TMP = -Im / -Re and phi_bc negates it again
        rhs[(2 * i) * n + (size_t)j * (NZ + 2) + k] = -(-CR1[c->ic(i, k, j)].im);
        rhs[(2 * i + 1) * n + (size_t)j * (NZ + 2) + k] = -(-CR1[c->ic(i, k, j)].re);
      }
  }
  const int st = mg_batch(c, rhs.data(), phi.data(), kx2.data(), 2 * nmode, nullptr);
  for (int i = 0; i < nmode; ++i)
    for (int j = 0; j <= NY + 1; ++j)
      for (int k = 0; k <= NZ + 1; ++k) {
        double re = phi[(2 * i + 1) * n + (size_t)j * (NZ + 2) + k];
        double im = phi[(2 * i) * n + (size_t)j * (NZ + 2) + k];
        if (c->p.quirk_phi_fp32) {  // CMPLX(P_TMP2,P_TMP) without KIND (duct.F90:2664)
          re = (double)(float)re;
          im = (double)(float)im;
        }
        CR1[c->ic(i, k, j)] = cplx{re, im};
      }
  // face-velocity correction (duct.F90:2709-2724)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        auto P = [&](int kk, int jj) { return CR1[c->ic(i, kk, jj)]; };
        CU2b[c->ic(i, k, j)] = csub(csub(CU2b[c->ic(i, k, j)], cscale(c->M3(c->gmat_22, k, j, 1), csub(P(k, j), P(k, j - 1)))),
                                    cscale(0.25 * c->M3(c->gmat_12, k, j, 1),
                                           csub(csub(cadd(P(k + 1, j), P(k + 1, j - 1)), P(k - 1, j)), P(k - 1, j - 1))));
        CU3b[c->ic(i, k, j)] = csub(csub(CU3b[c->ic(i, k, j)], cscale(c->M3(c->gmat_11, k, j, 2), csub(P(k, j), P(k - 1, j)))),
                                    cscale(0.25 * c->M3(c->gmat_12, k, j, 2),
                                           csub(csub(cadd(P(k, j + 1), P(k - 1, j + 1)), P(k, j - 1)), P(k - 1, j - 1))));
      }
  // cell-centre correction (duct.F90:2729-2750)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        auto P = [&](int kk, int jj) { return CR1[c->ic(i, kk, jj)]; };
        const double jac = c->JAC(k, j);
        CU1[c->ic(i, k, j)] = csub(CU1[c->ic(i, k, j)], cmul(cplx{0.0, c->KXP[i]}, P(k, j)));
        // Fortran term order: a - b + c - d
        const cplx t2 = csub(cadd(csub(cscale(c->M3(c->cjob_22, k, j + 1, 1), cadd(P(k, j), P(k, j + 1))),
                            cscale(c->M3(c->cjob_22, k, j, 1), cadd(P(k, j), P(k, j - 1)))),
                       cscale(c->M3(c->cjob_12, k + 1, j, 2), cadd(P(k + 1, j), P(k, j)))),
                  cscale(c->M3(c->cjob_12, k, j, 2), cadd(P(k, j), P(k - 1, j))));
        const cplx u2c = cscale(0.5, t2);
        CU2[c->ic(i, k, j)] = csub(CU2[c->ic(i, k, j)], cplx{u2c.re / jac, u2c.im / jac});
        cplx t3 = csub(cadd(csub(cscale(c->M3(c->cjob_11, k + 1, j, 2), cadd(P(k, j), P(k + 1, j))),
                                 cscale(c->M3(c->cjob_11, k, j, 2), cadd(P(k, j), P(k - 1, j)))),
                            cscale(c->M3(c->cjob_21, k, j + 1, 1), cadd(P(k, j + 1), P(k, j)))),
                       cscale(c->M3(c->cjob_21, k, j, 1), cadd(P(k, j), P(k, j - 1))));
        const cplx u3c = cscale(0.5, t3);
        CU3[c->ic(i, k, j)] = csub(CU3[c->ic(i, k, j)], cplx{u3c.re / jac, u3c.im / jac});
      }
  // divergence after projection (duct.F90:2754-2806)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        const cplx ikj = cmul(cplx{0.0, c->KXP[i]}, cplx{c->JAC(k, j), 0.0});
        CS1[c->ic(i, k, j)] = cadd(cadd(cmul(ikj, CU1[c->ic(i, k, j)]), csub(CU2b[c->ic(i, k, j + 1)], CU2b[c->ic(i, k, j)])),
                                   csub(CU3b[c->ic(i, k + 1, j)], CU3b[c->ic(i, k, j)]));
      }
  to_physical(c, CS1, c->S1, 0, NY + 1, 0, NZ + 1);
  std::vector<double> part(NY + 2, 0.0);
#pragma omp parallel for schedule(static)
  for (int j = 2; j <= NY - 1; ++j) {
    double s = 0.0;
    for (int k = 2; k <= NZ - 1; ++k)
      for (int i = 1; i <= c->NXP; ++i) s += std::fabs(c->S1[c->ip(i, k, j)]);
    part[j] = s;
  }
  double div = 0.0;
  for (int j = 2; j <= NY - 1; ++j) div += part[j];
  div = div / ((double)(c->NXP) * (double)NY * (double)NZ);
  c->last_div = div;
  if (std::isnan(div)) return fail(c, EK_ERR_NAN, "DIV is a NaN");
  // IF (DELTA_T .LT. 1.0E-4) STOP 'DELTA_T is zero' (duct.F90:2812), a REAL*4 bound
  if (c->p.delta_t < static_cast<double>(1.0e-4f)) return fail(c, EK_ERR_DT, "DELTA_T is zero");
  return st == EK_ERR_NOT_CONVERGED ? EK_OK : st;  // the reference ignores ierror
}

extern "C" int ekref_last_divergence(ekref_ctx *c, double *d) {
  *d = c->last_div;
  return EK_OK;
}
extern "C" int ekref_last_mg_stats(ekref_ctx *c, ek_mg_stats *s) {
  *s = c->last_stats;
  return EK_OK;
}

// Nonlinear + cross-diffusion flux of a field phi (duct.F90:735-761 for U1):
// S1 = -(U2b-flux) + 1/4 nu G12 terms ; S2 likewise in zeta ; S1 += S2.
static void flux_terms(ekref_ctx *c, const std::vector<double> &phi, double visc, int js, int je, int zs, int ze) {
  auto &S1 = c->S1, &S2 = c->S2, &U2b = c->U2b, &U3b = c->U3b;
#pragma omp parallel for schedule(static)
  for (int j = js; j <= je; ++j)
    for (int k = zs; k <= ze; ++k) {
      const double g12a = c->M3(c->gmat_12, k + 1, j, 2), g12b = c->M3(c->gmat_12, k, j, 2);
      const double g12c = c->M3(c->gmat_12, k, j + 1, 1), g12d = c->M3(c->gmat_12, k, j, 1);
      for (int i = 0; i <= c->NXP; ++i) {
        auto F = [&](int kk, int jj) { return phi[c->ip(i, kk, jj)]; };
        double s1 = 0.5 * U2b[c->ip(i, k, j + 1)] * (F(k, j) + F(k, j + 1)) - 0.5 * U2b[c->ip(i, k, j)] * (F(k, j) + F(k, j - 1));
        double s2 = 0.5 * U3b[c->ip(i, k + 1, j)] * (F(k, j) + F(k + 1, j)) - 0.5 * U3b[c->ip(i, k, j)] * (F(k, j) + F(k - 1, j));
        s1 = -s1 + 0.25 * visc * (g12a * (F(k + 1, j + 1) + F(k, j + 1) - F(k, j - 1) - F(k + 1, j - 1)) -
                                  g12b * (F(k - 1, j + 1) + F(k, j + 1) - F(k, j - 1) - F(k - 1, j - 1)));
        s2 = -s2 + 0.25 * visc * (g12c * (F(k + 1, j + 1) + F(k + 1, j) - F(k - 1, j + 1) - F(k - 1, j)) -
                                  g12d * (F(k + 1, j) + F(k + 1, j - 1) - F(k - 1, j) - F(k - 1, j - 1)));
        S1[c->ip(i, k, j)] = s1 + s2;
        S2[c->ip(i, k, j)] = s2;
      }
    }
}

// CF(i) -= CIKXP*CS1 over the range
static void sub_ik(ekref_ctx *c, std::vector<cplx> &CF, const std::vector<cplx> &CS, int js, int je, int zs, int ze) {
#pragma omp parallel for schedule(static)
  for (int j = js; j <= je; ++j)
    for (int k = zs; k <= ze; ++k)
      for (int i = 0; i <= c->NX2P; ++i)
        CF[c->ic(i, k, j)] = csub(CF[c->ic(i, k, j)], cmul(cplx{0.0, c->KXP[i]}, CS[c->ic(i, k, j)]));
}
static void add_c(ekref_ctx *c, std::vector<cplx> &CF, const std::vector<cplx> &CS, int js, int je, int zs, int ze) {
#pragma omp parallel for schedule(static)
  for (int j = js; j <= je; ++j)
    for (int k = zs; k <= ze; ++k)
      for (int i = 0; i <= c->NX2P; ++i) CF[c->ic(i, k, j)] = cadd(CF[c->ic(i, k, j)], CS[c->ic(i, k, j)]);
}

// RK_DUCT (duct.F90:237-2469)
extern "C" int ekref_rk_substep(ekref_ctx *c, int rk) {
  if (!c->have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
  if (rk < 1 || rk > 3) return fail(c, EK_ERR_ARG, "rk_step must be 1..3");
  if (c->p.les && !c->have_les_metrics) return fail(c, EK_ERR_STATE, "LES metrics not set");
  const ek_params &p = c->p;
  const int NX2P = c->NX2P, NXP = c->NXP, NY = c->NY, NZ = c->NZ;
  const int JS = c->JSTART, JE = c->JEND, ZS = c->ZSTART, ZE = c->ZEND;
  const int JST = c->JSTART_TH, JET = c->JEND_TH, ZST = c->ZSTART_TH, ZET = c->ZEND_TH;
  const double NU = p.nu;
  const double TEMP1 = NU * c->H_BAR[rk] / 2.0;
  const double TEMP2 = c->H_BAR[rk] / 2.0;
  const double TEMP3 = c->ZETA_BAR[rk] * c->H_BAR[rk];
  const double TEMP4 = c->H_BAR[rk];
  const double TEMP5 = c->BETA_BAR[rk] * c->H_BAR[rk];
  auto &CU1 = c->CU1, &CU2 = c->CU2, &CU3 = c->CU3, &CP = c->CP, &CTH = c->CTH;
  auto &CF1 = c->CF1, &CF2 = c->CF2, &CF3 = c->CF3, &CFTH = c->CFTH;
  auto &CR1 = c->CR1, &CR2 = c->CR2, &CR3 = c->CR3, &CRTH = c->CRTH, &CS1 = c->CS1, &CS2 = c->CS2;
  const bool th = p.n_th > 0;

  // (a1) explicit RHS in Fourier space (duct.F90:299-409)
  for (auto *v : {&CR1, &CR2, &CR3}) std::fill(v->begin(), v->end(), cplx{0, 0});
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k) {
      const double jac = c->JAC(k, j);
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        CR1[q] = cscale(jac, CU1[q]);
        CR2[q] = cscale(jac, CU2[q]);
        CR3[q] = cscale(jac, CU3[q]);
        if (rk > 1) {
          CR1[q] = cadd(CR1[q], cscale(TEMP3, CF1[q]));
          CR2[q] = cadd(CR2[q], cscale(TEMP3, CF2[q]));
          CR3[q] = cadd(CR3[q], cscale(TEMP3, CF3[q]));
        }
      }
    }
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        auto P = [&](int kk, int jj) { return CP[c->ic(i, kk, jj)]; };
        const size_t q = c->ic(i, k, j);
        // a - b + c - d in Fortran order
        CS1[q] = csub(cadd(csub(cscale(0.5 * c->M3(c->cjob_11, k + 1, j, 2), cadd(P(k, j), P(k + 1, j))),
                                cscale(0.5 * c->M3(c->cjob_11, k, j, 2), cadd(P(k, j), P(k - 1, j)))),
                           cscale(0.5 * c->M3(c->cjob_21, k, j + 1, 1), cadd(P(k, j), P(k, j + 1)))),
                      cscale(0.5 * c->M3(c->cjob_21, k, j, 1), cadd(P(k, j), P(k, j - 1))));
        CS2[q] = csub(cadd(csub(cscale(0.5 * c->M3(c->cjob_12, k + 1, j, 2), cadd(P(k, j), P(k + 1, j))),
                                cscale(0.5 * c->M3(c->cjob_12, k, j, 2), cadd(P(k, j), P(k - 1, j)))),
                           cscale(0.5 * c->M3(c->cjob_22, k, j + 1, 1), cadd(P(k, j), P(k, j + 1)))),
                      cscale(0.5 * c->M3(c->cjob_22, k, j, 1), cadd(P(k, j), P(k, j - 1))));
        // CR1 -= TEMP4*CIKXP*J*CP ; CR2 -= TEMP4*CS2 ; CR3 -= TEMP4*CS1
        const cplx t = cmul(cscale(c->JAC(k, j), cscale(TEMP4, cplx{0.0, c->KXP[i]})), P(k, j));
        CR1[q] = csub(CR1[q], t);
        CR2[q] = csub(CR2[q], cscale(TEMP4, CS2[q]));
        CR3[q] = csub(CR3[q], cscale(TEMP4, CS1[q]));
      }
  // mean-pressure forcing on mode 0 (duct.F90:411-455)
  if (p.f_type == 1 || p.f_type == 2) {
    const double px = (p.f_type == 1) ? p.px0 : (p.px0 + p.amp_omega0 * std::cos(p.omega0 * p.time));
    for (int j = JS; j <= JE; ++j)
      for (int k = ZS; k <= ZE; ++k) {
        const size_t q = c->ic(0, k, j);
        CR3[q] = csub(CR3[q], cplx{TEMP4 * px * c->JAC(k, j), 0.0});
      }
  }
  // (a1,a2) explicit terms CF (duct.F90:461-523)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k) {
      const double jac = c->JAC(k, j);
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        const double v = -NU * c->KX2P[i] * jac;
        CF1[q] = cscale(v, CU1[q]);
        CF2[q] = cscale(v, CU2[q]);
        CF3[q] = cscale(v, CU3[q]);
        // Coriolis on every kx (quirk of the reference, duct.F90:471-473)
        CF3[q] = cadd(CF3[q], cscale(jac, cscale(p.f0, cplx{CU1[q].re - p.u_bc_c1[EK_YMAX], CU1[q].im})));
        CF1[q] = csub(CF1[q], cscale(jac, cscale(p.f0, cplx{CU3[q].re - p.wbulk0, CU3[q].im})));
        if (th) CF2[q] = csub(CF2[q], cscale(jac * p.ri_tau, CTH[c->ic(i, k, j)]));
      }
    }
  if (th) {
    const double nupr = NU / p.pr;
    std::fill(CRTH.begin(), CRTH.end(), cplx{0, 0});
#pragma omp parallel for schedule(static)
    for (int j = JST; j <= JET; ++j)
      for (int k = ZST; k <= ZET; ++k) {
        const double jac = c->JAC(k, j);
        for (int i = 0; i <= NX2P; ++i) {
          const size_t q = c->ic(i, k, j);
          CRTH[q] = cscale(jac, CTH[q]);
          if (rk > 1) CRTH[q] = cadd(CRTH[q], cscale(TEMP3, CFTH[q]));
          CFTH[q] = cscale(-nupr * jac * c->KX2P[i], CTH[q]);
          if (p.cont_strat) {
            CFTH[q] = cadd(CFTH[q], cscale(jac, CU2[q]));
          } else {
            auto TB = [&](int kk, int jj) { return c->M2(c->th_bar, kk, jj); };
            const double g = 0.5 * c->M3(c->cjob_12, k + 1, j, 2) * (TB(k, j) + TB(k + 1, j)) -
                             0.5 * c->M3(c->cjob_12, k, j, 2) * (TB(k, j) + TB(k - 1, j)) +
                             0.5 * c->M3(c->cjob_22, k, j + 1, 1) * (TB(k, j) + TB(k, j + 1)) -
                             0.5 * c->M3(c->cjob_22, k, j, 1) * (TB(k, j) + TB(k, j - 1));
            CFTH[q] = csub(CFTH[q], cscale(g, CU2[q]));
            // with LES the coefficient takes KAPPA_T at the physical point
            // whose x index equals the mode index (duct.F90:610-618)
            const double kap = p.les ? (nupr + c->KAPPA_T[c->ip(i, k, j)]) : nupr;
            const double d =
                0.25 * kap *
                (+c->M3(c->gmat_12, k + 1, j, 2) * (TB(k + 1, j + 1) + TB(k, j + 1) - TB(k, j - 1) - TB(k + 1, j - 1)) -
                 c->M3(c->gmat_12, k, j, 2) * (TB(k - 1, j + 1) + TB(k, j + 1) - TB(k, j - 1) - TB(k - 1, j - 1)) +
                 c->M3(c->gmat_12, k, j + 1, 1) * (TB(k + 1, j + 1) + TB(k + 1, j) - TB(k - 1, j + 1) - TB(k - 1, j)) -
                 c->M3(c->gmat_12, k, j, 1) * (TB(k + 1, j) + TB(k + 1, j - 1) - TB(k - 1, j) - TB(k - 1, j - 1)) +
                 4.0 * (c->M3(c->gmat_11, k + 1, j, 2) * (TB(k + 1, j) - TB(k, j)) - c->M3(c->gmat_11, k, j, 2) * (TB(k, j) - TB(k - 1, j))) +
                 4.0 * (c->M3(c->gmat_22, k, j + 1, 1) * (TB(k, j + 1) - TB(k, j)) - c->M3(c->gmat_22, k, j, 1) * (TB(k, j) - TB(k, j - 1))));
            CFTH[q] = cadd(CFTH[q], cplx{d, 0.0});
          }
        }
      }
  }
  if (th && p.sponge_type != 0) sponge_th(c);  // duct.F90:635, inside the scalar loop
  const bool les = c->les_active();
  if (les) {
    // les_chan / les_chan_th (duct.F90:641-654) leave the fields in physical space
    les_chan(c, rk);
    if (th) les_chan_th(c);
  } else {
    // to physical space (duct.F90:656-673)
    to_physical(c, CU1, c->U1, 0, NY + 1, 0, NZ + 1);
    to_physical(c, CU2, c->U2, 0, NY + 1, 0, NZ + 1);
    to_physical(c, CU3, c->U3, 0, NY + 1, 0, NZ + 1);
    if (th) to_physical(c, CTH, c->TH, 0, NY + 1, 0, NZ + 1);
  }
  auto &U1 = c->U1, &U2 = c->U2, &U3 = c->U3, &TH = c->TH, &S1 = c->S1;

  // nonlinear terms (duct.F90:683-1121)
  auto product = [&](const std::vector<double> &a, const std::vector<double> &b, int js, int je, int zs, int ze) {
#pragma omp parallel for schedule(static)
    for (int j = js; j <= je; ++j)
      for (int k = zs; k <= ze; ++k) {
        const double jac = c->JAC(k, j);
        for (int i = 0; i <= NXP; ++i) S1[c->ip(i, k, j)] = jac * a[c->ip(i, k, j)] * b[c->ip(i, k, j)];
      }
  };
  product(U1, U1, JS, JE, ZS, ZE);
  to_fourier(c, S1, CS1, JS, JE, ZS, ZE);
  sub_ik(c, CF1, CS1, JS, JE, ZS, ZE);
  // contravariant face velocities (duct.F90:721-732)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE + 1; ++j)
    for (int k = ZS; k <= ZE + 1; ++k)
      for (int i = 0; i <= NXP; ++i) {
        c->U2b[c->ip(i, k, j)] = 0.5 * c->M3(c->cjob_22, k, j, 1) * (U2[c->ip(i, k, j)] + U2[c->ip(i, k, j - 1)]) +
                                 0.5 * c->M3(c->cjob_21, k, j, 1) * (U3[c->ip(i, k, j)] + U3[c->ip(i, k, j - 1)]);
        c->U3b[c->ip(i, k, j)] = 0.5 * c->M3(c->cjob_11, k, j, 2) * (U3[c->ip(i, k, j)] + U3[c->ip(i, k - 1, j)]) +
                                 0.5 * c->M3(c->cjob_12, k, j, 2) * (U2[c->ip(i, k, j)] + U2[c->ip(i, k - 1, j)]);
      }
  flux_terms(c, U1, NU, JS, JE, ZS, ZE);
  to_fourier(c, S1, CS1, JS, JE, ZS, ZE);
  add_c(c, CF1, CS1, JS, JE, ZS, ZE);
  product(U1, U2, JS, JE, ZS, ZE);
  to_fourier(c, S1, CS1, JS, JE, ZS, ZE);
  sub_ik(c, CF2, CS1, JS, JE, ZS, ZE);
  flux_terms(c, U2, NU, JS, JE, ZS, ZE);
  to_fourier(c, S1, CS1, JS, JE, ZS, ZE);
  add_c(c, CF2, CS1, JS, JE, ZS, ZE);
  product(U1, U3, JS, JE, ZS, ZE);
  to_fourier(c, S1, CS1, JS, JE, ZS, ZE);
  sub_ik(c, CF3, CS1, JS, JE, ZS, ZE);
  flux_terms(c, U3, NU, JS, JE, ZS, ZE);
  to_fourier(c, S1, CS1, JS, JE, ZS, ZE);
  add_c(c, CF3, CS1, JS, JE, ZS, ZE);
  if (les) les_cross_terms(c);  // duct.F90:990-1120
  // CR += TEMP5*CF (duct.F90:1127-1149), R to physical
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        CR1[q] = cadd(CR1[q], cscale(TEMP5, CF1[q]));
        CR2[q] = cadd(CR2[q], cscale(TEMP5, CF2[q]));
        CR3[q] = cadd(CR3[q], cscale(TEMP5, CF3[q]));
      }
  to_physical(c, CR1, c->R1, JS, JE, ZS, ZE);
  to_physical(c, CR2, c->R2, JS, JE, ZS, ZE);
  to_physical(c, CR3, c->R3, JS, JE, ZS, ZE);
  if (th) {
    product(TH, U1, JST, JET, ZST, ZET);
    to_fourier(c, S1, CS1, JST, JET, ZST, ZET);
    sub_ik(c, CFTH, CS1, JST, JET, ZST, ZET);
    flux_terms(c, TH, NU / p.pr, JST, JET, ZST, ZET);
    to_fourier(c, S1, CS1, JST, JET, ZST, ZET);
    add_c(c, CFTH, CS1, JST, JET, ZST, ZET);
    if (les) les_cross_terms_th(c);  // duct.F90:1266-1311
#pragma omp parallel for schedule(static)
    for (int j = JST; j <= JET; ++j)
      for (int k = ZST; k <= ZET; ++k)
        for (int i = 0; i <= NX2P; ++i) {
          const size_t q = c->ic(i, k, j);
          CRTH[q] = cadd(CRTH[q], cscale(TEMP5, CFTH[q]));
        }
    to_physical(c, CRTH, c->RTH, JST, JET, ZST, ZET);
    // ADI for TH (duct.F90:1334-1625), then corner copies (1610-1624)
    const LesAdi la{&c->KAPPA_T, &c->gmat_11, &c->gmat_22, TEMP2};
    adi_field(c, 0, TEMP1 / p.pr, TH, c->RTH, JST, JET, ZST, ZET, les ? &la : nullptr);
    if (p.th_bc[EK_ZMAX] == 1)
      for (int i = 0; i <= NXP; ++i) {
        TH[c->ip(i, NZ + 1, NY + 1)] = TH[c->ip(i, NZ, NY + 1)];
        TH[c->ip(i, NZ + 1, 0)] = TH[c->ip(i, NZ, 0)];
        TH[c->ip(i, 0, NY + 1)] = TH[c->ip(i, 1, NY + 1)];
        TH[c->ip(i, 0, 0)] = TH[c->ip(i, 1, 0)];
      }
    if (p.th_bc[EK_ZMIN] == 6)
      for (int i = 0; i <= NXP; ++i) {
        TH[c->ip(i, NZ + 1, NY + 1)] = TH[c->ip(i, 1, NY + 1)];
        TH[c->ip(i, NZ + 1, 0)] = TH[c->ip(i, 1, 0)];
        TH[c->ip(i, 0, NY + 1)] = TH[c->ip(i, NZ, NY + 1)];
        TH[c->ip(i, 0, 0)] = TH[c->ip(i, NZ, 0)];
      }
  }
  const LesAdi l1{&c->NU_T, &c->gmat_11, &c->gmat_22, TEMP2}, l2{&c->NU_T, &c->g11y, &c->g22y, TEMP2},
      l3{&c->NU_T, &c->g11z, &c->g22z, TEMP2};
  adi_field(c, 1, TEMP1, U1, c->R1, JS, JE, ZS, ZE, les ? &l1 : nullptr);
  adi_field(c, 2, TEMP1, U2, c->R2, JS, JE, ZS, ZE, les ? &l2 : nullptr);
  adi_field(c, 3, TEMP1, U3, c->R3, JS, JE, ZS, ZE, les ? &l3 : nullptr);
  // COURANT_CURV_MPI (duct.F90:2417-2419, 3605-3674)
  if (p.variable_dt && rk == 3 && p.time_step % p.update_dt == 0) {
    double dt = 999.0;
    const double dx = p.lx / (double)c->NX;
    for (int j = JS; j <= JE; ++j)
      for (int k = ZS; k <= ZE; ++k)
        for (int i = 0; i <= NXP; ++i) {
          const size_t q = c->ip(i, k, j), qj = c->ip(i, k, j - 1), qk = c->ip(i, k - 1, j);
          const double u2b = 0.5 * c->M3(c->cjob_22, k, j, 1) * (U2[q] + U2[qj]) +
                             0.5 * c->M3(c->cjob_21, k, j, 1) * (U3[q] + U3[qj]);
          const double u3b = 0.5 * c->M3(c->cjob_11, k, j, 2) * (U3[q] + U3[qk]) +
                             0.5 * c->M3(c->cjob_12, k, j, 2) * (U2[q] + U2[qk]);
          const double dt_x = p.cfl * dx / std::fabs(U1[q]);
          const double dt_y = p.cfl * c->JAC(k, j) / std::fabs(u2b);
          const double dt_z = p.cfl * c->JAC(k, j) / std::fabs(u3b);
          dt = std::min(std::min(std::min(dt, dt_x), dt_y), dt_z);
        }
    if (dt > 0.0) {
      c->p.delta_t = (dt >= p.delta_t_set) ? p.delta_t_set : dt;
      c->H_BAR[1] = c->p.delta_t * (8.0 / 15.0);
      c->H_BAR[2] = c->p.delta_t * (2.0 / 15.0);
      c->H_BAR[3] = c->p.delta_t * (5.0 / 15.0);
    }
  }
  // back to Fourier space (duct.F90:2421-2451)
  to_fourier(c, U1, CU1, 0, NY + 1, 0, NZ + 1);
  to_fourier(c, U2, CU2, 0, NY + 1, 0, NZ + 1);
  to_fourier(c, U3, CU3, 0, NY + 1, 0, NZ + 1);
  if (th) to_fourier(c, TH, CTH, 0, NY + 1, 0, NZ + 1);
  // projection and pressure update (duct.F90:2455-2466)
  const int st = ekref_rem_div(c);
  if (st != EK_OK) return st;
#pragma omp parallel for schedule(static)
  for (int j = JS - 1; j <= JE + 1; ++j)
    for (int k = ZS - 1; k <= ZE + 1; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        CP[q] = cadd(CP[q], cplx{CR1[q].re / TEMP4, CR1[q].im / TEMP4});
      }
  return EK_OK;
}

extern "C" int ekref_step(ekref_ctx *c, int nsteps) {
  for (int n = 0; n < nsteps; ++n) {
    c->p.time_step += 1;  // DO TIME_STEP = TIME_STEP+1, ... (diablo.F90:109)
    for (int rk = 1; rk <= 3; ++rk) {
      const int st = ekref_rk_substep(c, rk);
      if (st != EK_OK) return st;
    }
    c->p.time += c->p.delta_t;
    c->first_time = false;  // diablo.F90:157
  }
  return EK_OK;
}

// ---------------------------------------------------------------------------
// SAVE_STATS_CURVI (flow_statistics.F90:2-1023) with NP = 1 and N_TH <= 1:
// the plane statistics and the state round trip; the file output
// (time_bulk.txt, plot_binary, Tecplot, plane dumps) and the TKE budget are
// left out.  Loops and expression order follow the Fortran; arrays the
// reference leaves unassigned after ALLOCATE are zero.
extern "C" int ekref_save_stats(ekref_ctx *c, ek_stats *st) {
  if (!c->have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
  const int NX = c->NX, NY = c->NY, NZ = c->NZ, NZ2 = c->NZ2;
  const size_t n2 = (size_t)c->NZ2 * c->NY2;
  const bool th = c->p.n_th > 0;
  auto pl = [&]() { return std::vector<double>(n2, 0.0); };
  auto A = [&](std::vector<double> &a, int k, int j) -> double & { return a[(size_t)j * NZ2 + k]; };
  // CR*X = CU*X (flow_statistics.F90:99-112; the MPI broadcasts are copies)
  const std::vector<cplx> CR1 = c->CU1, CR2 = c->CU2, CR3 = c->CU3;
  auto R1 = [&](int k, int j) { return CR1[c->ic(0, k, j)].re; };
  auto R2 = [&](int k, int j) { return CR2[c->ic(0, k, j)].re; };
  auto R3 = [&](int k, int j) { return CR3[c->ic(0, k, j)].re; };
  // UBULK, VBULK (:80-95)
  double ubulk = 0.0, vbulk = 0.0;
  for (int J = 1; J <= NY; ++J)
    for (int K = 1; K <= NZ; ++K) {
      ubulk = ubulk + 0.25 * (R3(K, J) + R3(K - 1, J) + R3(K - 1, J - 1) + R3(K, J - 1));
      vbulk = vbulk + 0.25 * (R1(K, J) + R1(K - 1, J) + R1(K - 1, J - 1) + R1(K, J - 1));
    }
  const double ncell = (double)(float)(NY * NZ);
  ubulk = ubulk / ncell;
  vbulk = vbulk / ncell;
  std::vector<double> p_mean = pl();
  for (int k = 1; k <= NZ; ++k)
    for (int j = 1; j <= NY; ++j) A(p_mean, k, j) = c->CP[c->ic(0, k, j)].re;
  // to physical space (:156-160); P into the scratch S1
  to_physical(c, c->CU1, c->U1, 0, NY + 1, 0, NZ + 1);
  to_physical(c, c->CU2, c->U2, 0, NY + 1, 0, NZ + 1);
  to_physical(c, c->CU3, c->U3, 0, NY + 1, 0, NZ + 1);
  to_physical(c, c->CP, c->S1, 0, NY + 1, 0, NZ + 1);
  const std::vector<double> &U1 = c->U1, &U2 = c->U2, &U3 = c->U3, &PX = c->S1;
  std::vector<double> tke = pl(), urms = pl(), vrms = pl(), wrms = pl();
  std::vector<double> uv = pl(), uw = pl(), wv = pl(), pu = pl(), pv = pl();
  const bool scaled = c->p.amp_omega0 != 0.0;
  const double fac = scaled ? std::pow(c->p.amp_omega0 / c->p.omega0, -2.0) : 1.0;
  for (int k = 0; k <= NZ + 1; ++k)
    for (int j = 0; j <= NY + 1; ++j) {
      const double e = R1(k, j) * R1(k, j) + R2(k, j) * R2(k, j) + R3(k, j) * R3(k, j);
      A(tke, k, j) = scaled ? e * fac : e;
    }
  const int imax = NX - 1;  // MIN(NXP, NXP_L) on rank 0
  for (int k = 0; k <= NZ + 1; ++k)
    for (int j = 0; j <= NY + 1; ++j) {
      double su = 0.0, sv = 0.0, sw = 0.0;
      for (int i = 0; i <= imax; ++i) {
        const double a = U1[c->ip(i, k, j)] - R1(k, j), b = U2[c->ip(i, k, j)] - R2(k, j);
        const double w = U3[c->ip(i, k, j)] - R3(k, j);
        su = su + a * a;
        sv = sv + b * b;
        sw = sw + w * w;
      }
      A(urms, k, j) = su;
      A(vrms, k, j) = sv;
      A(wrms, k, j) = sw;
    }
  for (int k = 1; k <= NZ; ++k)
    for (int j = 0; j <= NY + 1; ++j) {
      double s12 = 0.0, s32 = 0.0, s13 = 0.0, s3p = 0.0, s2p = 0.0;
      for (int i = 0; i <= imax; ++i) {
        const size_t q = c->ip(i, k, j);
        const double a = U1[q] - R1(k, j), b = U2[q] - R2(k, j), w = U3[q] - R3(k, j);
        const double pp = PX[q] - A(p_mean, k, j);
        s12 = s12 + a * b;
        s32 = s32 + w * b;
        s13 = s13 + a * w;
        s3p = s3p + w * pp;
        s2p = s2p + b * pp;
      }
      const double nx = (double)(float)NX;
      A(uv, k, j) = s12 / nx;
      A(uw, k, j) = s13 / nx;
      A(wv, k, j) = s32 / nx;
      A(pu, k, j) = s3p / nx;
      A(pv, k, j) = s2p / nx;
    }
  auto cav = [&](const std::vector<double> &m, int K, int J) {
    return 0.125 * (c->M3(m, K, J, 1) + c->M3(m, K, J + 1, 1) + c->M3(m, K, J, 2) + c->M3(m, K + 1, J, 2));
  };
  std::vector<double> dudy = pl(), dwdy = pl(), dudz = pl(), dwdz = pl(), omx = pl();
  for (int K = c->ZSTART; K <= c->ZEND; ++K)
    for (int J = c->JSTART; J <= c->JEND; ++J) {
      const double a12 = cav(c->cjob_12, K, J), a22 = cav(c->cjob_22, K, J);
      A(dudy, K, J) = (a12 * (R1(K + 1, J) - R1(K - 1, J)) + a22 * (R1(K, J + 1) - R1(K, J - 1))) / c->JAC(K, J);
      A(dwdy, K, J) = (a12 * (R3(K + 1, J) - R3(K - 1, J)) + a22 * (R3(K, J + 1) - R3(K, J - 1))) / c->JAC(K, J);
    }
  for (int k = 1; k <= NZ; ++k) {
    A(dudy, k, 0) = A(dudy, k, 1);
    A(dwdy, k, 0) = A(dwdy, k, 1);
    A(dudy, k, NY + 1) = A(dudy, k, NY);
    A(dwdy, k, NY + 1) = A(dwdy, k, NY);
  }
  for (int K = 1; K <= NZ; ++K)
    for (int J = 1; J <= NY; ++J) {
      const double a21 = cav(c->cjob_21, K, J), a11 = cav(c->cjob_11, K, J);
      A(dudz, K, J) = (a21 * (R1(K, J + 1) - R1(K, J - 1)) + a11 * (R1(K + 1, J) - R1(K - 1, J))) / c->JAC(K, J);
      A(dwdz, K, J) = (a21 * (R3(K, J + 1) - R3(K, J - 1)) + a11 * (R3(K + 1, J) - R3(K - 1, J))) / c->JAC(K, J);
    }
  for (int k = 1; k <= NZ; ++k) {
    A(dudz, k, 0) = A(dudz, k, 1);
    A(dwdz, k, 0) = A(dwdz, k, 1);
    A(dudz, k, NY + 1) = A(dudz, k, NY);
    A(dwdz, k, NY + 1) = A(dwdz, k, NY);
  }
  for (int j = 1; j <= NY; ++j) {
    A(dwdz, 1, j) = A(dwdz, 2, j);
    A(dudz, 1, j) = A(dudz, 2, j);
  }
  for (int K = 1; K <= NZ; ++K)
    for (int J = 1; J <= NY; ++J) {
      const double a12 = cav(c->cjob_12, K, J), a22 = cav(c->cjob_22, K, J);
      const double a21 = cav(c->cjob_21, K, J), a11 = cav(c->cjob_11, K, J);
      A(omx, K, J) = (a12 * (R3(K + 1, J) - R3(K - 1, J)) + a22 * (R3(K, J + 1) - R3(K, J - 1))) / c->JAC(K, J) -
                     (a21 * (R2(K, J + 1) - R2(K, J - 1)) + a11 * (R2(K + 1, J) - R2(K - 1, J))) / c->JAC(K, J);
    }
  for (int k = 1; k <= NZ; ++k) {
    A(omx, k, 0) = A(omx, k, 1);
    A(omx, k, NY + 1) = A(omx, k, NY);
  }
  // the scalar (:417-555)
  std::vector<double> thrms = pl(), thv = pl(), thw = pl(), dthdy = pl(), dthdz = pl(), rig = pl();
  double thbulk = 0.0;
  if (th) {
    const std::vector<cplx> CRT = c->CTH;
    auto T = [&](int k, int j) { return CRT[c->ic(0, k, j)].re; };
    auto TB = [&](int k, int j) { return c->M2(c->th_bar, k, j); };
    to_physical(c, c->CTH, c->TH, 0, NY + 1, 0, NZ + 1);
    const std::vector<double> &THX = c->TH;
    for (int j = 0; j <= NY + 1; ++j)
      for (int k = 0; k <= NZ + 1; ++k) {
        double s = 0.0;
        for (int i = 0; i <= imax; ++i) {
          const double a = std::fabs(THX[c->ip(i, k, j)] - T(k, j));
          s = s + a * a;
        }
        A(thrms, k, j) = s;
      }
    for (int k = 1; k <= NZ; ++k)
      for (int j = 1; j <= NY; ++j) {
        const double a12 = cav(c->cjob_12, k, j), a22 = cav(c->cjob_22, k, j);
        A(dthdy, k, j) = (a12 * (T(k + 1, j) - T(k - 1, j)) + a22 * (T(k, j + 1) - T(k, j - 1))) / c->JAC(k, j);
        if (!c->p.cont_strat)
          A(dthdy, k, j) = A(dthdy, k, j) +
                           (a12 * (TB(k + 1, j) - TB(k - 1, j)) + a22 * (TB(k, j + 1) - TB(k, j - 1))) / c->JAC(k, j);
      }
    for (int j = 1; j <= NY; ++j) {
      A(dthdy, 0, j) = A(dthdy, 1, j);
      A(dthdy, NZ + 1, j) = A(dthdy, NZ, j);
    }
    for (int k = 0; k <= NZ + 1; ++k) {
      A(dthdy, k, 0) = 2.0 * A(dthdy, k, 1) - A(dthdy, k, 2);
      A(dthdy, k, NY + 1) = 2.0 * A(dthdy, k, NY) - A(dthdy, k, NY - 1);
    }
    for (int j = 0; j <= NY + 1; ++j)
      for (int k = 0; k <= NZ + 1; ++k) {
        double s2 = 0.0, s3 = 0.0;
        for (int i = 0; i <= imax; ++i) {
          const size_t q = c->ip(i, k, j);
          const double t = THX[q] - T(k, j);
          s2 = s2 + t * (U2[q] - R2(k, j));
          s3 = s3 + t * (U3[q] - R3(k, j));
        }
        A(thv, k, j) = s2 / (double)(float)NX;
        A(thw, k, j) = s3 / (double)(float)NX;
      }
    for (int k = 1; k <= NZ; ++k)
      for (int j = 1; j <= NY; ++j) {
        const double a21 = cav(c->cjob_21, k, j), a11 = cav(c->cjob_11, k, j);
        A(dthdz, k, j) = (a21 * (T(k, j + 1) - T(k, j - 1)) + a11 * (T(k + 1, j) - T(k - 1, j))) / c->JAC(k, j);
      }
    for (int j = 1; j <= NY; ++j) {
      A(dthdz, 0, j) = A(dthdz, 1, j);
      A(dthdz, NZ + 1, j) = A(dthdz, NZ, j);
    }
    for (int k = 0; k <= NZ + 1; ++k) {
      A(dthdz, k, 0) = 2.0 * A(dthdz, k, 1) - A(dthdz, k, 2);
      A(dthdz, k, NY + 1) = 2.0 * A(dthdz, k, NY) - A(dthdz, k, NY - 1);
    }
    const double ri = c->p.ri_tau;
    for (int J = 1; J <= NY; ++J)
      for (int K = 1; K <= NZ; ++K) {
        thbulk = thbulk + 0.25 * (T(K, J) + T(K - 1, J) + T(K - 1, J - 1) + T(K, J - 1));
        const double b = c->p.cont_strat ? A(dthdy, K, J) - 1.0 : A(dthdy, K, J);
        if (A(dwdy, K, J) == 0.0)
          A(rig, K, J) = -ri * b * 1.0e18;
        else
          A(rig, K, J) = -ri * b / (A(dwdy, K, J) * A(dwdy, K, J) + A(dudy, K, J) * A(dudy, K, J));
      }
    thbulk = thbulk / ncell;
    to_fourier(c, c->TH, c->CTH, 0, NY + 1, 0, NZ + 1);  // REAL_FOURIER_TRANS_TH(.true.) (:821)
  }
  // rms and their bulk averages (:846-879), scalar rms (:914-920)
  double ub = 0.0, vb = 0.0, wb = 0.0, area = 0.0;
  for (int k = 0; k <= NZ + 1; ++k)
    for (int j = 0; j <= NY + 1; ++j) {
      A(urms, k, j) = std::sqrt(A(urms, k, j) / (double)NX);
      A(vrms, k, j) = std::sqrt(A(vrms, k, j) / (double)NX);
      A(wrms, k, j) = std::sqrt(A(wrms, k, j) / (double)NX);
    }
  for (int k = 1; k <= NZ; ++k)
    for (int j = 1; j <= NY; ++j) {
      const double J = c->JAC(k, j);
      area = area + J;
      ub = ub + 0.25 * (A(urms, k, j) + A(urms, k, j - 1) + A(urms, k - 1, j) + A(urms, k - 1, j - 1)) * J;
      vb = vb + 0.25 * (A(vrms, k, j) + A(vrms, k, j - 1) + A(vrms, k - 1, j) + A(vrms, k - 1, j - 1)) * J;
      wb = wb + 0.25 * (A(wrms, k, j) + A(wrms, k, j - 1) + A(wrms, k - 1, j) + A(wrms, k - 1, j - 1)) * J;
    }
  if (th)
    for (int j = 0; j <= NY + 1; ++j)
      for (int k = 0; k <= NZ + 1; ++k) A(thrms, k, j) = std::sqrt(A(thrms, k, j) / (double)(float)NX);
  // back to Fourier space and CF1X..CF3X = 0 (:951-963)
  to_fourier(c, c->U1, c->CU1, 0, NY + 1, 0, NZ + 1);
  to_fourier(c, c->U2, c->CU2, 0, NY + 1, 0, NZ + 1);
  to_fourier(c, c->U3, c->CU3, 0, NY + 1, 0, NZ + 1);
  to_fourier(c, c->S1, c->CP, 0, NY + 1, 0, NZ + 1);
  for (auto *f : {&c->CF1, &c->CF2, &c->CF3}) std::fill(f->begin(), f->end(), cplx{0.0, 0.0});
  std::vector<double> m1 = pl(), m2 = pl(), m3 = pl(), mp = pl(), mt = pl();
  for (int k = 0; k <= NZ + 1; ++k)
    for (int j = 0; j <= NY + 1; ++j) {
      A(m1, k, j) = c->CU1[c->ic(0, k, j)].re;
      A(m2, k, j) = c->CU2[c->ic(0, k, j)].re;
      A(m3, k, j) = c->CU3[c->ic(0, k, j)].re;
      A(mp, k, j) = c->CP[c->ic(0, k, j)].re;
      A(mt, k, j) = th ? c->CTH[c->ic(0, k, j)].re : 0.0;
    }
  st->ubulk = ubulk;
  st->vbulk = vbulk;
  st->thbulk = thbulk;
  st->urms_b = ub / area;
  st->vrms_b = vb / area;
  st->wrms_b = wb / area;
  st->u3_probe = U3[c->ip(NX + 1, 2, NY)];
  st->u1_probe = U1[c->ip(NX + 1, 2, NY)];
  auto out = [&](double *dst, const std::vector<double> &src) {
    if (dst) std::copy(src.begin(), src.end(), dst);
  };
  out(st->urms, urms); out(st->vrms, vrms); out(st->wrms, wrms);
  out(st->uv, uv); out(st->uw, uw); out(st->wv, wv); out(st->pu, pu); out(st->pv, pv);
  out(st->tke, tke); out(st->dudy, dudy); out(st->dwdy, dwdy); out(st->dudz, dudz); out(st->dwdz, dwdz);
  out(st->omega_x, omx);
  out(st->thrms, thrms); out(st->thv, thv); out(st->thw, thw); out(st->dthdy, dthdy); out(st->dthdz, dthdz);
  out(st->rig, rig);
  out(st->mean_u1, m1); out(st->mean_u2, m2); out(st->mean_u3, m3); out(st->mean_p, mp); out(st->mean_th, mt);
  return EK_OK;
}
