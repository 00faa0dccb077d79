// Oracle (test infrastructure): the LES subgrid model restated from the
// reference for one MPI rank:
//   les_chan            src/les_chan.F90:1-1622, LES_MODEL_TYPE = 2 (dynamic
//                       Smagorinsky, LES_IMPLICIT = .FALSE. as set at :41)
//   compute_strain_chan src/les_chan.F90:1623-1718
//   les_filter_chan     src/les_chan.F90:1719-1839 through FILTER_VAR
//                       (src/mpi_duct.F90:834-852)
//   les_chan_th         src/les_chan_th.F90:1-461, LES_MODEL_TYPE_TH = 1
//   compute_scalar_grad src/les_chan_th.F90:462-540
//   the GMAT_12 eddy-viscosity cross terms of RK_DUCT (src/duct.F90:990-1120,
//   1266-1311).
// Loop ranges, expression order and the persistent scratch arrays (Sij,
// CSij, S2X) follow the Fortran.  Diagnostics that only feed output files
// (Sij_mean, TAU_mean, NU_T_MEAN, tke_sgs, the plane_les files, U*_BAR_les)
// are left out.  The LES variants GMAT_*_y / GMAT_*_z of JACOBI_TRANS are
// restated in ekref_metrics.cpp.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ekref_ctx.h"

using namespace ekref_detail;

namespace {

// les_chan.F90:30,37 REAL*8 alpha; PARAMETER (alpha = 2.44950): a default-REAL
// literal, so alpha is 2.4495 rounded to single precision, widened.
constexpr double kAlpha = static_cast<double>(2.44950f);
constexpr double kBeta = 1.0;       // PARAMETER (beta = 1.d0)

inline cplx cdiv_r(cplx a, double r) { return {a.re / r, a.im / r}; }

// The face-weighted difference that compute_strain_chan (and the CF
// additions of les_chan) apply to a field X at (i, k, j):
//   0.5*A(K+1,J,2)*(X+X(K+1)) - 0.5*A(K,J,2)*(X+X(K-1))
//     + 0.5*B(K,J+1,1)*(X+X(J+1)) - 0.5*B(K,J,1)*(X+X(J-1))
// with (A, B) = (CJOB_12, CJOB_22) (the eta form) or (CJOB_11, CJOB_21)
// (the zeta form).  The four terms are returned so that callers can sum
// them in the Fortran order.
template <typename T>
struct Four {
  T t1, t2, t3, t4;
};
inline double radd(double a, double b) { return a + b; }
inline cplx radd(cplx a, cplx b) { return cadd(a, b); }
inline double rsc(double s, double a) { return s * a; }
inline cplx rsc(double s, cplx a) { return cscale(s, a); }
inline double rsub(double a, double b) { return a - b; }
inline cplx rsub(cplx a, cplx b) { return csub(a, b); }

template <typename T, typename Idx>
Four<T> face_terms(const ekref_ctx *c, const std::vector<double> &A, const std::vector<double> &B,
                   const std::vector<T> &X, Idx idx, int i, int k, int j) {
  const T x0 = X[idx(i, k, j)];
  return Four<T>{rsc(0.5 * c->M3(A, k + 1, j, 2), radd(x0, X[idx(i, k + 1, j)])),
                 rsc(0.5 * c->M3(A, k, j, 2), radd(x0, X[idx(i, k - 1, j)])),
                 rsc(0.5 * c->M3(B, k, j + 1, 1), radd(x0, X[idx(i, k, j + 1)])),
                 rsc(0.5 * c->M3(B, k, j, 1), radd(x0, X[idx(i, k, j - 1)]))};
}
template <typename T>
T sum4(const Four<T> &f) {  // ((t1 - t2) + t3) - t4
  return rsub(radd(rsub(f.t1, f.t2), f.t3), f.t4);
}

// les_filter_chan with filter_type = 2 (weights 1/4, 1/2, 1/4; x periodic
// over I = 0..NX-1) on every (K, J) line, as FILTER_VAR(2) applies it.
void filter2(ekref_ctx *c, std::vector<double> &a) {
  const int NX = c->NX, NXM = NX - 1;
  const double Wm2 = 0.0, Wm1 = 1.0 / 4.0, W0 = 1.0 / 2.0, W1 = 1.0 / 4.0, W2 = 0.0;
  std::vector<int> im2(NX), im1(NX), ip1(NX), ip2(NX);
  for (int i = 2; i <= NXM; ++i) im2[i] = i - 2;
  im2[1] = NXM;
  im2[0] = NX - 2;
  for (int i = 1; i <= NXM; ++i) im1[i] = i - 1;
  im1[0] = NXM;
  for (int i = 0; i <= NX - 2; ++i) ip1[i] = i + 1;
  ip1[NXM] = 0;
  for (int i = 0; i <= NX - 3; ++i) ip2[i] = i + 2;
  ip2[NX - 2] = 0;
  ip2[NXM] = 1;
#pragma omp parallel
  {
    std::vector<double> b(NX);
#pragma omp for collapse(2) schedule(static)
    for (int j = 0; j <= c->NY + 1; ++j)
      for (int k = 0; k <= c->NZ + 1; ++k) {
        double *A = &a[c->ip(0, k, j)];
        for (int i = 0; i <= NXM; ++i)
          b[i] = Wm2 * A[im2[i]] + Wm1 * A[im1[i]] + W0 * A[i] + W1 * A[ip1[i]] + W2 * A[ip2[i]];
        for (int i = 0; i <= NXM; ++i) A[i] = b[i];
      }
  }
}

// Ghost copies of a subgrid stress (les_chan.F90:961-971): the J rows first,
// then the K columns.
void ghost_copies(ekref_ctx *c, std::vector<double> &s) {
  const int NY = c->NY, NZ = c->NZ, NXP = c->NXP;
  for (int k = 0; k <= NZ + 1; ++k)
    for (int i = 0; i <= NXP; ++i) {
      s[c->ip(i, k, NY + 1)] = s[c->ip(i, k, NY)];
      s[c->ip(i, k, 0)] = s[c->ip(i, k, 1)];
    }
  for (int j = 0; j <= NY + 1; ++j)
    for (int i = 0; i <= NXP; ++i) {
      s[c->ip(i, NZ + 1, j)] = s[c->ip(i, NZ, j)];
      s[c->ip(i, 0, j)] = s[c->ip(i, 1, j)];
    }
}

// GMAT_12-form eddy-viscosity cross term of a field U with viscosity nu
// (duct.F90:990-1004 for U1; 1266-1283 for TH with KAPPA_T).
double cross_term(const ekref_ctx *c, const std::vector<double> &G, const std::vector<double> &nu,
                  const std::vector<double> &U, int i, int k, int j) {
  auto F = [&](int kk, int jj) { return U[c->ip(i, kk, jj)]; };
  auto N = [&](int kk, int jj) { return nu[c->ip(i, kk, jj)]; };
  const double t1 = c->M3(G, k + 1, j, 2) * 0.5 * (N(k + 1, j) + N(k, j)) * (F(k + 1, j + 1) + F(k, j + 1) - F(k, j - 1) - F(k + 1, j - 1));
  const double t2 = c->M3(G, k, j, 2) * 0.5 * (N(k, j) + N(k - 1, j)) * (F(k - 1, j + 1) + F(k, j + 1) - F(k, j - 1) - F(k - 1, j - 1));
  const double t3 = c->M3(G, k, j + 1, 1) * 0.5 * (N(k, j) + N(k, j + 1)) * (F(k + 1, j + 1) + F(k + 1, j) - F(k - 1, j + 1) - F(k - 1, j));
  const double t4 = c->M3(G, k, j, 1) * 0.5 * (N(k, j) + N(k, j - 1)) * (F(k + 1, j) + F(k + 1, j - 1) - F(k - 1, j) - F(k - 1, j - 1));
  return 0.25 * (t1 - t2 + t3 - t4);
}

}  // namespace

void les_alloc(ekref_ctx *c) {
  const size_t np = (size_t)c->LDX * c->NZ2 * c->NY2, nc = (size_t)c->LDC * c->NZ2 * c->NY2;
  c->NU_T.assign(np, 0.0);
  c->KAPPA_T.assign(np, 0.0);
  c->S2X.assign(np, 0.0);
  c->C_DYN.assign((size_t)c->NZ2 * c->NY2, 0.0);
  for (int ij = 0; ij < 6; ++ij) {
    c->Sij[ij].assign(np, 0.0);
    c->CSij[ij].assign(nc, cplx{0.0, 0.0});
  }
}

// les_chan, LES_MODEL_TYPE = 2 (les_chan.F90:332-1351): strain rates, the
// dynamic coefficient C_DYN (recomputed at RK_STEP 1 of every fifth step and
// in every substep of the run's first step), NU_T, the explicit part of the
// subgrid stress and its divergence added to CF1..CF3.  Also leaves U1..U3
// in physical space, as the REAL_FOURIER_TRANS_U* calls inside it do.
void les_chan(ekref_ctx *c, int rk) {
  const ek_params &p = c->p;
  const int NX = c->NX, NY = c->NY, NZ = c->NZ, NXP = c->NXP, NX2P = c->NX2P;
  const int JS = c->JSTART, JE = c->JEND, ZS = c->ZSTART, ZE = c->ZEND;
  auto &Sij = c->Sij;
  auto &CSij = c->CSij;
  auto ipf = [c](int i, int k, int j) { return c->ip(i, k, j); };
  auto icf = [c](int i, int k, int j) { return c->ic(i, k, j); };
  const size_t np = c->U1.size();
  // DELTA_Y (les_chan.F90:343-348)
  std::vector<double> DY((size_t)c->NZ2 * c->NY2);
  const double DX1 = p.lx / NX;  // DX(1) = LX/NX (diablo.F90:409)
  for (int j = 0; j <= NY + 1; ++j)
    for (int k = 0; k <= NZ + 1; ++k) DY[(size_t)j * c->NZ2 + k] = std::pow(kBeta * DX1 * c->JAC(k, j), 1.0 / 3.0);
  auto Dlt = [&](int k, int j) { return DY[(size_t)j * c->NZ2 + k]; };

  // compute_strain_chan (les_chan.F90:1623-1718)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k) {
      const double jac = c->JAC(k, j);
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        const cplx ik{0.0, c->KXP[i]};
        CSij[0][q] = cmul(ik, c->CU1[q]);
        CSij[1][q] = cdiv_r(sum4(face_terms(c, c->cjob_12, c->cjob_22, c->CU2, icf, i, k, j)), jac);
        CSij[2][q] = cdiv_r(sum4(face_terms(c, c->cjob_11, c->cjob_21, c->CU3, icf, i, k, j)), jac);
        CSij[3][q] = cscale(0.5, cadd(cdiv_r(sum4(face_terms(c, c->cjob_12, c->cjob_22, c->CU1, icf, i, k, j)), jac),
                                      cmul(ik, c->CU2[q])));
        CSij[4][q] = cscale(0.5, cadd(cdiv_r(sum4(face_terms(c, c->cjob_11, c->cjob_21, c->CU1, icf, i, k, j)), jac),
                                      cmul(ik, c->CU3[q])));
        const auto a = face_terms(c, c->cjob_11, c->cjob_21, c->CU2, icf, i, k, j);
        const auto b = face_terms(c, c->cjob_12, c->cjob_22, c->CU3, icf, i, k, j);
        // 0.5*( a1 - a2 + a3 - a4 + b1 - b2 + b3 - b4 )/INT_JACOB, left to right
        cplx s = csub(cadd(csub(cadd(csub(cadd(csub(a.t1, a.t2), a.t3), a.t4), b.t1), b.t2), b.t3), b.t4);
        CSij[5][q] = cdiv_r(cscale(0.5, s), jac);
      }
    }
  for (int ij = 0; ij < 6; ++ij) to_physical(c, CSij[ij], Sij[ij], 0, NY + 1, 0, NZ + 1);

  // |S| (les_chan.F90:357-377)
  auto &S2X = c->S2X;
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= NXP; ++i) {
        const size_t q = c->ip(i, k, j);
        const double s1 = Sij[0][q], s2 = Sij[1][q], s3 = Sij[2][q], s4 = Sij[3][q], s5 = Sij[4][q], s6 = Sij[5][q];
        S2X[q] = std::sqrt(2.0 * (s1 * s1) + 4.0 * (s4 * s4) + 4.0 * (s5 * s5) + 2.0 * (s2 * s2) + 4.0 * (s6 * s6) +
                           2.0 * (s3 * s3));
      }
  for (int k = 0; k <= NZ + 1; ++k)
    for (int i = 0; i <= NXP; ++i) {
      S2X[c->ip(i, k, 0)] = S2X[c->ip(i, k, 1)];
      S2X[c->ip(i, k, NY + 1)] = S2X[c->ip(i, k, NY)];
    }

  // REAL_FOURIER_TRANS_U1..3 (les_chan.F90:422-424) and the test-filtered
  // velocities U_BAR_TIL (431-471)
  to_physical(c, c->CU1, c->U1, 0, NY + 1, 0, NZ + 1);
  to_physical(c, c->CU2, c->U2, 0, NY + 1, 0, NZ + 1);
  to_physical(c, c->CU3, c->U3, 0, NY + 1, 0, NZ + 1);
  const std::vector<double> *U[3] = {&c->U1, &c->U2, &c->U3};
  std::vector<double> UB[3] = {c->U1, c->U2, c->U3};
  for (auto &v : UB) filter2(c, v);

  // C_DYN (les_chan.F90:475-821)
  if ((p.time_step % 5 == 0 && rk == 1) || c->first_time) {
    static const int ui1[6] = {0, 1, 2, 0, 0, 1}, ui2[6] = {0, 1, 2, 1, 2, 2};  // U_index1/2 - 1
    std::vector<double> S_2BAR = S2X;
    filter2(c, S_2BAR);
    std::fill(c->C_DYN.begin(), c->C_DYN.end(), 0.0);
    std::vector<double> num_sum((size_t)c->NZ2 * c->NY2, 0.0), den_sum((size_t)c->NZ2 * c->NY2, 0.0);
    std::vector<double> temp(np), Mij(np);
    for (int ij = 0; ij < 6; ++ij) {
      const double cross = (ij < 3) ? 1.0 : 2.0;
      temp = Sij[ij];
      filter2(c, temp);
#pragma omp parallel for schedule(static)
      for (int j = 0; j <= NY + 1; ++j)
        for (int k = 0; k <= NZ + 1; ++k) {
          const double ad = kAlpha * Dlt(k, j), d = Dlt(k, j);
          for (int i = 0; i <= NXP; ++i) {
            const size_t q = c->ip(i, k, j);
            temp[q] = temp[q] * (ad * ad) * S_2BAR[q];
            Mij[q] = (d * d) * S2X[q] * Sij[ij][q];
          }
        }
      filter2(c, Mij);
      for (size_t q = 0; q < np; ++q) Mij[q] = temp[q] - Mij[q];
      const std::vector<double> &Ua = *U[ui1[ij]], &Ub = *U[ui2[ij]];
      for (size_t q = 0; q < np; ++q) temp[q] = Ua[q] * Ub[q];
      filter2(c, temp);
      const std::vector<double> &Ba = UB[ui1[ij]], &Bb = UB[ui2[ij]];
#pragma omp parallel for schedule(static)
      for (int j = 0; j <= NY + 1; ++j)
        for (int k = 0; k <= NZ + 1; ++k) {
          double sn = 0.0, sd = 0.0;
          for (int i = 0; i <= NX - 1; ++i) {
            const size_t q = c->ip(i, k, j);
            sn += Mij[q] * (temp[q] - Ba[q] * Bb[q]);
            sd += Mij[q] * Mij[q];
          }
          const size_t m = (size_t)j * c->NZ2 + k;
          den_sum[m] = den_sum[m] + cross * sd;
          num_sum[m] = num_sum[m] + cross * sn;
        }
    }
    for (int j = JS; j <= JE; ++j)
      for (int k = ZS; k <= ZE; ++k) {
        const size_t m = (size_t)j * c->NZ2 + k;
        c->C_DYN[m] = (den_sum[m] != 0.0) ? -0.5 * num_sum[m] / den_sum[m] : 0.0;
      }
    for (double &v : c->C_DYN)
      if (v < 0.0) v = 0.0;
  }
  auto CD = [&](int k, int j) { return c->C_DYN[(size_t)j * c->NZ2 + k]; };

  // NU_T (les_chan.F90:828-834)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k) {
      const double d = Dlt(k, j);
      for (int i = 0; i <= NXP; ++i) c->NU_T[c->ip(i, k, j)] = CD(k, j) * (d * d) * S2X[c->ip(i, k, j)];
    }

  // explicit subgrid stress (les_chan.F90:839-973) and its transform (1178-1193)
  for (int ij = 0; ij < 6; ++ij) {
    std::vector<double> &s = Sij[ij];
    if (ij == 0) {
      for (int j = 1; j <= NY + 1; ++j)
        for (int k = 1; k <= NZ + 1; ++k) {
          const double d = Dlt(k, j);
          for (int i = 0; i <= NXP; ++i) {
            const size_t q = c->ip(i, k, j);
            s[q] = -2.0 * CD(k, j) * (d * d) * S2X[q] * s[q];
          }
        }
    } else if (ij == 1 || ij == 2) {
      for (int j = (ij == 1) ? 1 : 0; j <= NY + 1; ++j)
        for (int k = 1; k <= NZ + 1; ++k)
          for (int i = 0; i <= NXP; ++i) s[c->ip(i, k, j)] = 0.0;
    } else {
      // tau_12, tau_13, tau_23 less their implicit parts: 0.5*d(U1)/d(eta),
      // 0.5*d(U1)/d(zeta), 0.5*d(U2)/d(zeta)
      const std::vector<double> &A = (ij == 3) ? c->cjob_12 : c->cjob_11;
      const std::vector<double> &B = (ij == 3) ? c->cjob_22 : c->cjob_21;
      const std::vector<double> &F = (ij == 5) ? c->U2 : c->U1;
#pragma omp parallel for schedule(static)
      for (int j = JS; j <= JE; ++j)
        for (int k = ZS; k <= ZE; ++k) {
          const double d = Dlt(k, j), jac = c->JAC(k, j);
          for (int i = 0; i <= NXP; ++i) {
            const size_t q = c->ip(i, k, j);
            const double g = sum4(face_terms(c, A, B, F, ipf, i, k, j));
            s[q] = -2.0 * CD(k, j) * (d * d) * S2X[q] * (s[q] - 0.5 * g / jac);
          }
        }
    }
    ghost_copies(c, s);
    to_fourier(c, s, CSij[ij], 0, NY + 1, 0, NZ + 1);
  }

  // CF additions, LES_IMPLICIT = .FALSE. (les_chan.F90:1306-1351)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k) {
      const double jac = c->JAC(k, j);
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        const cplx jik = cscale(jac, cplx{0.0, c->KXP[i]});
        auto Ey = [&](int ij) { return sum4(face_terms(c, c->cjob_12, c->cjob_22, CSij[ij], icf, i, k, j)); };
        auto Ez = [&](int ij) { return sum4(face_terms(c, c->cjob_11, c->cjob_21, CSij[ij], icf, i, k, j)); };
        c->CF1[q] = csub(csub(csub(c->CF1[q], cmul(jik, CSij[0][q])), Ey(3)), Ez(4));
        c->CF2[q] = csub(csub(csub(c->CF2[q], cmul(jik, CSij[3][q])), Ey(1)), Ez(5));
        c->CF3[q] = csub(csub(csub(c->CF3[q], cmul(jik, CSij[4][q])), Ey(5)), Ez(2));
      }
    }
}

// les_chan_th, LES_MODEL_TYPE_TH = 1 (les_chan_th.F90:45-105, 396-405):
// KAPPA_T = NU_T/PR, the x subgrid flux -KAPPA_T d(TH)/dx added to CFTH, and
// TH left in physical space (REAL_FOURIER_TRANS_TH).
void les_chan_th(ekref_ctx *c) {
  const int NY = c->NY, NZ = c->NZ, NXP = c->NXP, NX2P = c->NX2P;
  const int JS = c->JSTART, JE = c->JEND, ZS = c->ZSTART, ZE = c->ZEND;
  auto &Sij = c->Sij;
  auto &CSij = c->CSij;
  auto icf = [c](int i, int k, int j) { return c->ic(i, k, j); };
  const double PR = c->p.pr;
  // compute_scalar_grad (les_chan_th.F90:462-540)
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k) {
      const double jac = c->JAC(k, j);
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        CSij[0][q] = cmul(cplx{0.0, c->KXP[i]}, c->CTH[q]);
        CSij[1][q] = cdiv_r(sum4(face_terms(c, c->cjob_12, c->cjob_22, c->CTH, icf, i, k, j)), jac);
        CSij[2][q] = cdiv_r(sum4(face_terms(c, c->cjob_11, c->cjob_21, c->CTH, icf, i, k, j)), jac);
      }
    }
  for (int ij = 0; ij < 3; ++ij) to_physical(c, CSij[ij], Sij[ij], 0, NY + 1, 0, NZ + 1);
  if (!c->th_bar.empty()) {
    auto TB = [&](int k, int j) { return c->M2(c->th_bar, k, j); };
    for (int j = JS; j <= JE; ++j)
      for (int k = ZS; k <= ZE; ++k) {
        const double g = (0.5 * c->M3(c->cjob_12, k + 1, j, 2) * (TB(k, j) + TB(k + 1, j)) -
                          0.5 * c->M3(c->cjob_12, k, j, 2) * (TB(k, j) + TB(k - 1, j)) +
                          0.5 * c->M3(c->cjob_22, k, j + 1, 1) * (TB(k, j) + TB(k, j + 1)) -
                          0.5 * c->M3(c->cjob_22, k, j, 1) * (TB(k, j) + TB(k, j - 1))) /
                         c->JAC(k, j);
        for (int i = 0; i <= NXP; ++i) Sij[1][c->ip(i, k, j)] = Sij[1][c->ip(i, k, j)] + g;
      }
  }
  // KAPPA_T and the flux (les_chan_th.F90:50-105)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= NXP; ++i) c->KAPPA_T[c->ip(i, k, j)] = c->NU_T[c->ip(i, k, j)] / PR;
  for (int j = 0; j <= NY + 1; ++j)
    for (int k = 0; k <= NZ + 1; ++k)
      for (int i = 0; i <= NXP; ++i) {
        const size_t q = c->ip(i, k, j);
        Sij[0][q] = -(c->NU_T[q] / PR * Sij[0][q]);
      }
  ghost_copies(c, Sij[0]);
  to_fourier(c, Sij[0], CSij[0], 0, NY + 1, 0, NZ + 1);
  for (int j = 1; j <= NY + 1; ++j)
    for (int k = 0; k <= NZ + 1; ++k)
      for (int i = 0; i <= NX2P; ++i) {
        CSij[1][c->ic(i, k, j)] = cplx{0.0, 0.0};
        CSij[2][c->ic(i, k, j)] = cplx{0.0, 0.0};
      }
  to_physical(c, c->CTH, c->TH, 0, NY + 1, 0, NZ + 1);
  // CFTH -= INT_JACOB*CIKXP*CSij(1) (les_chan_th.F90:396-403)
  for (int j = c->JSTART_TH; j <= c->JEND_TH; ++j)
    for (int k = c->ZSTART_TH; k <= c->ZEND_TH; ++k) {
      const double jac = c->JAC(k, j);
      for (int i = 0; i <= NX2P; ++i) {
        const size_t q = c->ic(i, k, j);
        c->CFTH[q] = csub(c->CFTH[q], cmul(cscale(jac, cplx{0.0, c->KXP[i]}), CSij[0][q]));
      }
    }
}

// duct.F90:990-1120: the NU_T cross terms of U1 (GMAT_12), U2 (GMAT_12_y) and
// U3 (GMAT_12_z), each transformed and added to CF1..CF3.
void les_cross_terms(ekref_ctx *c) {
  const int JS = c->JSTART, JE = c->JEND, ZS = c->ZSTART, ZE = c->ZEND;
  const std::vector<double> *G[3] = {&c->gmat_12, &c->g12y, &c->g12z};
  const std::vector<double> *U[3] = {&c->U1, &c->U2, &c->U3};
  std::vector<cplx> *CF[3] = {&c->CF1, &c->CF2, &c->CF3};
  for (int f = 0; f < 3; ++f) {
#pragma omp parallel for schedule(static)
    for (int j = JS; j <= JE; ++j)
      for (int k = ZS; k <= ZE; ++k)
        for (int i = 0; i <= c->NXP; ++i) c->S1[c->ip(i, k, j)] = cross_term(c, *G[f], c->NU_T, *U[f], i, k, j);
    to_fourier(c, c->S1, c->CS1, JS, JE, ZS, ZE);
    for (int j = JS; j <= JE; ++j)
      for (int k = ZS; k <= ZE; ++k)
        for (int i = 0; i <= c->NX2P; ++i) (*CF[f])[c->ic(i, k, j)] = cadd((*CF[f])[c->ic(i, k, j)], c->CS1[c->ic(i, k, j)]);
  }
}

// duct.F90:1266-1311: the KAPPA_T cross term of TH added to CFTH.
void les_cross_terms_th(ekref_ctx *c) {
  const int JS = c->JSTART_TH, JE = c->JEND_TH, ZS = c->ZSTART_TH, ZE = c->ZEND_TH;
#pragma omp parallel for schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= c->NXP; ++i) c->S1[c->ip(i, k, j)] = cross_term(c, c->gmat_12, c->KAPPA_T, c->TH, i, k, j);
  to_fourier(c, c->S1, c->CS1, JS, JE, ZS, ZE);
  for (int j = JS; j <= JE; ++j)
    for (int k = ZS; k <= ZE; ++k)
      for (int i = 0; i <= c->NX2P; ++i) c->CFTH[c->ic(i, k, j)] = cadd(c->CFTH[c->ic(i, k, j)], c->CS1[c->ic(i, k, j)]);
}

extern "C" int ekref_set_les_metrics(ekref_ctx *c, const double *g11y, const double *g12y, const double *g22y,
                                     const double *g11z, const double *g12z, const double *g22z) {
  if (!c || !g11y || !g12y || !g22y || !g11z || !g12z || !g22z) return EK_ERR_ARG;
  const size_t n3 = (size_t)2 * (c->NZ + 3) * (c->NY + 3);
  c->g11y.assign(g11y, g11y + n3);
  c->g12y.assign(g12y, g12y + n3);
  c->g22y.assign(g22y, g22y + n3);
  c->g11z.assign(g11z, g11z + n3);
  c->g12z.assign(g12z, g12z + n3);
  c->g22z.assign(g22z, g22z + n3);
  c->have_les_metrics = true;
  return EK_OK;
}

extern "C" int ekref_les_set_first_time(ekref_ctx *c, int first_time) {
  if (!c) return EK_ERR_ARG;
  c->first_time = first_time != 0;
  return EK_OK;
}

extern "C" int ekref_les_get(ekref_ctx *c, double *nu_t, double *c_dyn) {
  if (!c || !c->p.les) return EK_ERR_STATE;
  if (nu_t) std::memcpy(nu_t, c->NU_T.data(), sizeof(double) * c->NU_T.size());
  if (c_dyn) std::memcpy(c_dyn, c->C_DYN.data(), sizeof(double) * c->C_DYN.size());
  return EK_OK;
}
