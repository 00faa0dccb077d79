// RK substep kernels of the GB300 duct path, FP64: the fused spectral
// right-hand side, contravariant face velocities, the CN-ADI line solves
// and the REM_DIV_CURV divergence / projection stencils.  Each kernel cites
// the loop nests of src/duct.F90 it replaces.
#include "ek_internal.h"

namespace ek {

namespace {

__device__ __forceinline__ cplx_t cadd(cplx_t a, cplx_t b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cplx_t csub(cplx_t a, cplx_t b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cplx_t cscl(double s, cplx_t a) { return {s * a.re, s * a.im}; }

// x / b for several x sharing one divisor b: r = RN(1/b) once, then per
// quotient q0 = RN(x r), e = x - b q0 (exact with an FMA), q = RN(q0 + e r),
// Markstein's correction step, which rounds the quotient correctly.  Saves
// the full FP64 division sequence per quotient on a GPU whose FP64 pipe is
// narrow.
struct DivBy {
  double b, r;
  __device__ explicit DivBy(double bb) : b(bb), r(1.0 / bb) {}
  __device__ DivBy(double bb, double rr) : b(bb), r(rr) {}
  __device__ double operator()(double x) const {
    const double q0 = x * r;
    return fma(fma(-b, q0, x), r, q0);
  }
};

struct SpecArgs {
  Dims d;
  Metrics m;
  const double *kx, *kx2;
  cplx_t *CU1, *CU2, *CU3, *CP, *CTH, *CF1, *CF2, *CF3, *CFTH, *CR1, *CR2, *CR3, *CRTH;
  double nu, nupr, T3, T4, px, f0, ubc_top, wbulk0, ri;
  int rk, th, cont_strat, forcing;
  // 1: CR holds only the explicit increment CR - J CU (the mixed path,
  // whose ADI takes S = R - J phi straight from its FP32 transform)
  int cr_inc;
  const double *nut;  // LES: NU_T of the previous substep (KAPPA_T = NU_T/PR), else null
  double pr;
  // sponge_th
  const double *sig, *sig_out, *sred;  // sred[1] != 0: dynamic branch active
  double amp, tgt1, tgt2, tgt3;
  int sponge, strat_per, reset;
};

// sponge_th's mean of Re CU3X(0,K,J) over J = NY_sponge..JEND,
// K = ZSTART..ZEND (duct.F90:3253-3277) and its dynamic-branch test
// |mean - WBULK0| > WBULK0 * 0.001 (duct.F90:3288).  One block.
__global__ void k_sponge_mean(Dims d, const cplx_t *CU3, int ny_sponge, double wbulk0, double *red) {
  __shared__ double s[256];
  double acc = 0.0;
  const int nk = d.ZE - d.ZS + 1, nj = d.JE - ny_sponge + 1;
  for (int t = threadIdx.x; t < nk * nj; t += blockDim.x) {
    const int k = d.ZS + t % nk, j = ny_sponge + t / nk;
    acc += CU3[d.ic(0, k, j)].re;
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double mean = (nk > 0 && nj > 0) ? s[0] / ((double)nk * (double)nj) : 0.0;
    red[0] = mean;
    red[1] = (fabs(mean - wbulk0) > wbulk0 * 0.001) ? 1.0 : 0.0;
  }
}

// Spectral explicit RHS: duct.F90:299-409 (CR = J CU + zeta h CF_prev, the
// curvilinear pressure gradient), 411-455 (mean forcing, mode 0),
// 461-523 (viscous x term, Coriolis on every kx, buoyancy) and 540-633
// (scalar RHS with the background stratification term).
// sum_t G[t] P[t] over the five pressure points (p0, p(k+1), p(k-1),
// p(j+1), p(j-1)) with the weights of coefficient planes g0..g0+4
__device__ __forceinline__ cplx_t pg_dot(const double *pg, size_t n2, int g0, size_t mm, cplx_t p0, cplx_t pkp,
                                         cplx_t pkm, cplx_t pjp, cplx_t pjm) {
  const double w0 = pg[(g0 + 0) * n2 + mm], w1 = pg[(g0 + 1) * n2 + mm], w2 = pg[(g0 + 2) * n2 + mm];
  const double w3 = pg[(g0 + 3) * n2 + mm], w4 = pg[(g0 + 4) * n2 + mm];
  cplx_t r;
  r.re = fma(w4, pjm.re, fma(w3, pjp.re, fma(w2, pkm.re, fma(w1, pkp.re, w0 * p0.re))));
  r.im = fma(w4, pjm.im, fma(w3, pjp.im, fma(w2, pkm.im, fma(w1, pkp.im, w0 * p0.im))));
  return r;
}

// The pressure-gradient weights and 1/J per cell, K = 1..NZ, J = 1..NY: the
// metric combinations that the spectral right-hand side and the projection
// would otherwise rebuild for every kx mode.  Planes 11 and 12 hold the
// TH_BAR terms of the scalar right-hand side (duct.F90:589-618), which
// depend on (K, J) only: the coefficient g of CU2 and the bracket that
// KAPPA/4 multiplies, each evaluated in the order of the per-mode formula
// it replaces, so the right-hand side is unchanged bit for bit.
constexpr int kPgPlanes = 13;
__global__ void k_metric_tables(Dims d, Metrics m) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  const size_t n2 = (size_t)d.LDM * (d.NY + 3);
  if (k > d.NZ + 2 || j > d.NY + 2) return;
  const size_t mm = d.m2(k, j);
  double w[kPgPlanes] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (k >= 1 && k <= d.NZ && j >= 1 && j <= d.NY) {
    const double *TB = m.thbar;
    auto tb = [&](int kk, int jj) { return TB[d.m2(kk, jj)]; };
    w[11] = 0.5 * m.c12[d.m3(k + 1, j, 2)] * (tb(k, j) + tb(k + 1, j)) -
            0.5 * m.c12[d.m3(k, j, 2)] * (tb(k, j) + tb(k - 1, j)) +
            0.5 * m.c22[d.m3(k, j + 1, 1)] * (tb(k, j) + tb(k, j + 1)) -
            0.5 * m.c22[d.m3(k, j, 1)] * (tb(k, j) + tb(k, j - 1));
    w[12] = (+m.g12[d.m3(k + 1, j, 2)] * (tb(k + 1, j + 1) + tb(k, j + 1) - tb(k, j - 1) - tb(k + 1, j - 1)) -
             m.g12[d.m3(k, j, 2)] * (tb(k - 1, j + 1) + tb(k, j + 1) - tb(k, j - 1) - tb(k - 1, j - 1)) +
             m.g12[d.m3(k, j + 1, 1)] * (tb(k + 1, j + 1) + tb(k + 1, j) - tb(k - 1, j + 1) - tb(k - 1, j)) -
             m.g12[d.m3(k, j, 1)] * (tb(k + 1, j) + tb(k + 1, j - 1) - tb(k - 1, j) - tb(k - 1, j - 1)) +
             4.0 * (m.g11[d.m3(k + 1, j, 2)] * (tb(k + 1, j) - tb(k, j)) - m.g11[d.m3(k, j, 2)] * (tb(k, j) - tb(k - 1, j))) +
             4.0 * (m.g22[d.m3(k, j + 1, 1)] * (tb(k, j + 1) - tb(k, j)) - m.g22[d.m3(k, j, 1)] * (tb(k, j) - tb(k, j - 1))));
    const double e = 0.5 * m.c12[d.m3(k + 1, j, 2)], f = 0.5 * m.c12[d.m3(k, j, 2)];
    const double g = 0.5 * m.c22[d.m3(k, j + 1, 1)], h = 0.5 * m.c22[d.m3(k, j, 1)];
    const double a = 0.5 * m.c11[d.m3(k + 1, j, 2)], b = 0.5 * m.c11[d.m3(k, j, 2)];
    const double c = 0.5 * m.c21[d.m3(k, j + 1, 1)], dd = 0.5 * m.c21[d.m3(k, j, 1)];
    w[0] = ((e - f) + g) - h; w[1] = e; w[2] = -f; w[3] = g; w[4] = -h;
    w[5] = ((a - b) + c) - dd; w[6] = a; w[7] = -b; w[8] = c; w[9] = -dd;
    w[10] = 1.0 / m.jac[mm];
  }
  for (int t = 0; t < kPgPlanes; ++t) m.pg[t * n2 + mm] = w[t];
}

__global__ void k_spectral_rhs(SpecArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, j = blockIdx.z;
  if (i > d.NX2P) return;
  const size_t q = d.ic(i, k, j);
  const double jac = a.m.jac[d.m2(k, j)];
  const bool vel = (j >= d.JS && j <= d.JE && k >= d.ZS && k <= d.ZE);
  const bool sca = a.th && (j >= d.JST && j <= d.JET && k >= d.ZST && k <= d.ZET);
  cplx_t F1{}, F2{}, F3{}, FT{};
  if (vel) {
    const cplx_t cu1 = a.CU1[q], cu2 = a.CU2[q], cu3 = a.CU3[q];
    // the explicit-increment form leaves J CU out of CR (no products spent on it)
    cplx_t r1{}, r2{}, r3{};
    if (!a.cr_inc) {
      r1 = cscl(jac, cu1);
      r2 = cscl(jac, cu2);
      r3 = cscl(jac, cu3);
    }
    if (a.rk > 1) {
      r1 = cadd(r1, cscl(a.T3, a.CF1[q]));
      r2 = cadd(r2, cscl(a.T3, a.CF2[q]));
      r3 = cadd(r3, cscl(a.T3, a.CF3[q]));
    }
    const cplx_t *CP = a.CP;
    const cplx_t p0 = CP[q];
    const cplx_t pkp = CP[d.ic(i, k + 1, j)], pkm = CP[d.ic(i, k - 1, j)];
    const cplx_t pjp = CP[d.ic(i, k, j + 1)], pjm = CP[d.ic(i, k, j - 1)];
    // the curvilinear pressure gradient (duct.F90:371-409) from the
    // per-cell weight planes
    const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
    const cplx_t cs1 = pg_dot(a.m.pg, n2, 5, mm, p0, pkp, pkm, pjp, pjm);
    const cplx_t cs2 = pg_dot(a.m.pg, n2, 0, mm, p0, pkp, pkm, pjp, pjm);
    // - T4 J (i kx) p0, with the zero real part of i kx dropped: GB300's
    // FP64 pipe is this kernel's limit, so every product that is known to
    // vanish or can be shared is left out (the terms are those of
    // duct.F90:371-409, regrouped: results agree to rounding)
    const double s1 = (jac * a.T4) * a.kx[i];
    r1.re = fma(s1, p0.im, r1.re);
    r1.im = fma(-s1, p0.re, r1.im);
    r2.re = fma(-a.T4, cs2.re, r2.re);
    r2.im = fma(-a.T4, cs2.im, r2.im);
    r3.re = fma(-a.T4, cs1.re, r3.re);
    r3.im = fma(-a.T4, cs1.im, r3.im);
    if (i == 0 && a.forcing) r3.re = r3.re - a.T4 * a.px * jac;
    a.CR1[q] = r1;
    a.CR2[q] = r2;
    a.CR3[q] = r3;
    const double v = -a.nu * a.kx2[i] * jac;
    cplx_t f1 = cscl(v, cu1), f2 = cscl(v, cu2), f3 = cscl(v, cu3);
    // Coriolis on every kx (duct.F90:461-473), J f0 shared by both terms
    const double jf = jac * a.f0;
    f3.re = fma(jf, cu1.re - a.ubc_top, f3.re);
    f3.im = fma(jf, cu1.im, f3.im);
    f1.re = fma(-jf, cu3.re - a.wbulk0, f1.re);
    f1.im = fma(-jf, cu3.im, f1.im);
    if (a.th) {
      const double jr = jac * a.ri;
      const cplx_t cth = a.CTH[q];
      f2.re = fma(-jr, cth.re, f2.re);
      f2.im = fma(-jr, cth.im, f2.im);
    }
    F1 = f1;
    F2 = f2;
    F3 = f3;
  }
  if (sca) {
    const cplx_t cth = a.CTH[q];
    cplx_t rt = a.cr_inc ? cplx_t{0.0, 0.0} : cscl(jac, cth);
    if (a.rk > 1) rt = cadd(rt, cscl(a.T3, a.CFTH[q]));
    a.CRTH[q] = rt;
    cplx_t ft = cscl(-a.nupr * jac * a.kx2[i], cth);
    if (a.cont_strat) {
      ft = cadd(ft, cscl(jac, a.CU2[q]));
    } else {
      // the TH_BAR terms from their per-cell planes (k_metric_tables)
      const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
      ft = csub(ft, cscl(a.m.pg[11 * n2 + mm], a.CU2[q]));
      // with LES the coefficient is NU/PR + KAPPA_T at the physical point whose
      // x index is the mode index (duct.F90:610-618)
      const double kap = a.nut ? a.nupr + a.nut[d.ip(i, k, j)] / a.pr : a.nupr;
      ft.re = ft.re + 0.25 * kap * a.m.pg[12 * n2 + mm];
    }
    FT = ft;
  }
  if (a.sponge) {
    // sponge_th (duct.F90:3196-3362), in its statement order; each term is
    // ((amplitude * sigma) * (CU - target)) * J as the Fortran evaluates it
    cplx_t cu2 = a.CU2[q];
    if (vel) {
      const cplx_t cu1 = a.CU1[q], cu3 = a.CU3[q];
      const cplx_t cth = sca ? a.CTH[q] : cplx_t{};
      const double sg = a.amp * a.sig[j], so = a.amp * a.sig_out[k];
      auto damp = [&](cplx_t f, double s, cplx_t u, double tgt, double w) {
        return csub(f, cscl(w, cscl(s, cplx_t{u.re - tgt, u.im})));
      };
      if (i >= 1) {
        F1 = damp(F1, sg, cu1, 0.0, jac);
        F2 = damp(F2, sg, cu2, 0.0, jac);
        F3 = damp(F3, sg, cu3, 0.0, jac);
        if (sca) FT = damp(FT, sg, cth, 0.0, jac);
        F1 = damp(F1, so, cu1, 0.0, jac);
        F2 = damp(F2, so, cu2, 0.0, jac);
        F3 = damp(F3, so, cu3, 0.0, jac);
        if (sca) FT = damp(FT, so, cth, 0.0, jac);
      } else {
        if (a.sred[1] != 0.0) {
          F1 = damp(F1, sg, cu1, a.tgt1, jac);
          F2 = damp(F2, sg, cu2, a.tgt2, jac);
          F3 = damp(F3, sg, cu3, a.tgt3, jac);
          if (sca) FT = damp(FT, sg, cth, 0.0, jac);
        } else {
          F2 = damp(F2, sg, cu2, a.tgt2, jac);
          F1 = damp(F1, sg, cu1, a.tgt1, jac);
        }
        if (a.strat_per) {
          // CF2X(0,:,:) -= Sponge_Amp*(CU2X(0,:,:)-target)*INT_JACOB(K,J), with K, J
          // left at ZEND+1, JEND+1 by the loops before it
          F2 = damp(F2, a.amp, cu2, a.tgt2, a.m.jac[d.m2(d.ZE + 1, d.JE + 1)]);
          if (a.reset) cu2 = cplx_t{0.0, 0.0};
        }
        const double so2 = (2.0 * a.amp) * a.sig_out[k];
        F1 = damp(F1, so2, cu1, 0.0, jac);
        F2 = damp(F2, so2, cu2, 0.0, jac);
        F3 = damp(F3, so2, cu3, a.tgt3, jac);
        if (sca) FT = damp(FT, so2, cth, 0.0, jac);
      }
    }
    // CU2X(0,:,:) = 0 on the whole plane, after every use above
    if (i == 0 && a.strat_per && a.reset) {
      // the explicit-increment form takes phi_old from the reset CU2, so CR
      // keeps J times the part the reset removes (R itself still holds it)
      if (a.cr_inc && vel) a.CR2[q] = cadd(a.CR2[q], cscl(jac, a.CU2[q]));
      a.CU2[q] = cplx_t{0.0, 0.0};
    }
  }
  if (vel) {
    a.CF1[q] = F1;
    a.CF2[q] = F2;
    a.CF3[q] = F3;
  }
  if (sca) a.CFTH[q] = FT;
}

// Contravariant face velocities U2b, U3b (duct.F90:721-732); U3b is stored
// right after U2b.
__global__ void k_face_velocity(Dims d, Metrics m, const double *U2, const double *U3, double *U2b, const float *U2f,
                                const float *U3f, float *U2bf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = d.ZS + blockIdx.y, j = d.JS + blockIdx.z;
  if (i >= d.NX) return;
  double *U3b = U2b + d.nphys();
  const size_t c = d.ip(i, k, j);
  const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  if (U2bf) {
    // only the FP32 flux transforms read the face velocities: the same sums
    // in FP32 from the FP32 copies of U2, U3 (no FP64 instruction; the
    // metrics are rounded on the integer pipe, the halving is exact)
    const float h22 = 0.5f * d2f_bits(m.c22[d.m3(k, j, 1)]), h21 = 0.5f * d2f_bits(m.c21[d.m3(k, j, 1)]);
    const float h11 = 0.5f * d2f_bits(m.c11[d.m3(k, j, 2)]), h12 = 0.5f * d2f_bits(m.c12[d.m3(k, j, 2)]);
    const float u2 = U2f[c], u3 = U3f[c];
    U2bf[c] = h22 * (u2 + U2f[c - sJ]) + h21 * (u3 + U3f[c - sJ]);
    U2bf[c + d.nphys()] = h11 * (u3 + U3f[c - sK]) + h12 * (u2 + U2f[c - sK]);
  } else {
    U2b[c] = 0.5 * m.c22[d.m3(k, j, 1)] * (U2[c] + U2[c - sJ]) + 0.5 * m.c21[d.m3(k, j, 1)] * (U3[c] + U3[c - sJ]);
    U3b[c] = 0.5 * m.c11[d.m3(k, j, 2)] * (U3[c] + U3[c - sK]) + 0.5 * m.c12[d.m3(k, j, 2)] * (U2[c] + U2[c - sK]);
  }
}


struct AdiArgs {
  Dims d;
  Metrics m;
  const double *R, *phi_old, *phs;  // R: c2r(CR); phi_old: field before ADI; phs: y-sweep output
  double *out;                      // y: phs, z: field
  const double *fa, *fib, *fu;      // factors [line][row]
  BcSet bc;
  const double *bcw;
  double coef;
  int js, je, zs, ze;
  const double *tab;  // per-cell right-hand-side weights of this sweep (k_adi_tab)
  // LES (k_adi_les): NU_T, the per-cell row weights of this sweep
  // (k_adi_les_tab) and two scratch fields for the reciprocal of the
  // eliminated diagonal and the upper diagonal
  const double *nut, *ltab;
  double *scr_b, *scr_u;
  // the float-float variant (k_adi_les_ff): NU_T in FP32 and the weights of
  // both tables split into float-float planes (0..3 right-hand side, 4..10 row)
  const float *nutf;
  const float2 *ftab;
  // the explicit-increment form (mixed path): S = R - J phi_old in FP32 in
  // R's slots, and the weights of k_adi_tab with the J phi_old halves folded
  // in; null: R in FP64
  const float *Sf;
  // float-float fields (k_adi_ffs): the old field, the y-sweep result and
  // the output as high/low float planes; the right-hand-side weights and the
  // line's Thomas factors as float pairs
  const float *po_h, *po_l, *ps_h, *ps_l;
  float *out_h, *out_l;
  const float2 *tab2, *fa2, *fib2, *fu2;
  // increment form (k_adi_inc): the field's FP32 copy, the y sweep's
  // increment and the sweep's output (y: that increment; z: the total);
  // brk: on the rows that copy another row (periodic ghosts) the FP32
  // transform of the spectral difference phi_old(src) - phi_old(row)
  const float *phf, *dsf, *brk;
  float *incf;
};

// Right-hand-side weights of one ADI sweep per cell (tab[t * n2 + m2(k, j)]),
// so that the line kernel forms each row with four or five multiply-adds
// instead of rebuilding the metric terms for every x point:
//   y sweep: v = 0.5 R + t0 phi + t1 phi(k+1) + t2 phi(k-1)
//            t0 = 0.5 J - c (G11(k+1) + G11(k)), t1 = c G11(k+1), t2 = c G11(k)
//   z sweep: v = 0.5 R + t3 phi + t0 phs + t1 phs(j+1) + t2 phs(j-1)
//            t0 = J - c (G22(j+1) + G22(j)), t1 = c G22(j+1), t2 = c G22(j), t3 = -0.5 J
// (c = NU H/2 [/PR]; the same algebra as duct.F90:1640-1660, 1877-1905, ...)
template <bool ZS>
__global__ void k_adi_tab(Dims d, Metrics m, double coef, int sform, double *tab, float2 *tab2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (k > d.NZ + 1 || j > d.NY + 1 || k < 1 || j < 1) return;
  const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
  const double jac = m.jac[mm];
  double w[4];
  // R/2 = S/2 + J phi_old/2: with S in place of R the y sweep's J/2 becomes J
  // and the z sweep's -J phi_old/2 term cancels
  if (!ZS) {
    const double gp = m.g11[d.m3(k + 1, j, 2)], gm = m.g11[d.m3(k, j, 2)];
    w[0] = (sform ? jac : 0.5 * jac) - coef * (gp + gm);
    w[1] = coef * gp;
    w[2] = coef * gm;
  } else {
    const double gp = m.g22[d.m3(k, j + 1, 1)], gm = m.g22[d.m3(k, j, 1)];
    w[0] = jac - coef * (gp + gm);
    w[1] = coef * gp;
    w[2] = coef * gm;
    w[3] = sform ? 0.0 : -0.5 * jac;
  }
  for (int t = 0; t < (ZS ? 4 : 3); ++t) {
    tab[t * n2 + mm] = w[t];
    // the float-float sweeps read the same weights as float pairs
    if (tab2) {
      const FF f(w[t]);
      tab2[t * n2 + mm] = make_float2(f.hi, f.lo);
    }
  }
}

// A double array split into float-float pairs (hi, lo).
__global__ void k_split_ff(size_t n, const double *in, float2 *out) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const FF f(in[q]);
    out[q] = make_float2(f.hi, f.lo);
  }
}

// Per-cell weights of one LES ADI sweep (seven planes, ltab[t * n2 + m2(k, j)]):
//   t0 = -c Gb(lo), t1 = -c Gb(up), t2 = J + c (Gb(up) + Gb(lo))   the plain row
//   t3 = h Gm(lo),  t4 = h Gm(up)     eddy-viscosity face weights of the row
//   t5 = h Gr(+),   t6 = h Gr(-)      and of the explicit term across the line
// with c = NU H/2 [/PR], h = TEMP2/2 [/PR] (KAPPA_T = NU_T/PR for TH); Gb the
// plain metric of the line direction (GMAT_22 for y, GMAT_11 for z), Gm the
// LES metric of the line direction and Gr that of the other direction
// (GMAT_*, GMAT_*_y for U2, GMAT_*_z for U3).  Faces: y lines lo = (k,j,1),
// up = (k,j+1,1), across (k+1,j,2) / (k,j,2); z lines lo = (k,j,2),
// up = (k+1,j,2), across (k,j+1,1) / (k,j,1).
template <bool ZS>
__global__ void k_adi_les_tab(Dims d, Metrics m, const double *gb, const double *gm, const double *gr, double c,
                              double h, double *tab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (k < 1 || k > d.NZ || j < 1 || j > d.NY) return;
  const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
  const size_t lo = ZS ? d.m3(k, j, 2) : d.m3(k, j, 1), up = ZS ? d.m3(k + 1, j, 2) : d.m3(k, j + 1, 1);
  const size_t xp = ZS ? d.m3(k, j + 1, 1) : d.m3(k + 1, j, 2), xm = ZS ? d.m3(k, j, 1) : d.m3(k, j, 2);
  tab[mm] = -c * gb[lo];
  tab[n2 + mm] = -c * gb[up];
  tab[2 * n2 + mm] = m.jac[mm] + c * (gb[up] + gb[lo]);
  tab[3 * n2 + mm] = h * gm[lo];
  tab[4 * n2 + mm] = h * gm[up];
  tab[5 * n2 + mm] = h * gr[xp];
  tab[6 * n2 + mm] = h * gr[xm];
}

// Rows per chunk of the line-solve kernels below: a thread issues every
// load of a chunk's rows before its recurrence consumes them (the
// x-dependent LES rows hold more values per row than the plain ones).
constexpr int kAdiChunk = 8, kLesChunk = 4, kIncChunkY = 8, kIncChunkZ = 4;

// CN-ADI line solves with the LES eddy viscosity (duct.F90:1373-1386,
// 1437-1450, 1489-1500, 1559-1569 for TH; 1667-1680, 1720-1731, 1771-1784,
// 1821-1832 for U1; 1916-1929, 1963-1973, 2013-2026, 2081-2091 for U2 with
// GMAT_*_y; 2177-2190, 2224-2234, 2300-2313, 2358-2368 for U3 with GMAT_*_z):
// the matrix rows depend on x through NU_T, so each thread owns one system
// (one x point of one line) and builds every row -- the right-hand side of
// k_adi plus the NU_T term across the line, the tridiagonal row from the
// per-cell weights and the two face sums of NU_T, or the boundary row -- then
// runs the elimination of THOMAS_REAL (boundary.F90:53-84) with one
// reciprocal per row: the forward sweep parks 1/B and the upper diagonal in
// two scratch fields and the modified right-hand side in the output, the
// back substitution reads them back.  Consecutive threads take consecutive x
// points, so every access is coalesced; the work is FP64 arithmetic, about
// two dozen operations and one reciprocal per row.
template <bool ZS, bool SF>
__global__ void __launch_bounds__(128) k_adi_les(AdiArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int line = ZS ? (int)blockIdx.y : a.zs + (int)blockIdx.y;
  if (i >= d.NX) return;
  if (ZS && (line < a.js || line > a.je)) {
    for (int k = a.zs; k <= a.ze; ++k) a.out[d.ip(i, k, line)] = a.phs[d.ip(i, k, line)];
    return;
  }
  const int nrow = ZS ? d.NZ2 : d.NY2;
  const int r0 = ZS ? a.zs : a.js, r1 = ZS ? a.ze : a.je;
  const int n2 = d.LDM * (d.NY + 3);  // plane stride of the weight tables
  const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  const size_t sA = ZS ? sK : sJ;  // along the line
  const size_t sX = ZS ? sJ : sK;  // across: the direction of the explicit term
  const double *nut = a.nut, *R = a.R, *po = a.phi_old, *ps = a.phs;
  const double *px = ZS ? ps : po;  // field of the explicit term across the line
  // addresses advance along the line: the point by sA, the cell by 1 (z) or LDM (y)
  const size_t c0 = ZS ? d.ip(i, 0, line) : d.ip(i, line, 0);
  const int m0 = ZS ? line * d.LDM : line, mstep = ZS ? 1 : d.LDM;
  // chunked along y only (as in k_adi_seq)
  constexpr int CH = ZS ? 1 : kLesChunk, CB = ZS ? 1 : kAdiChunk;
  double rBp = 1.0, gp = 0.0, Up = 0.0;
  // rows CH at a time: the rows of a chunk are built (every load
  // issued) before the elimination runs through them
  for (int rc = 0; rc < nrow; rc += CH) {
    double Lv[CH], Dv[CH], Uv[CH], Vv[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      const size_t c = c0 + (size_t)r * sA;
      double L = 0.0, D = 1.0, U = 0.0, V = 0.0;
      if (r >= r0 && r <= r1) {
        const double *lt = a.ltab + (m0 + r * mstep), *tb = a.tab + (m0 + r * mstep);
        const double nu0 = nut[c], nap = nut[c + sA], nam = nut[c - sA];
        const double nxp = nut[c + sX], nxm = nut[c - sX];
        const double f0 = px[c], fxp = px[c + sX], fxm = px[c - sX];
        const double rv = SF ? f2d_bits(a.Sf[c]) : R[c];
        if (!ZS || SF) V = fma(0.5, rv, fma(tb[0], f0, fma(tb[n2], fxp, tb[2 * n2] * fxm)));
        else V = fma(0.5, rv, fma(tb[3 * n2], po[c], fma(tb[0], f0, fma(tb[n2], fxp, tb[2 * n2] * fxm))));
        const double tp = lt[5 * n2] * (nxp + nu0), tm = lt[6 * n2] * (nu0 + nxm);
        V = fma(tp, fxp - f0, fma(-tm, f0 - fxm, V));
        const double slo = nu0 + nam, sup = nu0 + nap;
        const double ml = lt[3 * n2], mu = lt[4 * n2];
        L = fma(-ml, slo, lt[0]);
        U = fma(-mu, sup, lt[n2]);
        D = fma(mu, sup, fma(ml, slo, lt[2 * n2]));
      }
      if (r < nrow)
        for (int b = 0; b < a.bc.n; ++b) {
          const BcRow &br = a.bc.r[b];
          if (br.row != r) continue;
          L = br.l;
          D = br.dg;
          U = br.u;
          if (br.kind == 0) V = br.val;
          else if (br.kind == 1) V = ZS ? ps[d.ip(i, br.src, line)] : po[d.ip(i, line, br.src)];
          else V = br.val * a.bcw[br.src + line];
        }
      Lv[u] = L;
      Dv[u] = D;
      Uv[u] = U;
      Vv[u] = V;
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      if (r >= nrow) break;
      const size_t c = c0 + (size_t)r * sA;
      double B, g;
      if (r == 0) {
        B = Dv[u];
        g = Vv[u];
      } else {
        const double am = -Lv[u] * rBp;
        B = fma(am, Up, Dv[u]);
        g = fma(am, gp, Vv[u]);
      }
      const double rB = __drcp_rn(B);
      a.out[c] = g;
      a.scr_b[c] = rB;
      a.scr_u[c] = Uv[u];
      rBp = rB;
      gp = g;
      Up = Uv[u];
    }
  }
  double x = gp * rBp;
  a.out[c0 + (size_t)(nrow - 1) * sA] = x;
  for (int rc = nrow - 2; rc >= 0; rc -= CB) {
    double gv[CB], uv[CB], bv[CB];
#pragma unroll
    for (int u = 0; u < CB; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        const size_t c = c0 + (size_t)r * sA;
        gv[u] = a.out[c];
        uv[u] = a.scr_u[c];
        bv[u] = a.scr_b[c];
      }
    }
#pragma unroll
    for (int u = 0; u < CB; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        x = fma(-uv[u], x, gv[u]) * bv[u];
        a.out[c0 + (size_t)r * sA] = x;
      }
    }
  }
}

// Float-float reciprocal: the FP32 reciprocal and one Newton step in
// float-float (about 46 bits).
__device__ __forceinline__ FF ff_rcp(FF b) {
  const float r0 = __frcp_rn(b.hi);
  float e = __fmaf_rn(-b.hi, r0, 1.0f);
  e = __fmaf_rn(-b.lo, r0, e);
  return ff_norm(r0, __fmul_rn(r0, e));
}
__device__ __forceinline__ FF ff2(float2 v) { return FF(v.x, v.y); }
__device__ __forceinline__ FF ff1(float v) { return FF(v, 0.0f); }

// The weights of one sweep's two tables split into float-float planes.
__global__ void k_adi_ff_tab(int n2, const double *rhs_tab, const double *row_tab, float2 *ftab) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n2) return;
  for (int p = 0; p < 11; ++p) {
    const double v = (p < 4) ? rhs_tab[(size_t)p * n2 + m] : row_tab[(size_t)(p - 4) * n2 + m];
    const FF f(v);
    ftab[(size_t)p * n2 + m] = make_float2(f.hi, f.lo);
  }
}

// k_adi_les in float-float arithmetic, for the mixed-precision method: the
// rows, the elimination and the back substitution run on the FP32 pipe at
// about 46 significant bits; the FP64 pipe only splits the five FP64 inputs
// of a row and joins the result.  The eliminated rows go to the scratch
// fields (and the modified right-hand side into the output) as float pairs
// in the same 8-byte slots.
template <bool ZS, bool SF>
__global__ void __launch_bounds__(128) k_adi_les_ff(AdiArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int line = ZS ? (int)blockIdx.y : a.zs + (int)blockIdx.y;
  if (i >= d.NX) return;
  if (ZS && (line < a.js || line > a.je)) {
    for (int k = a.zs; k <= a.ze; ++k) a.out[d.ip(i, k, line)] = a.phs[d.ip(i, k, line)];
    return;
  }
  const int nrow = ZS ? d.NZ2 : d.NY2;
  const int r0 = ZS ? a.zs : a.js, r1 = ZS ? a.ze : a.je;
  const int n2 = d.LDM * (d.NY + 3);
  const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  const size_t sA = ZS ? sK : sJ;
  const size_t sX = ZS ? sJ : sK;
  const float *nut = a.nutf;
  const double *R = a.R, *po = a.phi_old, *ps = a.phs;
  const double *px = ZS ? ps : po;
  float2 *gout = reinterpret_cast<float2 *>(a.out);
  float2 *sb = reinterpret_cast<float2 *>(a.scr_b), *su = reinterpret_cast<float2 *>(a.scr_u);
  const size_t c0 = ZS ? d.ip(i, 0, line) : d.ip(i, line, 0);
  const int m0 = ZS ? line * d.LDM : line, mstep = ZS ? 1 : d.LDM;
  // chunked along y only (as in k_adi_seq)
  constexpr int CH = ZS ? 1 : kLesChunk, CB = ZS ? 1 : kAdiChunk;
  FF rBp(1.0f, 0.0f), gp(0.0f, 0.0f), Up(0.0f, 0.0f);
  for (int rc = 0; rc < nrow; rc += CH) {
    FF Lv[CH], Dv[CH], Uv[CH], Vv[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      const size_t c = c0 + (size_t)r * sA;
      FF L(0.0f, 0.0f), D(1.0f, 0.0f), U(0.0f, 0.0f), V(0.0f, 0.0f);
      if (r >= r0 && r <= r1) {
        const float2 *t = a.ftab + (m0 + r * mstep);
        const float nu0 = nut[c], nap = nut[c + sA], nam = nut[c - sA], nxp = nut[c + sX], nxm = nut[c - sX];
        const FF f0(px[c]), fxp(px[c + sX]), fxm(px[c - sX]);
        const FF rr = SF ? FF(a.Sf[c], 0.0f) : FF(R[c]);
        FF v = FF(0.5f * rr.hi, 0.5f * rr.lo);
        if (!ZS) {
          v = v + ff2(t[0]) * f0 + ff2(t[n2]) * fxp + ff2(t[2 * n2]) * fxm;
        } else if (SF) {
          v = v + ff2(t[0]) * f0 + ff2(t[n2]) * fxp + ff2(t[2 * n2]) * fxm;
        } else {
          const FF p0(po[c]);
          v = v + ff2(t[3 * n2]) * p0 + ff2(t[0]) * f0 + ff2(t[n2]) * fxp + ff2(t[2 * n2]) * fxm;
        }
        const FF tp = ff2(t[9 * n2]) * (ff1(nxp) + ff1(nu0)), tm = ff2(t[10 * n2]) * (ff1(nu0) + ff1(nxm));
        V = v + tp * (fxp - f0) - tm * (f0 - fxm);
        const FF slo = ff1(nu0) + ff1(nam), sup = ff1(nu0) + ff1(nap);
        const FF ml = ff2(t[7 * n2]), mu = ff2(t[8 * n2]);
        L = ff2(t[4 * n2]) - ml * slo;
        U = ff2(t[5 * n2]) - mu * sup;
        D = ff2(t[6 * n2]) + mu * sup + ml * slo;
      }
      if (r < nrow)
        for (int b = 0; b < a.bc.n; ++b) {
          const BcRow &br = a.bc.r[b];
          if (br.row != r) continue;
          L = FF(br.l);
          D = FF(br.dg);
          U = FF(br.u);
          if (br.kind == 0) V = FF(br.val);
          else if (br.kind == 1) V = FF(ZS ? ps[d.ip(i, br.src, line)] : po[d.ip(i, line, br.src)]);
          else V = FF(br.val * a.bcw[br.src + line]);
        }
      Lv[u] = L;
      Dv[u] = D;
      Uv[u] = U;
      Vv[u] = V;
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      if (r >= nrow) break;
      const size_t c = c0 + (size_t)r * sA;
      FF B, g;
      if (r == 0) {
        B = Dv[u];
        g = Vv[u];
      } else {
        const FF am = -(Lv[u] * rBp);
        B = Dv[u] + am * Up;
        g = Vv[u] + am * gp;
      }
      const FF rB = ff_rcp(B);
      gout[c] = make_float2(g.hi, g.lo);
      sb[c] = make_float2(rB.hi, rB.lo);
      su[c] = make_float2(Uv[u].hi, Uv[u].lo);
      rBp = rB;
      gp = g;
      Up = Uv[u];
    }
  }
  FF x = gp * rBp;
  a.out[c0 + (size_t)(nrow - 1) * sA] = (double)x;
  for (int rc = nrow - 2; rc >= 0; rc -= CB) {
    float2 gv[CB], uv[CB], bv[CB];
#pragma unroll
    for (int u = 0; u < CB; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        const size_t c = c0 + (size_t)r * sA;
        gv[u] = gout[c];
        uv[u] = su[c];
        bv[u] = sb[c];
      }
    }
#pragma unroll
    for (int u = 0; u < CB; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        x = (ff2(gv[u]) - ff2(uv[u]) * x) * ff2(bv[u]);
        a.out[c0 + (size_t)r * sA] = (double)x;
      }
    }
  }
}

// CN-ADI line solves, one thread per system (one x point of one line).
// y sweep (ZS = false), duct.F90:1640-1739 for U1 (TH 1334-1433, U2
// 1877-1980, U3 2137-2233): R' = S/2 + J phi + coef d_zeta(G11 d_zeta phi),
// S = R - J phi; the solution of each (I,K) line goes to phs.
// z sweep (ZS = true), duct.F90:1741-1854 for U1 (TH 1437-1600, U2
// 1983-2115, U3 2257-2392): R'' = S/2 + J phi* + coef d_eta(G22 d_eta phi*);
// the solution of each (I,J) line goes into the field; rows J outside the
// solved range take the y-sweep values.
// The thread forms each row's right-hand side from the per-cell weights
// (k_adi_tab), runs the forward elimination of THOMAS_REAL with the line's
// host factors (broadcast loads: a block's threads share the line) and parks
// the modified right-hand side in the output, then back-substitutes.  Along
// y, rows go kAdiChunk at a time: every load of a chunk is issued before the
// recurrence consumes it, so a thread keeps that many rows' loads in flight
// instead of waiting out one memory latency per row.  (A block of eight
// warps that built the rows in shared memory while one warp ran the
// recurrences took twice as long: seven warps idled through the sequential
// part.)  In the z sweep the output is the field itself: a row's old value
// is loaded (with its chunk) before the row is stored.
template <bool ZS, bool SF>
__global__ void __launch_bounds__(128) k_adi_seq(AdiArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int line = ZS ? (int)blockIdx.y : a.zs + (int)blockIdx.y;
  if (i >= d.NX) return;
  if (ZS && (line < a.js || line > a.je)) {
    for (int k = a.zs; k <= a.ze; ++k) a.out[d.ip(i, k, line)] = a.phs[d.ip(i, k, line)];
    return;
  }
  const int nrow = ZS ? d.NZ2 : d.NY2;
  const int r0 = ZS ? a.zs : a.js, r1 = ZS ? a.ze : a.je;
  const int n2 = d.LDM * (d.NY + 3);
  const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  const size_t sA = ZS ? sK : sJ;
  const size_t sX = ZS ? sJ : sK;
  const double *R = a.R, *po = a.phi_old, *ps = a.phs;
  const double *px = ZS ? ps : po;
  const double *fa = a.fa + (size_t)line * nrow, *fib = a.fib + (size_t)line * nrow, *fu = a.fu + (size_t)line * nrow;
  const size_t c0 = ZS ? d.ip(i, 0, line) : d.ip(i, line, 0);
  const int m0 = ZS ? line * d.LDM : line, mstep = ZS ? 1 : d.LDM;
  // chunks along y; the z sweep (a field in place, rows LDX apart) measured
  // slower with them, so it keeps one row at a time
  constexpr int CH = ZS ? 1 : kAdiChunk;
  double prev = 0.0;
  for (int rc = 0; rc < nrow; rc += CH) {
    double vv[CH], av[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      double v = 0.0;
      if (r < nrow) {
        const size_t c = c0 + (size_t)r * sA;
        if (r >= r0 && r <= r1) {
          const double *tb = a.tab + (m0 + r * mstep);
          // SF: the explicit increment S in FP32 (a.Sf), no phi_old term in z
          const double rv = SF ? f2d_bits(a.Sf[c]) : R[c];
          if (!ZS || SF) v = fma(0.5, rv, fma(tb[0], px[c], fma(tb[n2], px[c + sX], tb[2 * n2] * px[c - sX])));
          else v = fma(0.5, rv, fma(tb[3 * n2], po[c], fma(tb[0], px[c], fma(tb[n2], px[c + sX], tb[2 * n2] * px[c - sX]))));
        }
        for (int b = 0; b < a.bc.n; ++b) {
          const BcRow &br = a.bc.r[b];
          if (br.row != r) continue;
          if (br.kind == 0) v = br.val;
          else if (br.kind == 1) v = ZS ? ps[d.ip(i, br.src, line)] : po[d.ip(i, line, br.src)];
          else v = br.val * a.bcw[br.src + line];
        }
      }
      vv[u] = v;
      av[u] = (r < nrow) ? fa[r] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      if (r < nrow) {
        prev = (r == 0) ? vv[u] : vv[u] + av[u] * prev;
        a.out[c0 + (size_t)r * sA] = prev;
      }
    }
  }
  double x = prev * fib[nrow - 1];
  a.out[c0 + (size_t)(nrow - 1) * sA] = x;
  for (int rc = nrow - 2; rc >= 0; rc -= CH) {
    double gv[CH], uv[CH], bv[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        gv[u] = a.out[c0 + (size_t)r * sA];
        uv[u] = fu[r];
        bv[u] = fib[r];
      }
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        x = (gv[u] - uv[u] * x) * bv[u];
        a.out[c0 + (size_t)r * sA] = x;
      }
    }
  }
}

// k_adi_seq (explicit-increment form) on float-float fields, for the mixed
// path: the old field, the y-sweep result and the new field are float-float
// planes and every row runs in float-float arithmetic (about 48 bits) on the
// FP32 pipe, from the same per-cell weights and host Thomas factors split
// into float pairs; the only FP64 work left is a boundary row's constant.
template <bool ZS>
__global__ void __launch_bounds__(128) k_adi_ffs(AdiArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int line = ZS ? (int)blockIdx.y : a.zs + (int)blockIdx.y;
  if (i >= d.NX) return;
  if (ZS && (line < a.js || line > a.je)) {
    for (int k = a.zs; k <= a.ze; ++k) {
      const size_t c = d.ip(i, k, line);
      a.out_h[c] = a.ps_h[c];
      a.out_l[c] = a.ps_l[c];
    }
    return;
  }
  const int nrow = ZS ? d.NZ2 : d.NY2;
  const int r0 = ZS ? a.zs : a.js, r1 = ZS ? a.ze : a.je;
  const int n2 = d.LDM * (d.NY + 3);
  const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  const size_t sA = ZS ? sK : sJ;
  const size_t sX = ZS ? sJ : sK;
  // the y sweep reads the old field, the z sweep the y sweep's result
  const float *xh = ZS ? a.ps_h : a.po_h, *xl = ZS ? a.ps_l : a.po_l;
  const float2 *fa = a.fa2 + (size_t)line * nrow, *fib = a.fib2 + (size_t)line * nrow;
  const float2 *fu = a.fu2 + (size_t)line * nrow;
  const size_t c0 = ZS ? d.ip(i, 0, line) : d.ip(i, line, 0);
  const int m0 = ZS ? line * d.LDM : line, mstep = ZS ? 1 : d.LDM;
  constexpr int CH = ZS ? 1 : kAdiChunk;
  FF prev(0.0f, 0.0f);
  for (int rc = 0; rc < nrow; rc += CH) {
    FF vv[CH];
    float2 av[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      FF v(0.0f, 0.0f);
      if (r < nrow) {
        const size_t c = c0 + (size_t)r * sA;
        if (r >= r0 && r <= r1) {
          const float2 *tb = a.tab2 + (m0 + r * mstep);
          v = FF(0.5f * a.Sf[c], 0.0f) + ff2(tb[0]) * FF(xh[c], xl[c]) + ff2(tb[n2]) * FF(xh[c + sX], xl[c + sX]) +
              ff2(tb[2 * n2]) * FF(xh[c - sX], xl[c - sX]);
        }
        for (int b = 0; b < a.bc.n; ++b) {
          const BcRow &br = a.bc.r[b];
          if (br.row != r) continue;
          if (br.kind == 0) {
            v = FF(br.val);
          } else if (br.kind == 1) {
            const size_t q = ZS ? d.ip(i, br.src, line) : d.ip(i, line, br.src);
            v = FF(xh[q], xl[q]);
          } else {
            v = FF(br.val * a.bcw[br.src + line]);
          }
        }
      }
      vv[u] = v;
      av[u] = (r < nrow) ? fa[r] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      if (r < nrow) {
        prev = (r == 0) ? vv[u] : vv[u] + ff2(av[u]) * prev;
        const size_t c = c0 + (size_t)r * sA;
        a.out_h[c] = prev.hi;
        a.out_l[c] = prev.lo;
      }
    }
  }
  FF x = prev * ff2(fib[nrow - 1]);
  {
    const size_t c = c0 + (size_t)(nrow - 1) * sA;
    a.out_h[c] = x.hi;
    a.out_l[c] = x.lo;
  }
  for (int rc = nrow - 2; rc >= 0; rc -= CH) {
    FF gv[CH];
    float2 uv[CH], bv[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        const size_t c = c0 + (size_t)r * sA;
        gv[u] = FF(a.out_h[c], a.out_l[c]);
        uv[u] = fu[r];
        bv[u] = fib[r];
      }
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        x = (gv[u] - ff2(uv[u]) * x) * ff2(bv[u]);
        const size_t c = c0 + (size_t)r * sA;
        a.out_h[c] = x.hi;
        a.out_l[c] = x.lo;
      }
    }
  }
}

// The ADI in increment form, FP32 (the mixed path with ff_arith = 2).  Each
// sweep's tridiagonal system M phi_new = v (the rows of k_adi_seq: interior
// rows (J - c A_line) with v = S/2 + (J + c A_across) phi_base, the boundary
// rows of APPLY_BC_*, identity rows elsewhere) is solved for the increment
// over its base field, M (phi_new - phi_base) = v - M phi_base.  For an
// interior row that right-hand side is S/2 + c (A_k + A_j) phi_base: the
// J phi terms cancel algebraically, so nothing of size J phi is rounded to
// FP32, only the O(h) increment S and the O(c) viscous differences.  The y
// sweep's base is phi_old (the field's FP32 copy) and its output the
// increment d*; the z sweep's base is phi* = phi_old + d* (d* = 0 on the
// lines the y sweep leaves alone) and its output the total increment
// phi_new - phi_old, whose FP32 forward transform is added to the spectral
// state.  The same host Thomas factors and per-cell weights, rounded to
// FP32, drive the elimination.
template <bool ZS>
__global__ void __launch_bounds__(128) k_adi_inc(AdiArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int line = ZS ? (int)blockIdx.y : a.zs + (int)blockIdx.y;
  if (i >= d.NX) return;
  const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  const float *ph = a.phf, *ds = a.dsf;
  float *out = a.incf;
  // the base field of the sweep at point q (row k along z)
  auto base = [&](size_t q, int k) -> float {
    return (ZS && k >= a.zs && k <= a.ze) ? ph[q] + ds[q] : ph[q];
  };
  if (ZS && (line < a.js || line > a.je)) {
    // phi_new = phi* on the y sweep's lines, phi_old elsewhere
    for (int k = 0; k < d.NZ2; ++k) {
      const size_t q = d.ip(i, k, line);
      out[q] = (k >= a.zs && k <= a.ze) ? ds[q] : 0.0f;
    }
    return;
  }
  const int nrow = ZS ? d.NZ2 : d.NY2;
  const int r0 = ZS ? a.zs : a.js, r1 = ZS ? a.ze : a.je;
  const int n2 = d.LDM * (d.NY + 3);
  const size_t sA = ZS ? sK : sJ;
  const float2 *fa = a.fa2 + (size_t)line * nrow, *fib = a.fib2 + (size_t)line * nrow;
  const float2 *fu = a.fu2 + (size_t)line * nrow;
  // per-cell weights c G11(k+1), c G11(k) (the y table) and c G22(j+1),
  // c G22(j) (the z table), high parts of the float pairs
  const float2 *wk = a.tab2, *wj = a.tab2 + 4 * (size_t)n2;
  const size_t c0 = ZS ? d.ip(i, 0, line) : d.ip(i, line, 0);
  const size_t sX = ZS ? sJ : sK;
  // rows go CH at a time: the chunk's base values along the line (rows
  // rc-1 .. rc+CH) are loaded once and shared by neighbouring rows, and
  // every load of the chunk is issued before the recurrence consumes it
  constexpr int CH = ZS ? kIncChunkZ : kIncChunkY;
  auto base_row = [&](int r) -> float {
    if (r < 0 || r >= nrow) return 0.0f;
    return base(c0 + (size_t)r * sA, ZS ? r : line);
  };
  float prev = 0.0f;
  for (int rc = 0; rc < nrow; rc += CH) {
    float vv[CH], av[CH], bp[CH + 2];
#pragma unroll
    for (int u = 0; u < CH + 2; ++u) bp[u] = base_row(rc - 1 + u);
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      float v = 0.0f;
      if (r < nrow) {
        const size_t q = c0 + (size_t)r * sA;
        const int k = ZS ? r : line, j = ZS ? line : r;
        const float p0 = bp[u + 1];
        if (r >= r0 && r <= r1) {
          const int m = d.m2(k, j);
          // along the line: bp; across it: rows of the neighbouring lines
          const float pap = bp[u + 2], pam = bp[u];
          const float pxp = base(q + sX, k), pxm = base(q - sX, k);
          const float pkp = ZS ? pap : pxp, pkm = ZS ? pam : pxm;
          const float pjp = ZS ? pxp : pap, pjm = ZS ? pxm : pam;
          v = 0.5f * a.Sf[q] + (wk[n2 + m].x * (pkp - p0) - wk[2 * n2 + m].x * (p0 - pkm)) +
              (wj[n2 + m].x * (pjp - p0) - wj[2 * n2 + m].x * (p0 - pjm));
        } else {
          v = -p0;  // identity row: phi_new = 0
        }
        for (int b = 0; b < a.bc.n; ++b) {
          const BcRow &br = a.bc.r[b];
          if (br.row != r) continue;
          if (br.kind == 1) {
            // the lagged copy (an identity row): phi_base(src) - phi_base(row)
            // = (phi_old(src) - phi_old(row)) + (d*(src) - d*(row)) in z,
            // the first part from the spectral difference, so the FP32
            // roundings of the two old values never enter the ghost rows
            float dv = a.brk[q];
            if (ZS) {
              const size_t qs = d.ip(i, br.src, line);
              if (br.src >= a.zs && br.src <= a.ze) dv += ds[qs];
              if (k >= a.zs && k <= a.ze) dv -= ds[q];
            }
            v = dv;
            continue;
          }
          const float vb = (br.kind == 0) ? (float)br.val : (float)(br.val * a.bcw[br.src + line]);
          float mrow = (float)br.dg * p0;
          if (r > 0) mrow += (float)br.l * bp[u];
          if (r + 1 < nrow) mrow += (float)br.u * bp[u + 2];
          v = vb - mrow;
        }
      }
      vv[u] = v;
      av[u] = (r < nrow) ? fa[r].x : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc + u;
      if (r < nrow) {
        prev = (r == 0) ? vv[u] : fmaf(av[u], prev, vv[u]);
        out[c0 + (size_t)r * sA] = prev;  // parked until the back substitution
      }
    }
  }
  // back substitution; the z sweep adds d* to its increment for the total
  float x = prev * fib[nrow - 1].x;
  {
    const size_t q = c0 + (size_t)(nrow - 1) * sA;
    const int k = ZS ? nrow - 1 : line;
    out[q] = (ZS && k >= a.zs && k <= a.ze) ? x + ds[q] : x;
  }
  for (int rc = nrow - 2; rc >= 0; rc -= CH) {
    float gv[CH], uv[CH], bv[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        gv[u] = out[c0 + (size_t)r * sA];
        uv[u] = fu[r].x;
        bv[u] = fib[r].x;
      }
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int r = rc - u;
      if (r >= 0) {
        x = (gv[u] - uv[u] * x) * bv[u];
        const size_t q = c0 + (size_t)r * sA;
        const int k = ZS ? r : line;
        out[q] = (ZS && k >= a.zs && k <= a.ze) ? x + ds[q] : x;
      }
    }
  }
}

// TH corner copies (duct.F90:1606-1624) in increment form: the corner's new
// value is its neighbour's, so its increment is phi_old(nb) + d(nb) -
// phi_old(corner).
__global__ void k_th_corners_inc(Dims d, const float *TH, float *dTH, int zmax1, int zmin6) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NX) return;
  const int NZ = d.NZ, NY = d.NY;
  auto cp = [&](int kd, int jd, int ks, int js) {
    const size_t q = d.ip(i, kd, jd), s = d.ip(i, ks, js);
    dTH[q] = (TH[s] + dTH[s]) - TH[q];
  };
  if (zmax1) {
    cp(NZ + 1, NY + 1, NZ, NY + 1);
    cp(NZ + 1, 0, NZ, 0);
    cp(0, NY + 1, 1, NY + 1);
    cp(0, 0, 1, 0);
  }
  if (zmin6) {
    cp(NZ + 1, NY + 1, 1, NY + 1);
    cp(NZ + 1, 0, 1, 0);
    cp(0, NY + 1, NZ, NY + 1);
    cp(0, 0, NZ, 0);
  }
}

// Corner copies after the TH solve (duct.F90:1606-1624); T = double, or
// float for each plane of a float-float field.
template <typename T>
__global__ void k_th_corners(Dims d, T *TH, int zmax1, int zmin6) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.NX) return;
  const int NZ = d.NZ, NY = d.NY;
  if (zmax1) {
    TH[d.ip(i, NZ + 1, NY + 1)] = TH[d.ip(i, NZ, NY + 1)];
    TH[d.ip(i, NZ + 1, 0)] = TH[d.ip(i, NZ, 0)];
    TH[d.ip(i, 0, NY + 1)] = TH[d.ip(i, 1, NY + 1)];
    TH[d.ip(i, 0, 0)] = TH[d.ip(i, 1, 0)];
  }
  if (zmin6) {
    TH[d.ip(i, NZ + 1, NY + 1)] = TH[d.ip(i, 1, NY + 1)];
    TH[d.ip(i, NZ + 1, 0)] = TH[d.ip(i, 1, 0)];
    TH[d.ip(i, 0, NY + 1)] = TH[d.ip(i, NZ, NY + 1)];
    TH[d.ip(i, 0, 0)] = TH[d.ip(i, NZ, 0)];
  }
}

// REM_DIV_CURV face velocities CU2b, CU3b (duct.F90:2511-2522), zero
// elsewhere (2501-2503); CU3b follows CU2b in memory.
__global__ void k_rem_faces(Dims d, Metrics m, const cplx_t *CU2, const cplx_t *CU3, cplx_t *CU2b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, j = blockIdx.z;
  if (i > d.NX2P) return;
  cplx_t *CU3b = CU2b + d.nspec();
  const size_t q = d.ic(i, k, j);
  if (j >= d.JS && j <= d.JE + 1 && k >= d.ZS && k <= d.ZE + 1) {
    const size_t sK = d.LDC, sJ = (size_t)d.LDC * d.NZ2;
    CU2b[q] = cadd(cscl(0.5 * m.c22[d.m3(k, j, 1)], cadd(CU2[q], CU2[q - sJ])),
                   cscl(0.5 * m.c21[d.m3(k, j, 1)], cadd(CU3[q], CU3[q - sJ])));
    CU3b[q] = cadd(cscl(0.5 * m.c11[d.m3(k, j, 2)], cadd(CU3[q], CU3[q - sK])),
                   cscl(0.5 * m.c12[d.m3(k, j, 2)], cadd(CU2[q], CU2[q - sK])));
  } else {
    CU2b[q] = cplx_t{0.0, 0.0};
    CU3b[q] = cplx_t{0.0, 0.0};
  }
}

// Divergence (duct.F90:2527-2535) written straight into the multigrid
// right-hand side: problem p = 2I (real part) or 2I+1 (imaginary part) of
// mode I, MUDPACK point (K+1, J+1); RHS_TMP is zero outside the range
// (2631-2651) and phi_bc negates -Re/-Im back.
__global__ void k_div_rhs(Dims d, const double *kx, const cplx_t *CU1, const cplx_t *CU2b, const double *jacm,
                          double *rhs, int P) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, j = blockIdx.z;  // full 0..NZ+1, 0..NY+1
  if (p >= P) return;
  const int I = p >> 1;
  double v = 0.0;
  if (j >= d.JS && j <= d.JE && k >= d.ZS && k <= d.ZE) {
    const cplx_t *CU3b = CU2b + d.nspec();
    const size_t q = d.ic(I, k, j);
    const size_t sK = d.LDC, sJ = (size_t)d.LDC * d.NZ2;
    // only the part this problem needs: i kx J CU1 has real part
    // -kx J Im CU1 and imaginary part kx J Re CU1 (the zero real part of
    // i kx dropped; GB300's FP64 pipe is the limit here)
    const double kj = kx[I] * jacm[d.m2(k, j)];
    if (p & 1) v = (kj * CU1[q].re + (CU2b[q + sJ].im - CU2b[q].im)) + (CU3b[q + sK].im - CU3b[q].im);
    else v = (-(kj * CU1[q].im) + (CU2b[q + sJ].re - CU2b[q].re)) + (CU3b[q + sK].re - CU3b[q].re);
  }
  const int nfx = d.NZ2;
  rhs[((size_t)j * nfx + k) * P + p] = v;
}

// phi back into CR1 (CMPLX(P_TMP2,P_TMP), duct.F90:2662-2666; REAL*4
// rounding under quirk_phi_fp32), modes above the solved set are zero, and
// the pressure update CP += CR1/h (duct.F90:2460-2466) when requested.
__global__ void k_phi_to_cr1(Dims d, const double *phif, int P, cplx_t *CR1, cplx_t *CP, double temp4, double rtemp4,
                             int update_p,
                             int fp32) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, j = blockIdx.z;
  if (I > d.NX2P) return;
  cplx_t v{0.0, 0.0};
  if (2 * I + 1 < P) {
    const size_t b = ((size_t)j * d.NZ2 + k) * P + 2 * I;
    v.re = phif[b];
    v.im = phif[b + 1];
    if (fp32) {
      v.re = (double)(float)v.re;
      v.im = (double)(float)v.im;
    }
  }
  const size_t q = d.ic(I, k, j);
  CR1[q] = v;
  if (update_p && j >= d.JS - 1 && j <= d.JE + 1 && k >= d.ZS - 1 && k <= d.ZE + 1) {
    const cplx_t o = CP[q];
    const DivBy div(temp4, rtemp4);
    CP[q] = cplx_t{o.re + div(v.re), o.im + div(v.im)};
  }
}

// Face-velocity correction (duct.F90:2709-2724).
__global__ void k_correct_faces(Dims d, Metrics m, const cplx_t *CR1, cplx_t *CU2b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = d.ZS + blockIdx.y, j = d.JS + blockIdx.z;
  if (i > d.NX2P) return;
  cplx_t *CU3b = CU2b + d.nspec();
  const size_t q = d.ic(i, k, j);
  const size_t sK = d.LDC, sJ = (size_t)d.LDC * d.NZ2;
  auto P = [&](int dk, int dj) { return CR1[q + (long)dk * (long)sK + (long)dj * (long)sJ]; };
  // the same terms with each metric product fused into its subtraction
  const cplx_t p00 = P(0, 0), p0m = P(0, -1), pm0 = P(-1, 0), pmm = P(-1, -1);
  const cplx_t p10 = P(1, 0), p1m = P(1, -1), p01 = P(0, 1), pm1 = P(-1, 1);
  const double a22 = m.g22[d.m3(k, j, 1)], a12 = 0.25 * m.g12[d.m3(k, j, 1)];
  const double b11 = m.g11[d.m3(k, j, 2)], b12 = 0.25 * m.g12[d.m3(k, j, 2)];
  const cplx_t u = CU2b[q], w = CU3b[q];
  CU2b[q] = cplx_t{fma(-a12, ((p10.re + p1m.re) - pm0.re) - pmm.re, fma(-a22, p00.re - p0m.re, u.re)),
                   fma(-a12, ((p10.im + p1m.im) - pm0.im) - pmm.im, fma(-a22, p00.im - p0m.im, u.im))};
  CU3b[q] = cplx_t{fma(-b12, ((p01.re + pm1.re) - p0m.re) - pmm.re, fma(-b11, p00.re - pm0.re, w.re)),
                   fma(-b12, ((p01.im + pm1.im) - p0m.im) - pmm.im, fma(-b11, p00.im - pm0.im, w.im))};
}

// Cell-centre correction (duct.F90:2729-2750).
__global__ void k_correct_cells(Dims d, Metrics m, const double *kx, const cplx_t *CR1, cplx_t *CU1, cplx_t *CU2,
                                cplx_t *CU3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = d.ZS + blockIdx.y, j = d.JS + blockIdx.z;
  if (i > d.NX2P) return;
  const size_t q = d.ic(i, k, j);
  const size_t sK = d.LDC, sJ = (size_t)d.LDC * d.NZ2;
  auto P = [&](int dk, int dj) { return CR1[q + (long)dk * (long)sK + (long)dj * (long)sJ]; };
  const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
  const cplx_t p00 = P(0, 0), p10 = P(1, 0), pm0 = P(-1, 0), p01 = P(0, 1), p0m = P(0, -1);
  const cplx_t o1 = CU1[q];
  CU1[q] = cplx_t{fma(kx[i], p00.im, o1.re), fma(-kx[i], p00.re, o1.im)};  // CU1 -= i kx phi
  const double rj = m.pg[10 * n2 + mm];
  const cplx_t u2 = pg_dot(m.pg, n2, 0, mm, p00, p10, pm0, p01, p0m);  // 0.5 (CJOB_22, CJOB_12 terms)
  const cplx_t o2 = CU2[q];
  CU2[q] = cplx_t{fma(-u2.re, rj, o2.re), fma(-u2.im, rj, o2.im)};
  const cplx_t u3 = pg_dot(m.pg, n2, 5, mm, p00, p10, pm0, p01, p0m);  // 0.5 (CJOB_11, CJOB_21 terms)
  const cplx_t o3 = CU3[q];
  CU3[q] = cplx_t{fma(-u3.re, rj, o3.re), fma(-u3.im, rj, o3.im)};
}

// Divergence after the projection (duct.F90:2754-2761) into CS.
__global__ void k_div_check(Dims d, const double *kx, const double *jacm, const cplx_t *CU1, const cplx_t *CU2b,
                            cplx_t *CS) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y, j = blockIdx.z;
  if (i > d.NX2P) return;
  const size_t q = d.ic(i, k, j);
  cplx_t v{0.0, 0.0};
  if (j >= d.JS && j <= d.JE && k >= d.ZS && k <= d.ZE) {
    const cplx_t *CU3b = CU2b + d.nspec();
    const size_t sK = d.LDC, sJ = (size_t)d.LDC * d.NZ2;
    const double kj = kx[i] * jacm[d.m2(k, j)];
    const cplx_t u1 = CU1[q], a0 = CU2b[q], a1 = CU2b[q + sJ], b0 = CU3b[q], b1 = CU3b[q + sK];
    v.re = (-(kj * u1.im) + (a1.re - a0.re)) + (b1.re - b0.re);
    v.im = (kj * u1.re + (a1.im - a0.im)) + (b1.im - b0.im);
  }
  CS[q] = v;
}

// The same sums from the FP32 plane of the mixed path's FP32 transform (its
// values are exactly the FP32 results the FP64 plane would hold widened):
// each thread accumulates in float-float on the FP32 pipe, then the block
// reduces in FP64 as above.  GB300's FP64 pipe made the FP64 sums of 50 M
// values a 0.3 ms kernel.
__global__ void k_div_sum_f(Dims d, const float *S, double *part) {
  const int j = 2 + blockIdx.x;
  __shared__ double red[256];
  // four accumulators over consecutive K, so four dependent chains interleave
  FF s[4] = {FF(0.0f, 0.0f), FF(0.0f, 0.0f), FF(0.0f, 0.0f), FF(0.0f, 0.0f)};
  for (int i = 1 + threadIdx.x; i <= d.NX + 1; i += blockDim.x) {
    int k = 2;
    for (; k + 3 <= d.NZ - 1; k += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) s[u] = s[u] + FF(fabsf(S[d.ip(i, k + u, j)]), 0.0f);
    }
    for (; k <= d.NZ - 1; ++k) s[0] = s[0] + FF(fabsf(S[d.ip(i, k, j)]), 0.0f);
  }
  red[threadIdx.x] = (double)((s[0] + s[1]) + (s[2] + s[3]));
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Sum of |div| over I = 1..NXP, K = 2..NZ-1 per line J (duct.F90:2790-2798);
// one block per J, fixed summation order.
__global__ void k_div_sum(Dims d, const double *S, double *part) {
  const int j = 2 + blockIdx.x;
  __shared__ double red[256];
  double s = 0.0;
  for (int k = 2; k <= d.NZ - 1; ++k)
    for (int i = 1 + threadIdx.x; i <= d.NX + 1; i += blockDim.x) s += fabs(S[d.ip(i, k, j)]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

}  // namespace

void launch_metric_tables(Ctx &c) {
  const Dims &d = c.d;
  k_metric_tables<<<dim3((unsigned)((d.NZ + 3 + 63) / 64), (unsigned)(d.NY + 3)), 64, 0, c.stream>>>(d, c.m);
  after_launch(c);
  EK_CUDA(cudaStreamSynchronize(c.stream));
}

void launch_spectral_rhs(Ctx &c, int rk) {
  SpecArgs a;
  a.d = c.d;
  a.m = c.m;
  a.kx = c.kx;
  a.kx2 = c.kx2;
  a.CU1 = c.CU1; a.CU2 = c.CU2; a.CU3 = c.CU3; a.CP = c.CP; a.CTH = c.CTH;
  a.CF1 = c.CF1; a.CF2 = c.CF2; a.CF3 = c.CF3; a.CFTH = c.CFTH;
  a.CR1 = c.CR1; a.CR2 = c.CR2; a.CR3 = c.CR3; a.CRTH = c.CRTH;
  const ek_params &p = c.p;
  a.cr_inc = explicit_increment_form(c) ? 1 : 0;
  a.nu = p.nu;
  a.nupr = p.nu / p.pr;
  a.T3 = c.ZETA_BAR[rk] * c.H_BAR[rk];
  a.T4 = c.H_BAR[rk];
  a.forcing = (p.f_type == 1 || p.f_type == 2);
  a.px = (p.f_type == 1) ? p.px0 : (p.px0 + p.amp_omega0 * cos(p.omega0 * p.time));
  a.f0 = p.f0;
  a.ubc_top = p.u_bc_c1[EK_YMAX];
  a.wbulk0 = p.wbulk0;
  a.ri = p.ri_tau;
  a.rk = rk;
  a.th = p.n_th > 0;
  a.cont_strat = p.cont_strat;
  a.nut = p.les ? c.les.nut : nullptr;
  a.pr = p.pr;
  // sponge_th runs inside the scalar loop (duct.F90:635), so only with N_TH >= 1
  a.sponge = (p.sponge_type != 0 && p.n_th > 0) ? 1 : 0;
  a.sig = c.sponge_sig;
  a.sig_out = c.sponge_sig_out;
  a.sred = c.sponge_red;
  a.amp = 0.1 / p.delta_t;
  a.tgt1 = p.v_bc_c1[EK_YMAX];
  a.tgt2 = p.u_bc_c1[EK_YMAX];
  a.tgt3 = p.wbulk0;
  a.strat_per = (p.v_bc[EK_ZMAX] == 6 && p.u_bc[EK_ZMAX] == 6 && p.w_bc[EK_ZMAX] == 6 && p.ri_tau != 0.0) ? 1 : 0;
  a.reset = (a.strat_per && p.save_stats_int > 0 && (2 * p.time_step) % p.save_stats_int == 0) ? 1 : 0;
  a.d = spec_dims(c);
  dim3 grid((a.d.NX2P + 1 + 63) / 64, c.d.NZ2, c.d.NY2);
  KScope ks(c, KC_SPECTRAL, 16.0 * c.d.nspec() * (a.d.NX2P + 1.0) / c.d.LDC * (5 + (rk > 1 ? 4 : 0) + 8));
  if (a.sponge) {
    const int nys = (p.ny_s_t > p.ny) ? (2 * p.ny) / 3 : p.ny_s_t;
    k_sponge_mean<<<1, 256, 0, c.stream>>>(c.d, c.CU3, nys, p.wbulk0, c.sponge_red);
    after_launch(c);
  }
  k_spectral_rhs<<<grid, 64, 0, c.stream>>>(a);
  after_launch(c);
}

// COURANT_CURV_MPI (duct.F90:3605-3674): the minimum over I = 0..NXP,
// K = ZSTART..ZEND, J = JSTART..JEND of CFL*DX/|U1|, CFL*J/|U2b|, CFL*J/|U3b|
// (face velocities as duct.F90:3631-3636), starting from 999.  All terms
// are positive, so the minimum of their bit patterns is the minimum.
// a physical field value: FP64, or the sum of a float-float field's planes
__device__ __forceinline__ double fld(const double *U, const float *H, const float *L, size_t c) {
  return H ? f2d_bits(H[c]) + f2d_bits(L[c]) : U[c];
}

__global__ void k_courant(Dims d, Metrics m, const double *U1, const double *U2, const double *U3, const float *H1,
                          const float *L1, const float *H2, const float *L2, const float *H3, const float *L3,
                          double cfl, double dx, unsigned long long *out) {
  __shared__ unsigned long long s[256];
  unsigned long long best = (unsigned long long)__double_as_longlong(999.0);
  const int ni = d.NX + 2, nk = d.ZE - d.ZS + 1, nj = d.JE - d.JS + 1;
  const long n = (long)ni * nk * nj;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t % ni), k = d.ZS + (int)((t / ni) % nk), j = d.JS + (int)(t / ((long)ni * nk));
    // the padding points x = NX, NX+1 hold zero velocity (infinite steps,
    // no effect on the minimum); plane forms do not keep them
    if (H1 && i >= d.NX) continue;
    const size_t c = d.ip(i, k, j);
    const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
    const double u2 = fld(U2, H2, L2, c), u3 = fld(U3, H3, L3, c);
    const double u2b = 0.5 * m.c22[d.m3(k, j, 1)] * (u2 + fld(U2, H2, L2, c - sJ)) +
                       0.5 * m.c21[d.m3(k, j, 1)] * (u3 + fld(U3, H3, L3, c - sJ));
    const double u3b = 0.5 * m.c11[d.m3(k, j, 2)] * (u3 + fld(U3, H3, L3, c - sK)) +
                       0.5 * m.c12[d.m3(k, j, 2)] * (u2 + fld(U2, H2, L2, c - sK));
    const double jac = m.jac[d.m2(k, j)];
    const double dtx = cfl * dx / fabs(fld(U1, H1, L1, c));
    const double dty = cfl * jac / fabs(u2b);
    const double dtz = cfl * jac / fabs(u3b);
    for (double v : {dtx, dty, dtz}) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(v);
      if (v == v && b < best) best = b;
    }
  }
  s[threadIdx.x] = best;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w && s[threadIdx.x + w] < s[threadIdx.x]) s[threadIdx.x] = s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMin(out, s[0]);
}

__global__ void k_set_double(double *a, double v) { *a = v; }

void launch_courant(Ctx &c) {
  const Dims &d = c.d;
  KScope ks(c, KC_FACE, 8.0 * 5 * (double)(d.NX + 2) * (d.ZE - d.ZS + 1) * (d.JE - d.JS + 1));
  k_set_double<<<1, 1, 0, c.stream>>>(c.cfl_dt, 999.0);
  after_launch(c);
  // float-float fields: the two planes; increment form: phi_old's FP32 copy
  // plus the ADI's total increment
  const bool ffp = ff_fields(c), inc = inc_fields(c);
  const bool pl = ffp || inc;
  float *l1 = inc ? inc_plane(c, c.R1) : ff_lo(c.U1), *l2 = inc ? inc_plane(c, c.R2) : ff_lo(c.U2);
  float *l3 = inc ? inc_plane(c, c.R3) : ff_lo(c.U3);
  k_courant<<<2 * 152, 256, 0, c.stream>>>(d, c.m, c.U1, c.U2, c.U3, pl ? c.U1f : nullptr, l1, pl ? c.U2f : nullptr,
                                          l2, pl ? c.U3f : nullptr, l3, c.p.cfl, c.p.lx / c.p.nx,
                                          reinterpret_cast<unsigned long long *>(c.cfl_dt));
  after_launch(c);
}

void launch_face_velocity(Ctx &c) {
  const Dims &d = c.d;
  dim3 grid((d.NX + 127) / 128, d.ZE - d.ZS + 2, d.JE - d.JS + 2);
  // read U2, U3 and write U2b, U3b: FP64, or FP32 copies on the mixed path
  KScope ks(c, KC_FACE, (c.p.fft_fp32 ? 16.0 : 32.0) * d.NX * (d.ZE - d.ZS + 2) * (d.JE - d.JS + 2));
  k_face_velocity<<<grid, 128, 0, c.stream>>>(d, c.m, c.U2, c.U3, c.U2b, c.U2f, c.U3f, c.p.fft_fp32 ? c.U2bf : nullptr);
  after_launch(c);
}

void launch_adi(Ctx &c, int field, int rk) {
  const Dims &d = c.d;
  double *phi = (field == 0) ? c.TH : (field == 1) ? c.U1 : (field == 2) ? c.U2 : c.U3;
  const double *R = (field == 0) ? c.RTH : (field == 1) ? c.R1 : (field == 2) ? c.R2 : c.R3;
  double coef = c.p.nu * c.H_BAR[rk] / 2.0;
  if (field == 0) coef = coef / c.p.pr;
  AdiArgs a;
  a.d = d;
  a.m = c.m;
  a.R = R;
  const int sform = explicit_increment_form(c) ? 1 : 0;
  a.Sf = sform ? reinterpret_cast<const float *>(R) : nullptr;
  a.phi_old = phi;
  a.phs = c.PHS;
  a.bcw = c.bc_weights;
  a.coef = coef;
  a.js = (field == 0) ? d.JST : d.JS;
  a.je = (field == 0) ? d.JET : d.JE;
  a.zs = (field == 0) ? d.ZST : d.ZS;
  a.ze = (field == 0) ? d.ZET : d.ZE;
  const size_t n2 = (size_t)d.LDM * (d.NY + 3);
  if (!c.adi_tab) {
    EK_CUDA(cudaMalloc(&c.adi_tab, sizeof(double) * 8 * n2));
    c.allocs.push_back(c.adi_tab);
  }
  const bool ffp = ff_fields(c), inc = inc_fields(c);
  if ((ffp || inc) && !c.adi_tab2) {
    EK_CUDA(cudaMalloc(&c.adi_tab2, sizeof(float2) * 8 * n2));
    c.allocs.push_back(c.adi_tab2);
  }
  // the increment form keeps each field's weights and scratch apart, so the
  // four fields' sweeps may run concurrently
  if (inc && !c.adi_tab_f[field]) {
    EK_CUDA(cudaMalloc(&c.adi_tab_f[field], sizeof(double) * 8 * n2));
    c.allocs.push_back(c.adi_tab_f[field]);
    EK_CUDA(cudaMalloc(&c.adi_tab2_f[field], sizeof(float2) * 8 * n2));
    c.allocs.push_back(c.adi_tab2_f[field]);
    if (field == 0) {
      c.inc_scr[0] = ff_lo(c.PHS);
    } else {
      EK_CUDA(cudaMalloc(&c.inc_scr[field], sizeof(float) * 2 * d.nphys()));
      c.allocs.push_back(c.inc_scr[field]);
    }
  }
  double *tab = inc ? c.adi_tab_f[field] : c.adi_tab;
  float2 *tab2 = inc ? c.adi_tab2_f[field] : c.adi_tab2;
  a.tab = tab;
  {
    const dim3 tg((unsigned)((d.NZ + 2 + 63) / 64), (unsigned)(d.NY + 2));
    k_adi_tab<false><<<tg, 64, 0, c.stream>>>(d, c.m, coef, sform, tab, (ffp || inc) ? tab2 : nullptr);
    after_launch(c);
    k_adi_tab<true><<<tg, 64, 0, c.stream>>>(d, c.m, coef, sform, tab + 4 * n2, (ffp || inc) ? tab2 + 4 * n2 : nullptr);
    after_launch(c);
  }
  if (les_active(c)) {
    // LES: x-dependent rows, one thread per system
    const size_t np = d.nphys();
    if (!c.adi_scr) {
      EK_CUDA(cudaMalloc(&c.adi_scr, sizeof(double) * 2 * np));
      c.allocs.push_back(c.adi_scr);
      EK_CUDA(cudaMalloc(&c.adi_les_tab, sizeof(double) * 14 * n2));
      c.allocs.push_back(c.adi_les_tab);
    }
    a.scr_b = c.adi_scr;
    a.scr_u = c.adi_scr + np;
    a.nut = c.les.nut;
    // KAPPA_T = NU_T/PR for TH: the 1/PR goes into the eddy-viscosity weights
    const double h = 0.5 * (c.H_BAR[rk] / 2.0) * ((field == 0) ? 1.0 / c.p.pr : 1.0);
    const double *l11 = (field == 2) ? c.m.g11y : (field == 3) ? c.m.g11z : c.m.g11;
    const double *l22 = (field == 2) ? c.m.g22y : (field == 3) ? c.m.g22z : c.m.g22;
    {
      const dim3 tg((unsigned)((d.NZ + 2 + 63) / 64), (unsigned)(d.NY + 2));
      k_adi_les_tab<false><<<tg, 64, 0, c.stream>>>(d, c.m, c.m.g22, l22, l11, coef, h, c.adi_les_tab);
      after_launch(c);
      k_adi_les_tab<true><<<tg, 64, 0, c.stream>>>(d, c.m, c.m.g11, l11, l22, coef, h, c.adi_les_tab + 7 * n2);
      after_launch(c);
    }
    // the mixed-precision method (FP32 LES kernels) eliminates in float-float
    const bool ff = c.les.lowp;
    if (ff) {
      if (!c.adi_ff_tab) {
        EK_CUDA(cudaMalloc(&c.adi_ff_tab, sizeof(float2) * 22 * n2));
        c.allocs.push_back(c.adi_ff_tab);
      }
      const unsigned nb = (unsigned)((n2 + 127) / 128);
      k_adi_ff_tab<<<nb, 128, 0, c.stream>>>((int)n2, c.adi_tab, c.adi_les_tab, c.adi_ff_tab);
      after_launch(c);
      k_adi_ff_tab<<<nb, 128, 0, c.stream>>>((int)n2, c.adi_tab + 4 * n2, c.adi_les_tab + 7 * n2, c.adi_ff_tab + 11 * n2);
      after_launch(c);
      a.nutf = c.les.nutf;
    }
    a.out = c.PHS;
    a.bc = c.bc[field][0];
    a.ltab = c.adi_les_tab;
    a.ftab = c.adi_ff_tab;
    {
      dim3 grid((d.NX + 127) / 128, a.ze - a.zs + 1);
      // algorithmic: read R, the field and NU_T, write the result
      KScope ks(c, KC_ADI_Y, 32.0 * d.NX * d.NY2 * (a.ze - a.zs + 1));
      if (ff && a.Sf) k_adi_les_ff<false, true><<<grid, 128, 0, c.stream>>>(a);
      else if (ff) k_adi_les_ff<false, false><<<grid, 128, 0, c.stream>>>(a);
      else if (a.Sf) k_adi_les<false, true><<<grid, 128, 0, c.stream>>>(a);
      else k_adi_les<false, false><<<grid, 128, 0, c.stream>>>(a);
      after_launch(c);
    }
    a.tab = c.adi_tab + 4 * n2;
    a.out = phi;
    a.bc = c.bc[field][1];
    a.ltab = c.adi_les_tab + 7 * n2;
    a.ftab = c.adi_ff_tab ? c.adi_ff_tab + 11 * n2 : nullptr;
    {
      dim3 grid((d.NX + 127) / 128, d.NY2);
      // read R, the old field, the y-sweep result and NU_T, write the result
      KScope ks(c, KC_ADI_Z, 40.0 * d.NX * d.NZ2 * (a.je - a.js + 1));
      if (ff && a.Sf) k_adi_les_ff<true, true><<<grid, 128, 0, c.stream>>>(a);
      else if (ff) k_adi_les_ff<true, false><<<grid, 128, 0, c.stream>>>(a);
      else if (a.Sf) k_adi_les<true, true><<<grid, 128, 0, c.stream>>>(a);
      else k_adi_les<true, false><<<grid, 128, 0, c.stream>>>(a);
      after_launch(c);
    }
    return;
  }
  if (inc) {
    float *phf = (field == 0) ? c.THf : (field == 1) ? c.U1f : (field == 2) ? c.U2f : c.U3f;
    const cplx_t *cu = (field == 0) ? c.CTH : (field == 1) ? c.CU1 : (field == 2) ? c.CU2 : c.CU3;
    float *dstar = c.inc_scr[field];
    float *brk = c.inc_scr[field] + d.nphys();
    // copy rows: the FP32 transform of CU(src) - CU(row) on their lines
    auto brackets = [&](const BcSet &bs, int dir) {
      for (int b = 0; b < bs.n; ++b) {
        const BcRow &br = bs.r[b];
        if (br.kind != 1) continue;
        C2rArgs t{};
        const long shift = (dir == 0) ? (long)d.ic(0, 0, br.src) - (long)d.ic(0, 0, br.row)
                                      : (long)d.ic(0, br.src, 0) - (long)d.ic(0, br.row, 0);
        t.src = cu + shift;
        t.src2 = cu;
        t.scale2 = -1.0;
        t.dstf = brk;
        t.lowp = 1;
        if (dir == 0) {
          t.j0 = t.j1 = br.row;
          t.k0 = 0;
          t.k1 = d.NZ + 1;
        } else {
          t.k0 = t.k1 = br.row;
          t.j0 = 0;
          t.j1 = d.NY + 1;
        }
        launch_c2r(c, t);
      }
    };
    brackets(c.bc[field][0], 0);
    a.phf = phf;
    a.dsf = dstar;
    a.brk = brk;
    a.incf = dstar;
    a.tab2 = tab2;
    a.fa2 = c.adi[field][rk][0].a2;
    a.fib2 = c.adi[field][rk][0].ib2;
    a.fu2 = c.adi[field][rk][0].u2;
    a.bc = c.bc[field][0];
    {
      // read S and the FP32 field (8 bytes), write the increment (4)
      KScope ks(c, KC_ADI_Y, 12.0 * d.NX * d.NY2 * (a.ze - a.zs + 1));
      const dim3 grid((d.NX + 127) / 128, a.ze - a.zs + 1);
      k_adi_inc<false><<<grid, 128, 0, c.stream>>>(a);
      after_launch(c);
    }
    brackets(c.bc[field][1], 1);
    a.incf = inc_plane(c, const_cast<double *>(R));
    a.fa2 = c.adi[field][rk][1].a2;
    a.fib2 = c.adi[field][rk][1].ib2;
    a.fu2 = c.adi[field][rk][1].u2;
    a.bc = c.bc[field][1];
    {
      // read S, the FP32 field and the y increment, write the total increment
      KScope ks(c, KC_ADI_Z, 16.0 * d.NX * d.NZ2 * d.NY2);
      const dim3 grid((d.NX + 127) / 128, d.NY2);
      k_adi_inc<true><<<grid, 128, 0, c.stream>>>(a);
      after_launch(c);
    }
    return;
  }
  if (ffp) {
    // float-float fields: the high planes are the FP32 copies, the low ones
    // the first half of the FP64 buffers; PHS holds the y sweep's planes
    float *hi = (field == 0) ? c.THf : (field == 1) ? c.U1f : (field == 2) ? c.U2f : c.U3f;
    float *lo = ff_lo(phi);
    float *ph = ff_lo(c.PHS), *pl = ff_lo(c.PHS) + d.nphys();
    a.po_h = hi;
    a.po_l = lo;
    a.ps_h = ph;
    a.ps_l = pl;
    a.out_h = ph;
    a.out_l = pl;
    a.tab2 = c.adi_tab2;
    a.fa2 = c.adi[field][rk][0].a2;
    a.fib2 = c.adi[field][rk][0].ib2;
    a.fu2 = c.adi[field][rk][0].u2;
    a.bc = c.bc[field][0];
    {
      // read S (4 bytes) and the old field (8), write the planes (8)
      KScope ks(c, KC_ADI_Y, 20.0 * d.NX * d.NY2 * (a.ze - a.zs + 1));
      const dim3 grid((d.NX + 127) / 128, a.ze - a.zs + 1);
      k_adi_ffs<false><<<grid, 128, 0, c.stream>>>(a);
      after_launch(c);
    }
    a.out_h = hi;
    a.out_l = lo;
    a.tab2 = c.adi_tab2 + 4 * n2;
    a.fa2 = c.adi[field][rk][1].a2;
    a.fib2 = c.adi[field][rk][1].ib2;
    a.fu2 = c.adi[field][rk][1].u2;
    a.bc = c.bc[field][1];
    {
      // read S and the y-sweep planes, write the field's planes
      KScope ks(c, KC_ADI_Z, 20.0 * d.NX * d.NZ2 * (a.je - a.js + 1));
      const dim3 grid((d.NX + 127) / 128, d.NY2);
      k_adi_ffs<true><<<grid, 128, 0, c.stream>>>(a);
      after_launch(c);
    }
    return;
  }
  // y sweep
  a.out = c.PHS;
  a.fa = c.adi[field][rk][0].a;
  a.fib = c.adi[field][rk][0].ib;
  a.fu = c.adi[field][rk][0].u;
  a.bc = c.bc[field][0];
  {
    KScope ks(c, KC_ADI_Y, 24.0 * d.NX * d.NY2 * (a.ze - a.zs + 1));
    const dim3 grid((d.NX + 127) / 128, a.ze - a.zs + 1);
    if (a.Sf) k_adi_seq<false, true><<<grid, 128, 0, c.stream>>>(a);
    else k_adi_seq<false, false><<<grid, 128, 0, c.stream>>>(a);
    after_launch(c);
  }
  // z sweep
  a.tab = c.adi_tab + 4 * n2;
  a.out = phi;
  a.fa = c.adi[field][rk][1].a;
  a.fib = c.adi[field][rk][1].ib;
  a.fu = c.adi[field][rk][1].u;
  a.bc = c.bc[field][1];
  {
    KScope ks(c, KC_ADI_Z, 32.0 * d.NX * d.NZ2 * (a.je - a.js + 1));
    const dim3 grid((d.NX + 127) / 128, d.NY2);
    if (a.Sf) k_adi_seq<true, true><<<grid, 128, 0, c.stream>>>(a);
    else k_adi_seq<true, false><<<grid, 128, 0, c.stream>>>(a);
    after_launch(c);
  }
}

void launch_th_corners(Ctx &c) {
  const int zmax1 = c.p.th_bc[EK_ZMAX] == 1, zmin6 = c.p.th_bc[EK_ZMIN] == 6;
  if (!zmax1 && !zmin6) return;
  KScope ks(c, KC_ADI_Z, 64.0 * c.d.NX);
  if (inc_fields(c)) {
    k_th_corners_inc<<<(c.d.NX + 127) / 128, 128, 0, c.stream>>>(c.d, c.THf, inc_plane(c, c.RTH), zmax1, zmin6);
  } else if (ff_fields(c)) {
    k_th_corners<float><<<(c.d.NX + 127) / 128, 128, 0, c.stream>>>(c.d, c.THf, zmax1, zmin6);
    after_launch(c);
    k_th_corners<float><<<(c.d.NX + 127) / 128, 128, 0, c.stream>>>(c.d, ff_lo(c.TH), zmax1, zmin6);
  } else {
    k_th_corners<double><<<(c.d.NX + 127) / 128, 128, 0, c.stream>>>(c.d, c.TH, zmax1, zmin6);
  }
  after_launch(c);
}

void launch_divergence_rhs(Ctx &c, double *rhs, int P) {
  const Dims &d = c.d;
  const Dims ds = spec_dims(c);
  const double fm = (ds.NX2P + 1.0) / d.LDC;  // share of the modes processed
  KScope ks(c, KC_DIVERGENCE, 16.0 * d.nspec() * fm * 4 + (16.0 * d.nspec() * 3 + 8.0 * P * d.NZ2 * d.NY2));
  dim3 g1((ds.NX2P + 1 + 63) / 64, d.NZ2, d.NY2);
  k_rem_faces<<<g1, 64, 0, c.stream>>>(ds, c.m, c.CU2, c.CU3, c.CU2b);
  after_launch(c);
  dim3 g2((P + 63) / 64, d.NZ2, d.NY2);
  k_div_rhs<<<g2, 64, 0, c.stream>>>(d, c.kx, c.CU1, c.CU2b, c.m.jac, rhs, P);
  after_launch(c);
}

void launch_projection(Ctx &c, const double *phif, int P, double temp4, bool update_p) {
  const Dims &d = c.d;
  const bool side = c.graph_slot >= 0 && !c.timing;
  const Dims ds = spec_dims(c);
  const double fm = (ds.NX2P + 1.0) / d.LDC;
  dim3 g0((ds.NX2P + 1 + 63) / 64, d.NZ2, d.NY2);
  {
  KScope ks(c, KC_PROJECTION, (16.0 * d.nspec() * (1 + 1 + (update_p ? 2 : 0)) + 16.0 * d.nspec() * (5 + 7 + 4)) * fm);
  k_phi_to_cr1<<<g0, 64, 0, c.stream>>>(ds, phif, P, c.CR1, c.CP, temp4, 1.0 / temp4, update_p ? 1 : 0,
                                       c.p.quirk_phi_fp32);
  after_launch(c);
  dim3 g1((ds.NX2P + 1 + 63) / 64, d.ZE - d.ZS + 1, d.JE - d.JS + 1);
  k_correct_faces<<<g1, 64, 0, c.stream>>>(ds, c.m, c.CR1, c.CU2b);
  after_launch(c);
  k_correct_cells<<<g1, 64, 0, c.stream>>>(ds, c.m, c.kx, c.CR1, c.CU1, c.CU2, c.CU3);
  after_launch(c);
  if (!side) {
    k_div_check<<<g0, 64, 0, c.stream>>>(ds, c.kx, c.m.jac, c.CU1, c.CU2b, c.CS);
    after_launch(c);
  }
  }
  const cudaStream_t main = c.stream;
  if (side) {
    // a captured step checks the divergence on the side stream, alongside
    // the next substep's right-hand side and transforms; the work that next
    // writes CU1 or the face velocities waits for it (div_join)
    EK_CUDA(cudaEventRecord(c.div_ev[0], main));
    EK_CUDA(cudaStreamWaitEvent(c.div_stream, c.div_ev[0], 0));
    c.stream = c.div_stream;
    k_div_check<<<g0, 64, 0, c.stream>>>(ds, c.kx, c.m.jac, c.CU1, c.CU2b, c.CS);
    after_launch(c);
  }
  C2rArgs ca{};
  ca.src = c.CS;
  ca.dst = c.SPH;
  ca.j0 = 2;
  ca.j1 = d.NY - 1;
  ca.k0 = 2;
  ca.k1 = d.NZ - 1;
  // the check's transform is linear in the (small) divergence itself: on the
  // mixed path FP32 arithmetic keeps it to ~1e-7 relative, into an FP32 plane
  const bool lp = explicit_increment_form(c);
  ca.lowp = lp ? 1 : 0;
  if (lp) {
    ca.dst = nullptr;
    ca.dstf = reinterpret_cast<float *>(c.SPH);
  }
  launch_c2r(c, ca);
  KScope ks(c, KC_DIVERGENCE, (lp ? 4.0 : 8.0) * (d.NX + 2) * (d.NZ - 2) * (d.NY - 2));
  if (lp) k_div_sum_f<<<d.NY - 2, 256, 0, c.stream>>>(d, reinterpret_cast<const float *>(c.SPH), c.div_part);
  else k_div_sum<<<d.NY - 2, 256, 0, c.stream>>>(d, c.SPH, c.div_part);
  after_launch(c);
  if (side) {
    div_final(c);
    EK_CUDA(cudaEventRecord(c.div_ev[1], c.stream));
    c.stream = main;
    c.div_pending = true;
  }
}

// Mean |div| from the per-line partial sums, in J order (duct.F90:2800).
namespace {
// The mean |div| from the per-line sums, in the order and arithmetic of the
// host reduction below, written to a step graph's statistics slot.
__global__ void k_div_final(const double *part, int n, double scale_den, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int t = 0; t < n; ++t) s += part[t];
  *out = s / scale_den;
}
}  // namespace

// a captured step's mean |div| into its statistics slot
void div_final(Ctx &c) {
  const Dims &d = c.d;
  k_div_final<<<1, 32, 0, c.stream>>>(c.div_part, d.NY - 2, (double)(d.NX + 1) * (double)d.NY * (double)d.NZ,
                                       &c.step_stats_dev[c.graph_slot].div);
  after_launch(c);
}

void div_join(Ctx &c) {
  if (!c.div_pending) return;
  EK_CUDA(cudaStreamWaitEvent(c.stream, c.div_ev[1], 0));
  c.div_pending = false;
}

int finish_divergence(Ctx &c, double *div_out) {
  const Dims &d = c.d;
  if (c.graph_slot >= 0) {
    // a captured step reads the value after the step (the side stream's
    // check has written it already)
    if (!c.div_pending) div_final(c);
    return EK_OK;
  }
  std::vector<double> part(d.NY - 2);
  EK_CUDA(cudaMemcpyAsync(part.data(), c.div_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, c.stream));
  EK_CUDA(cudaStreamSynchronize(c.stream));
  double s = 0.0;
  for (double v : part) s += v;
  s = s / ((double)(d.NX + 1) * (double)d.NY * (double)d.NZ);
  c.last_div = s;
  if (div_out) *div_out = s;
  return (s != s) ? EK_ERR_NAN : EK_OK;
}

}  // namespace ek

namespace ek {
// The RK kernels use the default shared-memory limit.
void rk_init_attributes() {}
}  // namespace ek

namespace ek {
bool ff_fields(const Ctx &c) { return c.p.ff_arith == 1 && c.p.fft_fp32 == 1 && !les_active(c); }
bool inc_fields(const Ctx &c) { return c.p.ff_arith == 2 && c.p.fft_fp32 == 1 && !les_active(c); }

void split_ff(Ctx &c, const double *in, float2 *out, size_t n) {
  if (n == 0) return;
  const unsigned nb = (unsigned)std::min<size_t>((n + 255) / 256, 4 * 152);
  k_split_ff<<<nb, 256, 0, c.stream>>>(n, in, out);
  after_launch(c);
}
}  // namespace ek

namespace ek {
// The modes the spectral kernels process: all NX/2+1 on the plain path, as
// the reference does; on the mixed path the ones up to NX/3 only.  The x
// transforms read and write no mode above NX/3, and no spectral operation
// couples modes, so those modes of CF and CR (which the reference's
// Coriolis term on every kx fills) never reach a field that is kept.
Dims spec_dims(const Ctx &c) {
  Dims d = c.d;
  if (explicit_increment_form(c)) d.NX2P = d.NKX;
  return d;
}
}  // namespace ek
