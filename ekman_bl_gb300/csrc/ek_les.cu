// LES subgrid model of the duct substep on the GPU, FP64: the dynamic
// Smagorinsky model of les_chan (src/les_chan.F90, LES_MODEL_TYPE = 2,
// LES_IMPLICIT = .FALSE.), the eddy diffusivity of les_chan_th
// (src/les_chan_th.F90, LES_MODEL_TYPE_TH = 1) and the eddy-viscosity cross
// terms of RK_DUCT (src/duct.F90:990-1120, 1266-1311).  The implicit NU_T
// terms of the ADI are in k_adi_les (ek_rk.cu).
//
// The reference transforms every strain-rate and stress component on its own
// (six inverse and nine forward transforms per substep).  Here the
// x-transforms are linear and the eta/zeta differences act per (K, J), so:
//   * only the x derivatives d(U1,U2,U3)/dx (and d(TH)/dx) come from inverse
//     transforms of i kx CU; the eta/zeta derivatives of compute_strain_chan
//     are taken on the physical fields, which equal the inverse transforms of
//     the spectral differences;
//   * one block per (K, J) line forms the six strain rates and |S|, applies
//     the test filter in shared memory, reduces the Germano sums over x to
//     C_DYN(K, J) (no atomics: one block owns the line), and writes NU_T and
//     the explicit stresses tau_11, tau_12, tau_13, tau_23 (tau_22 = tau_33 =
//     0 in model 2);
//   * the stresses enter the nonlinear-term transforms that already exist:
//     J tau_1i joins the product J U1 Ui of CF_i (the -INT_JACOB CIKXP CSij
//     terms), and the eta/zeta divergence of the stresses joins the flux
//     transform of CF_i together with the GMAT_12 eddy-viscosity term, so
//     LES adds four inverse transforms and no forward one.
// The reference's stress arrays are kept between calls; on the planes next
// to the boundaries they hold the ghost copies J=0 <- 1, J=NY+1 <- NY, then
// K=0 <- 1, K=NZ+1 <- NZ (les_chan.F90:961-971), and on the other planes
// outside the solved range zero (C_DYN is zero there, and the off-diagonal
// stresses there keep the zero transforms they start from).  k_les_extra
// reads the stresses through that map.
#include <cmath>

#include "ek_internal.h"

namespace ek {

namespace {

constexpr double kAlpha = 2.44950;  // les_chan.F90 PARAMETER alpha (test-filter width ratio)
constexpr int kLineThreads = 256;

struct LesLineArgs {
  Dims d;
  Metrics m;
  const double *U1, *U2, *U3;
  double *t0, *t1, *t2;  // in: d(U1,U2,U3)/dx; out: tau_11, tau_12, tau_13
  double *t23, *nut, *cdyn;
  double dx1;  // DX(1) = LX/NX
};

// Strain rates of compute_strain_chan (les_chan.F90:1623-1718) at x point i
// of the line at base: S = (S11, S22, S33, S12, S13, S23), plus the implicit
// parts d(U1)/d(eta)/J, d(U1)/d(zeta)/J, d(U2)/d(zeta)/J that les_chan takes
// out of tau_12, tau_13, tau_23 (les_chan.F90:874-937).
struct Strain {
  double S[6];
  double ay1, az1, az2;
};

__device__ __forceinline__ Strain strain_at(const LesLineArgs &a, size_t c, const double *wy, const double *wz,
                                            double rJ, size_t sK, size_t sJ) {
  auto Dy = [&](const double *F) {
    return fma(wy[4], F[c - sJ], fma(wy[3], F[c + sJ], fma(wy[2], F[c - sK], fma(wy[1], F[c + sK], wy[0] * F[c]))));
  };
  auto Dz = [&](const double *F) {
    return fma(wz[4], F[c - sJ], fma(wz[3], F[c + sJ], fma(wz[2], F[c - sK], fma(wz[1], F[c + sK], wz[0] * F[c]))));
  };
  Strain s;
  s.ay1 = Dy(a.U1) * rJ;
  s.az1 = Dz(a.U1) * rJ;
  const double dz2 = Dz(a.U2), dy3 = Dy(a.U3);
  s.az2 = dz2 * rJ;
  s.S[0] = a.t0[c];
  s.S[1] = Dy(a.U2) * rJ;
  s.S[2] = Dz(a.U3) * rJ;
  s.S[3] = 0.5 * (s.ay1 + a.t1[c]);
  s.S[4] = 0.5 * (s.az1 + a.t2[c]);
  s.S[5] = 0.5 * (dz2 + dy3) * rJ;
  return s;
}

// |S| = sqrt(2 S11^2 + 4 S12^2 + 4 S13^2 + 2 S22^2 + 4 S23^2 + 2 S33^2)
// in the order of les_chan.F90:360-367
__device__ __forceinline__ double smag(const double *S) {
  return sqrt(2.0 * (S[0] * S[0]) + 4.0 * (S[3] * S[3]) + 4.0 * (S[4] * S[4]) + 2.0 * (S[1] * S[1]) +
              4.0 * (S[5] * S[5]) + 2.0 * (S[2] * S[2]));
}

// One block per (K, J) line of the velocity range.  DYN: also recompute
// C_DYN(K, J) (les_chan.F90:475-821): test filter FILTER_VAR(2) (weights
// 1/4, 1/2, 1/4, periodic over I = 0..NX-1) of U, |S|, S_ij,
// DELTA^2 |S| S_ij and U_a U_b in shared memory; M_ij = (alpha DELTA)^2
// filt(|S|) filt(S_ij) - filt(DELTA^2 |S| S_ij), L_ij = filt(U_a U_b) -
// filt(U_a) filt(U_b); C = -0.5 sum(w M L) / sum(w M M) with w = 1 on the
// diagonal and 2 off it, zero when the denominator is zero, clipped at 0.
// Then NU_T = C DELTA^2 |S| (828-834) and the explicit stresses (839-937).
template <bool DYN>
__global__ void __launch_bounds__(kLineThreads) k_les_line(LesLineArgs a) {
  extern __shared__ double sh[];  // DYN: U1 U2 U3 S11 S22 S33 S12 S13 S23 |S|, NX each
  __shared__ double red[2][kLineThreads / 32];
  __shared__ double cbc;
  const Dims &d = a.d;
  const int nk = d.ZE - d.ZS + 1;
  const int k = d.ZS + (int)(blockIdx.x % nk), j = d.JS + (int)(blockIdx.x / nk);
  const int NX = d.NX;
  const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
  double wy[5], wz[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    wy[t] = a.m.pg[t * n2 + mm];
    wz[t] = a.m.pg[(5 + t) * n2 + mm];
  }
  const double rJ = a.m.pg[10 * n2 + mm];
  const double delta = pow(a.dx1 * a.m.jac[mm], 1.0 / 3.0);  // (beta DX(1) INT_JACOB)^(1/3), beta = 1
  const double d2 = delta * delta;
  const size_t base = d.ip(0, k, j), sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  double C;
  if (DYN) {
    double *sU = sh, *sS = sh + 3 * (size_t)NX, *sM = sh + 9 * (size_t)NX;
    for (int i = threadIdx.x; i < NX; i += blockDim.x) {
      const size_t c = base + i;
      const Strain s = strain_at(a, c, wy, wz, rJ, sK, sJ);
      sU[i] = a.U1[c];
      sU[NX + i] = a.U2[c];
      sU[2 * NX + i] = a.U3[c];
#pragma unroll
      for (int t = 0; t < 6; ++t) sS[t * NX + i] = s.S[t];
      sM[i] = smag(s.S);
    }
    __syncthreads();
    const double ad = kAlpha * delta, ad2 = ad * ad;
    double num = 0.0, den = 0.0;
    for (int i = threadIdx.x; i < NX; i += blockDim.x) {
      const int im = (i == 0) ? NX - 1 : i - 1, ip = (i == NX - 1) ? 0 : i + 1;
      auto filt = [&](const double *v) { return 0.25 * v[im] + 0.5 * v[i] + 0.25 * v[ip]; };
      double ub[3];
#pragma unroll
      for (int t = 0; t < 3; ++t) ub[t] = filt(sU + t * NX);
      const double sbar = filt(sM);
      constexpr int ua[6] = {0, 1, 2, 0, 0, 1}, ubi[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        const double *Sv = sS + t * NX;
        const double shat = filt(Sv);
        const double mf = 0.25 * ((d2 * sM[im]) * Sv[im]) + 0.5 * ((d2 * sM[i]) * Sv[i]) + 0.25 * ((d2 * sM[ip]) * Sv[ip]);
        const double M = shat * ad2 * sbar - mf;
        const double *A = sU + ua[t] * NX, *B = sU + ubi[t] * NX;
        const double uu = 0.25 * (A[im] * B[im]) + 0.5 * (A[i] * B[i]) + 0.25 * (A[ip] * B[ip]);
        const double L = uu - ub[ua[t]] * ub[ubi[t]];
        const double w = (t < 3) ? 1.0 : 2.0;
        num = fma(w * M, L, num);
        den = fma(w * M, M, den);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      num += __shfl_xor_sync(0xffffffffu, num, o);
      den += __shfl_xor_sync(0xffffffffu, den, o);
    }
    const int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
      red[0][wid] = num;
      red[1][wid] = den;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double sn = 0.0, sd = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        sn += red[0][w];
        sd += red[1][w];
      }
      double cc = (sd != 0.0) ? -0.5 * sn / sd : 0.0;
      if (cc < 0.0) cc = 0.0;
      a.cdyn[(size_t)j * d.NZ2 + k] = cc;
      cbc = cc;
    }
    __syncthreads();
    C = cbc;
  } else {
    C = a.cdyn[(size_t)j * d.NZ2 + k];
  }
  const double cd2 = C * d2;
  for (int i = threadIdx.x; i < NX + 2; i += blockDim.x) {
    const size_t c = base + i;
    if (i >= NX) {
      a.nut[c] = 0.0;
      a.t0[c] = 0.0;
      a.t1[c] = 0.0;
      a.t2[c] = 0.0;
      a.t23[c] = 0.0;
      continue;
    }
    const Strain s = strain_at(a, c, wy, wz, rJ, sK, sJ);
    const double sm = smag(s.S);
    const double g = -2.0 * cd2 * sm;
    a.nut[c] = cd2 * sm;
    a.t0[c] = g * s.S[0];
    a.t1[c] = g * (s.S[3] - 0.5 * s.ay1);
    a.t2[c] = g * (s.S[4] - 0.5 * s.az1);
    a.t23[c] = g * (s.S[5] - 0.5 * s.az2);
  }
}

// les_chan_th, model 1 (les_chan_th.F90:50-105): the x flux of the scalar,
// -KAPPA_T d(TH)/dx with KAPPA_T = NU_T/PR, over the scalar range (NU_T is
// zero outside the velocity range).  In place on d(TH)/dx.
__global__ void k_les_th_flux(Dims d, const double *nut, double *tth, double pr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = d.ZST + (int)blockIdx.y, j = d.JST + (int)blockIdx.z;
  if (i >= d.LDX) return;
  const size_t c = d.ip(i, k, j);
  tth[c] = -(nut[c] / pr * tth[c]);
}

struct LesExtraArgs {
  Dims d;
  Metrics m;
  const double *U1, *U2, *U3, *TH, *nut;
  const double *t12, *t13, *t23;
  double *e1, *e2, *e3, *eth;
  double inv_pr;
  int th;
};

// GMAT_12-form eddy-viscosity cross term of a field F with viscosity
// nu = scale * NU_T (duct.F90:990-1004 for U1, with GMAT_12_y for U2 and
// GMAT_12_z for U3; 1266-1283 for TH with KAPPA_T)
__device__ __forceinline__ double cross_term(const Dims &d, const double *G, const double *F, const double *nut,
                                             double scale, int i, int k, int j) {
  const size_t c = d.ip(i, k, j), sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  const double n0 = nut[c] * scale;
  const double nkp = nut[c + sK] * scale, nkm = nut[c - sK] * scale;
  const double njp = nut[c + sJ] * scale, njm = nut[c - sJ] * scale;
  const double fpp = F[c + sK + sJ], fpm = F[c + sK - sJ], fmp = F[c - sK + sJ], fmm = F[c - sK - sJ];
  const double fkp = F[c + sK], fkm = F[c - sK], fjp = F[c + sJ], fjm = F[c - sJ];
  const double t1 = G[d.m3(k + 1, j, 2)] * 0.5 * (nkp + n0) * (fpp + fjp - fjm - fpm);
  const double t2 = G[d.m3(k, j, 2)] * 0.5 * (n0 + nkm) * (fmp + fjp - fjm - fmm);
  const double t3 = G[d.m3(k, j + 1, 1)] * 0.5 * (n0 + njp) * (fpp + fkp - fmp - fkm);
  const double t4 = G[d.m3(k, j, 1)] * 0.5 * (n0 + njm) * (fkp + fpm - fkm - fmm);
  return 0.25 * (t1 - t2 + t3 - t4);
}

// The flux-transform additions: for U1 the eddy-viscosity cross term minus
// the eta divergence of tau_12 and the zeta divergence of tau_13 (the CF1X
// lines of les_chan.F90:1310-1320); for U2 minus the zeta divergence of
// tau_23 (tau_22 = 0); for U3 minus the eta divergence of tau_23 (tau_33 =
// 0); for TH the KAPPA_T cross term.  The divergences use the
// pressure-gradient weight planes (the same CJOB combinations with their
// 0.5), and the stresses through the ghost map of the file comment.
__global__ void k_les_extra(LesExtraArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = (int)blockIdx.y, j = (int)blockIdx.z;
  if (i >= d.NX) return;
  const bool vel = (j >= d.JS && j <= d.JE && k >= d.ZS && k <= d.ZE);
  const bool sca = a.th && (j >= d.JST && j <= d.JET && k >= d.ZST && k <= d.ZET);
  if (!vel && !sca) return;
  const size_t c = d.ip(i, k, j);
  if (vel) {
    const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
    auto tau = [&](const double *T, int kk, int jj) {
      kk = (kk == 0) ? 1 : (kk == d.NZ + 1) ? d.NZ : kk;
      jj = (jj == 0) ? 1 : (jj == d.NY + 1) ? d.NY : jj;
      const bool in = (jj >= d.JS && jj <= d.JE && kk >= d.ZS && kk <= d.ZE);
      return in ? T[d.ip(i, kk, jj)] : 0.0;
    };
    auto div = [&](const double *T, int g0) {
      const double *pg = a.m.pg;
      return fma(pg[(g0 + 4) * n2 + mm], tau(T, k, j - 1),
                 fma(pg[(g0 + 3) * n2 + mm], tau(T, k, j + 1),
                     fma(pg[(g0 + 2) * n2 + mm], tau(T, k - 1, j),
                         fma(pg[(g0 + 1) * n2 + mm], tau(T, k + 1, j), pg[g0 * n2 + mm] * tau(T, k, j)))));
    };
    a.e1[c] = cross_term(d, a.m.g12, a.U1, a.nut, 1.0, i, k, j) - div(a.t12, 0) - div(a.t13, 5);
    a.e2[c] = cross_term(d, a.m.g12y, a.U2, a.nut, 1.0, i, k, j) - div(a.t23, 5);
    a.e3[c] = cross_term(d, a.m.g12z, a.U3, a.nut, 1.0, i, k, j) - div(a.t23, 0);
  }
  if (sca) a.eth[c] = cross_term(d, a.m.g12, a.TH, a.nut, a.inv_pr, i, k, j);
}

}  // namespace

bool les_active(const Ctx &c) { return c.p.les && (!c.p.create_new_flow || c.p.time_step > 1); }

void les_alloc(Ctx &c) {
  const size_t np = c.d.nphys();
  LesState &L = c.les;
  auto field = [&](double *&p, size_t n) {
    EK_CUDA(cudaMalloc(&p, sizeof(double) * n));
    c.allocs.push_back(p);
    EK_CUDA(cudaMemset(p, 0, sizeof(double) * n));
  };
  field(L.nut, np);
  field(L.cdyn, (size_t)c.d.NZ2 * c.d.NY2);
  for (double *&t : L.t) field(t, np);
  field(L.t23, np);
  field(L.tth, np);
  for (double *&e : L.ext) field(e, np);
}

size_t les_line_smem(const Dims &d) { return sizeof(double) * 10 * (size_t)d.NX; }

// The LES part of a substep, after U1..U3 (and TH) are in physical space:
// the x derivatives, the line kernel (C_DYN recomputed at RK_STEP 1 of every
// fifth step and in every substep of the run's first step,
// les_chan.F90:475), the scalar flux and the flux-transform additions.
void launch_les(Ctx &c, int rk) {
  const Dims &d = c.d;
  const ek_params &p = c.p;
  LesState &L = c.les;
  const bool th = p.n_th > 0;
  {
    C2rArgs a{};
    a.ik = 1;
    a.j0 = d.JS; a.j1 = d.JE; a.k0 = d.ZS; a.k1 = d.ZE;
    a.src = c.CU1; a.dst = L.t[0]; launch_c2r(c, a);
    a.src = c.CU2; a.dst = L.t[1]; launch_c2r(c, a);
    a.src = c.CU3; a.dst = L.t[2]; launch_c2r(c, a);
    if (th) {
      a.j0 = d.JST; a.j1 = d.JET; a.k0 = d.ZST; a.k1 = d.ZET;
      a.src = c.CTH; a.dst = L.tth; launch_c2r(c, a);
    }
  }
  LesLineArgs la;
  la.d = d;
  la.m = c.m;
  la.U1 = c.U1; la.U2 = c.U2; la.U3 = c.U3;
  la.t0 = L.t[0]; la.t1 = L.t[1]; la.t2 = L.t[2];
  la.t23 = L.t23; la.nut = L.nut; la.cdyn = L.cdyn;
  la.dx1 = p.lx / p.nx;
  const unsigned nlines = (unsigned)((d.ZE - d.ZS + 1) * (d.JE - d.JS + 1));
  const bool dyn = (p.time_step % 5 == 0 && rk == 1) || L.first_time;
  {
    // algorithmic bytes: read d(U1,U2,U3)/dx and U1..U3, write NU_T and four stresses
    KScope ks(c, KC_LES, 8.0 * 11.0 * (double)d.NX * nlines);
    if (dyn) k_les_line<true><<<nlines, kLineThreads, les_line_smem(d), c.stream>>>(la);
    else k_les_line<false><<<nlines, kLineThreads, 0, c.stream>>>(la);
    after_launch(c);
  }
  if (th) {
    KScope ks(c, KC_LES, 24.0 * d.LDX * (d.ZET - d.ZST + 1) * (d.JET - d.JST + 1));
    dim3 grid((d.LDX + 127) / 128, d.ZET - d.ZST + 1, d.JET - d.JST + 1);
    k_les_th_flux<<<grid, 128, 0, c.stream>>>(d, L.nut, L.tth, p.pr);
    after_launch(c);
  }
  {
    LesExtraArgs ea;
    ea.d = d;
    ea.m = c.m;
    ea.U1 = c.U1; ea.U2 = c.U2; ea.U3 = c.U3; ea.TH = c.TH; ea.nut = L.nut;
    ea.t12 = L.t[1]; ea.t13 = L.t[2]; ea.t23 = L.t23;
    ea.e1 = L.ext[0]; ea.e2 = L.ext[1]; ea.e3 = L.ext[2]; ea.eth = L.ext[3];
    ea.inv_pr = 1.0 / p.pr;
    ea.th = th ? 1 : 0;
    // read U1..U3, TH, NU_T and three stresses, write four additions (interior points)
    KScope ks(c, KC_LES, 8.0 * 12.0 * (double)d.NX * nlines);
    dim3 grid((d.NX + 127) / 128, d.NZ2, d.NY2);
    k_les_extra<<<grid, 128, 0, c.stream>>>(ea);
    after_launch(c);
  }
}

void les_init_attributes() {
  EK_CUDA(cudaFuncSetAttribute(k_les_line<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
}

}  // namespace ek
