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
// With fft_fp32 >= 1 (the mixed-precision method, whose nonlinear-term
// transforms already run in FP32) the LES kernels compute in FP32 from the
// FP32 copies of the fields and per-cell FP32 weights, and hand the stresses
// to the FP32 transforms in FP32; NU_T is stored in FP64 for the ADI either
// way.  Conversions go through the integer-pipe helpers of ek_ffbits.h.
//
// The reference's stress arrays are kept between calls; on the planes next
// to the boundaries they hold the ghost copies J=0 <- 1, J=NY+1 <- NY, then
// K=0 <- 1, K=NZ+1 <- NZ (les_chan.F90:961-971), and on the other planes
// outside the solved range zero (C_DYN is zero there, and the off-diagonal
// stresses there keep the zero transforms they start from).  k_les_extra
// reads the stresses through that map.
#include <cmath>

#include "ek_ffbits.h"
#include "ek_internal.h"

namespace ek {

namespace {

// les_chan.F90:30,37 REAL*8 alpha; PARAMETER (alpha=2.44950): the test-filter
// width ratio.  The literal is default REAL, so the parameter holds 2.4495
// rounded to single precision (2.4495000839...), not the decimal value.
constexpr double kAlpha = static_cast<double>(2.44950f);
constexpr int kLineThreads = 256;
// planes of the FP32 weight table: pg[0..9] (eta and zeta differences),
// 1/J, then the GMAT_12, GMAT_12_y, GMAT_12_z faces (K+1,J,2), (K,J,2),
// (K,J+1,1), (K,J,1)
constexpr int kTabRJ = 10, kTabG12 = 11, kTabPlanes = 23;

template <typename T> __device__ __forceinline__ T cvt(double x);
template <> __device__ __forceinline__ double cvt<double>(double x) { return x; }
template <> __device__ __forceinline__ float cvt<float>(double x) { return d2f_bits(x); }
__device__ __forceinline__ double wide(double x) { return x; }
__device__ __forceinline__ double wide(float x) { return f2d_bits(x); }
__device__ __forceinline__ double ssqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float ssqrt(float x) { return sqrtf(x); }

// Per-cell FP32 weights of the FP32 LES kernels (K = 1..NZ, J = 1..NY).
__global__ void k_les_tab(Dims d, Metrics m, float *tab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (k < 1 || k > d.NZ || j < 1 || j > d.NY) return;
  const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
  for (int t = 0; t <= kTabRJ; ++t) tab[t * n2 + mm] = d2f_bits(m.pg[t * n2 + mm]);
  const double *g[3] = {m.g12, m.g12y, m.g12z};
  for (int v = 0; v < 3; ++v) {
    tab[(kTabG12 + 4 * v + 0) * n2 + mm] = d2f_bits(g[v][d.m3(k + 1, j, 2)]);
    tab[(kTabG12 + 4 * v + 1) * n2 + mm] = d2f_bits(g[v][d.m3(k, j, 2)]);
    tab[(kTabG12 + 4 * v + 2) * n2 + mm] = d2f_bits(g[v][d.m3(k, j + 1, 1)]);
    tab[(kTabG12 + 4 * v + 3) * n2 + mm] = d2f_bits(g[v][d.m3(k, j, 1)]);
  }
}

// DELTA_Y(K, J) = (beta DX(1) INT_JACOB(K, J))^(1/3), beta = 1
// (les_chan.F90:343-348), once per metric set.
__global__ void k_les_delta(Dims d, Metrics m, double dx1, double *delta) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (k > d.NZ + 1 || j > d.NY + 1) return;
  delta[d.m2(k, j)] = pow(dx1 * m.jac[d.m2(k, j)], 1.0 / 3.0);
}

struct LesLineArgs {
  Dims d;
  Metrics m;
  const float *tabf;
  const double *U1, *U2, *U3;     // FP64 kernels
  const float *U1f, *U2f, *U3f;   // FP32 kernels
  double *t0, *t1, *t2, *t23;     // FP64: in d(U1,U2,U3)/dx; out tau_11, tau_12, tau_13, tau_23
  float *f0, *f1, *f2, *f23;      // FP32: the same
  double *nut, *cdyn;
  float *nutf;
  const double *delta;  // DELTA(K, J)
};

template <typename T>
__device__ __forceinline__ const T *ufield(const LesLineArgs &a, int f) {
  if constexpr (sizeof(T) == 8) return f == 0 ? a.U1 : f == 1 ? a.U2 : a.U3;
  else return f == 0 ? a.U1f : f == 1 ? a.U2f : a.U3f;
}
template <typename T>
__device__ __forceinline__ T *tfield(const LesLineArgs &a, int f) {
  if constexpr (sizeof(T) == 8) return f == 0 ? a.t0 : f == 1 ? a.t1 : f == 2 ? a.t2 : a.t23;
  else return f == 0 ? a.f0 : f == 1 ? a.f1 : f == 2 ? a.f2 : a.f23;
}

// Strain rates of compute_strain_chan (les_chan.F90:1623-1718) at point c:
// S = (S11, S22, S33, S12, S13, S23), plus the implicit parts
// d(U1)/d(eta)/J, d(U1)/d(zeta)/J, d(U2)/d(zeta)/J that les_chan takes out
// of tau_12, tau_13, tau_23 (les_chan.F90:874-937).
template <typename T>
struct Strain {
  T S[6];
  T ay1, az1, az2;
};

template <typename T>
__device__ __forceinline__ Strain<T> strain_at(const LesLineArgs &a, size_t c, const T *wy, const T *wz, T rJ,
                                               size_t sK, size_t sJ) {
  const T *U1 = ufield<T>(a, 0), *U2 = ufield<T>(a, 1), *U3 = ufield<T>(a, 2);
  auto Dy = [&](const T *F) {
    return fma(wy[4], F[c - sJ], fma(wy[3], F[c + sJ], fma(wy[2], F[c - sK], fma(wy[1], F[c + sK], wy[0] * F[c]))));
  };
  auto Dz = [&](const T *F) {
    return fma(wz[4], F[c - sJ], fma(wz[3], F[c + sJ], fma(wz[2], F[c - sK], fma(wz[1], F[c + sK], wz[0] * F[c]))));
  };
  const T h = T(0.5);
  Strain<T> s;
  s.ay1 = Dy(U1) * rJ;
  s.az1 = Dz(U1) * rJ;
  const T dz2 = Dz(U2), dy3 = Dy(U3);
  s.az2 = dz2 * rJ;
  s.S[0] = tfield<T>(a, 0)[c];
  s.S[1] = Dy(U2) * rJ;
  s.S[2] = Dz(U3) * rJ;
  s.S[3] = h * (s.ay1 + tfield<T>(a, 1)[c]);
  s.S[4] = h * (s.az1 + tfield<T>(a, 2)[c]);
  s.S[5] = h * (dz2 + dy3) * rJ;
  return s;
}

// |S| = sqrt(2 S11^2 + 4 S12^2 + 4 S13^2 + 2 S22^2 + 4 S23^2 + 2 S33^2)
// in the order of les_chan.F90:360-367
template <typename T>
__device__ __forceinline__ T smag(const T *S) {
  const T two = T(2.0), four = T(4.0);
  return ssqrt(two * (S[0] * S[0]) + four * (S[3] * S[3]) + four * (S[4] * S[4]) + two * (S[1] * S[1]) +
               four * (S[5] * S[5]) + two * (S[2] * S[2]));
}

// One block per (K, J) line of the velocity range.  DYN: also recompute
// C_DYN(K, J) (les_chan.F90:475-821): test filter FILTER_VAR(2) (weights
// 1/4, 1/2, 1/4, periodic over I = 0..NX-1) of U, |S|, S_ij,
// DELTA^2 |S| S_ij and U_a U_b in shared memory; M_ij = (alpha DELTA)^2
// filt(|S|) filt(S_ij) - filt(DELTA^2 |S| S_ij), L_ij = filt(U_a U_b) -
// filt(U_a) filt(U_b); C = -0.5 sum(w M L) / sum(w M M) with w = 1 on the
// diagonal and 2 off it, zero when the denominator is zero, clipped at 0.
// Then NU_T = C DELTA^2 |S| (828-834) and the explicit stresses (839-937).
template <typename T, bool DYN>
__global__ void __launch_bounds__(kLineThreads) k_les_line(LesLineArgs a) {
  extern __shared__ __align__(16) unsigned char sh_raw[];  // DYN: U1 U2 U3 S11 S22 S33 S12 S13 S23 |S|
  __shared__ T red[2][kLineThreads / 32];
  __shared__ T cbc;
  T *sh = reinterpret_cast<T *>(sh_raw);
  const Dims &d = a.d;
  const int nk = d.ZE - d.ZS + 1;
  const int k = d.ZS + (int)(blockIdx.x % nk), j = d.JS + (int)(blockIdx.x / nk);
  const int NX = d.NX;
  const size_t n2 = (size_t)d.LDM * (d.NY + 3), mm = d.m2(k, j);
  T wy[5], wz[5], rJ;
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int t = 0; t < 5; ++t) {
      wy[t] = a.m.pg[t * n2 + mm];
      wz[t] = a.m.pg[(5 + t) * n2 + mm];
    }
    rJ = a.m.pg[kTabRJ * n2 + mm];
  } else {
#pragma unroll
    for (int t = 0; t < 5; ++t) {
      wy[t] = a.tabf[t * n2 + mm];
      wz[t] = a.tabf[(5 + t) * n2 + mm];
    }
    rJ = a.tabf[kTabRJ * n2 + mm];
  }
  const double delta64 = a.delta[mm];  // DELTA(K, J), k_les_delta
  const T delta = cvt<T>(delta64);
  const T d2 = delta * delta;
  const size_t base = d.ip(0, k, j), sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  T C;
  if (DYN) {
    T *sU = sh, *sS = sh + 3 * (size_t)NX, *sM = sh + 9 * (size_t)NX;
    for (int i = threadIdx.x; i < NX; i += blockDim.x) {
      const size_t c = base + i;
      const Strain<T> s = strain_at<T>(a, c, wy, wz, rJ, sK, sJ);
#pragma unroll
      for (int f = 0; f < 3; ++f) sU[f * NX + i] = ufield<T>(a, f)[c];
#pragma unroll
      for (int t = 0; t < 6; ++t) sS[t * NX + i] = s.S[t];
      sM[i] = smag(s.S);
    }
    __syncthreads();
    const T ad = cvt<T>(kAlpha * delta64), ad2 = ad * ad;
    const T q = T(0.25), hf = T(0.5);
    T num = T(0.0), den = T(0.0);
    for (int i = threadIdx.x; i < NX; i += blockDim.x) {
      const int im = (i == 0) ? NX - 1 : i - 1, ip = (i == NX - 1) ? 0 : i + 1;
      auto filt = [&](const T *v) { return q * v[im] + hf * v[i] + q * v[ip]; };
      T ub[3];
#pragma unroll
      for (int t = 0; t < 3; ++t) ub[t] = filt(sU + t * NX);
      const T sbar = filt(sM);
      constexpr int ua[6] = {0, 1, 2, 0, 0, 1}, ubi[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        const T *Sv = sS + t * NX;
        const T shat = filt(Sv);
        const T mf = q * ((d2 * sM[im]) * Sv[im]) + hf * ((d2 * sM[i]) * Sv[i]) + q * ((d2 * sM[ip]) * Sv[ip]);
        const T M = shat * ad2 * sbar - mf;
        const T *A = sU + ua[t] * NX, *B = sU + ubi[t] * NX;
        const T uu = q * (A[im] * B[im]) + hf * (A[i] * B[i]) + q * (A[ip] * B[ip]);
        const T L = uu - ub[ua[t]] * ub[ubi[t]];
        const T w = (t < 3) ? T(1.0) : T(2.0);
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
      T sn = T(0.0), sd = T(0.0);
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        sn += red[0][w];
        sd += red[1][w];
      }
      T cc = (sd != T(0.0)) ? T(-0.5) * sn / sd : T(0.0);
      if (cc < T(0.0)) cc = T(0.0);
      a.cdyn[(size_t)j * d.NZ2 + k] = wide(cc);
      cbc = cc;
    }
    __syncthreads();
    C = cbc;
  } else {
    C = cvt<T>(a.cdyn[(size_t)j * d.NZ2 + k]);
  }
  const T cd2 = C * d2;
  T *o0 = tfield<T>(a, 0), *o1 = tfield<T>(a, 1), *o2 = tfield<T>(a, 2), *o3 = tfield<T>(a, 3);
  for (int i = threadIdx.x; i < NX + 2; i += blockDim.x) {
    const size_t c = base + i;
    if (i >= NX) {
      a.nut[c] = 0.0;
      if constexpr (sizeof(T) == 4) a.nutf[c] = 0.0f;
      o0[c] = o1[c] = o2[c] = o3[c] = T(0.0);
      continue;
    }
    const Strain<T> s = strain_at<T>(a, c, wy, wz, rJ, sK, sJ);
    const T sm = smag(s.S);
    const T g = T(-2.0) * cd2 * sm;
    const T hf = T(0.5);
    const T nu = cd2 * sm;
    a.nut[c] = wide(nu);
    if constexpr (sizeof(T) == 4) a.nutf[c] = nu;
    o0[c] = g * s.S[0];
    o1[c] = g * (s.S[3] - hf * s.ay1);
    o2[c] = g * (s.S[4] - hf * s.az1);
    o3[c] = g * (s.S[5] - hf * s.az2);
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
__global__ void k_les_th_flux_f(Dims d, const float *nut, float *tth, float inv_pr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = d.ZST + (int)blockIdx.y, j = d.JST + (int)blockIdx.z;
  if (i >= d.LDX) return;
  const size_t c = d.ip(i, k, j);
  tth[c] = -(nut[c] * inv_pr * tth[c]);
}

struct LesExtraArgs {
  Dims d;
  Metrics m;
  const float *tabf;
  const double *U1, *U2, *U3, *TH, *nut, *t12, *t13, *t23;
  const float *U1f, *U2f, *U3f, *THf, *nutf, *f12, *f13, *f23;
  double *e1, *e2, *e3, *eth;
  float *g1, *g2, *g3, *gth;
  double inv_pr;
  int th;
};

// GMAT_12-form eddy-viscosity cross term of a field F with viscosity
// nu = scale * NU_T (duct.F90:990-1004 for U1, with GMAT_12_y for U2 and
// GMAT_12_z for U3; 1266-1283 for TH with KAPPA_T); G = the faces
// (K+1,J,2), (K,J,2), (K,J+1,1), (K,J,1)
template <typename T>
__device__ __forceinline__ T cross_term(const T *G, const T *F, const T *nut, T scale, size_t c, size_t sK,
                                        size_t sJ) {
  const T n0 = nut[c] * scale;
  const T nkp = nut[c + sK] * scale, nkm = nut[c - sK] * scale;
  const T njp = nut[c + sJ] * scale, njm = nut[c - sJ] * scale;
  const T fpp = F[c + sK + sJ], fpm = F[c + sK - sJ], fmp = F[c - sK + sJ], fmm = F[c - sK - sJ];
  const T fkp = F[c + sK], fkm = F[c - sK], fjp = F[c + sJ], fjm = F[c - sJ];
  const T h = T(0.5);
  const T t1 = G[0] * h * (nkp + n0) * (fpp + fjp - fjm - fpm);
  const T t2 = G[1] * h * (n0 + nkm) * (fmp + fjp - fjm - fmm);
  const T t3 = G[2] * h * (n0 + njp) * (fpp + fkp - fmp - fkm);
  const T t4 = G[3] * h * (n0 + njm) * (fkp + fpm - fkm - fmm);
  return T(0.25) * (t1 - t2 + t3 - t4);
}

// The flux-transform additions: for U1 the eddy-viscosity cross term minus
// the eta divergence of tau_12 and the zeta divergence of tau_13 (the CF1X
// lines of les_chan.F90:1310-1320); for U2 minus the zeta divergence of
// tau_23 (tau_22 = 0); for U3 minus the eta divergence of tau_23 (tau_33 =
// 0); for TH the KAPPA_T cross term.  The divergences use the
// pressure-gradient weight planes (the same CJOB combinations with their
// 0.5), and the stresses through the ghost map of the file comment.
template <typename T>
__global__ void k_les_extra(LesExtraArgs a) {
  const Dims &d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = (int)blockIdx.y, j = (int)blockIdx.z;
  if (i >= d.NX) return;
  const bool vel = (j >= d.JS && j <= d.JE && k >= d.ZS && k <= d.ZE);
  const bool sca = a.th && (j >= d.JST && j <= d.JET && k >= d.ZST && k <= d.ZET);
  if (!vel && !sca) return;
  constexpr bool kF = sizeof(T) == 4;
  const size_t c = d.ip(i, k, j), sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  const size_t mm = d.m2(k, j);
  const int n2 = d.LDM * (d.NY + 3);  // plane stride of the weight tables (32-bit products)
  const T *nut;
  if constexpr (kF) nut = a.nutf; else nut = a.nut;
  auto faces = [&](int v, T *G) {
    if constexpr (kF) {
      const float *tb = a.tabf + mm;
      for (int t = 0; t < 4; ++t) G[t] = tb[(kTabG12 + 4 * v + t) * n2];
    } else {
      const double *g = (v == 0) ? a.m.g12 : (v == 1) ? a.m.g12y : a.m.g12z;
      G[0] = g[d.m3(k + 1, j, 2)];
      G[1] = g[d.m3(k, j, 2)];
      G[2] = g[d.m3(k, j + 1, 1)];
      G[3] = g[d.m3(k, j, 1)];
    }
  };
  T G[4];
  if (vel) {
    // the stresses at (k, j) and its four neighbours through the ghost map:
    // an offset from c and a flag per point, the same for the whole block row
    long long off[5];
    bool in[5];
    {
      const int dk[5] = {0, 1, -1, 0, 0}, dj[5] = {0, 0, 0, 1, -1};
#pragma unroll
      for (int n = 0; n < 5; ++n) {
        int kk = k + dk[n], jj = j + dj[n];
        kk = (kk == 0) ? 1 : (kk == d.NZ + 1) ? d.NZ : kk;
        jj = (jj == 0) ? 1 : (jj == d.NY + 1) ? d.NY : jj;
        in[n] = (jj >= d.JS && jj <= d.JE && kk >= d.ZS && kk <= d.ZE);
        const long long ok = (kk == k) ? 0LL : (kk > k ? (long long)sK : -(long long)sK);
        const long long oj = (jj == j) ? 0LL : (jj > j ? (long long)sJ : -(long long)sJ);
        off[n] = ok + oj;
      }
    }
    auto tau = [&](const T *S, int n) { return in[n] ? S[(long long)c + off[n]] : T(0.0); };
    auto w = [&](int t) -> T {
      if constexpr (kF) return a.tabf[mm + t * n2];
      else return a.m.pg[mm + t * n2];
    };
    // w0 X + w1 X(k+1) + w2 X(k-1) + w3 X(j+1) + w4 X(j-1)
    auto div = [&](const T *S, int g0) {
      return fma(w(g0 + 4), tau(S, 4),
                 fma(w(g0 + 3), tau(S, 3), fma(w(g0 + 2), tau(S, 2), fma(w(g0 + 1), tau(S, 1), w(g0) * tau(S, 0)))));
    };
    const T *U1, *U2, *U3, *t12, *t13, *t23;
    T *e1, *e2, *e3;
    if constexpr (kF) {
      U1 = a.U1f; U2 = a.U2f; U3 = a.U3f; t12 = a.f12; t13 = a.f13; t23 = a.f23; e1 = a.g1; e2 = a.g2; e3 = a.g3;
    } else {
      U1 = a.U1; U2 = a.U2; U3 = a.U3; t12 = a.t12; t13 = a.t13; t23 = a.t23; e1 = a.e1; e2 = a.e2; e3 = a.e3;
    }
    faces(0, G);
    e1[c] = cross_term<T>(G, U1, nut, T(1.0), c, sK, sJ) - div(t12, 0) - div(t13, 5);
    faces(1, G);
    e2[c] = cross_term<T>(G, U2, nut, T(1.0), c, sK, sJ) - div(t23, 5);
    faces(2, G);
    e3[c] = cross_term<T>(G, U3, nut, T(1.0), c, sK, sJ) - div(t23, 0);
  }
  if (sca) {
    faces(0, G);
    if constexpr (kF) a.gth[c] = cross_term<T>(G, a.THf, nut, (T)d2f_bits(a.inv_pr), c, sK, sJ);
    else a.eth[c] = cross_term<T>(G, a.TH, nut, a.inv_pr, c, sK, sJ);
  }
}

size_t les_line_smem(const Dims &d, bool lowp) { return (lowp ? 4 : 8) * 10 * (size_t)d.NX; }

}  // namespace

bool les_active(const Ctx &c) { return c.p.les && (!c.p.create_new_flow || c.p.time_step > 1); }

// NU_T and C_DYN in FP64; the work fields in the precision the kernels use.
void les_alloc(Ctx &c) {
  const size_t np = c.d.nphys();
  LesState &L = c.les;
  L.lowp = c.p.fft_fp32 >= 1;
  auto field = [&](auto *&p, size_t n) {
    using E = std::remove_reference_t<decltype(*p)>;
    EK_CUDA(cudaMalloc(&p, sizeof(E) * n));
    c.allocs.push_back(p);
    EK_CUDA(cudaMemset(p, 0, sizeof(E) * n));
  };
  field(L.nut, np);
  field(L.cdyn, (size_t)c.d.NZ2 * c.d.NY2);
  field(L.delta, (size_t)c.d.LDM * (c.d.NY + 3));
  if (L.lowp) {
    for (float *&t : L.tf) field(t, np);
    field(L.t23f, np);
    field(L.tthf, np);
    for (float *&e : L.extf) field(e, np);
    field(L.nutf, np);
    field(L.tabf, (size_t)kTabPlanes * c.d.LDM * (c.d.NY + 3));
  } else {
    for (double *&t : L.t) field(t, np);
    field(L.t23, np);
    field(L.tth, np);
    for (double *&e : L.ext) field(e, np);
  }
}

// The LES part of a substep, after U1..U3 (and TH) are in physical space:
// the x derivatives, the line kernel (C_DYN recomputed at RK_STEP 1 of every
// fifth step and in every substep of the run's first step,
// les_chan.F90:475), the scalar flux and the flux-transform additions.
void launch_les(Ctx &c, int rk) {
  const Dims &d = c.d;
  const ek_params &p = c.p;
  LesState &L = c.les;
  const bool th = p.n_th > 0;
  const bool lowp = L.lowp;
  if (!L.tab_ok) {
    const dim3 tg((unsigned)((d.NZ + 2 + 63) / 64), (unsigned)(d.NY + 2));
    k_les_delta<<<tg, 64, 0, c.stream>>>(d, c.m, p.lx / p.nx, L.delta);
    after_launch(c);
    if (lowp) {
      k_les_tab<<<tg, 64, 0, c.stream>>>(d, c.m, L.tabf);
      after_launch(c);
    }
    L.tab_ok = true;
  }
  {
    C2rArgs a{};
    a.ik = 1;
    a.lowp = lowp ? 1 : 0;
    a.j0 = d.JS; a.j1 = d.JE; a.k0 = d.ZS; a.k1 = d.ZE;
    const cplx_t *src[3] = {c.CU1, c.CU2, c.CU3};
    for (int f = 0; f < 3; ++f) {
      a.src = src[f];
      a.dst = lowp ? nullptr : L.t[f];
      a.dstf = lowp ? L.tf[f] : nullptr;
      launch_c2r(c, a);
    }
    if (th) {
      a.j0 = d.JST; a.j1 = d.JET; a.k0 = d.ZST; a.k1 = d.ZET;
      a.src = c.CTH;
      a.dst = lowp ? nullptr : L.tth;
      a.dstf = lowp ? L.tthf : nullptr;
      launch_c2r(c, a);
    }
  }
  LesLineArgs la{};
  la.d = d;
  la.m = c.m;
  la.tabf = L.tabf;
  la.U1 = c.U1; la.U2 = c.U2; la.U3 = c.U3;
  la.U1f = c.U1f; la.U2f = c.U2f; la.U3f = c.U3f;
  la.t0 = L.t[0]; la.t1 = L.t[1]; la.t2 = L.t[2]; la.t23 = L.t23;
  la.f0 = L.tf[0]; la.f1 = L.tf[1]; la.f2 = L.tf[2]; la.f23 = L.t23f;
  la.nut = L.nut; la.nutf = L.nutf; la.cdyn = L.cdyn;
  la.delta = L.delta;
  const unsigned nlines = (unsigned)((d.ZE - d.ZS + 1) * (d.JE - d.JS + 1));
  const bool dyn = (p.time_step % 5 == 0 && rk == 1) || L.first_time;
  const double wb = lowp ? 4.0 : 8.0;  // bytes per value of the work fields
  {
    // algorithmic bytes: read d(U1,U2,U3)/dx and U1..U3, write NU_T (FP64) and four stresses
    KScope ks(c, KC_LES, (10.0 * wb + 8.0 + (lowp ? 4.0 : 0.0)) * (double)d.NX * nlines);
    const size_t sm = les_line_smem(d, lowp);
    if (lowp) {
      if (dyn) k_les_line<float, true><<<nlines, kLineThreads, sm, c.stream>>>(la);
      else k_les_line<float, false><<<nlines, kLineThreads, 0, c.stream>>>(la);
    } else {
      if (dyn) k_les_line<double, true><<<nlines, kLineThreads, sm, c.stream>>>(la);
      else k_les_line<double, false><<<nlines, kLineThreads, 0, c.stream>>>(la);
    }
    after_launch(c);
  }
  if (th) {
    KScope ks(c, KC_LES, 3.0 * wb * d.LDX * (d.ZET - d.ZST + 1) * (d.JET - d.JST + 1));
    dim3 grid((d.LDX + 127) / 128, d.ZET - d.ZST + 1, d.JET - d.JST + 1);
    if (lowp) k_les_th_flux_f<<<grid, 128, 0, c.stream>>>(d, L.nutf, L.tthf, (float)(1.0 / p.pr));
    else k_les_th_flux<<<grid, 128, 0, c.stream>>>(d, L.nut, L.tth, p.pr);
    after_launch(c);
  }
  {
    LesExtraArgs ea{};
    ea.d = d;
    ea.m = c.m;
    ea.tabf = L.tabf;
    ea.U1 = c.U1; ea.U2 = c.U2; ea.U3 = c.U3; ea.TH = c.TH; ea.nut = L.nut;
    ea.t12 = L.t[1]; ea.t13 = L.t[2]; ea.t23 = L.t23;
    ea.U1f = c.U1f; ea.U2f = c.U2f; ea.U3f = c.U3f; ea.THf = c.THf; ea.nutf = L.nutf;
    ea.f12 = L.tf[1]; ea.f13 = L.tf[2]; ea.f23 = L.t23f;
    ea.e1 = L.ext[0]; ea.e2 = L.ext[1]; ea.e3 = L.ext[2]; ea.eth = L.ext[3];
    ea.g1 = L.extf[0]; ea.g2 = L.extf[1]; ea.g3 = L.extf[2]; ea.gth = L.extf[3];
    ea.inv_pr = 1.0 / p.pr;
    ea.th = th ? 1 : 0;
    // read U1..U3, TH, NU_T and three stresses, write four additions (interior points)
    KScope ks(c, KC_LES, wb * 12.0 * (double)d.NX * nlines);
    dim3 grid((d.NX + 127) / 128, d.NZ2, d.NY2);
    if (lowp) k_les_extra<float><<<grid, 128, 0, c.stream>>>(ea);
    else k_les_extra<double><<<grid, 128, 0, c.stream>>>(ea);
    after_launch(c);
  }
}

void les_init_attributes() {
  EK_CUDA(cudaFuncSetAttribute(k_les_line<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  EK_CUDA(cudaFuncSetAttribute(k_les_line<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
}

}  // namespace ek
