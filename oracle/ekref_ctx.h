// Oracle (test infrastructure): the context and FFT helpers shared by the
// oracle's translation units.  Not part of the product.
#ifndef EKREF_CTX_H
#define EKREF_CTX_H

#include <cmath>
#include <complex>
#include <memory>
#include <string>
#include <vector>

#include "ekref.h"
#include "ekref_mud.h"

namespace ekref_detail {

struct cplx {
  double re, im;
};
inline cplx cadd(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
inline cplx csub(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
inline cplx cscale(double s, cplx a) { return {s * a.re, s * a.im}; }
inline cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// Radix-2 complex FFT, sign = -1 forward, +1 inverse (unnormalised).
struct FFT {
  int n = 0;
  std::vector<std::complex<double>> tw;
  std::vector<int> rev;
  explicit FFT(int n_) : n(n_), tw(n_ / 2), rev(n_) {
    for (int k = 0; k < n / 2; ++k) tw[k] = std::polar(1.0, -2.0 * M_PI * k / n);
    int lg = 0;
    while ((1 << lg) < n) ++lg;
    for (int i = 0; i < n; ++i) {
      int r = 0;
      for (int b = 0; b < lg; ++b) r |= ((i >> b) & 1) << (lg - 1 - b);
      rev[i] = r;
    }
  }
  void run(std::complex<double> *a, int sign) const {
    for (int i = 0; i < n; ++i)
      if (i < rev[i]) std::swap(a[i], a[rev[i]]);
    for (int len = 2; len <= n; len <<= 1) {
      const int step = n / len;
      for (int s = 0; s < n; s += len)
        for (int k = 0; k < len / 2; ++k) {
          std::complex<double> w = tw[k * step];
          if (sign > 0) w = std::conj(w);
          const std::complex<double> u = a[s + k], v = a[s + k + len / 2] * w;
          a[s + k] = u + v;
          a[s + k + len / 2] = u - v;
        }
    }
  }
};

inline void r2c_line(const FFT &f, int nkx, const double *in, cplx *out, std::complex<double> *buf) {
  const int n = f.n;
  for (int i = 0; i < n; ++i) buf[i] = std::complex<double>(in[i], 0.0);
  f.run(buf, -1);
  const double s = 1.0 / n;
  for (int k = 0; k <= n / 2; ++k)
    out[k] = (k <= nkx) ? cplx{buf[k].real() * s, buf[k].imag() * s} : cplx{0.0, 0.0};
}

inline void c2r_line(const FFT &f, int nkx, const cplx *in, double *out, std::complex<double> *buf) {
  const int n = f.n;
  for (int i = 0; i < n; ++i) buf[i] = 0.0;
  buf[0] = std::complex<double>(in[0].re, 0.0);
  for (int k = 1; k <= nkx && k < n / 2; ++k) {
    buf[k] = std::complex<double>(in[k].re, in[k].im);
    buf[n - k] = std::complex<double>(in[k].re, -in[k].im);
  }
  f.run(buf, +1);
  for (int i = 0; i < n; ++i) out[i] = buf[i].real();
  out[n] = 0.0;
  out[n + 1] = 0.0;
}

}  // namespace ekref_detail

using ekref_detail::cplx;
using ekref_detail::FFT;

struct ekref_ctx {
  ek_params p{};
  std::string err;
  int NX, NY, NZ, NKX, NX2P, NXP;
  int LDX, LDC;      // physical and spectral line lengths (NX+2, NX/2+1)
  int NZ2, NY2;      // NZ+2, NY+2 lines
  int JSTART, JEND, ZSTART, ZEND, JSTART_TH, JEND_TH, ZSTART_TH, ZEND_TH;
  double H_BAR[4], BETA_BAR[4], ZETA_BAR[4];
  std::vector<double> KXP, KX2P;
  std::vector<double> int_jacob, gmat_11, gmat_12, gmat_22, cjob_11, cjob_12, cjob_21, cjob_22, th_bar;
  std::vector<double> sponge_sigma, sponge_sigma_out;  // (0:NY+1), (0:NZ+1); zero by default
  bool have_metrics = false;
  // spectral fields
  std::vector<cplx> CU1, CU2, CU3, CP, CTH, CF1, CF2, CF3, CFTH, CR1, CR2, CR3, CRTH, CS1, CS2, CU2b, CU3b;
  // physical fields
  std::vector<double> U1, U2, U3, TH, R1, R2, R3, RTH, S1, S2, U2b, U3b;
  std::unique_ptr<FFT> fft;
  ekref::MudOpts mud{};
  // left null vector of the finest kx = 0 operator (the residual rule's
  // well-posed kx = 0 solve); built on first use, cleared with the metrics
  std::vector<double> mg_z;
  double last_div = 0.0;
  ek_mg_stats last_stats{};
  // LES (les_chan / les_chan_th): the module arrays they keep between
  // calls.  Sij, CSij and S2X persist like the reference's static scratch
  // arrays (zero at program start), so values that the reference reads from
  // earlier calls are read here too.
  std::vector<double> g11y, g12y, g22y, g11z, g12z, g22z;  // GMAT_*_y, GMAT_*_z (M3 layout)
  bool have_les_metrics = false;
  bool first_time = true;                                   // FIRST_TIME (diablo.F90:88,157)
  std::vector<double> NU_T, KAPPA_T, S2X;                   // physical layout
  std::vector<double> C_DYN;                                // (0:NZ+1, 0:NY+1), K fastest
  std::vector<double> Sij[6];
  std::vector<cplx> CSij[6];
  bool les_active() const { return p.les && (!p.create_new_flow || p.time_step > 1); }

  size_t ip(int i, int k, int j) const { return ((size_t)j * NZ2 + k) * LDX + i; }
  size_t ic(int i, int k, int j) const { return ((size_t)j * NZ2 + k) * LDC + i; }
  double M2(const std::vector<double> &a, int k, int j) const { return a[(size_t)j * (NZ + 3) + k]; }
  double M3(const std::vector<double> &a, int k, int j, int f) const {
    return a[(size_t)(f - 1) * (NZ + 3) * (NY + 3) + (size_t)j * (NZ + 3) + k];
  }
  double JAC(int k, int j) const { return M2(int_jacob, k, j); }
};


// x-transforms over the (j, k) planes j0..j1, k0..k1 (ekref_step.cpp)
void to_fourier(ekref_ctx *c, const std::vector<double> &in, std::vector<cplx> &out, int j0, int j1, int k0, int k1);
void to_physical(ekref_ctx *c, const std::vector<cplx> &in, std::vector<double> &out, int j0, int j1, int k0, int k1);

// LES pieces (ekref_les.cpp)
void les_alloc(ekref_ctx *c);
void les_chan(ekref_ctx *c, int rk);
void les_chan_th(ekref_ctx *c);
void les_cross_terms(ekref_ctx *c);
void les_cross_terms_th(ekref_ctx *c);
// The LES terms of one field's ADI (duct.F90:1373-1386, 1437-1450, 1489-1500,
// 1559-1569 for TH; 1667-1854 U1; 1916-2094 U2; 2177-2372 U3): nu is NU_T or
// KAPPA_T; g11 weighs the zeta (K) differences, g22 the eta (J) ones
// (GMAT_11/22, or their _y variants for U2 and _z variants for U3).
struct LesAdi {
  const std::vector<double> *nu;
  const std::vector<double> *g11, *g22;
  double temp2;
};

#endif
