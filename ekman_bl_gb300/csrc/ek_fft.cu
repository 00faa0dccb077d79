// Batched x-direction real FFTs of the duct substep, FP64.
//
// The reference transforms every field line along x through
// REAL_FOURIER_TRANS_* (src/mpi_duct.F90:271-717) and the missing
// FFT_X_TO_FOURIER_OP / FFT_X_TO_PHYSICAL_OP (FFTW 2 rfftw).  Here one warp
// owns one x-line: a length-NX real transform is done as a length-NX/2
// complex radix-2 DIF FFT in shared memory plus the split/merge twiddle
// step.  Forward transforms keep modes 0..NX/3 and scale by 1/NX; the
// inverse reads modes 0..NX/3 (imaginary part of mode 0 ignored) and zeroes
// the two padding points x = NX, NX+1, as the reference's copy loops do.
//
// The forward kernel fuses its producer and consumer:
//   prologue PRO_LOAD  x = a
//            PRO_PROD  x = J a b            (duct.F90:685-691 products)
//            PRO_FLUX  x = flux stencil of a (duct.F90:735-761 form)
//            (with LES, + J tau or + the eddy-viscosity terms: ek_les.cu)
//   epilogue EPI_STORE dst  = X            (modes > NX/3 set to 0)
//            EPI_ADD   dst += X            (duct.F90:779-785)
//            EPI_SUB_IK dst -= i kx X      (duct.F90:712-718)
// so no product or transform temporary ever reaches HBM.
#include <map>
#include <type_traits>
#include <mutex>
#include <utility>

#include "ek_internal.h"

namespace ek {

namespace {

constexpr int kWarpsPerBlock = 4;

struct FftConst {
  Dims d;
  int M, logM;
  const double2 *tw_m, *tw_n;
  const float2 *tw_mf, *tw_nf;  // the same tables rounded to FP32
  const float4 *tw_mff, *tw_nff;  // and split into float-float (re.hi, re.lo, im.hi, im.lo)
  const double *kx;
  Metrics m;
  double inv_nx;  // 1/NX, divided once on the host
};

// T: the arithmetic type of a transform (double; float with the fields still
// stored in FP64; or FF); V: its complex pair.
template <typename T> struct Cx;
template <> struct Cx<double> {
  using V = double2;
  __device__ static V make(double x, double y) { return make_double2(x, y); }
};
template <> struct Cx<float> {
  using V = float2;
  __device__ static V make(float x, float y) { return make_float2(x, y); }
};
struct FF2 {
  FF x, y;
};
template <> struct Cx<FF> {
  using V = FF2;
  __device__ static V make(FF x, FF y) { return FF2{x, y}; }
};
template <typename T> __device__ __forceinline__ const typename Cx<T>::V *tw_m(const FftConst &f);
template <> __device__ __forceinline__ const double2 *tw_m<double>(const FftConst &f) { return f.tw_m; }
template <> __device__ __forceinline__ const float2 *tw_m<float>(const FftConst &f) { return f.tw_mf; }
template <> __device__ __forceinline__ const FF2 *tw_m<FF>(const FftConst &f) {
  return reinterpret_cast<const FF2 *>(f.tw_mff);
}
template <typename T> __device__ __forceinline__ const typename Cx<T>::V *tw_n(const FftConst &f);
template <> __device__ __forceinline__ const double2 *tw_n<double>(const FftConst &f) { return f.tw_n; }
template <> __device__ __forceinline__ const float2 *tw_n<float>(const FftConst &f) { return f.tw_nf; }
template <> __device__ __forceinline__ const FF2 *tw_n<FF>(const FftConst &f) {
  return reinterpret_cast<const FF2 *>(f.tw_nff);
}

// an FP64 value in the arithmetic type T; to float on the integer pipe
// (a plain cast is an F2F on the narrow FP64 pipe)
template <typename T> __device__ __forceinline__ T from_f64(double x) { return (T)x; }
template <> __device__ __forceinline__ float from_f64<float>(double x) { return d2f_bits(x); }

template <typename V>
__device__ __forceinline__ V cmul(V a, V b) {
  V r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

__device__ __forceinline__ unsigned brev(unsigned v, int logM) { return __brev(v) >> (32 - logM); }

// In-place radix-2 DIF over z[0..M), bit-reversed output.  conj_tw selects
// the inverse transform.
template <typename V>
__device__ __forceinline__ void dif_fft(V *z, int M, const V *tw, bool conj_tw, int lane) {
  for (int s = M >> 1; s >= 1; s >>= 1) {
    const int stride = (M >> 1) / s;  // twiddle step M/(2s)
    for (int q = lane; q < (M >> 1); q += 32) {
      const int t = q & (s - 1);
      const int a = ((q - t) << 1) + t;
      const int b = a + s;
      const V u = z[a], v = z[b];
      V sum, dlt;
      sum.x = u.x + v.x;
      sum.y = u.y + v.y;
      dlt.x = u.x - v.x;
      dlt.y = u.y - v.y;
      z[a] = sum;
      if (t != 0) {
        V w = tw[t * stride];
        if (conj_tw) w.y = -w.y;
        dlt = cmul(dlt, w);
      }
      z[b] = dlt;
    }
    __syncwarp();
  }
}

// One value exchanged with the lane whose index differs in the bits of m.
__device__ __forceinline__ float2 shfl_x(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
template <typename V>
__device__ __forceinline__ V csub(V a, V b) {
  V r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
template <typename V>
__device__ __forceinline__ V caddv(V a, V b) {
  V r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}

// The same radix-2 DIF (same butterflies, same twiddles, bit-reversed
// output in z) with the warp's M = 32 E points held in registers: lane l
// keeps points l + 32 t, t < E.  The log2(E) stages whose pairs are 32 or
// more apart run between a lane's own registers; the five stages below run
// between lanes through shuffles, where a lane's twiddle depends only on the
// lane.  Shared memory is touched once to load and once to store, instead
// of twice per stage.
template <int E, typename V>
__device__ __forceinline__ void dif_fft_reg(V *z, const V *tw, bool conj_tw, int lane) {
  constexpr int M = 32 * E;
  V v[E];
#pragma unroll
  for (int t = 0; t < E; ++t) v[t] = z[lane + 32 * t];
#pragma unroll
  for (int h = E / 2; h >= 1; h >>= 1) {
    // span s = 32 h: pairs (t, t + h) within each block of 2h registers
    const int stride = M / (64 * h);  // M / (2 s)
#pragma unroll
    for (int t = 0; t < E; ++t) {
      if (t & h) continue;
      const V a = v[t], b = v[t + h];
      v[t] = caddv(a, b);
      const int tt = lane + 32 * (t & (h - 1));  // n mod s
      V dlt = csub(a, b);
      if (tt != 0) {
        V w = tw[tt * stride];
        if (conj_tw) w.y = -w.y;
        dlt = cmul(dlt, w);
      }
      v[t + h] = dlt;
    }
  }
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
    const int tt = lane & (s - 1);
    V w = tw[tt * (M / (2 * s))];
    if (conj_tw) w.y = -w.y;
#pragma unroll
    for (int t = 0; t < E; ++t) {
      const V p = shfl_x(v[t], s);
      if (!upper) {
        v[t] = caddv(v[t], p);
      } else {
        V dlt = csub(p, v[t]);
        if (tt != 0) dlt = cmul(dlt, w);
        v[t] = dlt;
      }
    }
  }
  // v[t] holds DIF position p = lane + 32 t, i.e. frequency brev(p) =
  // rev5(lane) E + revE(t); it goes to its natural-order slot with one pad
  // element every E (fslot), so that this store and the readers' runs of
  // consecutive frequencies fall in distinct banks (the bit-reversed order
  // puts a warp's 32 frequencies E elements apart)
  const int r5 = (int)(__brev((unsigned)lane) >> 27);
#pragma unroll
  for (int t = 0; t < E; ++t) {
    int rt = 0;
#pragma unroll
    for (int b = 1, q = E >> 1; b < E; b <<= 1, q >>= 1)
      if (t & b) rt |= q;
    z[r5 * (E + 1) + rt] = v[t];
  }
  __syncwarp();
}

// Where frequency f of a transform of M = 32 E points sits after
// dif_fft_any<E>: natural order with a pad element every E (the register
// form), bit-reversed order (the shared-memory loop, E = 0).
template <int E>
__device__ __forceinline__ int fslot(int f, int logM) {
  if constexpr (E > 0) return f + f / E;
  else return (int)brev((unsigned)f, logM);
}
// Per-warp stride of the spectra in shared memory: room for the pad slots
template <int E>
__device__ __forceinline__ int fstride(int M) { return (E > 0) ? M + 32 : M; }

// The register form for M = 32 E (E > 0, chosen per launch so that each
// size gets its own register budget), the shared-memory loop otherwise.
template <int E, typename V>
__device__ __forceinline__ void dif_fft_any(V *z, int M, const V *tw, bool conj_tw, int lane) {
  __syncwarp();
  if constexpr (E > 0) dif_fft_reg<E>(z, tw, conj_tw, lane);
  else dif_fft(z, M, tw, conj_tw, lane);
}

// The flux form of the eta/zeta convection plus the GMAT_12 cross diffusion
// of field a (duct.F90:735-761; the TH version at 1210-1241 has visc =
// NU/PR) along one x-line, into zr: from the FP32 copies (fin) or FP64.
// b is U2b, followed in memory by U3b (see the launch).
template <typename T>
__device__ __forceinline__ void flux_line(T *zr, const FftConst &fc, int k, int j, size_t base, int lane, bool fin,
                                          const double *a, const double *b, const float *af, const float *bf,
                                          double visc) {
  const Dims &d = fc.d;
  const int NX = d.NX;
  const T g12a = from_f64<T>(fc.m.g12[d.m3(k + 1, j, 2)]), g12b = from_f64<T>(fc.m.g12[d.m3(k, j, 2)]);
  const T g12c = from_f64<T>(fc.m.g12[d.m3(k, j + 1, 1)]), g12d = from_f64<T>(fc.m.g12[d.m3(k, j, 1)]);
  const T qv = from_f64<T>(0.25 * visc);
  const T h = (T)0.5;
  const size_t sK = d.LDX, sJ = (size_t)d.LDX * d.NZ2;
  if (fin) {
    const float *F = af, *U2b = bf, *U3b = bf + d.nphys();
    for (int n = lane; n < NX; n += 32) {
      const size_t c = base + n;
      const T f = (T)(double)F[c], fkp = (T)(double)F[c + sK], fkm = (T)(double)F[c - sK];
      const T fjp = (T)(double)F[c + sJ], fjm = (T)(double)F[c - sJ];
      const T fpp = (T)(double)F[c + sK + sJ], fpm = (T)(double)F[c + sK - sJ];
      const T fmp = (T)(double)F[c - sK + sJ], fmm = (T)(double)F[c - sK - sJ];
      T s1 = h * (T)(double)U2b[c + sJ] * (f + fjp) - h * (T)(double)U2b[c] * (f + fjm);
      T s2 = h * (T)(double)U3b[c + sK] * (f + fkp) - h * (T)(double)U3b[c] * (f + fkm);
      s1 = -s1 + qv * (g12a * (fpp + fjp - fjm - fpm) - g12b * (fmp + fjp - fjm - fmm));
      s2 = -s2 + qv * (g12c * (fpp + fkp - fmp - fkm) - g12d * (fkp + fpm - fkm - fmm));
      zr[n] = s1 + s2;
    }
  } else {
    const double *F = a, *U2b = b, *U3b = b + d.nphys();
    for (int n = lane; n < NX; n += 32) {
      const size_t c = base + n;
      const T f = (T)F[c], fkp = (T)F[c + sK], fkm = (T)F[c - sK], fjp = (T)F[c + sJ], fjm = (T)F[c - sJ];
      const T fpp = (T)F[c + sK + sJ], fpm = (T)F[c + sK - sJ], fmp = (T)F[c - sK + sJ], fmm = (T)F[c - sK - sJ];
      T s1 = h * (T)U2b[c + sJ] * (f + fjp) - h * (T)U2b[c] * (f + fjm);
      T s2 = h * (T)U3b[c + sK] * (f + fkp) - h * (T)U3b[c] * (f + fkm);
      s1 = -s1 + qv * (g12a * (fpp + fjp - fjm - fpm) - g12b * (fmp + fjp - fjm - fmm));
      s2 = -s2 + qv * (g12c * (fpp + fkp - fmp - fkm) - g12d * (fkp + fpm - fkm - fmm));
      zr[n] = s1 + s2;
    }
  }
}

// The FP32 register form asks for 8 blocks an SM (64 registers, a 16-byte
// spill; 72 registers left 7): the step's forward transforms 10.6 -> 9.8 ms
// on 512 x 385 x 257.  A minimum of 0 leaves the other forms' allocation
// as the compiler chooses it.
template <typename T, int E>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, (sizeof(T) == 4 && E > 0) ? 8 : 0)
    k_r2c(FftConst fc, R2cArgs args) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *smem_c = reinterpret_cast<V *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Dims &d = fc.d;
  const int nk = args.k1 - args.k0 + 1;
  // grid (ceil(nk / kWarpsPerBlock), nj): no index division (a 64-bit one
  // is a long integer sequence with FP64 steps)
  const int kw = (int)blockIdx.x * kWarpsPerBlock + warp;
  if (kw >= nk) return;
  const int k = args.k0 + kw;
  const int j = args.j0 + (int)blockIdx.y;
  const int NX = d.NX, M = fc.M;
  V *z = smem_c + (size_t)warp * fstride<E>(M);
  T *zr = reinterpret_cast<T *>(z);
  const size_t base = d.ip(0, k, j);
  constexpr bool kF = sizeof(T) == 4;
  const bool fin = kF && args.af != nullptr;  // FP32 copies of the inputs
  if (args.pro == PRO_LOAD) {
    if constexpr (std::is_same_v<T, FF>) {
      if (args.alo) {
        // a float-float field: the pair as it is, no FP64 split
        for (int n = lane; n < NX; n += 32) zr[n] = FF(args.af[base + n], args.alo[base + n]);
      } else {
        for (int n = lane; n < NX; n += 32) zr[n] = (T)args.a[base + n];
      }
    } else if (fin) {
      // an FP32 field (the increment of the state)
      for (int n = lane; n < NX; n += 32) zr[n] = (T)args.af[base + n];
    } else {
      for (int n = lane; n < NX; n += 32) zr[n] = (T)args.a[base + n];
    }
  } else if (args.pro == PRO_PROD) {
    const T jac = from_f64<T>(fc.m.jac[d.m2(k, j)]);
    if (fin)
      for (int n = lane; n < NX; n += 32) zr[n] = jac * (T)(double)args.af[base + n] * (T)(double)args.bf[base + n];
    else
      for (int n = lane; n < NX; n += 32) zr[n] = jac * (T)args.a[base + n] * (T)args.b[base + n];
  } else {
    flux_line<T>(zr, fc, k, j, base, lane, fin, args.a, args.b, args.af, args.bf, args.visc);
  }
  if (args.pro != PRO_LOAD && (args.extra || args.extraf)) {
    // LES additions: jac * tau for a product, the precomputed terms for a flux
    const T es = (args.pro == PRO_PROD) ? from_f64<T>(fc.m.jac[d.m2(k, j)]) : (T)1.0;
    if (kF && args.extraf)
      for (int n = lane; n < NX; n += 32) zr[n] = zr[n] + es * (T)args.extraf[base + n];
    else if (args.extra)
      for (int n = lane; n < NX; n += 32) zr[n] = zr[n] + es * (T)args.extra[base + n];
  }
  // with fuse_flux the same line's flux term (PRO_FLUX of a2 against b2, and
  // its LES addition) goes through a second transform in the same warp
  const bool fuse = args.fuse_flux != 0;
  V *z2 = smem_c + (size_t)(kWarpsPerBlock + warp) * fstride<E>(M);
  if (fuse) {
    T *zr2 = reinterpret_cast<T *>(z2);
    const bool fin2 = kF && args.a2f != nullptr;
    flux_line<T>(zr2, fc, k, j, base, lane, fin2, args.a2, args.b2, args.a2f, args.b2f, args.visc2);
    if (kF && args.extraf2)
      for (int n = lane; n < NX; n += 32) zr2[n] = zr2[n] + (T)1.0 * (T)args.extraf2[base + n];
    else if (args.extra2)
      for (int n = lane; n < NX; n += 32) zr2[n] = zr2[n] + (T)1.0 * (T)args.extra2[base + n];
  }
  __syncwarp();
  dif_fft_any<E>(z, M, tw_m<T>(fc), false, lane);
  if (fuse) dif_fft_any<E>(z2, M, tw_m<T>(fc), false, lane);
  // split: X[k] = E + W^k O, E = (Z_k + conj Z_{M-k})/2, O = -i (Z_k - conj Z_{M-k})/2
  cplx_t *dst = args.dst + d.ic(0, k, j);
  const T inv = from_f64<T>(fc.inv_nx);
  const T h = (T)0.5;
  const int NKX = d.NKX;
  const V *twn = tw_n<T>(fc);
  for (int kk = lane; kk <= d.NX2P; kk += 32) {
    if (kk > NKX) {
      if (args.epi == EPI_STORE || args.zero_hi) dst[kk] = cplx_t{0.0, 0.0};
      continue;
    }
    const int ik = fslot<E>(kk & (M - 1), fc.logM), im = fslot<E>((M - kk) & (M - 1), fc.logM);
    const V w = twn[kk];
    auto split = [&](const V *zz, T &tr, T &ti) {
      const V zk = zz[ik], zm = zz[im];
      const T er = h * (zk.x + zm.x), ei = h * (zk.y - zm.y);
      const T orr = h * (zk.y + zm.y), oi = -h * (zk.x - zm.x);
      tr = (er + (w.x * orr - w.y * oi)) * inv;
      ti = (ei + (w.x * oi + w.y * orr)) * inv;
    };
    T tr, ti;
    split(z, tr, ti);
    if (fuse) {
      // dst -= i kx X, then dst += X2: the two launches' FP64 updates in order
      T tr2, ti2;
      split(z2, tr2, ti2);
      const cplx_t o = dst[kk];
      if constexpr (kF) {
        const T kv = from_f64<T>(fc.kx[kk]);
        const cplx_t o1{o.re - f2d_bits((float)(T(0) * tr - kv * ti)), o.im - f2d_bits((float)(T(0) * ti + kv * tr))};
        dst[kk] = cplx_t{o1.re + f2d_bits((float)tr2), o1.im + f2d_bits((float)ti2)};
      } else {
        const double xr = (double)tr, xi = (double)ti, kv = fc.kx[kk];
        const cplx_t o1{o.re - (0.0 * xr - kv * xi), o.im - (0.0 * xi + kv * xr)};
        dst[kk] = cplx_t{o1.re + (double)tr2, o1.im + (double)ti2};
      }
      continue;
    }
    if constexpr (kF) {
      // the FP32 result enters the FP64 field with one exact widening and
      // one FP64 add per component
      const cplx_t o = (args.epi == EPI_STORE) ? cplx_t{0.0, 0.0} : dst[kk];
      if (args.epi == EPI_STORE) {
        dst[kk] = cplx_t{f2d_bits((float)tr), f2d_bits((float)ti)};
      } else if (args.epi == EPI_ADD) {
        dst[kk] = cplx_t{o.re + f2d_bits((float)tr), o.im + f2d_bits((float)ti)};
      } else {
        const T kv = from_f64<T>(fc.kx[kk]);
        dst[kk] = cplx_t{o.re - f2d_bits((float)(T(0) * tr - kv * ti)), o.im - f2d_bits((float)(T(0) * ti + kv * tr))};
      }
      continue;
    } else {
    const double xr = (double)tr, xi = (double)ti;
    if (args.epi == EPI_STORE) {
      dst[kk] = cplx_t{xr, xi};
    } else if (args.epi == EPI_ADD) {
      const cplx_t o = dst[kk];
      dst[kk] = cplx_t{o.re + xr, o.im + xi};
    } else {
      // CF = CF - CIKXP*CS with CIKXP = (0, kx)
      const double kv = fc.kx[kk];
      const cplx_t o = dst[kk];
      dst[kk] = cplx_t{o.re - (0.0 * xr - kv * xi), o.im - (0.0 * xi + kv * xr)};
    }
    }
  }
}

template <typename T, int E>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_c2r(FftConst fc, C2rArgs args) {
  using V = typename Cx<T>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *smem_c = reinterpret_cast<V *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Dims &d = fc.d;
  const int nk = args.k1 - args.k0 + 1;
  // grid (ceil(nk / kWarpsPerBlock), nj): no index division (a 64-bit one
  // is a long integer sequence with FP64 steps)
  const int kw = (int)blockIdx.x * kWarpsPerBlock + warp;
  if (kw >= nk) return;
  const int k = args.k0 + kw;
  const int j = args.j0 + (int)blockIdx.y;
  const int M = fc.M, NKX = d.NKX;
  V *z = smem_c + (size_t)warp * fstride<E>(M);
  const cplx_t *src = args.src + d.ic(0, k, j);
  const cplx_t *src2 = args.src2 ? args.src2 + d.ic(0, k, j) : nullptr;
  auto X = [&](int kk) -> V {
    if (kk > NKX || kk >= M) return Cx<T>::make(T(0.0), T(0.0));
    cplx_t v = src[kk];
    if (src2) {
      const cplx_t w = src2[kk];
      v.re = v.re + args.scale2 * w.re;
      v.im = v.im + args.scale2 * w.im;
    }
    if (args.ik) {  // CIKXP * v
      const double kv = fc.kx[kk], re = v.re;
      v.re = -(kv * v.im);
      v.im = kv * re;
    }
    if (kk == 0) v.im = 0.0;
    return Cx<T>::make(from_f64<T>(v.re), from_f64<T>(v.im));
  };
  // merge: Z'[k] = (X_k + conj X_{M-k}) + i (X_k - conj X_{M-k}) W^{-k}.
  // The spectrum is staged in z first, so that each mode's prologue (FP64
  // loads, the scale2 combination, the split into T) runs once; then each
  // lane merges the pair (k, M-k) in place (X_M = 0: k = 0 pairs with zero).
  for (int kk = lane; kk < M; kk += 32) z[kk] = X(kk);
  __syncwarp();
  const V *twn = tw_n<T>(fc);
  auto merge = [&](V a, V b, V w) {
    const T sr = a.x + b.x, si = a.y - b.y;  // X_k + conj X_{M-k}
    const T dr = a.x - b.x, di = a.y + b.y;  // X_k - conj X_{M-k}
    const T tr = dr * w.x + di * w.y, ti = di * w.x - dr * w.y;  // (d)*conj(w)
    return Cx<T>::make(sr - ti, si + tr);   // + i*t
  };
  for (int kk = lane; kk <= (M >> 1); kk += 32) {
    const V a = z[kk];
    const V b = (kk == 0) ? Cx<T>::make(T(0.0), T(0.0)) : z[M - kk];
    z[kk] = merge(a, b, twn[kk]);
    if (kk != 0 && 2 * kk != M) z[M - kk] = merge(b, a, twn[M - kk]);
  }
  __syncwarp();
  dif_fft_any<E>(z, M, tw_m<T>(fc), true, lane);
  const T *zr = reinterpret_cast<const T *>(z);
  double *dst = args.dst ? args.dst + d.ip(0, k, j) : nullptr;
  float *dstf = args.dstf ? args.dstf + d.ip(0, k, j) : nullptr;
  const int NX = d.NX;
  if constexpr (std::is_same_v<T, FF>) {
    if (args.dstlo) {
      // float-float planes: the high part is also the field's FP32 copy
      float *dlo = args.dstlo + d.ip(0, k, j);
      for (int n = lane; n < NX + 2; n += 32) {
        FF v(0.0f, 0.0f);
        if (n < NX) v = zr[2 * fslot<E>(n >> 1, fc.logM) + (n & 1)];
        dstf[n] = v.hi;
        dlo[n] = v.lo;
      }
      return;
    }
  }
  for (int n = lane; n < NX + 2; n += 32) {
    T v = T(0.0);
    if (n < NX) {
      const int m = n >> 1;
      v = zr[2 * fslot<E>(m, fc.logM) + (n & 1)];
    }
    if constexpr (sizeof(T) == 4) {
      if (dst) dst[n] = f2d_bits((float)v);
      if (dstf) dstf[n] = (float)v;
    } else {
      if (dst) dst[n] = (double)v;
      if (dstf) dstf[n] = d2f_bits((double)v);
    }
  }
}

// Launch a transform.  The register form of the FFT pays in the FP32
// transforms (measured on 512 x 385 x 257: the inverse 0.34 -> 0.23 ms per
// launch; the forward ones, since each launch fuses a component's product
// and flux transforms, 13.9 -> 11.7 ms a step); in the FP64 and float-float
// ones its extra registers cost more than the shared-memory passes it
// saves, so they keep the loop.
template <typename T>
void run_r2c(dim3 grid, size_t smem, cudaStream_t s, const FftConst &fc, const R2cArgs &a) {
  const unsigned nt = 32 * kWarpsPerBlock;
  if constexpr (std::is_same_v<T, float>) {
    switch (fc.M) {
      case 32: k_r2c<T, 1><<<grid, nt, smem, s>>>(fc, a); return;
      case 64: k_r2c<T, 2><<<grid, nt, smem, s>>>(fc, a); return;
      case 128: k_r2c<T, 4><<<grid, nt, smem, s>>>(fc, a); return;
      case 256: k_r2c<T, 8><<<grid, nt, smem, s>>>(fc, a); return;
      case 512: k_r2c<T, 16><<<grid, nt, smem, s>>>(fc, a); return;
      default: break;
    }
  }
  k_r2c<T, 0><<<grid, nt, smem, s>>>(fc, a);
}
template <typename T>
void run_c2r(dim3 grid, size_t smem, cudaStream_t s, const FftConst &fc, const C2rArgs &a) {
  const unsigned nt = 32 * kWarpsPerBlock;
  if constexpr (std::is_same_v<T, float>) {
    switch (fc.M) {
      case 32: k_c2r<T, 1><<<grid, nt, smem, s>>>(fc, a); return;
      case 64: k_c2r<T, 2><<<grid, nt, smem, s>>>(fc, a); return;
      case 128: k_c2r<T, 4><<<grid, nt, smem, s>>>(fc, a); return;
      case 256: k_c2r<T, 8><<<grid, nt, smem, s>>>(fc, a); return;
      case 512: k_c2r<T, 16><<<grid, nt, smem, s>>>(fc, a); return;
      default: break;
    }
  }
  k_c2r<T, 0><<<grid, nt, smem, s>>>(fc, a);
}
template <typename T>
void smem_attributes() {
  const int b = 96 * 1024;
  EK_CUDA(cudaFuncSetAttribute(k_r2c<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
  EK_CUDA(cudaFuncSetAttribute(k_c2r<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
  if constexpr (std::is_same_v<T, float>) {
    EK_CUDA(cudaFuncSetAttribute(k_c2r<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_r2c<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_r2c<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_r2c<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_r2c<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_r2c<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_c2r<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_c2r<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_c2r<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    EK_CUDA(cudaFuncSetAttribute(k_c2r<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
  }
}

FftConst make_const(Ctx &c) {
  FftConst f;
  f.d = c.d;
  f.M = c.d.NX / 2;
  int lg = 0;
  while ((1 << lg) < f.M) ++lg;
  f.logM = lg;
  f.tw_m = c.tw_m;
  f.tw_n = c.tw_n;
  f.tw_mf = c.tw_mf;
  f.tw_nf = c.tw_nf;
  f.tw_mff = c.tw_mff;
  f.tw_nff = c.tw_nff;
  f.kx = c.kx;
  f.inv_nx = 1.0 / c.d.NX;
  f.m = c.m;
  return f;
}

}  // namespace

// FP32 arithmetic for this transform?  fft_fp32 = 1: only the transforms
// marked low-precision (the nonlinear products and fluxes, whose results
// enter the step multiplied by the time step); 2: every transform.
bool fft_lowp(const Ctx &c, int lowp) { return c.p.fft_fp32 >= 2 || (c.p.fft_fp32 == 1 && lowp); }
// float-float for the other transforms under ff_arith
bool fft_ff(const Ctx &c, int lowp) { return c.p.ff_arith && !fft_lowp(c, lowp); }

void launch_r2c(Ctx &c, const R2cArgs &a) {
  const FftConst fc = make_const(c);
  const long nlines = (long)(a.k1 - a.k0 + 1) * (a.j1 - a.j0 + 1);
  if (nlines <= 0) return;
  const dim3 grid((unsigned)((a.k1 - a.k0 + 1 + kWarpsPerBlock - 1) / kWarpsPerBlock), (unsigned)(a.j1 - a.j0 + 1));
  if (a.fuse_flux && (a.pro != PRO_PROD || a.epi != EPI_SUB_IK))
    throw CudaError("r2c: a fused flux goes with a product and dst -= i kx X");
  // a fused launch holds both lines' spectra
  const size_t smem = sizeof(double2) * fc.M * kWarpsPerBlock * (a.fuse_flux ? 2 : 1);
  // algorithmic bytes: the input planes read (the flux's field, U2b and U3b;
  // a fused launch reads its product's second factor once, as the flux's
  // field) at the size of the copy the kernel reads, and the spectrum
  // (an FP32 kernel reading FP32 copies: 4 bytes an element; FP64 fields,
  // or float-float planes as hi and lo: 8)
  const bool lp = fft_lowp(c, a.lowp);
  const double elt = (lp && a.af) ? 4.0 : 8.0;
  const int nops = (a.pro == PRO_LOAD) ? 1 : (a.pro == PRO_PROD) ? (a.fuse_flux ? 4 : 2) : 3;
  const double epi = (a.epi == EPI_STORE) ? 16.0 * (c.d.NX2P + 1) : 32.0 * (c.d.NKX + 1);
  KScope ks(c, KC_R2C, nlines * (elt * c.d.NX * nops + epi));
  // FP32 spectra: 8 bytes an element, with the register form's pad slots
  const size_t smem_f = sizeof(float2) * (fc.M + 32) * kWarpsPerBlock * (a.fuse_flux ? 2 : 1);
  if (lp) run_r2c<float>(grid, smem_f, c.stream, fc, a);
  else if (fft_ff(c, a.lowp)) run_r2c<FF>(grid, smem, c.stream, fc, a);
  else run_r2c<double>(grid, smem, c.stream, fc, a);
  after_launch(c);
}

void launch_c2r(Ctx &c, const C2rArgs &a) {
  const FftConst fc = make_const(c);
  const long nlines = (long)(a.k1 - a.k0 + 1) * (a.j1 - a.j0 + 1);
  if (nlines <= 0) return;
  const dim3 grid((unsigned)((a.k1 - a.k0 + 1 + kWarpsPerBlock - 1) / kWarpsPerBlock), (unsigned)(a.j1 - a.j0 + 1));
  const size_t smem = sizeof(double2) * fc.M * kWarpsPerBlock;
  // algorithmic bytes: the spectra read, the planes written (FP64, FP32 copy
  // and float-float low part as given)
  const double out = (a.dst ? 8.0 : 0.0) + (a.dstf ? 4.0 : 0.0) + (a.dstlo ? 4.0 : 0.0);
  KScope ks(c, KC_C2R, nlines * (16.0 * (c.d.NKX + 1) * (a.src2 ? 2 : 1) + out * (c.d.NX + 2)));
  const size_t smem_f = sizeof(float2) * (fc.M + 32) * kWarpsPerBlock;
  if (fft_lowp(c, a.lowp)) run_c2r<float>(grid, smem_f, c.stream, fc, a);
  else if (fft_ff(c, a.lowp)) run_c2r<FF>(grid, smem, c.stream, fc, a);
  else run_c2r<double>(grid, smem, c.stream, fc, a);
  after_launch(c);
}

}  // namespace ek

namespace ek {
void fft_init_attributes() {
  static std::once_flag once;
  std::call_once(once, [] {
  smem_attributes<double>();
  smem_attributes<float>();
  smem_attributes<FF>();
  });
}
}  // namespace ek

// ---------------------------------------------------------------------------
// Context-free batched x-transforms: the FFT_X_TO_FOURIER_OP /
// FFT_X_TO_PHYSICAL_OP pair that the reference calls (e.g. duct.F90:700 and
// mpi_duct.F90:308) and whose source (fft.F90) is missing from its tree.
namespace ek {
namespace {

thread_local std::string t_last_error;

__global__ void k_twiddles(double2 *tw_m, double2 *tw_n, int nx) {
  const int M = nx / 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t <= M; t += gridDim.x * blockDim.x) {
    double s, c;
    if (t < M / 2) {
      sincospi(-2.0 * t / M, &s, &c);
      tw_m[t] = make_double2(c, s);
    }
    sincospi(-2.0 * t / nx, &s, &c);
    tw_n[t] = make_double2(c, s);
  }
}

bool fft_args_ok(int nx, int nkx, long nlines, const void *in, const void *out) {
  if (nx < 8 || nx > 1024 || (nx & (nx - 1))) {
    t_last_error = "nx must be a power of two in [8, 1024]";
    return false;
  }
  if (nkx < 0 || nkx >= nx / 2) {
    t_last_error = "nkx must be in [0, nx/2)";
    return false;
  }
  if (nlines < 0 || nlines > (1L << 30) || (nlines > 0 && (!in || !out))) {
    t_last_error = "bad line count or NULL buffer";
    return false;
  }
  return true;
}

// Twiddle tables of the context-free transforms: cudaMalloc'd once per
// (device, nx) and kept for the life of the process.  Their size in double2,
// shared with the fixed table of the allocation-free entry point below.
constexpr int twiddle_count(int nx) { return (nx / 2) / 2 + nx / 2 + 1; }
std::mutex g_tw_mu;
std::map<std::pair<int, int>, double2 *> g_tw_cache;
double2 *cached_twiddles(int nx, cudaStream_t s) {
  int dev = 0;
  EK_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto &cache = g_tw_cache;
  auto it = cache.find({dev, nx});
  if (it != cache.end()) return it->second;
  const int M = nx / 2;
  double2 *tw = nullptr;
  EK_CUDA(cudaMalloc(&tw, sizeof(double2) * twiddle_count(nx)));
  k_twiddles<<<4, 256, 0, s>>>(tw, tw + M / 2, nx);
  EK_CUDA(cudaPeekAtLastError());
  EK_CUDA(cudaStreamSynchronize(s));
  cache[{dev, nx}] = tw;
  return tw;
}

FftConst standalone_const(int nx, int nkx, long nlines, const double2 *tw) {
  FftConst f{};
  Dims &d = f.d;
  d.NX = nx;
  d.NKX = nkx;
  d.NX2P = nx / 2;
  d.LDX = nx + 2;
  d.LDC = nx / 2 + 1;
  d.NZ2 = (int)nlines;  // lines are indexed as (k, j = 0)
  d.NY2 = 1;
  f.M = nx / 2;
  int lg = 0;
  while ((1 << lg) < f.M) ++lg;
  f.logM = lg;
  f.tw_m = tw;
  f.tw_n = tw + f.M / 2;
  f.inv_nx = 1.0 / nx;
  return f;
}

int run_standalone(bool forward, int nx, int nkx, long nlines, const double *in, double *out, cudaStream_t s,
                   const double2 *tw) {
  if (nlines == 0) return EK_OK;
  const FftConst fc = standalone_const(nx, nkx, nlines, tw);
  const dim3 grid((unsigned)((nlines + kWarpsPerBlock - 1) / kWarpsPerBlock), 1u);
  const size_t smem = sizeof(double2) * fc.M * kWarpsPerBlock;
  if (forward) {
    R2cArgs a{};
    a.a = in;
    a.dst = reinterpret_cast<cplx_t *>(out);
    a.pro = PRO_LOAD;
    a.epi = EPI_STORE;
    a.k0 = 0; a.k1 = (int)nlines - 1; a.j0 = 0; a.j1 = 0;
    run_r2c<double>(grid, smem, s, fc, a);
  } else {
    C2rArgs a{};
    a.src = reinterpret_cast<const cplx_t *>(in);
    a.dst = out;
    a.k0 = 0; a.k1 = (int)nlines - 1; a.j0 = 0; a.j1 = 0;
    run_c2r<double>(grid, smem, s, fc, a);
  }
  EK_CUDA(cudaPeekAtLastError());
  return EK_OK;
}

int standalone(bool forward, int nx, int nkx, long nlines, const double *in, double *out, void *stream) {
  if (!fft_args_ok(nx, nkx, nlines, in, out)) return EK_ERR_ARG;
  try {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    fft_init_attributes();
    const double2 *tw = cached_twiddles(nx, s);
    return run_standalone(forward, nx, nkx, nlines, in, out, s, tw);
  } catch (const CudaError &e) {
    t_last_error = e.msg;
    return EK_ERR_CUDA;
  }
}

}  // namespace

const char *last_global_error() { return t_last_error.c_str(); }

}  // namespace ek

extern "C" int ekgpu_fft_table_count(void) {
  std::lock_guard<std::mutex> lk(ek::g_tw_mu);
  return (int)ek::g_tw_cache.size();
}

extern "C" int ekgpu_fft_x_to_fourier(int nx, int nkx, long nlines, const double *in_dev, double *out_dev,
                                      void *stream) {
  return ek::standalone(true, nx, nkx, nlines, in_dev, out_dev, stream);
}

extern "C" int ekgpu_fft_x_to_physical(int nx, int nkx, long nlines, const double *in_dev, double *out_dev,
                                       void *stream) {
  return ek::standalone(false, nx, nkx, nlines, in_dev, out_dev, stream);
}

// ---------------------------------------------------------------------------
// ekgpu_fft_x_to_fourier_noalloc: the forward transform above with its
// twiddle scratch in a fixed device array instead of cudaMalloc'd memory.
namespace ek {
namespace {

// Largest nx the array holds: (nx/4 + nx/2 + 1) twiddles = 769 for nx = 1024
// (12.3 KB, resident on every GPU that loads the library until exit).
constexpr int kNoAllocMaxNx = 1024;
constexpr int kNoAllocTw = kNoAllocMaxNx / 4 + kNoAllocMaxNx / 2 + 1;
static_assert(kNoAllocTw == twiddle_count(kNoAllocMaxNx), "the fixed table must hold the cached layout at nx = 1024");
static __device__ __align__(256) double2 g_noalloc_twiddles[kNoAllocTw];

// Device address of g_noalloc_twiddles, looked up once per device (the host
// symbol itself is only a stand-in and must never reach a kernel).
double2 *noalloc_scratch(int &err) {
  static std::mutex mu;
  static double2 *addr[128] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) {
    t_last_error = std::string("ekgpu_fft_x_to_fourier_noalloc: cudaGetDevice: ") + cudaGetErrorString(e);
    err = EK_ERR_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
    if (e != cudaSuccess || !p) {
      t_last_error = std::string("ekgpu_fft_x_to_fourier_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      err = EK_ERR_CUDA;
      return nullptr;
    }
    addr[dev] = static_cast<double2 *>(p);
  }
  return addr[dev];
}

}  // namespace
}  // namespace ek

extern "C" int ekgpu_fft_x_to_fourier_noalloc(int nx, int nkx, long nlines, const double *in_dev, double *out_dev,
                                              void *stream) {
  using namespace ek;
  if (nx > kNoAllocMaxNx) {
    t_last_error = "ekgpu_fft_x_to_fourier_noalloc: nx exceeds the fixed scratch maximum of 1024";
    return EK_ERR_ARG;
  }
  if (!fft_args_ok(nx, nkx, nlines, in_dev, out_dev)) return EK_ERR_ARG;
  int err = EK_OK;
  double2 *tw = noalloc_scratch(err);
  if (!tw) return err;
  try {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    fft_init_attributes();
    // the whole table is rewritten on every call, before the transform reads it
    k_twiddles<<<4, 256, 0, s>>>(tw, tw + nx / 4, nx);
    EK_CUDA(cudaPeekAtLastError());
    return run_standalone(true, nx, nkx, nlines, in_dev, out_dev, s, tw);
  } catch (const CudaError &e) {
    t_last_error = e.msg;
    return EK_ERR_CUDA;
  }
}
