// Learned initial guess for the per-kx Poisson problems: a small U-Net on
// the problems' right-hand sides, trained on (rhs, solution) pairs that the
// solver itself produced, and its kernels.
//
// Network (per problem, one image): 4 levels of two 3x3 convolutions with
// ReLU and C channels at every level, 2x2 average pooling down,
// nearest-neighbour upsampling up, the skip tensor joined as channels
// C..2C-1 of the first decoder convolution, and a final 3x3 convolution to
// one channel.  Activations are BF16 (NHWC, a one-pixel zero border around
// every image so that a shifted read never needs a bounds check); weights
// are kept in FP32 (master copy, Adam moments) and rounded to BF16 when a
// tile is staged; gradients are FP32.
//
// All three convolution passes run on one tensor-core GEMM kernel
// (mma.sync m16n8k16, BF16 x BF16 -> FP32) with different operand loaders:
//   forward     M = pixels, N = Cout,  K = 9 Cin     A = shifted input, B = W
//   input grad  M = pixels, N = Cin,   K = 9 Cout    A = shifted dZ,    B = W^T
//   weight grad M = Cout,   N = 9 Cin, K = pixels    A = dZ^T,          B = shifted input
// (the weight gradient is split over pixels and summed with FP32 atomics).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ek_internal.h"
#include "ek_unet.h"

namespace ek {
namespace unet {

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8, NT = 128;

__device__ __forceinline__ unsigned short f2bf(float f) {
  // round to nearest even; NaN kept quiet
  unsigned u = __float_as_uint(f);
  if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x7fffffu)) return (unsigned short)((u >> 16) | 0x40u);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (unsigned short)(u >> 16);
}
__device__ __forceinline__ float bf2f(unsigned short h) { return __uint_as_float((unsigned)h << 16); }

// Image geometry: N images of H x W interior pixels, stored (H+2) x (W+2)
// with a zero border, C channels innermost.
struct Img {
  int N, H, W;
  __device__ __forceinline__ size_t at(int n, int y, int x, int C) const {
    return (((size_t)n * (H + 2) + (y + 1)) * (W + 2) + (x + 1)) * C;
  }
};

// One convolution's operands.  The input is the channel concatenation of
// x1 (c1 channels) and x2 (c2 channels, may be 0); activations BF16.
struct ConvArgs {
  Img g;
  const unsigned short *x1, *x2;
  int c1, c2, cin, cout;
  const float *w;       // [cout][9][cin]
  const float *bias;    // [cout]
  // forward output
  unsigned short *y;    // BF16 [.. cout], or
  float *y32;           // FP32 one channel (the last layer), no border
  int relu;
  // input-gradient pass
  const float *dz;      // FP32 [.. cout] with border
  float *dx1, *dx2;     // FP32 [.. c1], [.. c2] with border
  const unsigned short *m1, *m2;  // ReLU masks (the activations x1, x2), or null
  int acc1, acc2;       // accumulate into dx1 / dx2 instead of storing
  // weight-gradient pass
  float *dw;            // [cout][9][cin] accumulated
  int kchunk;           // pixels per block along K
};

__device__ __forceinline__ void pix(const Img &g, long m, int &n, int &y, int &x) {
  const long hw = (long)g.H * g.W;
  n = (int)(m / hw);
  const int r = (int)(m - (long)n * hw);
  y = r / g.W;
  x = r - y * g.W;
}

__device__ __forceinline__ float act_in(const ConvArgs &a, int n, int y, int x, int ci) {
  if (ci < a.c1) return bf2f(a.x1[a.g.at(n, y, x, a.c1) + ci]);
  return bf2f(a.x2[a.g.at(n, y, x, a.c2) + (ci - a.c1)]);
}

enum { PASS_FWD = 0, PASS_DX = 1, PASS_DW = 2 };

template <int PASS>
struct Ops;

// forward: A(m = pixel, k = tap*cin + ci) = x[pixel + offset(tap)][ci]
template <>
struct Ops<PASS_FWD> {
  static __device__ long M(const ConvArgs &a) { return (long)a.g.N * a.g.H * a.g.W; }
  static __device__ int N(const ConvArgs &a) { return a.cout; }
  static __device__ long K(const ConvArgs &a) { return 9L * a.cin; }
  static __device__ float A(const ConvArgs &a, long m, long k) {
    int n, y, x;
    pix(a.g, m, n, y, x);
    const int tap = (int)(k / a.cin), ci = (int)(k - (long)tap * a.cin);
    return act_in(a, n, y + tap / 3 - 1, x + tap % 3 - 1, ci);
  }
  static __device__ float B(const ConvArgs &a, int nn, long k) { return a.w[(size_t)nn * 9 * a.cin + k]; }
};

// input gradient: dX[p][ci] = sum_{tap,co} W[co][tap][ci] dZ[p - offset(tap)][co]
template <>
struct Ops<PASS_DX> {
  static __device__ long M(const ConvArgs &a) { return (long)a.g.N * a.g.H * a.g.W; }
  static __device__ int N(const ConvArgs &a) { return a.cin; }
  static __device__ long K(const ConvArgs &a) { return 9L * a.cout; }
  static __device__ float A(const ConvArgs &a, long m, long k) {
    int n, y, x;
    pix(a.g, m, n, y, x);
    const int tap = (int)(k / a.cout), co = (int)(k - (long)tap * a.cout);
    return a.dz[a.g.at(n, y - (tap / 3 - 1), x - (tap % 3 - 1), a.cout) + co];
  }
  static __device__ float B(const ConvArgs &a, int ci, long k) {
    const int tap = (int)(k / a.cout), co = (int)(k - (long)tap * a.cout);
    return a.w[((size_t)co * 9 + tap) * a.cin + ci];
  }
};

// weight gradient: dW[co][tap*cin + ci] = sum_p dZ[p][co] x[p + offset(tap)][ci]
template <>
struct Ops<PASS_DW> {
  static __device__ long M(const ConvArgs &a) { return a.cout; }
  static __device__ int N(const ConvArgs &a) { return 9 * a.cin; }
  static __device__ long K(const ConvArgs &a) { return (long)a.g.N * a.g.H * a.g.W; }
  static __device__ float A(const ConvArgs &a, long co, long p) {
    int n, y, x;
    pix(a.g, p, n, y, x);
    return a.dz[a.g.at(n, y, x, a.cout) + co];
  }
  static __device__ float B(const ConvArgs &a, int nn, long p) {
    int n, y, x;
    pix(a.g, p, n, y, x);
    const int tap = nn / a.cin, ci = nn - tap * a.cin;
    return act_in(a, n, y + tap / 3 - 1, x + tap % 3 - 1, ci);
  }
};

__device__ __forceinline__ void mma_bf16(float *d, const unsigned *a, const unsigned *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int PASS>
__device__ __forceinline__ void epilogue(const ConvArgs &a, long m, int nn, float v) {
  if (PASS == PASS_FWD) {
    v += a.bias[nn];
    if (a.relu) v = fmaxf(v, 0.f);
    if (a.y32) {
      a.y32[m] = v;
    } else {
      int n, y, x;
      pix(a.g, m, n, y, x);
      a.y[a.g.at(n, y, x, a.cout) + nn] = f2bf(v);
    }
  } else if (PASS == PASS_DX) {
    int n, y, x;
    pix(a.g, m, n, y, x);
    if (nn < a.c1) {
      const size_t q = a.g.at(n, y, x, a.c1) + nn;
      if (a.m1 && !(bf2f(a.m1[q]) > 0.f)) v = 0.f;
      a.dx1[q] = a.acc1 ? a.dx1[q] + v : v;
    } else {
      const size_t q = a.g.at(n, y, x, a.c2) + (nn - a.c1);
      if (a.m2 && !(bf2f(a.m2[q]) > 0.f)) v = 0.f;
      a.dx2[q] = a.acc2 ? a.dx2[q] + v : v;
    }
  } else {
    atomicAdd(&a.dw[(size_t)m * 9 * a.cin + nn], v);
  }
}

// The GEMM: a 64 x 64 tile per block of 4 warps (2 x 2, 32 x 32 each),
// K in steps of 32 staged through shared memory as BF16 with the K index
// contiguous (rows padded by 8 elements: the fragment loads of a warp hit
// 32 distinct banks).
template <int PASS>
__global__ void __launch_bounds__(NT) k_conv_gemm(ConvArgs a) {
  __shared__ __align__(16) unsigned short As[BM][BK + PAD];
  __shared__ __align__(16) unsigned short Bs[BN][BK + PAD];
  const long M = Ops<PASS>::M(a);
  const int Nn = Ops<PASS>::N(a);
  const long K = Ops<PASS>::K(a);
  const long m0 = (long)blockIdx.x * BM;
  const int n0 = (int)blockIdx.y * BN;
  long k0 = 0, k1 = K;
  if (PASS == PASS_DW) {
    k0 = (long)blockIdx.z * a.kchunk;
    k1 = min(K, k0 + (long)a.kchunk);
  }
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gq = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  for (long kb = k0; kb < k1; kb += BK) {
    // stage A and B; the weight-gradient pass walks pixels (its K) fastest
#pragma unroll 4
    for (int e = 0; e < BM * BK / NT; ++e) {
      const int idx = e * NT + tid;
      const int r = (PASS == PASS_DW) ? idx % BM : idx / BK;
      const int kk = (PASS == PASS_DW) ? idx / BM : idx % BK;
      const long m = m0 + r, k = kb + kk;
      const float v = (m < M && k < k1) ? Ops<PASS>::A(a, m, k) : 0.f;
      As[r][kk] = f2bf(v);
    }
#pragma unroll 4
    for (int e = 0; e < BN * BK / NT; ++e) {
      const int idx = e * NT + tid;
      const int r = (PASS == PASS_DW) ? idx % BN : idx / BK;
      const int kk = (PASS == PASS_DW) ? idx / BN : idx % BK;
      const int nn = n0 + r;
      const long k = kb + kk;
      const float v = (nn < Nn && k < k1) ? Ops<PASS>::B(a, nn, k) : 0.f;
      Bs[r][kk] = f2bf(v);
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      unsigned af[2][4], bq[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + gq;
        af[i][0] = *reinterpret_cast<const unsigned *>(&As[r][ks + 2 * tq]);
        af[i][1] = *reinterpret_cast<const unsigned *>(&As[r + 8][ks + 2 * tq]);
        af[i][2] = *reinterpret_cast<const unsigned *>(&As[r][ks + 2 * tq + 8]);
        af[i][3] = *reinterpret_cast<const unsigned *>(&As[r + 8][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int r = wn + j * 8 + gq;
        bq[j][0] = *reinterpret_cast<const unsigned *>(&Bs[r][ks + 2 * tq]);
        bq[j][1] = *reinterpret_cast<const unsigned *>(&Bs[r][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bq[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long m = m0 + wm + i * 16 + gq + ((q & 2) ? 8 : 0);
        const int nn = n0 + wn + j * 8 + 2 * tq + (q & 1);
        if (m < M && nn < Nn) epilogue<PASS>(a, m, nn, acc[i][j][q]);
      }
}

// ---------------------------------------------------------------------------
// Forward convolution on the 5th-generation tensor cores (tcgen05), for the
// layers with cin and cout multiples of 16 (cout <= 256): one CTA of 128
// threads computes a 128-pixel x cout tile as one GEMM D = A B^T with
// M = 128 pixels, N = cout, K = 9 cin.  The threads stage the whole K extent
// of A (the shifted input rows, BF16) and of B (the weights, rounded to
// BF16) in shared memory in the canonical no-swizzle K-major layout: 8-row x
// 16-byte core matrices, 128 contiguous bytes each, the K-adjacent ones 128
// bytes apart (leading byte offset) and the next 8 rows K*2 bytes apart
// (stride byte offset).  One elected thread issues the K/16 tcgen05.mma
// instructions (kind::f16, BF16 x BF16 -> FP32) into a TMEM accumulator of
// the CTA and commits them to an mbarrier; every warp then reads its 32
// rows of D from TMEM (tcgen05.ld 32x32b) for the epilogue (bias, ReLU,
// BF16 store).  The wait on the mbarrier is bounded: if it runs out the
// kernel flags the error, waits once more (bounded) for the MMAs it issued,
// frees its TMEM and leaves the tile unwritten.
namespace tc {

constexpr int kM = 128;
constexpr long kWaitLimit = 1L << 24;

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
// shared memory matrix descriptor: start, leading and stride byte offsets
// (>> 4), version 1, no swizzle
__device__ __forceinline__ unsigned long long sdesc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((addr >> 4) & 0x3fffu) | ((unsigned long long)((lbo >> 4) & 0x3fffu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, A and B BF16 and
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr unsigned idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(m >> 4) << 24);
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned phase, long limit) {
  for (long it = 0; it < limit; ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace tc

__global__ void __launch_bounds__(128, 1) k_conv_fwd_tc(ConvArgs a, int ncols, int *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int cin = a.cin, cout = a.cout;
  const int K = 9 * cin, KC = K / 8;
  unsigned char *As = smem;
  unsigned char *Bs = smem + (size_t)tc::kM * K * 2;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(Bs + (size_t)cout * K * 2);
  unsigned *tslot = reinterpret_cast<unsigned *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const long M = (long)a.g.N * a.g.H * a.g.W;
  const long ntile = (M + tc::kM - 1) / tc::kM;

  // TMEM: one warp allocates ncols (a power of two >= 32) columns, kept for
  // every tile of this CTA
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc::smem_u32(tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(tc::smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // B once per CTA: row co = the weights W[co][tap][ci] rounded to BF16
  for (int q = tid; q < cout * KC; q += 128) {
    const int co = q / KC, kc = q - co * KC;
    const float4 *w = reinterpret_cast<const float4 *>(a.w + (size_t)co * K + (size_t)kc * 8);
    const float4 w0 = w[0], w1 = w[1];
    const unsigned off = (unsigned)(co >> 3) * (unsigned)KC * 128u + (unsigned)kc * 128u + (unsigned)(co & 7) * 16u;
    *reinterpret_cast<uint4 *>(Bs + off) =
        make_uint4((unsigned)f2bf(w0.x) | ((unsigned)f2bf(w0.y) << 16), (unsigned)f2bf(w0.z) | ((unsigned)f2bf(w0.w) << 16),
                   (unsigned)f2bf(w1.x) | ((unsigned)f2bf(w1.y) << 16), (unsigned)f2bf(w1.z) | ((unsigned)f2bf(w1.w) << 16));
  }
  const unsigned barad = tc::smem_u32(bar);
  const unsigned rowoff = (unsigned)(tid >> 3) * (unsigned)KC * 128u + (unsigned)(tid & 7) * 16u;
  const unsigned arow = tc::smem_u32(As) + rowoff;
  bool ok = true;
  unsigned phase = 0;
  for (long tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const long m = tile * tc::kM + tid;
    // A: thread tid stages row tid (pixel m): per tap its cin channels as
    // 16-byte asynchronous copies (8 channels each) from x1, then x2, all in
    // flight together
    if (m < M) {
      int n, y, x;
      pix(a.g, m, n, y, x);
      for (int tap = 0; tap < 9; ++tap) {
        const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
        const unsigned short *s1 = a.x1 + a.g.at(n, yy, xx, a.c1);
        for (int c = 0; c < a.c1 / 8; ++c) {
          const int kc = (tap * cin) / 8 + c;
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(arow + (unsigned)kc * 128u), "l"(s1 + 8 * c)
                       : "memory");
        }
        if (a.c2) {
          const unsigned short *s2 = a.x2 + a.g.at(n, yy, xx, a.c2);
          for (int c = 0; c < a.c2 / 8; ++c) {
            const int kc = (tap * cin + a.c1) / 8 + c;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(arow + (unsigned)kc * 128u),
                         "l"(s2 + 8 * c)
                         : "memory");
          }
        }
      }
    } else {
      for (int kc = 0; kc < KC; ++kc) *reinterpret_cast<uint4 *>(As + rowoff + (unsigned)kc * 128u) = make_uint4(0, 0, 0, 0);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    // the stores must be visible to the tensor cores' async proxy
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const unsigned tmem = *tslot;
    if (tid == 0) {
      const unsigned idesc = tc::idesc_bf16(tc::kM, cout);
      const unsigned a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs);
      const unsigned sbo = (unsigned)KC * 128u;
      for (int ks = 0; ks < K / 16; ++ks) {
        const unsigned long long da = tc::sdesc(a0 + (unsigned)ks * 256u, 128u, sbo);
        const unsigned long long db = tc::sdesc(b0 + (unsigned)ks * 256u, 128u, sbo);
        const unsigned acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(barad)
                   : "memory");
    }
    bool done = tc::mbar_wait(barad, phase, tc::kWaitLimit);
    if (!done) {
      atomicExch(err, 1);
      done = tc::mbar_wait(barad, phase, tc::kWaitLimit);
    }
    phase ^= 1u;
    // every warp of the CTA takes the same branch (tcgen05.ld is .aligned)
    ok = __syncthreads_and(done) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (!ok) break;
    // warp w reads rows 32w..32w+31 (lane = its thread), 32 columns a load
    const unsigned tw = tmem + ((unsigned)(warp * 32) << 16);
    for (int c0 = 0; c0 < cout; c0 += 32) {
      unsigned r[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
          "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(tw + (unsigned)c0)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (m < M) {
        int n, y, x;
        pix(a.g, m, n, y, x);
        unsigned short *out = a.y + a.g.at(n, y, x, cout) + c0;
        const int nc = min(32, cout - c0);
#pragma unroll
        for (int j = 0; j < 32; j += 8) {
          if (j >= nc) break;
          unsigned pk[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            float v0 = __uint_as_float(r[j + 2 * e]) + a.bias[c0 + j + 2 * e];
            float v1 = __uint_as_float(r[j + 2 * e + 1]) + a.bias[c0 + j + 2 * e + 1];
            if (a.relu) {
              v0 = fmaxf(v0, 0.f);
              v1 = fmaxf(v1, 0.f);
            }
            pk[e] = (unsigned)f2bf(v0) | ((unsigned)f2bf(v1) << 16);
          }
          *reinterpret_cast<uint4 *>(out + j) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
    // the next tile's MMAs overwrite the accumulator and A: every thread's
    // TMEM reads and A copies of this tile end here
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(*tslot), "r"(ncols) : "memory");
  }
}

// The two thin convolutions of the network, on the CUDA cores with the same
// arithmetic as the tensor-core GEMMs (weights rounded to BF16, BF16
// activations, FP32 accumulation): the first (cin = cin of the network, a
// 9 cin-long K) and the last (cout = 1).  As GEMMs their K or N fills a
// small part of a tensor-core tile.
// first layer: one thread per pixel, all cout outputs (cout <= 64, cin <= 4)
__global__ void k_conv_first(ConvArgs a) {
  extern __shared__ float wsh[];  // [9 cin][cout] rounded weights, then bias
  const int cin = a.cin, cout = a.cout, K = 9 * cin;
  for (int q = threadIdx.x; q < K * cout; q += blockDim.x) {
    const int co = q % cout, k = q / cout;
    wsh[q] = bf2f(f2bf(a.w[(size_t)co * K + k]));
  }
  for (int q = threadIdx.x; q < cout; q += blockDim.x) wsh[K * cout + q] = a.bias[q];
  __syncthreads();
  const long M = (long)a.g.N * a.g.H * a.g.W;
  for (long m = (long)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (long)gridDim.x * blockDim.x) {
    int n, y, x;
    pix(a.g, m, n, y, x);
    float acc[64];
#pragma unroll
    for (int co = 0; co < 64; ++co) acc[co] = 0.f;
    for (int tap = 0; tap < 9; ++tap) {
      const unsigned short *src = a.x1 + a.g.at(n, y + tap / 3 - 1, x + tap % 3 - 1, cin);
      for (int ci = 0; ci < cin; ++ci) {
        const float v = bf2f(src[ci]);
        const float *wr = wsh + (tap * cin + ci) * cout;
#pragma unroll
        for (int co = 0; co < 64; ++co)
          if (co < cout) acc[co] = fmaf(v, wr[co], acc[co]);
      }
    }
    unsigned short *out = a.y + a.g.at(n, y, x, cout);
#pragma unroll
    for (int co = 0; co < 64; ++co) {
      if (co >= cout) break;
      float v = acc[co] + wsh[K * cout + co];
      if (a.relu) v = fmaxf(v, 0.f);
      out[co] = f2bf(v);
    }
  }
}

// last layer: one output channel in FP32, one thread per pixel
__global__ void k_conv_last(ConvArgs a) {
  extern __shared__ float wsh[];  // [9 cin] rounded weights
  const int cin = a.cin, K = 9 * cin;
  for (int q = threadIdx.x; q < K; q += blockDim.x) wsh[q] = bf2f(f2bf(a.w[q]));
  __syncthreads();
  const float b = a.bias[0];
  const long M = (long)a.g.N * a.g.H * a.g.W;
  for (long m = (long)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (long)gridDim.x * blockDim.x) {
    int n, y, x;
    pix(a.g, m, n, y, x);
    float acc = 0.f;
    for (int tap = 0; tap < 9; ++tap) {
      const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
      const float *wr = wsh + tap * cin;
      for (int ci = 0; ci < cin; ++ci) acc = fmaf(act_in(a, n, yy, xx, ci), wr[ci], acc);
    }
    float v = acc + b;
    if (a.relu) v = fmaxf(v, 0.f);
    a.y32[m] = v;
  }
}

// bias gradient: db[co] += sum over pixels of dZ[p][co]
__global__ void k_bias_grad(Img g, const float *dz, int cout, float *db) {
  const long npx = (long)g.N * g.H * g.W;
  const int co = threadIdx.x % cout;
  const int lanes = blockDim.x / cout;  // pixel lanes per block
  const int pl = threadIdx.x / cout;
  if (pl >= lanes) return;
  float s = 0.f;
  for (long m = (long)blockIdx.x * lanes + pl; m < npx; m += (long)gridDim.x * lanes) {
    int n, y, x;
    pix(g, m, n, y, x);
    s += dz[g.at(n, y, x, cout) + co];
  }
  atomicAdd(&db[co], s);
}

// 2 x 2 average pooling of s (H x W) into p (H/2 x W/2), BF16
__global__ void k_pool_fwd(Img gc, const unsigned short *s, unsigned short *p, int C) {
  const long n = (long)gc.N * gc.H * gc.W * C;
  Img gf{gc.N, gc.H * 2, gc.W * 2};
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C);
    int im, y, x;
    pix(gc, t / C, im, y, x);
    const float v = bf2f(s[gf.at(im, 2 * y, 2 * x, C) + c]) + bf2f(s[gf.at(im, 2 * y, 2 * x + 1, C) + c]) +
                    bf2f(s[gf.at(im, 2 * y + 1, 2 * x, C) + c]) + bf2f(s[gf.at(im, 2 * y + 1, 2 * x + 1, C) + c]);
    p[gc.at(im, y, x, C) + c] = f2bf(0.25f * v);
  }
}

// pooling backward: ds (+)= dp[parent] / 4, masked by s > 0
__global__ void k_pool_bwd(Img gf, const float *dp, const unsigned short *s, float *ds, int C, int acc) {
  const long n = (long)gf.N * gf.H * gf.W * C;
  Img gc{gf.N, gf.H / 2, gf.W / 2};
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C);
    int im, y, x;
    pix(gf, t / C, im, y, x);
    const size_t q = gf.at(im, y, x, C) + c;
    float v = 0.25f * dp[gc.at(im, y / 2, x / 2, C) + c];
    if (!(bf2f(s[q]) > 0.f)) v = 0.f;
    ds[q] = acc ? ds[q] + v : v;
  }
}

// nearest upsampling of d (H/2 x W/2) into u (H x W)
__global__ void k_up_fwd(Img gf, const unsigned short *d, unsigned short *u, int C) {
  const long n = (long)gf.N * gf.H * gf.W * C;
  Img gc{gf.N, gf.H / 2, gf.W / 2};
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C);
    int im, y, x;
    pix(gf, t / C, im, y, x);
    u[gf.at(im, y, x, C) + c] = d[gc.at(im, y / 2, x / 2, C) + c];
  }
}

// upsampling backward: dd = sum of the four children's du, masked by d > 0
__global__ void k_up_bwd(Img gc, const float *du, const unsigned short *d, float *dd, int C) {
  const long n = (long)gc.N * gc.H * gc.W * C;
  Img gf{gc.N, gc.H * 2, gc.W * 2};
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C);
    int im, y, x;
    pix(gc, t / C, im, y, x);
    const size_t q = gc.at(im, y, x, C) + c;
    float v = du[gf.at(im, 2 * y, 2 * x, C) + c] + du[gf.at(im, 2 * y, 2 * x + 1, C) + c] +
              du[gf.at(im, 2 * y + 1, 2 * x, C) + c] + du[gf.at(im, 2 * y + 1, 2 * x + 1, C) + c];
    if (!(bf2f(d[q]) > 0.f)) v = 0.f;
    dd[q] = v;
  }
}

// network input: FP32 [n][h][w][cin] (no border) -> BF16 bordered image
__global__ void k_load_input(Img g, const float *x, unsigned short *xb, int C) {
  const long n = (long)g.N * g.H * g.W * C;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C);
    int im, y, xx;
    pix(g, t / C, im, y, xx);
    xb[g.at(im, y, xx, C) + c] = f2bf(x[t]);
  }
}

// mean-square error over the valid hv x wv corner of each image and its
// gradient (bordered, one channel)
__global__ void k_mse(Img g, const float *y, const float *t, int hv, int wv, float *dy, double *loss) {
  const long n = (long)g.N * g.H * g.W;
  const double inv = 1.0 / ((double)g.N * hv * wv);
  double s = 0.0;
  for (long m = blockIdx.x * (long)blockDim.x + threadIdx.x; m < n; m += (long)gridDim.x * blockDim.x) {
    int im, yy, xx;
    pix(g, m, im, yy, xx);
    float d = 0.f;
    if (yy < hv && xx < wv) {
      d = y[m] - t[m];
      s += (double)d * d;
    }
    dy[g.at(im, yy, xx, 1)] = (float)(2.0 * inv) * d;
  }
  s *= inv;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

// Adam (Kingma & Ba), bias-corrected step size computed on the host
__global__ void k_adam(float *w, const float *g, float *m, float *v, long n, float lr_t, float b1, float b2,
                       float eps) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr_t * mi / (sqrtf(vi) + eps);
  }
}

}  // namespace unet
}  // namespace ek

// ---------------------------------------------------------------------------
namespace ek {
using namespace unet;

namespace {
unsigned gsz(long n, int bs) {
  long b = (n + bs - 1) / bs;
  if (b < 1) b = 1;
  if (b > 152L * 64) b = 152L * 64;
  return (unsigned)b;
}
size_t img_bytes(int n, int h, int w, int c, size_t es) { return (size_t)n * (h + 2) * (w + 2) * c * es; }

struct Launcher {
  long &count;
  void check() {
    ++count;
    const cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) throw CudaError(std::string("unet launch: ") + cudaGetErrorString(e));
  }
};
}  // namespace

void *UNet::alloc(size_t bytes, std::vector<void *> &list) {
  void *p = nullptr;
  EK_CUDA(cudaMalloc(&p, bytes));
  list.push_back(p);
  EK_CUDA(cudaMemset(p, 0, bytes));
  return p;
}

UNet::UNet(int cin_, int C_, int max_n_, int h_, int w_) : cin(cin_), C(C_), max_n(max_n_), h(h_), w(w_) {
  if (h < 8 || w < 8 || h % 8 || w % 8 || cin < 1 || C < 1 || C > 64 || max_n < 1)
    throw CudaError("unet: h and w must be multiples of 8, 1 <= C <= 64");
  const int spec[kLayers][4] = {{cin, C, cin, 0},  {C, C, C, 0}, {C, C, C, 0},     {C, C, C, 0}, {C, C, C, 0},
                                {C, C, C, 0},      {C, C, C, 0}, {C, C, C, 0},     {2 * C, C, C, C}, {C, C, C, 0},
                                {2 * C, C, C, C},  {C, C, C, 0}, {2 * C, C, C, C}, {C, C, C, 0}, {C, 1, C, 0}};
  long off = 0;
  for (int l = 0; l < kLayers; ++l) {
    Layer &L = L_[l];
    L.cin = spec[l][0];
    L.cout = spec[l][1];
    L.c1 = spec[l][2];
    L.c2 = spec[l][3];
    L.woff = off;
    L.boff = off + (long)L.cout * 9 * L.cin;
    L.relu = l < kLayers - 1;
    off = L.boff + L.cout;
  }
  nparam_ = off;
  try {
    param_ = (float *)alloc(sizeof(float) * nparam_, bufs_);
    grad_ = (float *)alloc(sizeof(float) * nparam_, bufs_);
    m_ = (float *)alloc(sizeof(float) * nparam_, bufs_);
    v_ = (float *)alloc(sizeof(float) * nparam_, bufs_);
    loss_ = (double *)alloc(sizeof(double), bufs_);
    xin_ = (unsigned short *)alloc(img_bytes(max_n, h, w, cin, 2), bufs_);
    for (int l = 0; l < kLevels; ++l) {
      const int hl = h >> l, wl = w >> l;
      t_[l] = (unsigned short *)alloc(img_bytes(max_n, hl, wl, C, 2), bufs_);
      s_[l] = (unsigned short *)alloc(img_bytes(max_n, hl, wl, C, 2), bufs_);
      if (l >= 1) p_[l] = (unsigned short *)alloc(img_bytes(max_n, hl, wl, C, 2), bufs_);
      if (l <= kLevels - 2) {
        u_[l] = (unsigned short *)alloc(img_bytes(max_n, hl, wl, C, 2), bufs_);
        vv_[l] = (unsigned short *)alloc(img_bytes(max_n, hl, wl, C, 2), bufs_);
        d_[l] = (unsigned short *)alloc(img_bytes(max_n, hl, wl, C, 2), bufs_);
      }
    }
    y_ = (float *)alloc(sizeof(float) * (size_t)max_n * h * w, bufs_);
    tc_err_ = (int *)alloc(sizeof(int), bufs_);
  } catch (...) {
    for (void *p : bufs_) cudaFree(p);
    bufs_.clear();
    throw;
  }
}

UNet::~UNet() {
  for (void *p : gbufs_) cudaFree(p);
  for (void *p : bufs_) cudaFree(p);
}

void UNet::alloc_grads(int n) {
  if (n <= gn_) return;
  for (void *p : gbufs_) cudaFree(p);
  gbufs_.clear();
  gn_ = 0;
  gy_ = (float *)alloc(img_bytes(n, h, w, 1, 4), gbufs_);
  for (int l = 0; l < kLevels; ++l) {
    const int hl = h >> l, wl = w >> l;
    gt_[l] = (float *)alloc(img_bytes(n, hl, wl, C, 4), gbufs_);
    gs_[l] = (float *)alloc(img_bytes(n, hl, wl, C, 4), gbufs_);
    if (l >= 1) gp_[l] = (float *)alloc(img_bytes(n, hl, wl, C, 4), gbufs_);
    if (l <= kLevels - 2) {
      gu_[l] = (float *)alloc(img_bytes(n, hl, wl, C, 4), gbufs_);
      gv_[l] = (float *)alloc(img_bytes(n, hl, wl, C, 4), gbufs_);
      gd_[l] = (float *)alloc(img_bytes(n, hl, wl, C, 4), gbufs_);
    }
  }
  gn_ = n;
}

void UNet::set_params(const float *host) {
  EK_CUDA(cudaMemcpy(param_, host, sizeof(float) * nparam_, cudaMemcpyHostToDevice));
  EK_CUDA(cudaMemset(m_, 0, sizeof(float) * nparam_));
  EK_CUDA(cudaMemset(v_, 0, sizeof(float) * nparam_));
  step_ = 0;
}

void UNet::get_params(float *host) const {
  EK_CUDA(cudaMemcpy(host, param_, sizeof(float) * nparam_, cudaMemcpyDeviceToHost));
}

void UNet::layer_shape(int l, int *ci, int *co) const {
  *ci = L_[l].cin;
  *co = L_[l].cout;
}

double UNet::forward_flops(int n) const {
  double f = 0.0;
  const int lev[kLayers] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
  for (int l = 0; l < kLayers; ++l)
    f += 2.0 * 9.0 * L_[l].cin * L_[l].cout * (double)n * (h >> lev[l]) * (w >> lev[l]);
  return f;
}

void UNet::run_forward(const float *x, int n, float *y, cudaStream_t s) {
  if (n < 1 || n > max_n) throw CudaError("unet: batch outside 1..max_n");
  Launcher K{launches_};
  Img g[kLevels];
  for (int l = 0; l < kLevels; ++l) g[l] = Img{n, h >> l, w >> l};
  auto conv = [&](int l, int lev, const unsigned short *x1, const unsigned short *x2, unsigned short *out,
                  float *out32) {
    const Layer &Ly = L_[l];
    ConvArgs a{};
    a.g = g[lev];
    a.x1 = x1;
    a.x2 = x2;
    a.c1 = Ly.c1;
    a.c2 = Ly.c2;
    a.cin = Ly.cin;
    a.cout = Ly.cout;
    a.w = param_ + Ly.woff;
    a.bias = param_ + Ly.boff;
    a.y = out;
    a.y32 = out32;
    a.relu = Ly.relu;
    const long M = (long)n * a.g.H * a.g.W;
    if (tc_ && !out32 && Ly.cin % 16 == 0 && Ly.c1 % 8 == 0 && Ly.c2 % 8 == 0 && Ly.cout % 16 == 0 &&
        Ly.cout <= 256) {
      const size_t smem = (size_t)(tc::kM + Ly.cout) * 9 * Ly.cin * 2 + 16;
      int ncols = 32;
      while (ncols < Ly.cout) ncols *= 2;
      static bool attr = false;
      if (!attr) {
        EK_CUDA(cudaFuncSetAttribute(k_conv_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
        attr = true;
      }
      if (smem > 220 * 1024) throw CudaError("unet: tcgen05 tile does not fit in shared memory");
      // persistent CTAs: as many as fit on the SMs (by shared memory), each
      // stages the weights once and loops over 128-pixel tiles
      static int nsm = 0;
      if (!nsm) EK_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0));
      const long ntile = (M + tc::kM - 1) / tc::kM;
      const long per_sm = std::max<long>(1, (long)(220 * 1024) / (long)smem);
      const long nblk = std::min<long>(ntile, (long)nsm * per_sm);
      k_conv_fwd_tc<<<(unsigned)nblk, 128, smem, s>>>(a, ncols, tc_err_);
    } else if (tc_ && out32 && Ly.cout == 1 && !Ly.c2) {
      k_conv_last<<<gsz(M, 256), 256, sizeof(float) * 9 * Ly.cin, s>>>(a);
    } else if (tc_ && !out32 && Ly.cin <= 4 && Ly.cout <= 64 && !Ly.c2) {
      k_conv_first<<<gsz(M, 128), 128, sizeof(float) * (9 * Ly.cin + 1) * Ly.cout, s>>>(a);
    } else {
      k_conv_gemm<PASS_FWD><<<dim3((unsigned)((M + BM - 1) / BM), (unsigned)((Ly.cout + BN - 1) / BN)), NT, 0, s>>>(a);
    }
    K.check();
  };
  auto pool = [&](int lev, const unsigned short *src, unsigned short *dst) {
    k_pool_fwd<<<gsz((long)n * g[lev].H * g[lev].W * C, 256), 256, 0, s>>>(g[lev], src, dst, C);
    K.check();
  };
  auto up = [&](int lev, const unsigned short *src, unsigned short *dst) {
    k_up_fwd<<<gsz((long)n * g[lev].H * g[lev].W * C, 256), 256, 0, s>>>(g[lev], src, dst, C);
    K.check();
  };
  k_load_input<<<gsz((long)n * h * w * cin, 256), 256, 0, s>>>(g[0], x, xin_, cin);
  K.check();
  conv(0, 0, xin_, nullptr, t_[0], nullptr);
  conv(1, 0, t_[0], nullptr, s_[0], nullptr);
  for (int l = 1; l < kLevels; ++l) {
    pool(l, s_[l - 1], p_[l]);
    conv(2 * l, l, p_[l], nullptr, t_[l], nullptr);
    conv(2 * l + 1, l, t_[l], nullptr, s_[l], nullptr);
  }
  const unsigned short *below = s_[kLevels - 1];
  for (int l = kLevels - 2; l >= 0; --l) {
    const int li = 8 + 2 * (kLevels - 2 - l);  // 8, 10, 12
    up(l, below, u_[l]);
    conv(li, l, u_[l], s_[l], vv_[l], nullptr);
    conv(li + 1, l, vv_[l], nullptr, d_[l], nullptr);
    below = d_[l];
  }
  conv(kLayers - 1, 0, d_[0], nullptr, nullptr, y);
}

void UNet::forward(const float *x, int n, float *y, cudaStream_t s) { run_forward(x, n, y, s); }

int UNet::tc_error(cudaStream_t s) {
  int v = 0;
  EK_CUDA(cudaMemcpyAsync(&v, tc_err_, sizeof(int), cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaStreamSynchronize(s));
  return v;
}

double UNet::forward_backward(const float *x, const float *t, int n, int hv, int wv, float *y, cudaStream_t s) {
  if (!y) y = y_;
  run_forward(x, n, y, s);
  alloc_grads(n);
  Launcher K{launches_};
  Img g[kLevels];
  for (int l = 0; l < kLevels; ++l) g[l] = Img{n, h >> l, w >> l};
  EK_CUDA(cudaMemsetAsync(grad_, 0, sizeof(float) * nparam_, s));
  EK_CUDA(cudaMemsetAsync(loss_, 0, sizeof(double), s));
  k_mse<<<gsz((long)n * h * w, 256), 256, 0, s>>>(g[0], y, t, hv, wv, gy_, loss_);
  K.check();
  // dW, db and (when dx1 is given) dX of layer l at level lev
  auto back = [&](int l, int lev, const unsigned short *x1, const unsigned short *x2, const float *dz, float *dx1,
                  const unsigned short *m1, float *dx2, const unsigned short *m2) {
    const Layer &Ly = L_[l];
    ConvArgs a{};
    a.g = g[lev];
    a.x1 = x1;
    a.x2 = x2;
    a.c1 = Ly.c1;
    a.c2 = Ly.c2;
    a.cin = Ly.cin;
    a.cout = Ly.cout;
    a.w = param_ + Ly.woff;
    a.dz = dz;
    a.dw = grad_ + Ly.woff;
    const long npx = (long)n * a.g.H * a.g.W;
    // pixels per block of the weight gradient: about 64 partial sums per
    // weight, each added with one FP32 atomic
    long kc = (npx + 63) / 64;
    kc = ((kc + BK - 1) / BK) * BK;
    if (kc < 4 * BK) kc = 4 * BK;
    a.kchunk = (int)kc;
    k_conv_gemm<PASS_DW><<<dim3(1, (unsigned)((9 * Ly.cin + BN - 1) / BN), (unsigned)((npx + kc - 1) / kc)), NT, 0,
                           s>>>(a);
    K.check();
    const int lanes = 256 / Ly.cout;
    const long nbg = std::min((npx + lanes - 1) / lanes, 4L * 152);
    k_bias_grad<<<(unsigned)nbg, 256, 0, s>>>(a.g, dz, Ly.cout, grad_ + Ly.boff);
    K.check();
    if (dx1) {
      a.dx1 = dx1;
      a.dx2 = dx2;
      a.m1 = m1;
      a.m2 = m2;
      k_conv_gemm<PASS_DX><<<dim3((unsigned)((npx + BM - 1) / BM), (unsigned)((Ly.cin + BN - 1) / BN)), NT, 0, s>>>(a);
      K.check();
    }
  };
  back(kLayers - 1, 0, d_[0], nullptr, gy_, gd_[0], d_[0], nullptr, nullptr);
  for (int l = 0; l <= kLevels - 2; ++l) {
    const int li = 8 + 2 * (kLevels - 2 - l);
    back(li + 1, l, vv_[l], nullptr, gd_[l], gv_[l], vv_[l], nullptr, nullptr);
    back(li, l, u_[l], s_[l], gv_[l], gu_[l], nullptr, gs_[l], s_[l]);
    // the upsampling's gradient into the level below (d of the decoder
    // below, or s of the bottleneck)
    float *dst = (l + 1 <= kLevels - 2) ? gd_[l + 1] : gs_[kLevels - 1];
    const unsigned short *msk = (l + 1 <= kLevels - 2) ? d_[l + 1] : s_[kLevels - 1];
    k_up_bwd<<<gsz((long)n * g[l + 1].H * g[l + 1].W * C, 256), 256, 0, s>>>(g[l + 1], gu_[l], msk, dst, C);
    K.check();
  }
  for (int l = kLevels - 1; l >= 1; --l) {
    back(2 * l + 1, l, t_[l], nullptr, gs_[l], gt_[l], t_[l], nullptr, nullptr);
    back(2 * l, l, p_[l], nullptr, gt_[l], gp_[l], nullptr, nullptr, nullptr);
    k_pool_bwd<<<gsz((long)n * g[l - 1].H * g[l - 1].W * C, 256), 256, 0, s>>>(g[l - 1], gp_[l], s_[l - 1],
                                                                                 gs_[l - 1], C, 1);
    K.check();
  }
  back(1, 0, t_[0], nullptr, gs_[0], gt_[0], t_[0], nullptr, nullptr);
  back(0, 0, xin_, nullptr, gt_[0], nullptr, nullptr, nullptr, nullptr);
  double loss = 0.0;
  EK_CUDA(cudaMemcpyAsync(&loss, loss_, sizeof(double), cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaStreamSynchronize(s));
  return loss;
}

double UNet::train_step(const float *x, const float *t, int n, int hv, int wv, double lr, cudaStream_t s) {
  const double loss = forward_backward(x, t, n, hv, wv, nullptr, s);
  ++step_;
  const double b1 = 0.9, b2 = 0.999;
  const double lr_t = lr * std::sqrt(1.0 - std::pow(b2, (double)step_)) / (1.0 - std::pow(b1, (double)step_));
  k_adam<<<gsz(nparam_, 256), 256, 0, s>>>(param_, grad_, m_, v_, nparam_, (float)lr_t, (float)b1, (float)b2, 1e-8f);
  ++launches_;
  const cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) throw CudaError(std::string("unet adam: ") + cudaGetErrorString(e));
  return loss;
}

}  // namespace ek
