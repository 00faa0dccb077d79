// Inputs and outputs of the learned Poisson initial guess.
//
// The network works on a coarser image of each non-singular (kx^2 != 0)
// problem: the finest multigrid grid (K = 0..NZ+1 across, J = 0..NY+1 down,
// problem index fastest in memory) averaged over f x f blocks, padded to a
// multiple of 8 with zeros.  Input channel 0 is the averaged right-hand
// side scaled to unit RMS; channel 1 is log(1 + kx^2 J)/8 with J the block
// average of INT_JACOB, the zero-order coefficient of the problem.  The
// training target is the averaged solution scaled to unit RMS.  The
// prediction comes back to the finest grid by bilinear interpolation; its
// magnitude is set afterwards by the least-squares factor the multigrid
// computes (so the scaling of the training pairs does not matter, and the
// guess never makes the starting residual larger than the right-hand side).
#include <algorithm>
#include <cmath>

#include "ek_internal.h"
#include "ek_unet.h"

namespace ek {
namespace {

struct PoolArgs {
  const double *src;  // [(J*nfx + K)*P + p]
  int P, nfx, nfy, f, h, w, hv, wv;
  const int *idx;     // image q -> problem p
  float *dst;         // dst[((q*h + y)*w + x)*nch + ch]
  int nch, ch;
  double *ss;         // [q]: sum of squares of the averaged values
};

__global__ void k_pool_src(PoolArgs a) {
  const int q = blockIdx.y;
  const int p = a.idx[q];
  float v2 = 0.f;
  const int hw = a.h * a.w;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < hw; t += gridDim.x * blockDim.x) {
    const int yy = t / a.w, xx = t - (t / a.w) * a.w;
    float v = 0.f;
    if (yy < a.hv && xx < a.wv) {
      double s = 0.0;
      int cnt = 0;
      for (int dj = 0; dj < a.f; ++dj) {
        const int J = yy * a.f + dj;
        if (J >= a.nfy) break;
        for (int dk = 0; dk < a.f; ++dk) {
          const int K = xx * a.f + dk;
          if (K >= a.nfx) break;
          s += a.src[((size_t)J * a.nfx + K) * a.P + p];
          ++cnt;
        }
      }
      v = (float)(s / cnt);
    }
    a.dst[((size_t)q * hw + t) * a.nch + a.ch] = v;
    v2 += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) v2 += __shfl_xor_sync(0xffffffffu, v2, o);
  __shared__ float red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v2;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    atomicAdd(&a.ss[q], (double)s);
  }
}

// scale channel ch to unit RMS over the valid pixels; with kx2 given, also
// fill channel ch+1 with log(1 + kx^2 J)/8
__global__ void k_pool_norm(PoolArgs a, const double *kx2, const double *jac, int ldm) {
  const int q = blockIdx.y;
  const int hw = a.h * a.w;
  const double ms = a.ss[q] / ((double)a.hv * a.wv);
  const float inv = ms > 0.0 ? (float)(1.0 / sqrt(ms)) : 0.f;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < hw; t += gridDim.x * blockDim.x) {
    float *d = a.dst + ((size_t)q * hw + t) * a.nch;
    d[a.ch] *= inv;
    if (kx2) {
      const int yy = t / a.w, xx = t - (t / a.w) * a.w;
      float v = 0.f;
      if (yy < a.hv && xx < a.wv) {
        double s = 0.0;
        int cnt = 0;
        for (int dj = 0; dj < a.f; ++dj) {
          const int J = yy * a.f + dj;
          if (J >= a.nfy) break;
          for (int dk = 0; dk < a.f; ++dk) {
            const int K = xx * a.f + dk;
            if (K >= a.nfx) break;
            s += jac[(size_t)J * ldm + K];
            ++cnt;
          }
        }
        v = (float)(0.125 * log1p(kx2[a.idx[q]] * (s / cnt)));
      }
      d[a.ch + 1] = v;
    }
  }
}

// bilinear interpolation of the prediction to the finest grid, written as
// the FP32 part of the float-float iterate: interior rows j = 1..ny and the
// periodic ghost columns i = 0 (copy of nx-1) and nx+1 (copy of 2)
__global__ void k_guess_up(const float *y, int h, int w, int hv, int wv, int f, const int *idx, int nq, int P,
                           int nx, int ny, float *phh) {
  const long n = (long)ny * (nx + 2) * nq;
  const float c = 0.5f * (float)(f - 1), inv = 1.f / (float)f;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int q = (int)(t % nq);
    const long r = t / nq;
    const int i = (int)(r % (nx + 2)), j = 1 + (int)(r / (nx + 2));
    const int is = (i == 0) ? nx - 1 : (i == nx + 1 ? 2 : i);
    const float u = ((float)(is - 1) - c) * inv, v = ((float)(j - 1) - c) * inv;
    const int x0 = min(max((int)floorf(u), 0), wv - 1), y0 = min(max((int)floorf(v), 0), hv - 1);
    const int x1 = min(x0 + 1, wv - 1), y1 = min(y0 + 1, hv - 1);
    const float fx = fminf(fmaxf(u - (float)x0, 0.f), 1.f), fy = fminf(fmaxf(v - (float)y0, 0.f), 1.f);
    const float *Y = y + (size_t)q * h * w;
    const float a0 = Y[y0 * w + x0] + fx * (Y[y0 * w + x1] - Y[y0 * w + x0]);
    const float a1 = Y[y1 * w + x0] + fx * (Y[y1 * w + x1] - Y[y1 * w + x0]);
    phh[((size_t)j * (nx + 2) + i) * P + idx[q]] = a0 + fy * (a1 - a0);
  }
}

unsigned blocks_for(long n, int bs, long cap) {
  long b = (n + bs - 1) / bs;
  return (unsigned)std::max(1L, std::min(b, cap));
}

}  // namespace

void guess_geometry(const Ctx &c, int f, int &h, int &w, int &hv, int &wv) {
  const int nfx = c.mg.nfx, nfy = c.mg.nfy;
  hv = (nfy + f - 1) / f;
  wv = (nfx + f - 1) / f;
  h = (hv + 7) / 8 * 8;
  w = (wv + 7) / 8 * 8;
}

// device buffers for nq images
static void guess_buffers(Ctx &c, int nq) {
  GuessState &G = c.guess;
  if (nq <= G.cap) return;
  for (void *p : {(void *)G.x, (void *)G.y, (void *)G.ss, (void *)G.idx}) cudaFree(p);
  G.x = G.y = nullptr;
  G.ss = nullptr;
  G.idx = nullptr;
  G.cap = 0;
  G.idx_host.clear();
  const size_t hw = (size_t)G.h * G.w;
  EK_CUDA(cudaMalloc(&G.x, sizeof(float) * hw * 2 * nq));
  EK_CUDA(cudaMalloc(&G.y, sizeof(float) * hw * nq));
  EK_CUDA(cudaMalloc(&G.ss, sizeof(double) * 2 * nq));
  EK_CUDA(cudaMalloc(&G.idx, sizeof(int) * nq));
  G.cap = nq;
}

void guess_free(Ctx &c) {
  GuessState &G = c.guess;
  for (void *p : {(void *)G.x, (void *)G.y, (void *)G.ss, (void *)G.idx, (void *)G.alpha}) cudaFree(p);
  G = GuessState{};
}

static void upload_idx(Ctx &c, const std::vector<int> &idx, cudaStream_t s) {
  GuessState &G = c.guess;
  if (G.idx_host == idx) return;
  EK_CUDA(cudaMemcpyAsync(G.idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, s));
  G.idx_host = idx;
}

// averaged, unit-RMS images of src for the problems idx (device list) into
// dst channel ch of nch; with kx2, channel ch+1 gets the kx term
static void pool_images(Ctx &c, const double *src, int P, int f, int h, int w, int hv, int wv, const int *idx, int nq,
                        float *dst, int nch, int ch, double *ss, const double *kx2, cudaStream_t s) {
  PoolArgs a{src, P, c.mg.nfx, c.mg.nfy, f, h, w, hv, wv, idx, dst, nch, ch, ss};
  EK_CUDA(cudaMemsetAsync(ss, 0, sizeof(double) * nq, s));
  const dim3 grid(blocks_for((long)h * w, 256, 64), (unsigned)nq);
  k_pool_src<<<grid, 256, 0, s>>>(a);
  after_launch(c);
  k_pool_norm<<<grid, 256, 0, s>>>(a, kx2, c.m.jac, c.d.LDM);
  after_launch(c);
}

void guess_predict(Ctx &c, int P, const double *rhs, const double *kx2_dev, const std::vector<int> &nonsing,
                   float *phh, cudaStream_t s) {
  GuessState &G = c.guess;
  const int nq = (int)nonsing.size();
  if (nq == 0) return;
  if (nq > G.net->max_n) throw CudaError("learned guess: more problems than the network's batch");
  guess_buffers(c, nq);
  upload_idx(c, nonsing, s);
  pool_images(c, rhs, P, G.factor, G.h, G.w, G.hv, G.wv, G.idx, nq, G.x, 2, 0, G.ss, kx2_dev, s);
  G.net->forward(G.x, nq, G.y, s);
  const long n = (long)c.mg.nfy * (c.mg.nfx + 2) * nq;
  k_guess_up<<<blocks_for(n, 256, 152L * 32), 256, 0, s>>>(G.y, G.h, G.w, G.hv, G.wv, G.factor, G.idx, nq, P,
                                                          c.mg.nfx, c.mg.nfy, phh);
  after_launch(c);
  G.calls++;
}

void guess_collect(Ctx &c, int P, const double *rhs, const double *phi, const double *kx2_dev,
                   const std::vector<double> &kx2_host, cudaStream_t s) {
  GuessState &G = c.guess;
  if (!G.sink_x || G.sink_count >= G.sink_cap) return;
  std::vector<int> nonsing;
  for (int p = 0; p < P && (int)nonsing.size() < G.sink_cap - G.sink_count; ++p)
    if (kx2_host[p] != 0.0) nonsing.push_back(p);
  const int nq = (int)nonsing.size();
  if (nq == 0) return;
  guess_buffers(c, nq);
  upload_idx(c, nonsing, s);
  const size_t hw = (size_t)G.h * G.w;
  float *xd = G.sink_x + hw * 2 * G.sink_count;
  float *td = G.sink_t + hw * G.sink_count;
  pool_images(c, rhs, P, G.factor, G.h, G.w, G.hv, G.wv, G.idx, nq, xd, 2, 0, G.ss, kx2_dev, s);
  pool_images(c, phi, P, G.factor, G.h, G.w, G.hv, G.wv, G.idx, nq, td, 1, 0, G.ss + nq, nullptr, s);
  G.sink_count += nq;
}

}  // namespace ek
