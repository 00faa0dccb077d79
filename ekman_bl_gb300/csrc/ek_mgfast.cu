// Mixed-precision multigrid for the tolerance-driven projection solves.
//
// Same discrete operator as the MUDPACK-exact path (dismd2cr's 9-point
// coefficients, periodic x with MUDPACK's ghost columns, Neumann y), a
// different iteration: FP64 iterative refinement around FP32 V-cycles.
//   r = b - A phi            float-float (~48 bits, FP32 pipe), ||r||, ||b||
//   stop if ||r|| <= tol ||b||
//   A e = r                  one FP32 V(1,1) cycle from e = 0 on MUDPACK's
//                            coarse-level operators, alternating-direction
//                            zebra line Gauss-Seidel smoother, MUDPACK's
//                            full-weighting restriction and cubic prolongation
//   phi = phi + e            float-float; phi is widened to FP64 at the end
// GB300 runs FP32 at ~60x its FP64 rate; with float-float refinement the
// solve never touches the FP64 pipe beyond splitting the rhs and widening
// the result, and reaches relative residuals down to ~1e-13.  On a grid stretched in y the strong coupling is
// along y near the wall and along x far from it; line relaxation in both
// directions smooths both regions, so each cycle cuts the residual ~10x
// where MUDPACK's point smoother (W-cycles) gets ~1.3x.
//
// Problems with kx^2 = 0 are singular (periodic x, Neumann y).  They are
// solved as well-posed problems in the same batch: the right-hand side loses
// its component along the operator's left null vector, the tolerance is the
// same as for every other problem, and the solution has zero mean.  Inside
// the FP32 cycle their coarsest-level correction is shifted to zero mean (a
// constant is in the null space at every level and prolongs to a constant).
#include <algorithm>

#include "ek_internal.h"
#include "ek_unet.h"

namespace ek {

namespace {

struct LvF {
  int nx, ny;
  float *e, *r, *cof, *cp;  // e: (0:nx+1,0:ny+1)xP; r: nx*ny*P; cof: 11*nx*ny; cp: line-solve scratch nx*ny*P
  const float4 *cf4;        // cof packed per point (MgLevelF::cf4), for the level residual
};
struct FastDev {
  int P, ngrid, orth;
  LvF lv[24];
  float *scr;              // finest-size scratch x P (residual / correction)
  double *rhs;              // FP64 finest rhs
  float *phh, *phl;         // float-float finest iterate, with ghosts (buffer 0)
  float *phh2, *phl2;       // buffer 1: problem p's iterate after n corrections is in buffer n & 1
  float *bh, *bl;           // float-float finest rhs
  const float2 *cf2;        // float-float finest coefficients, (hi, lo) interleaved
  int nfx, nfy;
  const double *kx2;
  double *phif;            // output (finest interior, problem fastest)
  double *red;             // 6 per problem: |b|^2, |r|^2, two unused, meas
  int *done, *cycles, *alldone;
  int *iter;               // corrections applied so far
  double tol;
};

__device__ __forceinline__ float &E(const LvF &L, int P, int i, int j, int p) {
  return L.e[((size_t)j * (L.nx + 2) + i) * P + p];
}

// r = b - A phi at the finest level in float-float (about 48 bits, on the
// FP32 pipe); r32 = r; per-problem |b|^2 and |r|^2.  With `update` the
// correction of the cycle just run is applied first, phi' = phi + e (the
// float-float sum), and written to the other iterate buffer, ghosts
// included; r is then the residual of phi'.  The iterate of problem p is in
// buffer cycles[p] & 1 (corrections applied so far).  Block row j = 1..ny,
// lanes over 32 problems; each warp walks a contiguous run of i with the
// values at i-1, i, i+1 of row j kept in registers.
constexpr int kRY = 8;
// (at most 64 registers: four blocks an SM; its loads need the warps)
template <bool UPDATE, bool ORTH>
__global__ void __launch_bounds__(32 * kRY, 4) k_f_resid_ff(FastDev g) {
  if (*g.alldone) return;
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  const int ty = threadIdx.y;
  const int nx = g.nfx, ny = g.nfy, j = 1 + (int)blockIdx.y;
  const size_t npt = (size_t)nx * ny;
  float sb = 0.f, sr = 0.f;
  const bool act = (p < P) && !g.done[p];
  if (act) {
    const int par = g.cycles[p] & 1;
    const float *__restrict__ sh = par ? g.phh2 : g.phh;
    const float *__restrict__ sl = par ? g.phl2 : g.phl;
    float *__restrict__ dh = par ? g.phh : g.phh2;
    float *__restrict__ dl = par ? g.phl : g.phl2;
    const float *__restrict__ ef = g.lv[g.ngrid - 1].e;
    const size_t si = P, sj = (size_t)(nx + 2) * P;
    const FF kx2(g.kx2[p]);
    auto V = [&](size_t q) {
      FF v(sh[q], sl[q]);
      if (UPDATE) v = v + FF(ef[q], 0.f);
      return v;
    };
    const int per = (nx + kRY - 1) / kRY;
    const int i0 = 1 + ty * per, i1 = min(nx, i0 + per - 1);
    const size_t row = (size_t)j * (nx + 2) * P + p;
    FF wm, wc;
    if (i0 <= i1) {
      wm = V(row + (size_t)(i0 - 1) * si);
      wc = V(row + (size_t)i0 * si);
    }
    for (int i = i0; i <= i1; ++i) {
      const size_t pt = (size_t)(j - 1) * nx + (i - 1);
      const size_t q = row + (size_t)i * si;
      auto CF = [&](int l) {
        const float2 v = g.cf2[l * npt + pt];
        return FF(v.x, v.y);
      };
      const FF wp = V(q + si), wn = V(q + sj), ws = V(q - sj);
      FF s = CF(0) * wp;
      if (!ORTH) s = s + CF(1) * V(q + si + sj);
      s = s + CF(2) * wn;
      if (!ORTH) s = s + CF(3) * V(q + sj - si);
      s = s + CF(4) * wm;
      if (!ORTH) s = s + CF(5) * V(q - si - sj);
      s = s + CF(6) * ws;
      if (!ORTH) s = s + CF(7) * V(q + si - sj);
      const FF c9 = ((-kx2 * CF(10)) - CF(8)) + CF(9);
      s = s + c9 * wc;
      const FF b(g.bh[pt * P + p], g.bl[pt * P + p]);
      const FF r = b - s;
      const float r32 = __fadd_rn(r.hi, r.lo);
      sb = fmaf(b.hi, b.hi, sb);
      sr = fmaf(r32, r32, sr);
      g.lv[g.ngrid - 1].r[pt * P + p] = r32;
      if (UPDATE) {
        dh[q] = wc.hi;
        dl[q] = wc.lo;
        if (i == nx - 1) {
          dh[row] = wc.hi;
          dl[row] = wc.lo;
        }
        if (i == 2) {
          dh[row + (size_t)(nx + 1) * si] = wc.hi;
          dl[row + (size_t)(nx + 1) * si] = wc.lo;
        }
      }
      wm = wc;
      wc = wp;
    }
  }
  __shared__ float red[2][kRY][32];
  red[0][ty][threadIdx.x] = sb;
  red[1][ty][threadIdx.x] = sr;
  __syncthreads();
  if (ty == 0 && act) {
    for (int y = 1; y < kRY; ++y) {
      sb += red[0][y][threadIdx.x];
      sr += red[1][y][threadIdx.x];
    }
    atomicAdd(&g.red[6 * p], (double)sb);
    atomicAdd(&g.red[6 * p + 1], (double)sr);
  }
}

// Learned initial guess: after k_f_resid_ff on the unscaled guess g
// (r = b - A g), <r, b> per problem; then the least-squares factor
// alpha = <A g, b> / |A g|^2 = (|b|^2 - <r,b>) / (|b|^2 - 2<r,b> + |r|^2),
// the residual ratio it leaves, |b - alpha A g| / |b|, in red[6p+5], and the
// accumulators cleared for the iteration.
__global__ void __launch_bounds__(32 * kRY) k_f_guess_rb(FastDev g) {
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  const int ty = threadIdx.y;
  const int nx = g.nfx, j = 1 + (int)blockIdx.y;
  const LvF &F = g.lv[g.ngrid - 1];
  float s = 0.f;
  const bool act = (p < P) && !g.done[p];
  if (act)
    for (int i = 1 + ty; i <= nx; i += kRY) {
      const size_t pt = (size_t)(j - 1) * nx + (i - 1);
      s = fmaf(F.r[pt * P + p], g.bh[pt * P + p], s);
    }
  __shared__ float red[kRY][32];
  red[ty][threadIdx.x] = s;
  __syncthreads();
  if (ty == 0 && act) {
    for (int y = 1; y < kRY; ++y) s += red[y][threadIdx.x];
    atomicAdd(&g.red[6 * p + 2], (double)s);
  }
}

__global__ void k_f_guess_alpha(FastDev g, float *alpha) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < g.P; p += gridDim.x * blockDim.x) {
    double a = 0.0;
    if (!g.done[p]) {
      const double bb = g.red[6 * p], rr = g.red[6 * p + 1], rb = g.red[6 * p + 2];
      const double num = bb - rb, den = bb - 2.0 * rb + rr;
      if (den > 0.0) a = num / den;
      const double rho2 = bb > 0.0 ? (bb - a * num) / bb : 0.0;
      g.red[6 * p + 5] = sqrt(fmax(rho2, 0.0));
    }
    alpha[p] = (float)a;
    for (int k = 0; k < 4; ++k) g.red[6 * p + k] = 0.0;
  }
}

__global__ void k_f_guess_scale(FastDev g, const float *alpha) {
  const size_t n = (size_t)(g.nfx + 2) * (g.nfy + 2) * g.P;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    g.phh[t] *= alpha[t % g.P];
}

// float-float rhs from the FP64 one (once per solve)
__global__ void k_f_split(const double *b, float *bh, float *bl, size_t n) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const FF v(b[t]);
    bh[t] = v.hi;
    bl[t] = v.lo;
  }
}

// Decide per problem after a residual; iter = corrections applied so far
// (the device counter plus incr).  A problem within the tolerance is done
// (1); at iter = maxit the rest stop (2); when none is left, alldone.  In a
// captured step graph the block also sets the condition of the while-node
// that repeats the correction cycle: 1 while any problem is active.
__global__ void k_f_check(FastDev g, int maxit, int incr, cudaGraphConditionalHandle cond, int use_cond) {
  if (*g.alldone) {
    if (use_cond && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
    return;
  }
  __shared__ int active;
  const int iter = *g.iter + incr;
  const bool last = iter >= maxit;
  if (threadIdx.x == 0) active = 0;
  __syncthreads();
  for (int p = threadIdx.x; p < g.P; p += blockDim.x) {
    if (g.done[p]) continue;
    g.cycles[p] = iter;
    const double bn = sqrt(g.red[6 * p]);
    const double meas = (bn > 0.0) ? sqrt(g.red[6 * p + 1]) / bn : 0.0;
    const bool conv = meas <= g.tol;
    g.red[6 * p + 4] = meas;
    for (int k = 0; k < 4; ++k) g.red[6 * p + k] = 0.0;
    if (conv) g.done[p] = 1;
    else if (last) g.done[p] = 2;
    else atomicAdd(&active, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *g.iter = iter;
    if (active == 0) *g.alldone = 1;
    if (use_cond) cudaGraphSetConditional(cond, active == 0 ? 0u : 1u);
  }
}

// The solve's statistics on the device (a step run as a graph reads them
// after the step): cycle range, problems stopped at the cap, largest final
// relative residual.  One block.
__global__ void k_f_stats(FastDev g, StepStats *out) {
  __shared__ int smin[256], smax[256], snc[256];
  __shared__ double sres[256];
  int mn = 1 << 30, mx = 0, nc = 0;
  double rs = 0.0;
  for (int p = threadIdx.x; p < g.P; p += blockDim.x) {
    mn = min(mn, g.cycles[p]);
    mx = max(mx, g.cycles[p]);
    nc += (g.done[p] != 1);
    rs = fmax(rs, g.red[6 * p + 4]);
  }
  smin[threadIdx.x] = mn;
  smax[threadIdx.x] = mx;
  snc[threadIdx.x] = nc;
  sres[threadIdx.x] = rs;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      smin[threadIdx.x] = min(smin[threadIdx.x], smin[threadIdx.x + w]);
      smax[threadIdx.x] = max(smax[threadIdx.x], smax[threadIdx.x + w]);
      snc[threadIdx.x] += snc[threadIdx.x + w];
      sres[threadIdx.x] = fmax(sres[threadIdx.x], sres[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out->min_cycles = smin[0];
    out->max_cycles = smax[0];
    out->n_not_converged = snc[0];
    out->nprob = g.P;
    out->max_residual = sres[0];
  }
}

// Line Gauss-Seidel.  The 9-point operator couples each point to its eight
// neighbours; a line solve takes the three couplings along the line into a
// tridiagonal system and the others from current values.  Zebra order: the
// lines of one colour do not couple to each other, so all of them (for all
// problems) are solved in parallel, one thread per (line, problem).
//
// y-line at column i: c7 e(i,j-1) + c9 e(i,j) + c3 e(i,j+1) = r(i,j) - c1 e(i+1,j)
// - c5 e(i-1,j) [- c2, c4, c6, c8 diagonal terms].  Rows j = 1 and ny have
// c7 = 0 and c3 = 0 after MUDPACK's Neumann folding.  c' is kept in cp, d'
// overwrites e until the back substitution.
constexpr int kChunk = 8;
// zero_nbr: the neighbouring lines hold zero (the first sweep of a cycle
// from e = 0), so their terms are left out and their stale values unread
__device__ __forceinline__ void yline_solve(const LvF &L, int P, int p, int i, float kx2, bool orth,
                                            bool zero_nbr = false) {
  const int nx = L.nx, ny = L.ny;
  const size_t npt = (size_t)nx * ny;
  const size_t si = P, sj = (size_t)(nx + 2) * P;
  const float *cf = L.cof;
  float cprev = 0.f, dprev = 0.f;
  // forward elimination, kChunk rows at a time: every load of a chunk is
  // issued before the recurrence consumes it
  for (int j0 = 1; j0 <= ny; j0 += kChunk) {
    float dv[kChunk], av[kChunk], bv[kChunk], cv[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int j = j0 + u;
      if (j > ny) break;
      const size_t pt = (size_t)(j - 1) * nx + (i - 1);
      const float *ep = &L.e[((size_t)j * (nx + 2) + i) * P + p];
      float d = L.r[pt * P + p];
      if (!zero_nbr) {
        d = d - cf[pt] * ep[si] - cf[4 * npt + pt] * ep[-(long)si];
        if (orth == false)
          d = d - cf[npt + pt] * ep[si + sj] - cf[3 * npt + pt] * ep[sj - si] -
              cf[5 * npt + pt] * ep[-(long)(si + sj)] - cf[7 * npt + pt] * ep[si - sj];
      }
      dv[u] = d;
      av[u] = cf[6 * npt + pt];
      cv[u] = cf[2 * npt + pt];
      bv[u] = ((-kx2 * cf[10 * npt + pt]) - cf[8 * npt + pt]) + cf[9 * npt + pt];
    }
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int j = j0 + u;
      if (j > ny) break;
      const size_t pt = (size_t)(j - 1) * nx + (i - 1);
      const float m = 1.f / (bv[u] - av[u] * cprev);
      cprev = cv[u] * m;
      dprev = (dv[u] - av[u] * dprev) * m;
      L.cp[pt * P + p] = cprev;
      L.e[((size_t)j * (nx + 2) + i) * P + p] = dprev;
    }
  }
  // back substitution; periodic ghosts written together with their sources
  float x = 0.f;
  for (int j0 = ny; j0 >= 1; j0 -= kChunk) {
    float dv[kChunk], cv[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int j = j0 - u;
      if (j < 1) break;
      const size_t pt = (size_t)(j - 1) * nx + (i - 1);
      dv[u] = L.e[((size_t)j * (nx + 2) + i) * P + p];
      cv[u] = L.cp[pt * P + p];
    }
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int j = j0 - u;
      if (j < 1) break;
      x = dv[u] - cv[u] * x;
      L.e[((size_t)j * (nx + 2) + i) * P + p] = x;
      if (i == nx - 1) E(L, P, 0, j, p) = x;
      if (i == 2) E(L, P, nx + 1, j, p) = x;
    }
  }
}

// x-line at row j: c5 e(i-1,j) + c9 e(i,j) + c1 e(i+1,j) = r(i,j) - c3 e(i,j+1)
// - c7 e(i,j-1) [- diagonal terms].  The periodic wrap couplings (i = 1 to
// the ghost e(0) = e(nx-1), i = nx to the ghost e(nx+1) = e(2)) are taken
// from the ghosts' current values, so the line system stays tridiagonal.
__device__ __forceinline__ void xline_solve(const LvF &L, int P, int p, int j, float kx2, bool orth) {
  const int nx = L.nx, ny = L.ny;
  const size_t npt = (size_t)nx * ny;
  const size_t si = P, sj = (size_t)(nx + 2) * P;
  const float *cf = L.cof;
  float *erow = &L.e[(size_t)j * (nx + 2) * P + p];  // erow[i * P] = e(i, j)
  float *cprow = &L.cp[(size_t)(j - 1) * nx * P + p];  // cprow[(i-1) * P]
  const size_t rb = (size_t)(j - 1) * nx;
  const float g0 = erow[0], g1 = erow[(size_t)(nx + 1) * si];
  float cprev = 0.f, dprev = 0.f;
  for (int i0 = 1; i0 <= nx; i0 += kChunk) {
    float dv[kChunk], av[kChunk], bv[kChunk], cv[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int i = i0 + u;
      if (i > nx) break;
      const size_t pt = rb + (i - 1);
      const float *ep = erow + (size_t)i * si;
      float d = L.r[pt * P + p] - cf[2 * npt + pt] * ep[sj] - cf[6 * npt + pt] * ep[-(long)sj];
      if (orth == false)
        d = d - cf[npt + pt] * ep[si + sj] - cf[3 * npt + pt] * ep[sj - si] - cf[5 * npt + pt] * ep[-(long)(si + sj)] -
            cf[7 * npt + pt] * ep[si - sj];
      float a = cf[4 * npt + pt], c = cf[pt];
      if (i == 1) { d -= a * g0; a = 0.f; }
      if (i == nx) { d -= c * g1; c = 0.f; }
      dv[u] = d;
      av[u] = a;
      cv[u] = c;
      bv[u] = ((-kx2 * cf[10 * npt + pt]) - cf[8 * npt + pt]) + cf[9 * npt + pt];
    }
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int i = i0 + u;
      if (i > nx) break;
      const float m = 1.f / (bv[u] - av[u] * cprev);
      cprev = cv[u] * m;
      dprev = (dv[u] - av[u] * dprev) * m;
      cprow[(size_t)(i - 1) * si] = cprev;
      erow[(size_t)i * si] = dprev;
    }
  }
  float x = 0.f;
  for (int i0 = nx; i0 >= 1; i0 -= kChunk) {
    float dv[kChunk], cv[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int i = i0 - u;
      if (i < 1) break;
      dv[u] = erow[(size_t)i * si];
      cv[u] = cprow[(size_t)(i - 1) * si];
    }
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int i = i0 - u;
      if (i < 1) break;
      x = dv[u] - cv[u] * x;
      erow[(size_t)i * si] = x;
      if (i == nx - 1) erow[0] = x;
      if (i == 2) erow[(size_t)(nx + 1) * si] = x;
    }
  }
}

// y-lines i = i0, i0+istep, ... (ncol of them), all problems
__global__ void __launch_bounds__(64) k_f_yline(FastDev g, int level, int i0, int istep, int ncol, int zero_nbr) {
  if (*g.alldone) return;
  const LvF L = g.lv[level - 1];
  const int P = g.P;
  const long n = (long)ncol * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    if (g.done[p]) continue;
    yline_solve(L, P, p, i0 + istep * (int)(t / P), (float)g.kx2[p], g.orth != 0, zero_nbr != 0);
  }
}

// x-lines j = j0, j0+2, ... (nrow of them), all problems
__global__ void __launch_bounds__(64) k_f_xline(FastDev g, int level, int j0, int nrow) {
  if (*g.alldone) return;
  const LvF L = g.lv[level - 1];
  const int P = g.P;
  const long n = (long)nrow * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    if (g.done[p]) continue;
    xline_solve(L, P, p, j0 + 2 * (int)(t / P), (float)g.kx2[p], g.orth != 0);
  }
}

// Partitioned line solve: one block per (line, LANES problems), lanes over
// the problems (coalesced, the layout is problem fastest), threadIdx.y over K
// segments of the line.  The line's n rows are K segments of <= SEG interior
// rows separated by K-1 separator rows.  Each thread row eliminates its
// segment in registers, expressing every row as x = delta + gamma X0 -
// beta x(next) with X0, X1 the separators before and after it; the first and
// last rows in terms of (X0, X1) give a tridiagonal system for the
// separators, solved from shared memory by parallel cyclic reduction (one
// thread row per separator, log2(K) combine steps); then every segment
// back-substitutes.
// XL: x-line (along i, the periodic wrap couplings taken from the ghosts'
// current values); else y-line (along j).
enum { SH_A, SH_B, SH_C, SH_D, SH_YF, SH_VF, SH_WF, SH_YL, SH_VL, SH_WL, SH_S, SH_N };
// 4-row segments are capped at 48 registers, so that two or three blocks
// share an SM (their per-thread arrays are half as large)
template <bool XL, bool ORTH, int LANES, int SEG>
// zero_e: the first sweep of a cycle from e = 0 (y-lines only): the
// neighbouring lines' terms are left out and their stale values unread.
__global__ void __launch_bounds__(1024) __maxnreg__(SEG == 4 ? 48 : 64) k_f_pline(FastDev g, int level, int l0, int lstep, int mb, int me, int zero_e) {
  constexpr int kSegMax = SEG;
  if (*g.alldone) return;
  extern __shared__ float sh[];
  const int K = blockDim.y;
  auto S = [&](int arr, int seg) -> float & { return sh[(arr * K + seg) * LANES + threadIdx.x]; };
  const LvF L = g.lv[level - 1];
  const int P = g.P;
  const int nx = L.nx, ny = L.ny;
  const int s = threadIdx.y;
  const int p = blockIdx.y * LANES + threadIdx.x;
  const bool act = (p < P) && !g.done[p];
  if (!__syncthreads_or(act)) return;  // every problem of the block converged
  const int pp = act ? p : 0;
  const int line = l0 + lstep * (int)blockIdx.x;
  const int m = mb + (s < me ? 1 : 0);
  const int lo = 1 + s * (mb + 1) + min(s, me);
  // 32-bit offsets: the host checks that (nx+2)(ny+2)P and 11 nx ny fit
  const unsigned npt = (unsigned)nx * (unsigned)ny;
  const unsigned si = (unsigned)P, sj = (unsigned)(nx + 2) * (unsigned)P;
  const float kx2 = (float)g.kx2[pp];
  const float *cf = L.cof;
  // row k of the line: a x(k-1) + b x(k) + c x(k+1) = d
  auto row = [&](int k, float &a, float &b, float &c, float &d) {
    const int i = XL ? k : line, j = XL ? line : k;
    const unsigned pt = (unsigned)((j - 1) * nx + (i - 1));
    const float *ep = L.e + ((unsigned)(j * (nx + 2) + i) * si + (unsigned)pp);
    const float *cp = cf + pt;
    b = ((-kx2 * cp[10 * npt]) - cp[8 * npt]) + cp[9 * npt];
    float dd = L.r[pt * si + (unsigned)pp];
    if (XL) {
      a = cp[4 * npt];
      c = cp[0];
      dd = dd - cp[2 * npt] * ep[sj] - cp[6 * npt] * *(ep - sj);
    } else {
      a = cp[6 * npt];
      c = cp[2 * npt];
      if (!zero_e) dd = dd - cp[0] * ep[si] - cp[4 * npt] * *(ep - si);
    }
    if (!ORTH && !zero_e)
      dd = dd - cp[npt] * ep[si + sj] - cp[3 * npt] * ep[sj - si] - cp[5 * npt] * *(ep - (si + sj)) -
           cp[7 * npt] * *(ep - (sj - si));
    d = dd;
  };
  auto store = [&](int k, float x) {
    const int i = XL ? k : line, j = XL ? line : k;
    float *erow = L.e + (unsigned)(j * (nx + 2)) * si + (unsigned)p;
    erow[(unsigned)i * si] = x;
    if (i == nx - 1) erow[0] = x;
    if (i == 2) erow[(unsigned)(nx + 1) * si] = x;
  };
  // phase 1: every load of the segment (rows past its end repeat its last
  // row, so all addresses are valid and no load waits on arithmetic)
  float av[kSegMax], bv[kSegMax], cv[kSegMax], dv[kSegMax];
#pragma unroll
  for (int u = 0; u < kSegMax; ++u) row(lo + min(u, m - 1), av[u], bv[u], cv[u], dv[u]);
  if (XL) {
    // the periodic wrap of an x-line: i = 1 couples to the ghost e(0) =
    // e(nx-1), i = nx to e(nx+1) = e(2), both taken from current values
    const float *erow = L.e + (unsigned)(line * (nx + 2)) * si + (unsigned)pp;
    if (s == 0) {
      dv[0] -= av[0] * erow[0];
      av[0] = 0.f;
    }
    if (s == K - 1) {
      const float gh = erow[(unsigned)(nx + 1) * si];
#pragma unroll
      for (int u = 0; u < kSegMax; ++u) {
        const bool hit = (u == m - 1);
        dv[u] = hit ? dv[u] - cv[u] * gh : dv[u];
        cv[u] = hit ? 0.f : cv[u];
      }
    }
  }
  // phase 2: elimination in place: cv <- beta, dv <- delta, av <- gamma, where
  // row u of the segment is x = delta + gamma X0 - beta x(next)
  float yl = 0.f, vl = 0.f, wl = 0.f;
  {
    float bprev = 0.f, dprev = 0.f, gprev = 1.f;
#pragma unroll
    for (int u = 0; u < kSegMax; ++u) {
      const float inv = __fdividef(1.f, bv[u] - av[u] * bprev);
      bprev = cv[u] * inv;
      dprev = (dv[u] - av[u] * dprev) * inv;
      gprev = -av[u] * gprev * inv;
      cv[u] = bprev;
      dv[u] = dprev;
      av[u] = gprev;
      const bool last = (u == m - 1);
      yl = last ? dprev : yl;
      vl = last ? gprev : vl;
      wl = last ? -bprev : wl;
    }
  }
  float yf = yl, vf = vl, wf = wl;
#pragma unroll
  for (int u = kSegMax - 2; u >= 0; --u)
    if (u < m - 1) {
      yf = dv[u] - cv[u] * yf;
      vf = av[u] - cv[u] * vf;
      wf = -cv[u] * wf;
    }
  S(SH_YF, s) = yf; S(SH_VF, s) = vf; S(SH_WF, s) = wf;
  S(SH_YL, s) = yl; S(SH_VL, s) = vl; S(SH_WL, s) = wl;
  if (s < K - 1) {
    float a, b, c, d;
    row(lo + m, a, b, c, d);
    S(SH_A, s) = a; S(SH_B, s) = b; S(SH_C, s) = c; S(SH_D, s) = d;
  }
  __syncthreads();
  // the K-1 separator unknowns, A S(t-1) + B S(t) + C S(t+1) = D, by
  // parallel cyclic reduction: thread row t owns separator t; after the
  // steps of stride 1, 2, 4, ... each row couples to nothing and S(t) = D/B
  const int nsep = K - 1;
  float eA = 0.f, eB = 1.f, eC = 0.f, eD = 0.f;
  if (s < nsep) {
    const float a = S(SH_A, s), c = S(SH_C, s);
    eA = (s > 0) ? a * S(SH_VL, s) : 0.f;
    eB = S(SH_B, s) + a * S(SH_WL, s) + c * S(SH_VF, s + 1);
    eC = (s < nsep - 1) ? c * S(SH_WF, s + 1) : 0.f;
    eD = S(SH_D, s) - a * S(SH_YL, s) - c * S(SH_YF, s + 1);
  }
  for (int d = 1; d < nsep; d <<= 1) {
    __syncthreads();
    if (s < nsep) {
      S(SH_A, s) = eA;
      S(SH_B, s) = eB;
      S(SH_C, s) = eC;
      S(SH_D, s) = eD;
    }
    __syncthreads();
    if (s < nsep) {
      float nA = 0.f, nC = 0.f, nB = eB, nD = eD;
      if (s - d >= 0) {
        const float al = __fdividef(eA, S(SH_B, s - d));
        nA = -al * S(SH_A, s - d);
        nB -= al * S(SH_C, s - d);
        nD -= al * S(SH_D, s - d);
      }
      if (s + d < nsep) {
        const float ga = __fdividef(eC, S(SH_B, s + d));
        nC = -ga * S(SH_C, s + d);
        nB -= ga * S(SH_A, s + d);
        nD -= ga * S(SH_D, s + d);
      }
      eA = nA;
      eB = nB;
      eC = nC;
      eD = nD;
    }
  }
  if (s < nsep) S(SH_S, s) = __fdividef(eD, eB);
  __syncthreads();
  if (!act) return;
  const float X0 = (s > 0) ? S(SH_S, s - 1) : 0.f;
  const float X1 = (s < K - 1) ? S(SH_S, s) : 0.f;
  float x = 0.f;
#pragma unroll
  for (int u = kSegMax - 1; u >= 0; --u)
    if (u < m) {
      x = dv[u] + av[u] * X0 - cv[u] * ((u == m - 1) ? X1 : x);
      store(lo + u, x);
    }
  if (s < K - 1) store(lo + m, X1);
}

struct LinePhase {
  int i0, istep, ncol;
};
// y-line colour col (1, 2) of a level with nx columns as one or two ordered
// phases.  With nx odd the colours are odd and even i.  With nx even (only
// possible on the coarsest level) the periodic wrap couples i = 1 to
// i = nx-1 and i = nx to i = 2, so i = 1 and i = nx go in phases of their own.
__host__ __device__ inline int line_phases(int nx, int col, LinePhase *ph) {
  if (nx % 2 == 1) {
    ph[0] = (col == 1) ? LinePhase{1, 2, (nx + 1) / 2} : LinePhase{2, 2, (nx - 1) / 2};
    return 1;
  }
  if (col == 1) {
    ph[0] = LinePhase{3, 2, nx / 2 - 1};
    ph[1] = LinePhase{1, 1, 1};
  } else {
    ph[0] = LinePhase{2, 2, nx / 2 - 1};
    ph[1] = LinePhase{nx, 1, 1};
  }
  return 2;
}

// The coarsest level: `sweeps` alternating-direction sweeps, one thread per
// problem (the level has a few tens of points), in the same order as the
// per-line kernels use.
__global__ void k_f_coarsest(FastDev g, int sweeps) {
  if (*g.alldone) return;
  const LvF L = g.lv[0];
  const int P = g.P;
  const bool orth = g.orth != 0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    if (g.done[p]) continue;
    const float kx2 = (float)g.kx2[p];
    for (int sw = 0; sw < sweeps; ++sw) {
      for (int col = 1; col <= 2; ++col) {
        LinePhase ph[2];
        const int nph = line_phases(L.nx, col, ph);
        for (int q = 0; q < nph; ++q)
          for (int c = 0; c < ph[q].ncol; ++c) yline_solve(L, P, p, ph[q].i0 + ph[q].istep * c, kx2, orth);
      }
      for (int col = 1; col <= 2; ++col)
        for (int j = col; j <= L.ny; j += 2) xline_solve(L, P, p, j, kx2, orth);
    }
    if (kx2 == 0.f) {
      // singular: keep the correction at zero mean, ghosts included
      float m = 0.f;
      for (int j = 1; j <= L.ny; ++j)
        for (int i = 1; i <= L.nx; ++i) m += E(L, P, i, j, p);
      m = m / (float)(L.nx * L.ny);
      for (int j = 1; j <= L.ny; ++j)
        for (int i = 0; i <= L.nx + 1; ++i) E(L, P, i, j, p) -= m;
    }
  }
}

// The elementwise multigrid kernels below use one block per grid row (or
// coarse row) and 32 problems: lanes over the problems (coalesced, the
// layout is problem fastest), the block's warps striding along the row.  No
// index needs a division.
constexpr int kRowWarps = 8;

// The level operations below act on one point of one problem: arrays with
// the problem index fastest (stride P, problem p), as the batched kernels
// keep them in global memory, or P = 1, p = 0 for one problem's arrays in
// shared memory (k_f_vtail).  One definition serves both, so a level gives
// the same numbers in either.

// residual of the correction equation at point (i, j) of a level (FP32)
__device__ __forceinline__ void f_resid_at(const float *__restrict__ cf, const float *__restrict__ ee,
                                           const float *__restrict__ rr, float *__restrict__ scr, int nx, int ny,
                                           int P, int p, int i, int j, float kx2, bool orth) {
  const size_t npt = (size_t)nx * ny;
  const size_t si = P, sj = (size_t)(nx + 2) * P;
  const size_t pt = (size_t)(j - 1) * nx + (i - 1);
  const float *ep = &ee[((size_t)j * (nx + 2) + i) * P + p];
  float s = cf[pt] * ep[si] + cf[2 * npt + pt] * ep[sj] + cf[4 * npt + pt] * ep[-(long)si] +
            cf[6 * npt + pt] * ep[-(long)sj];
  if (!orth)
    s += cf[npt + pt] * ep[si + sj] + cf[3 * npt + pt] * ep[sj - si] + cf[5 * npt + pt] * ep[-(long)(si + sj)] +
         cf[7 * npt + pt] * ep[si - sj];
  const float c9 = ((-kx2 * cf[10 * npt + pt]) - cf[8 * npt + pt]) + cf[9 * npt + pt];
  s += c9 * ep[0];
  scr[((size_t)j * (nx + 2) + i) * P + p] = rr[pt * P + p] - s;
}

// full weighting (res2, mudcom.f:120-257) of the fine residual in scr to the
// coarse rhs at (ic, jc), and e_coarse = 0 there (ghosts included: ic =
// 0..ncx+1, jc = 0..ncy+1)
__device__ __forceinline__ void f_restrict_at(const float *__restrict__ scr, float *__restrict__ ce,
                                              float *__restrict__ cr, int nx, int ny, int ncx, int ncy, int P, int p,
                                              int ic, int jc) {
  const int ix = (ncx == nx) ? 0 : 1, jy = (ncy == ny) ? 0 : 1;
  ce[((size_t)jc * (ncx + 2) + ic) * P + p] = 0.f;
  if (ic < 1 || ic > ncx || jc < 1 || jc > ncy) return;
  const int i = ic + ix * (ic - 1), j = jc + jy * (jc - 1);
  int im1 = i - 1, ip1 = i + 1, jm1 = j - 1, jp1 = j + 1;
  if (ic == 1 || ic == ncx) {
    im1 = max(i - 1, 2);
    ip1 = min(i + 1, nx - 1);
    if (i == 1) im1 = nx - 1;
    if (i == nx) ip1 = 2;
  }
  if (jc == 1 || jc == ncy) {
    jm1 = max(j - 1, 2);
    jp1 = min(j + 1, ny - 1);
  }
  auto R = [&](int a, int b) { return scr[((size_t)b * (nx + 2) + a) * P + p]; };
  cr[((size_t)(jc - 1) * ncx + (ic - 1)) * P + p] =
      (R(im1, jm1) + R(ip1, jm1) + R(im1, jp1) + R(ip1, jp1) + 2.f * (R(im1, j) + R(ip1, j) + R(i, jm1) + R(i, jp1)) +
       4.f * R(i, j)) * .0625f;
}

// the same residual from the packed coefficients (the same products and
// sums, in the same order): two or three vector loads for seven or eleven
// scalar ones
__device__ __forceinline__ void f_resid_at4(const float4 *__restrict__ cf4, const float *__restrict__ ee,
                                            const float *__restrict__ rr, float *__restrict__ scr, int nx, int P,
                                            int p, int i, int j, float kx2, bool orth) {
  const size_t si = P, sj = (size_t)(nx + 2) * P;
  const size_t pt = (size_t)(j - 1) * nx + (i - 1);
  const float *ep = &ee[((size_t)j * (nx + 2) + i) * P + p];
  const float4 q0 = cf4[3 * pt], q1 = cf4[3 * pt + 1];
  float s = q0.x * ep[si] + q0.y * ep[sj] + q0.z * ep[-(long)si] + q0.w * ep[-(long)sj];
  if (!orth) {
    const float4 q2 = cf4[3 * pt + 2];
    s += q2.x * ep[si + sj] + q2.y * ep[sj - si] + q2.z * ep[-(long)(si + sj)] + q2.w * ep[si - sj];
  }
  const float c9 = ((-kx2 * q1.z) - q1.x) + q1.y;
  s += c9 * ep[0];
  scr[((size_t)j * (nx + 2) + i) * P + p] = rr[pt * P + p] - s;
}

// residual of the correction equation at a level (FP32) into the scratch
__global__ void __launch_bounds__(32 * kRowWarps) k_f_resid32(FastDev g, int level) {
  if (*g.alldone) return;
  const LvF L = g.lv[level - 1];
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  if (p >= P || g.done[p]) return;
  const int nx = L.nx, j = 1 + (int)blockIdx.y;
  const float kx2 = (float)g.kx2[p];
  const bool orth = g.orth != 0;
#pragma unroll 4
  for (int i = 1 + (int)threadIdx.y; i <= nx; i += kRowWarps)
    f_resid_at4(L.cf4, L.e, L.r, g.scr, nx, P, p, i, j, kx2, orth);
}

// full weighting (res2, mudcom.f:120-257) to the coarse rhs; e_coarse = 0
// (block row jc = 0..ncy+1, ghosts included)
__global__ void __launch_bounds__(32 * kRowWarps) k_f_restrict(FastDev g, int level) {
  if (*g.alldone) return;
  const LvF F = g.lv[level - 1], C = g.lv[level - 2];
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  if (p >= P || g.done[p]) return;
  const int jc = (int)blockIdx.y;
#pragma unroll 4
  for (int ic = (int)threadIdx.y; ic <= C.nx + 1; ic += kRowWarps)
    f_restrict_at(g.scr, C.e, C.r, F.nx, F.ny, C.nx, C.ny, P, p, ic, jc);
}

// cubic/linear prolongation (prolon1/prolon2, mudcom.f:261-499) of the
// coarse correction, stage 1: rows given directly by prolon1, into scratch
template <typename F>
__device__ __forceinline__ float prolon1f(int i, int ncx, int nx, bool cubic, F p) {
  if (ncx == nx) return p(i);
  if (!cubic) {
    if (i & 1) return p((i + 1) / 2);
    return 0.5f * (p(i / 2) + p(i / 2 + 1));
  }
  auto q = [&](int ii) { return p((ii + 1) / 2); };
  if (i & 1) return q(i);
  if (i >= 4 && i <= nx - 3) return (-q(i - 3) + 9.f * (q(i - 1) + q(i + 1)) - q(i + 3)) * .0625f;
  if (i == 2) return (-q(nx - 2) + 9.f * (q(1) + q(3)) - q(5)) * .0625f;
  return (-q(nx - 4) + 9.f * (q(nx - 2) + q(nx)) - q(3)) * .0625f;
}

// fine row j = 2 rr + 1 (y coarsened) or rr + 1, point i: stage 1 into scr
__device__ __forceinline__ void f_prolong_x_at(const float *__restrict__ ce, float *__restrict__ scr, int nx, int ny,
                                               int ncx, int ncy, int P, int p, int i, int rr) {
  const bool ycoarse = ncy < ny;
  const bool cubic = ncx >= 4;
  const int j = ycoarse ? 2 * rr + 1 : rr + 1;
  const int jc = ycoarse ? j / 2 + 1 : j;
  auto pc = [&](int ic) { return ce[((size_t)jc * (ncx + 2) + ic) * P + p]; };
  scr[((size_t)j * (nx + 2) + i) * P + p] = prolon1f(i, ncx, nx, cubic, pc);
}

// stage 2 at fine point (i, j): the rows between (cubic or linear in y), then
// e += correction, with the periodic ghosts written together with their
// sources
__device__ __forceinline__ void f_prolong_y_at(const float *__restrict__ scr, float *__restrict__ ef, int nx, int ny,
                                               int ncy, int P, int p, int i, int j) {
  const bool ycoarse = ncy < ny;
  const bool cubic = ncy >= 4;
  const size_t rowj = (size_t)j * (nx + 2) * P + p;
  auto Q = [&](int jj) { return scr[((size_t)jj * (nx + 2) + i) * P + p]; };
  float v;
  if (ycoarse && !(j & 1)) {
    if (!cubic) v = 0.5f * (Q(j - 1) + Q(j + 1));
    else if (j >= 4 && j <= ny - 3) v = (-Q(j - 3) + 9.f * (Q(j - 1) + Q(j + 1)) - Q(j + 3)) * .0625f;
    else if (j == 2) v = (5.f * Q(1) + 15.f * Q(3) - 5.f * Q(5) + Q(7)) * .0625f;
    else v = (5.f * Q(ny) + 15.f * Q(ny - 2) - 5.f * Q(ny - 4) + Q(ny - 6)) * .0625f;
  } else {
    v = Q(j);
  }
  const float ne = ef[rowj + (size_t)i * P] + v;
  ef[rowj + (size_t)i * P] = ne;
  if (i == nx - 1) ef[rowj] = ne;
  if (i == 2) ef[rowj + (size_t)(nx + 1) * P] = ne;
}

// block row rr: fine row j = 2 rr + 1 (y coarsened) or rr + 1
__global__ void __launch_bounds__(32 * kRowWarps) k_f_prolong_x(FastDev g, int level) {
  if (*g.alldone) return;
  const LvF F = g.lv[level - 1], C = g.lv[level - 2];
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  if (p >= P || g.done[p]) return;
  const int rr = (int)blockIdx.y;
#pragma unroll 4
  for (int i = 1 + (int)threadIdx.y; i <= F.nx; i += kRowWarps) f_prolong_x_at(C.e, g.scr, F.nx, F.ny, C.nx, C.ny, P, p, i, rr);
}

// block row j - 1
__global__ void __launch_bounds__(32 * kRowWarps) k_f_prolong_y(FastDev g, int level) {
  if (*g.alldone) return;
  const LvF F = g.lv[level - 1], C = g.lv[level - 2];
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  if (p >= P || g.done[p]) return;
  const int j = 1 + (int)blockIdx.y;
#pragma unroll 4
  for (int i = 1 + (int)threadIdx.y; i <= F.nx; i += kRowWarps) f_prolong_y_at(g.scr, F.e, F.nx, F.ny, C.ny, P, p, i, j);
}

// The coarse end of a V(1,1) cycle in one launch: levels ltop, ltop-1, ..., 1
// of one problem per block, with the level arrays in shared memory and the
// (problem-independent) coefficients read through L1.  Each level down: the
// pre-smoothing sweep, the residual, the restriction; the coarsest level's
// `sweeps` alternating sweeps (and, for kx^2 = 0, its zero-mean shift); each
// level up: the prolongation and the post-smoothing sweep -- the operations
// and order of the per-level launches, with every line solved by one thread
// (lines of one colour are independent).  On the coarse levels a per-level
// launch does a few microseconds of work behind a launch and a grid-wide
// dependency; here the levels follow each other behind block barriers.
//
// A line's Thomas factors (m = 1 / (b - a c'), c' = c m, per row) depend on
// the problem's kx^2 and the level coefficients only, so k_f_tail_factors
// computes them once per solve; a sweep then runs the recurrences
// d' = (d - a d') m and x = d' - c' x, with no division on the chain.
// In: the restricted rhs of level ltop (global); out: its correction e,
// ghosts included (global).
constexpr int kTailThreads = 64;
constexpr int kTailMax = 12;
struct TailPlan {
  int ltop, sweeps;
  int nfac;  // factor floats per problem: (c', m) of the y-lines and of the x-lines, every level
  int fac0, scr, total;  // shared-memory offsets (floats): factor block, transfer scratch; total floats
  int nx[kTailMax], ny[kTailMax];
  int e[kTailMax], r[kTailMax];  // shared-memory offsets of e and r of level l + 1
  int f[kTailMax];               // offset of level l + 1's y-line factors in the factor block (x-lines follow)
};

TailPlan make_tail_plan(const MgPlan &PL, int ltop) {
  TailPlan t{};
  t.ltop = ltop;
  t.sweeps = std::max(8, (PL.lv[0].nx + PL.lv[0].ny) / 2);
  int off = 0, fo = 0;
  for (int l = 0; l < ltop; ++l) {
    const int nx = PL.lv[l].nx, ny = PL.lv[l].ny;
    t.nx[l] = nx;
    t.ny[l] = ny;
    t.e[l] = off;
    off += (nx + 2) * (ny + 2);
    t.r[l] = off;
    off += nx * ny;
    t.f[l] = fo;
    fo += 4 * nx * ny;
  }
  t.scr = off;
  off += (t.nx[ltop - 1] + 2) * (t.ny[ltop - 1] + 2);
  off = (off + 3) & ~3;  // the factor block is copied as float4
  t.fac0 = off;
  t.nfac = fo;
  t.total = off + fo;
  return t;
}

// one level of one problem in shared memory (P = 1, p = 0)
struct TailLv {
  int nx, ny;
  float *e, *r;
  const float2 *fy, *fx;  // (c', m) per point, point (i, j) at (j-1) nx + (i-1)
  const float *cof;
};
__device__ __forceinline__ TailLv tail_level_at(const TailPlan &t, const FastDev &g, float *sm, int l) {
  TailLv L;
  L.nx = t.nx[l];
  L.ny = t.ny[l];
  L.e = sm + t.e[l];
  L.r = sm + t.r[l];
  L.fy = reinterpret_cast<const float2 *>(sm + t.fac0 + t.f[l]);
  L.fx = L.fy + (size_t)L.nx * L.ny;
  L.cof = g.lv[l].cof;
  return L;
}

// y-line at column i with precomputed factors (the rows of yline_solve)
__device__ __forceinline__ void tail_yline(const TailLv &L, int i, bool orth) {
  const int nx = L.nx, ny = L.ny, npt = nx * ny, sj = nx + 2;
  const float *__restrict__ cf = L.cof;
  const float *__restrict__ r = L.r;
  const float2 *__restrict__ fy = L.fy;
  float *__restrict__ e = L.e;
  float dprev = 0.f;
  for (int j0 = 1; j0 <= ny; j0 += kChunk) {
    float dv[kChunk], av[kChunk], mv[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int j = j0 + u;
      if (j > ny) break;
      const int pt = (j - 1) * nx + (i - 1), q = j * sj + i;
      float d = r[pt] - cf[pt] * e[q + 1] - cf[4 * npt + pt] * e[q - 1];
      if (orth == false)
        d = d - cf[npt + pt] * e[q + 1 + sj] - cf[3 * npt + pt] * e[q + sj - 1] - cf[5 * npt + pt] * e[q - 1 - sj] -
            cf[7 * npt + pt] * e[q + 1 - sj];
      dv[u] = d;
      av[u] = cf[6 * npt + pt];
      mv[u] = fy[pt].y;
    }
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int j = j0 + u;
      if (j > ny) break;
      dprev = (dv[u] - av[u] * dprev) * mv[u];
      e[j * sj + i] = dprev;
    }
  }
  float x = 0.f;
  for (int j = ny; j >= 1; --j) {
    x = e[j * sj + i] - fy[(j - 1) * nx + (i - 1)].x * x;
    e[j * sj + i] = x;
    if (i == nx - 1) e[j * sj] = x;
    if (i == 2) e[j * sj + nx + 1] = x;
  }
}

// x-line at row j with precomputed factors (the rows of xline_solve)
__device__ __forceinline__ void tail_xline(const TailLv &L, int j, bool orth) {
  const int nx = L.nx, ny = L.ny, npt = nx * ny, sj = nx + 2;
  const float *__restrict__ cf = L.cof;
  const float *__restrict__ r = L.r;
  const float2 *__restrict__ fx = L.fx;
  float *__restrict__ erow = L.e + j * sj;
  const float g0 = erow[0], g1 = erow[nx + 1];
  const int rb = (j - 1) * nx;
  float dprev = 0.f;
  for (int i0 = 1; i0 <= nx; i0 += kChunk) {
    float dv[kChunk], av[kChunk], mv[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int i = i0 + u;
      if (i > nx) break;
      const int pt = rb + (i - 1);
      float d = r[pt] - cf[2 * npt + pt] * erow[i + sj] - cf[6 * npt + pt] * erow[i - sj];
      if (orth == false)
        d = d - cf[npt + pt] * erow[i + 1 + sj] - cf[3 * npt + pt] * erow[i + sj - 1] -
            cf[5 * npt + pt] * erow[i - 1 - sj] - cf[7 * npt + pt] * erow[i + 1 - sj];
      float a = cf[4 * npt + pt];
      if (i == 1) { d -= a * g0; a = 0.f; }
      if (i == nx) d -= cf[pt] * g1;
      dv[u] = d;
      av[u] = a;
      mv[u] = fx[pt].y;
    }
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      const int i = i0 + u;
      if (i > nx) break;
      dprev = (dv[u] - av[u] * dprev) * mv[u];
      erow[i] = dprev;
    }
  }
  float x = 0.f;
  for (int i = nx; i >= 1; --i) {
    x = erow[i] - fx[rb + (i - 1)].x * x;
    erow[i] = x;
    if (i == nx - 1) erow[0] = x;
    if (i == 2) erow[nx + 1] = x;
  }
}

// one alternating-direction zebra sweep (the order of the per-level relax)
__device__ __forceinline__ void tail_relax(const TailLv &L, bool orth, bool post) {
  for (int k = 0; k < 2; ++k) {
    const int col = post ? 2 - k : 1 + k;
    LinePhase ph[2];
    const int nph = line_phases(L.nx, col, ph);
    for (int q = 0; q < nph; ++q) {
      for (int c = threadIdx.x; c < ph[q].ncol; c += blockDim.x) tail_yline(L, ph[q].i0 + ph[q].istep * c, orth);
      __syncthreads();
    }
  }
  for (int k = 0; k < 2; ++k) {
    const int col = post ? 2 - k : 1 + k;
    const int nrow = (L.ny >= col) ? (L.ny - col) / 2 + 1 : 0;
    for (int c = threadIdx.x; c < nrow; c += blockDim.x) tail_xline(L, col + 2 * c, orth);
    __syncthreads();
  }
}

// Thomas factors of every line of the levels 1..ltop, per problem (one block
// per problem), into fac[p * nfac ...] in the shared-memory layout of the
// factor block; the same m and c' as yline_solve / xline_solve compute
__global__ void __launch_bounds__(kTailThreads) k_f_tail_factors(FastDev g, TailPlan t, float *fac) {
  const int p = (int)blockIdx.x;
  if (p >= g.P) return;
  const float kx2 = (float)g.kx2[p];
  float *fb = fac + (size_t)p * t.nfac;
  for (int l = 0; l < t.ltop; ++l) {
    const int nx = t.nx[l], ny = t.ny[l], npt = nx * ny;
    const float *__restrict__ cf = g.lv[l].cof;
    float2 *fy = reinterpret_cast<float2 *>(fb + t.f[l]);
    float2 *fx = fy + npt;
    for (int i = 1 + threadIdx.x; i <= nx; i += blockDim.x) {
      float cprev = 0.f;
      for (int j = 1; j <= ny; ++j) {
        const int pt = (j - 1) * nx + (i - 1);
        const float b = ((-kx2 * cf[10 * npt + pt]) - cf[8 * npt + pt]) + cf[9 * npt + pt];
        const float m = 1.f / (b - cf[6 * npt + pt] * cprev);
        cprev = cf[2 * npt + pt] * m;
        fy[pt] = make_float2(cprev, m);
      }
    }
    for (int j = 1 + threadIdx.x; j <= ny; j += blockDim.x) {
      float cprev = 0.f;
      for (int i = 1; i <= nx; ++i) {
        const int pt = (j - 1) * nx + (i - 1);
        const float b = ((-kx2 * cf[10 * npt + pt]) - cf[8 * npt + pt]) + cf[9 * npt + pt];
        const float a = (i == 1) ? 0.f : cf[4 * npt + pt];
        const float c = (i == nx) ? 0.f : cf[pt];
        const float m = 1.f / (b - a * cprev);
        cprev = c * m;
        fx[pt] = make_float2(cprev, m);
      }
    }
  }
}

__global__ void __launch_bounds__(kTailThreads) k_f_vtail(FastDev g, TailPlan t, const float *fac) {
  if (*g.alldone) return;
  const int p = (int)blockIdx.x;
  if (p >= g.P || g.done[p]) return;
  extern __shared__ __align__(16) float tsh[];
  const int P = g.P;
  const float kx2 = (float)g.kx2[p];
  const bool orth = g.orth != 0;
  const int ltop = t.ltop;
  float *const scr = tsh + t.scr;
  {
    // this problem's factors (contiguous), the rhs of level ltop, e = 0
    const float4 *src = reinterpret_cast<const float4 *>(fac + (size_t)p * t.nfac);
    float4 *dst = reinterpret_cast<float4 *>(tsh + t.fac0);
    for (int v = threadIdx.x; v < t.nfac / 4; v += blockDim.x) dst[v] = src[v];
    const TailLv T = tail_level_at(t, g, tsh, ltop - 1);
    const LvF &G = g.lv[ltop - 1];
    const int ne = (T.nx + 2) * (T.ny + 2), nr = T.nx * T.ny;
    for (int v = threadIdx.x; v < ne; v += blockDim.x) T.e[v] = 0.f;
    for (int v = threadIdx.x; v < nr; v += blockDim.x) T.r[v] = G.r[(size_t)v * P + p];
  }
  __syncthreads();
  for (int l = ltop; l >= 2; --l) {
    const TailLv F = tail_level_at(t, g, tsh, l - 1), C = tail_level_at(t, g, tsh, l - 2);
    tail_relax(F, orth, false);
    for (int v = threadIdx.x; v < F.nx * F.ny; v += blockDim.x)
      f_resid_at(F.cof, F.e, F.r, scr, F.nx, F.ny, 1, 0, 1 + v % F.nx, 1 + v / F.nx, kx2, orth);
    __syncthreads();
    for (int v = threadIdx.x; v < (C.nx + 2) * (C.ny + 2); v += blockDim.x)
      f_restrict_at(scr, C.e, C.r, F.nx, F.ny, C.nx, C.ny, 1, 0, v % (C.nx + 2), v / (C.nx + 2));
    __syncthreads();
  }
  {
    const TailLv L = tail_level_at(t, g, tsh, 0);
    for (int sw = 0; sw < t.sweeps; ++sw) tail_relax(L, orth, false);
    if (kx2 == 0.f) {
      // singular: keep the correction at zero mean, ghosts included (the
      // sum in k_f_coarsest's order)
      __shared__ float mean;
      if (threadIdx.x == 0) {
        float m = 0.f;
        for (int j = 1; j <= L.ny; ++j)
          for (int i = 1; i <= L.nx; ++i) m += L.e[j * (L.nx + 2) + i];
        mean = m / (float)(L.nx * L.ny);
      }
      __syncthreads();
      for (int v = threadIdx.x; v < L.ny * (L.nx + 2); v += blockDim.x) L.e[(L.nx + 2) + v] -= mean;
      __syncthreads();
    }
  }
  for (int l = 2; l <= ltop; ++l) {
    const TailLv F = tail_level_at(t, g, tsh, l - 1), C = tail_level_at(t, g, tsh, l - 2);
    const int nrr = (C.ny < F.ny) ? (F.ny + 1) / 2 : F.ny;
    for (int v = threadIdx.x; v < F.nx * nrr; v += blockDim.x)
      f_prolong_x_at(C.e, scr, F.nx, F.ny, C.nx, C.ny, 1, 0, 1 + v % F.nx, v / F.nx);
    __syncthreads();
    for (int v = threadIdx.x; v < F.nx * F.ny; v += blockDim.x)
      f_prolong_y_at(scr, F.e, F.nx, F.ny, C.ny, 1, 0, 1 + v % F.nx, 1 + v / F.nx);
    __syncthreads();
    tail_relax(F, orth, true);
  }
  {
    const TailLv T = tail_level_at(t, g, tsh, ltop - 1);
    const LvF &G = g.lv[ltop - 1];
    const int ne = (T.nx + 2) * (T.ny + 2);
    for (int v = threadIdx.x; v < ne; v += blockDim.x) G.e[(size_t)v * P + p] = T.e[v];
  }
}

// the FP64 solution (finest interior, problem fastest) from the float-float
// iterate, after the last correction
__global__ void __launch_bounds__(32 * kRY) k_f_phif(FastDev g) {
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  if (p >= P) return;
  const int nx = g.nfx, j = 1 + (int)blockIdx.y;
  const int par = g.cycles[p] & 1;
  const float *__restrict__ ph = par ? g.phh2 : g.phh;
  const float *__restrict__ pl = par ? g.phl2 : g.phl;
  for (int i = 1 + (int)threadIdx.y; i <= nx; i += kRY) {
    const size_t q = ((size_t)j * (nx + 2) + i) * P + p;
    g.phif[((size_t)(j - 1) * nx + (i - 1)) * P + p] = (double)FF(ph[q], pl[q]);
  }
}


// One partitioned line launch: lines l0, l0+lstep, ... (nline of them) of
// length n at level l, all problems, in the layout (lanes, seg): `lanes`
// problems per block (8, 16 or 32), segments of at most `seg` rows (4 or 8)
// separated by single rows, at most 128 segments and 1024 threads.  Lines
// the layout cannot hold fall back to one thread per line.
// K segments of at most seg rows and K-1 separator rows cover n rows when
// K (seg + 1) >= n + 1
int pline_segments(int n, int seg) { return std::max(1, (n + seg + 1) / (seg + 1)); }
bool pline_fits(int n, int lanes, int seg) {
  const int K = pline_segments(n, seg);
  return K <= 128 && K * lanes <= 1024;
}

void launch_pline(const FastDev &g, int l, bool xl, int l0, int lstep, int nline, int n, int lanes, int seg,
                  cudaStream_t s, bool zero_e = false) {
  if (zero_e && xl) throw CudaError("line solve: the zero-neighbour sweep is a y-line sweep");
  const int z = zero_e ? 1 : 0;
  const int K = pline_segments(n, seg);
  // the kernel indexes with 32-bit offsets
  if ((size_t)(g.nfx + 2) * (g.nfy + 2) * g.P >= (1ull << 31) || 11ull * g.nfx * g.nfy >= (1ull << 31))
    throw CudaError("line solve: grid x problems beyond 32-bit offsets");
  if (!pline_fits(n, lanes, seg)) {
    const unsigned b = (unsigned)(((long)nline * g.P + 63) / 64);
    if (xl) k_f_xline<<<b, 64, 0, s>>>(g, l, l0, nline);
    else k_f_yline<<<b, 64, 0, s>>>(g, l, l0, lstep, nline, z);
    return;
  }
  const int mb = (n - K + 1) / K, me = (n - K + 1) % K;
  const dim3 grid((unsigned)nline, (unsigned)((g.P + lanes - 1) / lanes)), blk(lanes, K);
  const size_t smem = sizeof(float) * SH_N * K * lanes;
#define EK_PLINE(W, S)                                                                             \
  do {                                                                                             \
    if (g.orth) {                                                                                  \
      if (xl) k_f_pline<true, true, W, S><<<grid, blk, smem, s>>>(g, l, l0, lstep, mb, me, z);        \
      else k_f_pline<false, true, W, S><<<grid, blk, smem, s>>>(g, l, l0, lstep, mb, me, z);          \
    } else {                                                                                       \
      if (xl) k_f_pline<true, false, W, S><<<grid, blk, smem, s>>>(g, l, l0, lstep, mb, me, z);       \
      else k_f_pline<false, false, W, S><<<grid, blk, smem, s>>>(g, l, l0, lstep, mb, me, z);         \
    }                                                                                              \
  } while (0)
  if (seg == 4) {
    if (lanes == 32) EK_PLINE(32, 4);
    else if (lanes == 16) EK_PLINE(16, 4);
    else EK_PLINE(8, 4);
  } else {
    if (lanes == 32) EK_PLINE(32, 8);
    else if (lanes == 16) EK_PLINE(16, 8);
    else EK_PLINE(8, 8);
  }
#undef EK_PLINE
}

// The layout the solver uses when nothing was tuned: 8-row segments, 32
// problems per block while a line has at most 32 segments (n <= 287), else 16.
int default_lanes(int n) { return (pline_segments(n, 8) <= 32) ? 32 : 16; }

FastDev make_fastdev(Ctx &c, int nprob, const double *kx2_dev) {
  const MgPlan &PL = c.mg;
  MgWork &w = c.mgw;
  FastDev g{};
  g.P = nprob;
  g.ngrid = PL.ngrid;
  g.orth = PL.orth ? 1 : 0;
  for (int l = 0; l < PL.ngrid; ++l) {
    const MgLevelF &F = c.mgf_levels[l];
    g.lv[l] = LvF{PL.lv[l].nx, PL.lv[l].ny, F.e, F.r, F.cof, F.cp, F.cf4};
  }
  g.scr = c.mgf_scratch;
  g.rhs = w.rhs[PL.ngrid - 1];
  g.phh = c.mgf_phh;
  g.phl = c.mgf_phl;
  g.phh2 = c.mgf_phh2;
  g.phl2 = c.mgf_phl2;
  g.bh = c.mgf_bh;
  g.bl = c.mgf_bl;
  g.cf2 = c.mgf_cf2;
  g.nfx = PL.nfx;
  g.nfy = PL.nfy;
  g.kx2 = kx2_dev;
  g.phif = w.phif;
  g.red = w.red;
  g.done = w.done;
  g.cycles = w.cycles;
  g.alldone = w.alldone;
  g.iter = w.iter;
  g.tol = c.p.mg_tol;
  return g;
}

// shared memory of k_f_vtail: at most this much.  Measured on the
// 512 x 385 x 257 workload (levels 3x4 .. 257x385): the levels up to 17 x 25
// in the tail (17 KB) beat up to 33 x 49 (62 KB) by 0.8 ms a step -- a level
// of ~1,600 points is cheaper as batched launches than on one block's
// thread chain, and the smaller blocks leave L1 to the coefficients.
constexpr size_t kTailSmem = 24 * 1024;
// the levels 1..ltop that k_f_vtail runs: the largest ltop below the finest
// level whose arrays fit kTailSmem bytes (0: none fits, k_f_coarsest)
int tail_level(const MgPlan &PL) {
  int ltop = 0;
  while (ltop + 1 < PL.ngrid && ltop + 1 <= kTailMax &&
         make_tail_plan(PL, ltop + 1).total * sizeof(float) <= kTailSmem)
    ++ltop;
  return ltop;
}

void launch_resid_ff(const FastDev &g, bool update, unsigned pch, cudaStream_t s) {
  const dim3 grid(pch, (unsigned)g.nfy), blk(32, kRY);
  if (update) {
    if (g.orth) k_f_resid_ff<true, true><<<grid, blk, 0, s>>>(g);
    else k_f_resid_ff<true, false><<<grid, blk, 0, s>>>(g);
  } else {
    if (g.orth) k_f_resid_ff<false, true><<<grid, blk, 0, s>>>(g);
    else k_f_resid_ff<false, false><<<grid, blk, 0, s>>>(g);
  }
}

unsigned nb(long n, int bs) {
  long b = (n + bs - 1) / bs;
  if (b < 1) b = 1;
  if (b > 65535L * 32) b = 65535L * 32;
  return (unsigned)b;
}

}  // namespace

int mgfast_tail_levels(const Ctx &c) { return c.mg.ngrid > 0 ? tail_level(c.mg) : 0; }

// FP32 copies of the level coefficients and the FP32 work arrays.
void mgfast_alloc(Ctx &c, int pmax) {
  MgPlan &PL = c.mg;
  if (c.mgf_pool) {
    cudaFree(c.mgf_pool);
    c.mgf_pool = nullptr;
  }
  size_t tot = 0;
  std::vector<size_t> off(PL.ngrid);
  for (int l = 0; l < PL.ngrid; ++l) {
    const MgLevel &L = PL.lv[l];
    off[l] = tot;
    tot += (size_t)(L.nx + 2) * (L.ny + 2) * pmax + 2 * (size_t)L.nx * L.ny * pmax + 11 * (size_t)L.nx * L.ny;
  }
  const size_t scr_off = tot;
  const size_t nph = (size_t)(PL.nfx + 2) * (PL.nfy + 2), nf = (size_t)PL.nfx * PL.nfy;
  tot += nph * pmax;
  const size_t ff_off = tot;
  tot += 4 * nph * pmax + 2 * nf * pmax + 22 * nf + 1;
  const int ltop = tail_level(PL);
  const size_t nfac = ltop ? (size_t)make_tail_plan(PL, ltop).nfac * pmax : 0;
  tot = (tot + 3) & ~(size_t)3;  // float4 reads of each problem's factor block
  const size_t fac_off = tot;
  tot += nfac;
  EK_CUDA(cudaMalloc(&c.mgf_pool, tot * sizeof(float)));
  c.mgf_levels.assign(PL.ngrid, {});
  // the packed coefficients (3 float4 per point and level)
  if (c.mgf_cf4_pool) {
    cudaFree(c.mgf_cf4_pool);
    c.mgf_cf4_pool = nullptr;
  }
  size_t n4 = 0;
  for (int l = 0; l < PL.ngrid; ++l) n4 += 3 * (size_t)PL.lv[l].nx * PL.lv[l].ny;
  EK_CUDA(cudaMalloc(&c.mgf_cf4_pool, n4 * sizeof(float4)));
  for (int l = 0; l < PL.ngrid; ++l) {
    const MgLevel &L = PL.lv[l];
    float *b = c.mgf_pool + off[l];
    MgLevelF &F = c.mgf_levels[l];
    F.e = b;
    F.r = F.e + (size_t)(L.nx + 2) * (L.ny + 2) * pmax;
    F.cp = F.r + (size_t)L.nx * L.ny * pmax;
    F.cof = F.cp + (size_t)L.nx * L.ny * pmax;
    std::vector<float> cf(PL.cof_host[l].begin(), PL.cof_host[l].end());
    EK_CUDA(cudaMemcpy(F.cof, cf.data(), sizeof(float) * cf.size(), cudaMemcpyHostToDevice));
    {
      const size_t npt = (size_t)L.nx * L.ny;
      size_t o4 = 0;
      for (int q = 0; q < l; ++q) o4 += 3 * (size_t)PL.lv[q].nx * PL.lv[q].ny;
      F.cf4 = c.mgf_cf4_pool + o4;
      std::vector<float4> pk(3 * npt);
      for (size_t pt = 0; pt < npt; ++pt) {
        auto C = [&](int t) { return cf[t * npt + pt]; };
        pk[3 * pt] = make_float4(C(0), C(2), C(4), C(6));
        pk[3 * pt + 1] = make_float4(C(8), C(9), C(10), 0.f);
        pk[3 * pt + 2] = make_float4(C(1), C(3), C(5), C(7));
      }
      EK_CUDA(cudaMemcpy(F.cf4, pk.data(), sizeof(float4) * pk.size(), cudaMemcpyHostToDevice));
    }
  }
  c.mgf_scratch = c.mgf_pool + scr_off;
  c.mgf_phh = c.mgf_pool + ff_off;
  c.mgf_phl = c.mgf_phh + nph * pmax;
  c.mgf_phh2 = c.mgf_phl + nph * pmax;
  c.mgf_phl2 = c.mgf_phh2 + nph * pmax;
  c.mgf_bh = c.mgf_phl2 + nph * pmax;
  c.mgf_bl = c.mgf_bh + nf * pmax;
  // 8-byte aligned for the float2 loads: the address itself decides (the
  // pool holds one float of slack)
  {
    float *cfb = c.mgf_bl + nf * pmax;
    if (reinterpret_cast<uintptr_t>(cfb) & 7) ++cfb;
    c.mgf_cf2 = reinterpret_cast<float2 *>(cfb);
  }
  c.mgf_tailfac = nfac ? c.mgf_pool + fac_off : nullptr;
  c.mgf_tailfac_n = nfac;
  // every context's tail fits kTailSmem, so one process-wide limit serves all
  // (set here, never during a stream capture)
  EK_CUDA(cudaFuncSetAttribute(k_f_vtail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTailSmem));
  {
    // the finest coefficients split into float-float pairs
    const std::vector<double> &cf = PL.cof_host[PL.ngrid - 1];
    std::vector<float2> hl(cf.size());
    for (size_t t = 0; t < cf.size(); ++t) {
      const float h = (float)cf[t];
      hl[t] = make_float2(h, (float)(cf[t] - (double)h));
    }
    EK_CUDA(cudaMemcpy(c.mgf_cf2, hl.data(), sizeof(float2) * hl.size(), cudaMemcpyHostToDevice));
  }
  c.mgf_pmax = pmax;
}

// Solve with the mixed-precision iteration; the finest rhs must be in
// c.mgw.rhs[ngrid-1] (FP64, problem fastest); the solution is left in
// c.mgw.phif.
int mgfast_solve(Ctx &c, int nprob, const double *kx2_dev, const double *kx2_host, ek_mg_stats *st) {
  MgPlan &PL = c.mg;
  MgWork &w = c.mgw;
  if (nprob > c.mgf_pmax || nprob > w.pmax) return EK_ERR_ARG;
  cudaStream_t s = c.stream;
  const int bs = 256;
  const long npt = (long)PL.nfx * PL.nfy;
  // the kx^2 = 0 problems (well posed by projection; the learned guess and
  // its statistics leave them out)
  std::vector<double> kxh;
  if (!kx2_host) {
    kxh.resize(nprob);
    EK_CUDA(cudaMemcpyAsync(kxh.data(), kx2_dev, sizeof(double) * nprob, cudaMemcpyDeviceToHost, s));
    EK_CUDA(cudaStreamSynchronize(s));
    kx2_host = kxh.data();
  }
  std::vector<char> is_sing(nprob, 0);
  int ns = 0;
  for (int p = 0; p < nprob; ++p)
    if (kx2_host[p] == 0.0) {
      is_sing[p] = 1;
      ++ns;
    }
  if (ns > 0) mg_null_project(c, w.rhs[PL.ngrid - 1], nprob, kx2_dev);
  FastDev g = make_fastdev(c, nprob, kx2_dev);

  {
    KScope ks(c, KC_MG_SETUP, 8.0 * (PL.nfx + 2) * (PL.nfy + 2) * nprob * 2);
    EK_CUDA(cudaMemsetAsync(w.flags, 0, sizeof(int) * (2 * w.pmax + 4), s));
    EK_CUDA(cudaMemsetAsync(w.red, 0, sizeof(double) * (6 * w.pmax + 8), s));
    const size_t nph = (size_t)(PL.nfx + 2) * (PL.nfy + 2) * nprob;
    EK_CUDA(cudaMemsetAsync(g.phh, 0, sizeof(float) * nph, s));
    EK_CUDA(cudaMemsetAsync(g.phl, 0, sizeof(float) * nph, s));
    EK_CUDA(cudaMemsetAsync(g.phh2, 0, sizeof(float) * nph, s));
    EK_CUDA(cudaMemsetAsync(g.phl2, 0, sizeof(float) * nph, s));
    // the finest correction: its ghost rows stay zero from here on, and each
    // cycle's first sweep leaves its other values unread
    EK_CUDA(cudaMemsetAsync(g.lv[PL.ngrid - 1].e, 0, sizeof(float) * nph, s));
    const size_t nf = (size_t)PL.nfx * PL.nfy * nprob;
    k_f_split<<<nb((long)nf, bs), bs, 0, s>>>(g.rhs, g.bh, g.bl, nf);
    after_launch(c);
  }
  const int gx = (nprob + 31) / 32;
  const unsigned pch = (unsigned)gx;  // 32-problem chunks of the row kernels
  // learned initial guess for the kx^2 != 0 problems, scaled by the
  // least-squares factor (a useless guess gets a factor near zero)
  const bool guessed = c.guess.net && c.guess.use && nprob > ns;
  if (guessed) {
    GuessState &G = c.guess;
    KScope ks(c, KC_GUESS, G.net->forward_flops(nprob - ns));
    std::vector<int> nonsing;
    for (int p = 0; p < nprob; ++p)
      if (!is_sing[p]) nonsing.push_back(p);
    guess_predict(c, nprob, g.rhs, kx2_dev, nonsing, g.phh, s);
    if (G.alpha_cap < nprob) {
      cudaFree(G.alpha);
      G.alpha = nullptr;
      G.alpha_cap = 0;
      EK_CUDA(cudaMalloc(&G.alpha, sizeof(float) * nprob));
      G.alpha_cap = nprob;
    }
    launch_resid_ff(g, false, pch, s);
    after_launch(c);
    k_f_guess_rb<<<dim3(pch, PL.nfy), dim3(32, kRY), 0, s>>>(g);
    after_launch(c);
    k_f_guess_alpha<<<nb(nprob, 128), 128, 0, s>>>(g, G.alpha);
    after_launch(c);
    k_f_guess_scale<<<nb((long)(PL.nfx + 2) * (PL.nfy + 2) * nprob, bs), bs, 0, s>>>(g, G.alpha);
    after_launch(c);
  }

  // one partitioned line launch, in the layout tuned for (level, direction)
  auto pline = [&](int l, bool xl, int l0, int lstep, int nline, int n, bool zero_e) {
    int lanes = default_lanes(n), seg = 8;
    const std::vector<int> &tl = xl ? PL.lanes_x : PL.lanes_y;
    const std::vector<int> &ts = xl ? PL.seg_x : PL.seg_y;
    if (l < (int)tl.size() && tl[l] > 0) lanes = tl[l];
    if (l < (int)ts.size() && ts[l] > 0) seg = ts[l];
    launch_pline(g, l, xl, l0, lstep, nline, n, lanes, seg, s, zero_e);
    after_launch(c);
  };


  // one alternating-direction zebra sweep at level l: y-lines (colours
  // 1, 2), then x-lines (rows 1, 3, ... then 2, 4, ...); the post-smoothing
  // sweep takes the colours in the reverse order.  (Post-smoothing with
  // x-lines only needs 8-9 corrections instead of 6-7 on the 256x257x193
  // grid, so it costs more than it saves.)
  // zero_first: e holds stale values that the cycle starts from zero
  // (the finest level, whose e is not cleared between cycles): the first
  // colour's y-lines take their neighbours as zero.  Needs odd nx (one
  // phase per colour, and no line of the first colour reads a line of the
  // same colour), which every level above the coarsest has.
  auto relax = [&](int l, bool post, bool zero_first) {
    const MgLevel &L = PL.lv[l - 1];
    KScope ks(c, KC_MG_RELAX, 4.0 * nprob * L.nx * L.ny * 10);
    for (int k = 0; k < 2; ++k) {
      const int col = post ? 2 - k : 1 + k;
      LinePhase ph[2];
      const int nph = line_phases(L.nx, col, ph);
      for (int q = 0; q < nph; ++q)
        if (ph[q].ncol > 0) pline(l, false, ph[q].i0, ph[q].istep, ph[q].ncol, L.ny, zero_first && k == 0);
    }
    for (int k = 0; k < 2; ++k) {
      const int col = post ? 2 - k : 1 + k;
      pline(l, true, col, 2, (L.ny - col) / 2 + 1, L.nx, false);
    }
  };

  const int maxit = c.p.mg_maxcy;
  // r = b - A phi and the per-problem decision (incr: count one more
  // correction); cond/use_cond: the while-node condition in a graph
  auto check = [&](int incr, cudaGraphConditionalHandle cond, int use_cond) {
    // bytes: b (2), r; phi (2), and with the update e and phi' (2)
    KScope ks(c, KC_MG_CHECK, 4.0 * nprob * npt * (incr ? 8.0 : 5.0));
    launch_resid_ff(g, incr != 0, pch, s);
    after_launch(c);
    k_f_check<<<1, 256, 0, s>>>(g, maxit, incr, cond, use_cond);
    after_launch(c);
  };
  // the levels 1..ltop run as one k_f_vtail launch
  const int ltop = tail_level(PL);
  const TailPlan tplan = ltop ? make_tail_plan(PL, ltop) : TailPlan{};
  const size_t tail_bytes = ltop ? tplan.total * sizeof(float) : 0;
  if (ltop) {
    if ((size_t)tplan.nfac * nprob > c.mgf_tailfac_n) throw CudaError("mixed solve: tail factor buffer too small");
    KScope ks(c, KC_MG_SETUP, 4.0 * nprob * tplan.nfac);
    k_f_tail_factors<<<(unsigned)nprob, kTailThreads, 0, s>>>(g, tplan, c.mgf_tailfac);
    after_launch(c);
  }
  // one FP32 V(1,1) cycle on A e = r from e = 0 (phi += e follows in the
  // next check's residual kernel).  The finest e is not cleared: the first
  // sweep reads none of it (odd nx, the MUDPACK grids' rule), else it is
  // cleared here.
  const bool fine_zero = PL.ngrid >= 2 && PL.lv[PL.ngrid - 1].nx % 2 == 1;
  auto correction = [&]() {
    if (!fine_zero) {
      const size_t nph = (size_t)(PL.nfx + 2) * (PL.nfy + 2) * nprob;
      EK_CUDA(cudaMemsetAsync(g.lv[PL.ngrid - 1].e, 0, sizeof(float) * nph, s));
    }
    for (int l = PL.ngrid; l >= 1; --l) {
      const MgLevel &L = PL.lv[l - 1];
      if (l == ltop) {
        // bytes: level ltop's rhs in and its correction out
        KScope ks(c, KC_MG_COARSE, 4.0 * nprob * (L.nx * L.ny + (L.nx + 2.0) * (L.ny + 2)));
        k_f_vtail<<<(unsigned)nprob, kTailThreads, tail_bytes, s>>>(g, tplan, c.mgf_tailfac);
        after_launch(c);
        break;
      }
      if (l == 1) {
        const int sweeps = std::max(8, (L.nx + L.ny) / 2);
        KScope ks(c, KC_MG_RELAX, 4.0 * nprob * L.nx * L.ny * 10 * sweeps);
        k_f_coarsest<<<nb(nprob, 64), 64, 0, s>>>(g, sweeps);
        after_launch(c);
        break;
      }
      relax(l, false, l == PL.ngrid && fine_zero);
      const MgLevel &C = PL.lv[l - 2];
      KScope ks(c, KC_MG_TRANSFER, 4.0 * nprob * (4.0 * L.nx * L.ny + 2.0 * (C.nx + 2) * (C.ny + 2)));
      k_f_resid32<<<dim3(pch, L.ny), dim3(32, kRowWarps), 0, s>>>(g, l);
      after_launch(c);
      k_f_restrict<<<dim3(pch, C.ny + 2), dim3(32, kRowWarps), 0, s>>>(g, l);
      after_launch(c);
    }
    for (int l = std::max(2, ltop + 1); l <= PL.ngrid; ++l) {
      const MgLevel &L = PL.lv[l - 1];
      {
        KScope ks(c, KC_MG_TRANSFER, 4.0 * nprob * 4.0 * L.nx * L.ny);
        const MgLevel &Cq = PL.lv[l - 2];
        k_f_prolong_x<<<dim3(pch, Cq.ny < L.ny ? (L.ny + 1) / 2 : L.ny), dim3(32, kRowWarps), 0, s>>>(g, l);
        after_launch(c);
        k_f_prolong_y<<<dim3(pch, L.ny), dim3(32, kRowWarps), 0, s>>>(g, l);
        after_launch(c);
      }
      relax(l, true, false);
    }
  };
  if (c.graph_slot < 0) {
    // eager: the host stops issuing cycles once the done flag it polls is set
    c.poll.init();
    c.poll.reset();
    check(0, 0, 0);
    bool stop = c.poll.after_check(w.alldone, s);
    for (int it = 1; it <= maxit && !stop; ++it) {
      correction();
      check(1, 0, 0);
      stop = c.poll.after_check(w.alldone, s);
    }
  } else {
    // captured: the cycles repeat in a conditional while-node whose
    // condition the check kernel sets, so no host decides between them
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    EK_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
    if (cs != cudaStreamCaptureStatusActive) throw CudaError("mixed solve: step graph capture is not active");
    cudaGraphConditionalHandle cond;
    EK_CUDA(cudaGraphConditionalHandleCreate(&cond, cg, 1u, cudaGraphCondAssignDefault));
    check(0, cond, 1);
    EK_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t wnode;
    EK_CUDA(cudaGraphAddNode(&wnode, cg, deps, nullptr, ndeps, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    EK_CUDA(cudaStreamUpdateCaptureDependencies(s, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    const cudaStream_t outer = s;
    s = c.cap_stream2;
    const long long l0 = c.launches;
    try {
      EK_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
      correction();
      check(1, cond, 1);
      cudaGraph_t done_body = nullptr;
      EK_CUDA(cudaStreamEndCapture(s, &done_body));
    } catch (...) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(c.cap_stream2, &junk);
      s = outer;
      throw;
    }
    s = outer;
    c.graph_body_launches = c.launches - l0;
  }
  {
    KScope ks(c, KC_MG_SETUP, 16.0 * nprob * npt);
    k_f_phif<<<dim3(pch, PL.nfy), dim3(32, kRY), 0, s>>>(g);
    after_launch(c);
  }
  if (ns > 0) mg_null_mean(c, w.phif, nprob, kx2_dev);
  if (c.graph_slot >= 0) {
    // a captured step reads the statistics after the step
    k_f_stats<<<1, 256, 0, s>>>(g, c.step_stats_dev + c.graph_slot);
    after_launch(c);
    return EK_OK;
  }
  std::vector<int> cyc(nprob), done(nprob);
  std::vector<double> meas(6 * nprob);
  EK_CUDA(cudaMemcpyAsync(cyc.data(), w.cycles, sizeof(int) * nprob, cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaMemcpyAsync(done.data(), w.done, sizeof(int) * nprob, cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaMemcpyAsync(meas.data(), w.red, sizeof(double) * 6 * nprob, cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaStreamSynchronize(s));
  ek_mg_stats S{};
  S.nprob = nprob;
  S.min_cycles = nprob ? (1 << 30) : 0;
  double csum = 0.0, rsum = 0.0;
  for (int p = 0; p < nprob; ++p) {
    S.min_cycles = std::min(S.min_cycles, cyc[p]);
    S.max_cycles = std::max(S.max_cycles, cyc[p]);
    if (done[p] != 1) S.n_not_converged++;
    S.max_residual = std::max(S.max_residual, meas[6 * p + 4]);
    if (is_sing[p]) continue;
    csum += cyc[p];
    rsum += guessed ? meas[6 * p + 5] : 1.0;
  }
  c.last_mean_cycles = (nprob > ns) ? csum / (nprob - ns) : 0.0;
  c.guess.last_rho = (nprob > ns) ? rsum / (nprob - ns) : 1.0;
  c.last_stats = S;
  if (st) *st = S;
  return S.n_not_converged ? EK_ERR_NOT_CONVERGED : EK_OK;
}


// Tile-shape autotuner of the line solves: for every level of the mixed
// solver and both line directions, time one full zebra sweep (both colours)
// in each valid layout -- 8, 16 or 32 problems per block, segments of 8 or 4
// rows -- on the solver's own arrays, `reps` times, and keep the fastest.  The level arrays are work
// space that every solve re-initialises, so the timing runs leave no trace.
int mgfast_autotune(Ctx &c, int reps, std::string &report) {
  MgPlan &PL = c.mg;
  MgWork &w = c.mgw;
  const int nprob = 2 * (c.d.NKX + 1);
  if (!c.p.mg_fast || nprob > c.mgf_pmax) return EK_ERR_STATE;
  cudaStream_t s = c.stream;
  FastDev g = make_fastdev(c, nprob, w.kx2);
  EK_CUDA(cudaMemsetAsync(w.flags, 0, sizeof(int) * (2 * w.pmax + 4), s));  // every problem active
  PL.lanes_y.assign(PL.ngrid + 1, 0);
  PL.lanes_x.assign(PL.ngrid + 1, 0);
  PL.seg_y.assign(PL.ngrid + 1, 0);
  PL.seg_x.assign(PL.ngrid + 1, 0);
  cudaEvent_t e0, e1;
  EK_CUDA(cudaEventCreate(&e0));
  EK_CUDA(cudaEventCreate(&e1));
  report = "[";
  bool first = true;
  try {
    // the levels k_f_vtail runs have no line-solve launches to tune
    for (int l = std::max(2, tail_level(PL) + 1); l <= PL.ngrid; ++l) {
      const MgLevel &L = PL.lv[l - 1];
      for (int dir = 0; dir < 2; ++dir) {
        const bool xl = dir == 1;
        const int n = xl ? L.nx : L.ny;
        auto sweep = [&](int lanes, int seg) {
          if (xl) {
            for (int col = 1; col <= 2; ++col) {
              launch_pline(g, l, true, col, 2, (L.ny - col) / 2 + 1, L.nx, lanes, seg, s);
              after_launch(c);
            }
          } else {
            for (int col = 1; col <= 2; ++col) {
              LinePhase ph[2];
              const int nph = line_phases(L.nx, col, ph);
              for (int q = 0; q < nph; ++q)
                if (ph[q].ncol > 0) {
                  launch_pline(g, l, false, ph[q].i0, ph[q].istep, ph[q].ncol, L.ny, lanes, seg, s);
                  after_launch(c);
                }
            }
          }
        };
        int best = 0, best_seg = 8;
        float best_ms = 0.f;
        std::string row;
        for (int seg : {8, 4})
          for (int lanes : {32, 16, 8}) {
            if (!pline_fits(n, lanes, seg)) continue;
            sweep(lanes, seg);  // warm-up
            EK_CUDA(cudaEventRecord(e0, s));
            for (int r = 0; r < reps; ++r) sweep(lanes, seg);
            EK_CUDA(cudaEventRecord(e1, s));
            EK_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            EK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            ms /= (float)reps;
            row += (row.empty() ? "" : ", ") + std::string("\"") + std::to_string(lanes) + "x" + std::to_string(seg) +
                   "\": " + std::to_string(1000.0 * ms);
            if (best == 0 || ms < best_ms) {
              best = lanes;
              best_seg = seg;
              best_ms = ms;
            }
          }
        (xl ? PL.lanes_x : PL.lanes_y)[l] = best;
        (xl ? PL.seg_x : PL.seg_y)[l] = best_seg;
        report += std::string(first ? "" : ", ") + "{\"level\": " + std::to_string(l) + ", \"dir\": \"" +
                  (xl ? "x" : "y") + "\", \"n\": " + std::to_string(n) + ", \"us\": {" + row +
                  "}, \"lanes\": " + std::to_string(best) + ", \"seg\": " + std::to_string(best_seg) + "}";
        first = false;
      }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  report += "]";
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  EK_CUDA(cudaStreamSynchronize(s));
  return EK_OK;
}

}  // namespace ek
