// Batched per-kx multigrid of the pressure projection, FP64.
//
// Replaces the per-mode loop of REM_DIV_CURV (src/duct.F90:2620-2669) over
// MULTIGRID_MUDPACK (src/mg_solver2d.F90:75-201 -> mud2cr, src/mud2cr.f).
// Every real 2-D problem of a batch is advanced in lockstep through the
// same MUDPACK operation sequence: trsfc2 injection, one FMG pass, then
// k-cycles with the convergence check after each (mud2cr1,
// mud2cr.f:211-338).  The sequence is generated on the host by simulating
// kcymd2cr's level counters (mud2cr.f:340-499).
//
// Layout: problems are the fastest index of every level array, so a warp
// touches 32 problems at one grid point (coalesced), and the kx-independent
// stencil coefficients are broadcast.  For the projection the problem index
// is 2*mode + {0 real, 1 imaginary}, which is the complex spectral layout
// itself.
//
// Relaxation is MUDPACK's four-colour point Gauss-Seidel (relmd2crp,
// mud2cr.f:1693-1795) in its exact order: colour c updates the points with
// i+j = c+1 (mod 4), row classes j = 1,2,3,4 (mod 4) one after another, and
// the periodic ghost columns are refreshed after each colour.  When every
// diagonal coefficient (c2, c4, c6, c8) is zero -- orthogonal grids -- the
// row classes of one colour do not couple and run as one phase; results
// are the same.
//
// Fine levels run as grid-wide phase kernels; levels 1..lc run inside one
// CTA per problem in shared memory, one launch per stretch of the schedule
// that stays below level lc+1.
#include <algorithm>
#include <cstdio>

#include <mutex>

#include "ek_internal.h"

namespace ek {

namespace {

struct LvDev {
  int nx, ny;
  double *phi, *rhs, *cof, *inv9;
};
struct MgDev {
  int P, ngrid, lc, orth;
  LvDev lv[24];
  double *scr;
  const double *kx2;
  double *phif;
  double *red;
  int *done, *cycles, *alldone;
  double tol;
  int stop_rule;
};

__device__ __forceinline__ double &PH(const LvDev &L, int P, int i, int j, int p) {
  return L.phi[((size_t)j * (L.nx + 2) + i) * P + p];
}
__device__ __forceinline__ size_t PT(const LvDev &L, int i, int j) { return (size_t)(j - 1) * L.nx + (i - 1); }

// --------------------------------------------------------------------------
// setup: 1/c9 per point and problem, c9 = (-kx2*J - s4) + corr9
__global__ void k_inv9(MgDev g, int level) {
  const LvDev L = g.lv[level - 1];
  const int P = g.P;
  const long n = (long)L.nx * L.ny * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    const long pt = t / P;
    const size_t npt = (size_t)L.nx * L.ny;
    const double s4 = L.cof[8 * npt + pt], corr = L.cof[9 * npt + pt], jac = L.cof[10 * npt + pt];
    const double ce = -g.kx2[p] * jac;
    const double c9 = (ce - s4) + corr;
    L.inv9[pt * P + p] = 1.0 / c9;
  }
}

// trsfc2 chain (mudcom.f:61-118) at the FMG start, plus swk2's zero ghosts
// (mudcom.f:32-59): phi = 0 on every level (the initial guess is zero),
// coarse rhs = injection of the finer rhs.
__global__ void k_zero(double *a, size_t n) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) a[t] = 0.0;
}
__global__ void k_inject(MgDev g, int level) {  // level -> level-1
  const LvDev F = g.lv[level - 1], C = g.lv[level - 2];
  const int P = g.P;
  const long n = (long)C.nx * C.ny * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    const long pt = t / P;
    const int ic = 1 + (int)(pt % C.nx), jc = 1 + (int)(pt / C.nx);
    const int i = (C.nx < F.nx) ? ic + ic - 1 : ic;
    const int j = (C.ny < F.ny) ? jc + jc - 1 : jc;
    C.rhs[PT(C, ic, jc) * P + p] = F.rhs[PT(F, i, j) * P + p];
  }
}

// --------------------------------------------------------------------------
// one point update of relmd2crp
__device__ __forceinline__ double relax_value(const double *ph, size_t si, size_t sj, const double *cof, size_t npt,
                                              size_t pt, double rhs, double inv9, bool orth) {
  // ph points at phi(i,j) of this problem; si, sj are the i and j strides
  const double c1 = cof[pt], c3 = cof[2 * npt + pt], c5 = cof[4 * npt + pt], c7 = cof[6 * npt + pt];
  double s;
  if (orth) {
    s = c1 * ph[si];
    s = s + c3 * ph[sj];
    s = s + c5 * ph[-(long)si];
    s = s + c7 * ph[-(long)sj];
  } else {
    const double c2 = cof[npt + pt], c4 = cof[3 * npt + pt], c6 = cof[5 * npt + pt], c8 = cof[7 * npt + pt];
    s = c1 * ph[si];
    s = s + c2 * ph[si + sj];
    s = s + c3 * ph[sj];
    s = s + c4 * ph[sj - si];
    s = s + c5 * ph[-(long)si];
    s = s + c6 * ph[-(long)(si + sj)];
    s = s + c7 * ph[-(long)sj];
    s = s + c8 * ph[si - sj];
  }
  return (rhs - s) * inv9;
}

// first i >= 1 of colour c (1..4) in row j: i + j = c + 1 (mod 4)
__device__ __forceinline__ int first_i(int c, int j) { return 1 + (((c + 1 - j - 1) % 4) + 4) % 4; }

// Fine-level relaxation phase: colour c, row class r (1..4) or all rows
// (r = 0, orthogonal path).  ghost_on_write: write the periodic ghost
// columns when i = nx-1 or i = 2 is updated.
__global__ void k_relax_phase(MgDev g, int level, int c, int r, int ghost_on_write) {
  if (*g.alldone) return;
  const LvDev L = g.lv[level - 1];
  const int P = g.P;
  const int nx = L.nx, ny = L.ny;
  const int ncol = (nx + 3) / 4 + 1;  // columns per row (upper bound)
  const int nrow = (r == 0) ? ny : (ny - r) / 4 + 1;
  const long npoint = (long)nrow * ncol;
  const size_t npt = (size_t)nx * ny;
  const size_t si = P, sj = (size_t)(nx + 2) * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < npoint * P; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    if (g.done[p]) continue;
    const long q = t / P;
    const int rowi = (int)(q / ncol), coli = (int)(q % ncol);
    const int j = (r == 0) ? 1 + rowi : r + 4 * rowi;
    if (j > ny) continue;
    const int i = first_i(c, j) + 4 * coli;
    if (i > nx) continue;
    const size_t pt = PT(L, i, j);
    double *ph = &PH(L, P, i, j, p);
    const double v = relax_value(ph, si, sj, L.cof, npt, pt, L.rhs[pt * P + p], L.inv9[pt * P + p], g.orth);
    *ph = v;
    if (ghost_on_write) {
      if (i == nx - 1) PH(L, P, 0, j, p) = v;
      if (i == 2) PH(L, P, nx + 1, j, p) = v;
    }
  }
}

// periodic virtual boundaries (mud2cr.f:1784-1789, mudcom.f:540-551)
__global__ void k_ghost(MgDev g, int level) {
  if (*g.alldone) return;
  const LvDev L = g.lv[level - 1];
  const int P = g.P;
  const long n = (long)L.ny * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    if (g.done[p]) continue;
    const int j = 1 + (int)(t / P);
    PH(L, P, 0, j, p) = PH(L, P, L.nx - 1, j, p);
    PH(L, P, L.nx + 1, j, p) = PH(L, P, 2, j, p);
  }
}

// residual on the fine level into the scratch array (resmd2cr,
// mud2cr.f:1618-1665), then full weighting to the coarse rhs (res2,
// mudcom.f:120-257) and phic = 0.
__global__ void k_resid(MgDev g, int level) {
  if (*g.alldone) return;
  const LvDev L = g.lv[level - 1];
  const int P = g.P;
  const size_t npt = (size_t)L.nx * L.ny;
  const size_t si = P, sj = (size_t)(L.nx + 2) * P;
  const long n = (long)npt * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    if (g.done[p]) continue;
    const long pt = t / P;
    const int i = 1 + (int)(pt % L.nx), j = 1 + (int)(pt / L.nx);
    const double *ph = &PH(L, P, i, j, p);
    const double *cf = L.cof;
    double s = cf[pt] * ph[si];
    s = s + cf[npt + pt] * ph[si + sj];
    s = s + cf[2 * npt + pt] * ph[sj];
    s = s + cf[3 * npt + pt] * ph[sj - si];
    s = s + cf[4 * npt + pt] * ph[-(long)si];
    s = s + cf[5 * npt + pt] * ph[-(long)(si + sj)];
    s = s + cf[6 * npt + pt] * ph[-(long)sj];
    s = s + cf[7 * npt + pt] * ph[si - sj];
    // c9 itself (not its reciprocal) enters the residual
    const double s4 = cf[8 * npt + pt], corr = cf[9 * npt + pt], jac = cf[10 * npt + pt];
    const double c9v = ((-g.kx2[p] * jac) - s4) + corr;
    s = s + c9v * ph[0];
    g.scr[((size_t)j * (L.nx + 2) + i) * P + p] = L.rhs[pt * P + p] - s;
  }
}

__global__ void k_res2(MgDev g, int level) {  // level -> level-1
  if (*g.alldone) return;
  const LvDev F = g.lv[level - 1], C = g.lv[level - 2];
  const int P = g.P;
  const int nx = F.nx, ny = F.ny, ncx = C.nx, ncy = C.ny;
  const int ix = (ncx == nx) ? 0 : 1, jy = (ncy == ny) ? 0 : 1;
  const long n = (long)(ncx + 2) * (ncy + 2) * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % P);
    if (g.done[p]) continue;
    const long q = t / P;
    const int ic = (int)(q % (ncx + 2)), jc = (int)(q / (ncx + 2));
    C.phi[q * P + p] = 0.0;
    if (ic < 1 || ic > ncx || jc < 1 || jc > ncy) continue;
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
    auto R = [&](int a, int b) { return g.scr[((size_t)b * (nx + 2) + a) * P + p]; };
    const double v = (R(im1, jm1) + R(ip1, jm1) + R(im1, jp1) + R(ip1, jp1) +
                      2. * (R(im1, j) + R(ip1, j) + R(i, jm1) + R(i, jp1)) + 4. * R(i, j)) * .0625;
    C.rhs[PT(C, ic, jc) * P + p] = v;
  }
}

// prolon1 (mudcom.f:404-499) value at fine index i from the coarse row p()
// (periodic x); cubic unless intpol == 1 or ncx < 4.
template <typename F>
__device__ __forceinline__ double prolon1_at(int i, int ncx, int nx, bool cubic, F p) {
  if (ncx == nx) return p(i);
  if (!cubic) {
    if (i & 1) return p((i + 1) / 2);
    return 0.5 * (p(i / 2) + p(i / 2 + 1));
  }
  auto q = [&](int ii) { return p((ii + 1) / 2); };  // odd ii only
  if (i & 1) return q(i);
  if (i >= 4 && i <= nx - 3) return (-q(i - 3) + 9. * (q(i - 1) + q(i + 1)) - q(i + 3)) * .0625;
  if (i == 2) return (-q(nx - 2) + 9. * (q(1) + q(3)) - q(5)) * .0625;
  // i == nx-1
  return (-q(nx - 4) + 9. * (q(nx - 2) + q(nx)) - q(3)) * .0625;
}

// prolon2 (mudcom.f:261-399) stage 1: rows set by prolon1.  mode 0 = into
// the scratch array (cor2), mode 1 = into phi of the fine level (FMG), where
// prolon1 also sets the ghost points of those rows.
__global__ void k_prolong_x(MgDev g, int level, int intpol, int mode) {  // coarse level-1 -> fine level
  if (*g.alldone) return;
  const LvDev F = g.lv[level - 1], C = g.lv[level - 2];
  const int P = g.P;
  const int nx = F.nx, ny = F.ny, ncx = C.nx, ncy = C.ny;
  const bool ycoarse = ncy < ny;
  const bool cubic_x = !(intpol == 1 || ncx < 4);
  const int nrows = ycoarse ? (ny + 1) / 2 : ny;
  const long n = (long)nrows * (nx + 2) * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int pp = (int)(t % P);
    if (g.done[pp]) continue;
    const long q = t / P;
    const int i = (int)(q % (nx + 2));
    const int rr = (int)(q / (nx + 2));
    const int j = ycoarse ? 2 * rr + 1 : rr + 1;
    const int jc = ycoarse ? j / 2 + 1 : j;
    auto pc = [&](int ic) { return PH(C, P, ic, jc, pp); };
    double v;
    if (i == 0) v = prolon1_at(nx - 1, ncx, nx, cubic_x, pc);
    else if (i == nx + 1) v = prolon1_at(2, ncx, nx, cubic_x, pc);
    else v = prolon1_at(i, ncx, nx, cubic_x, pc);
    if (mode == 0) g.scr[((size_t)j * (nx + 2) + i) * P + pp] = v;
    else PH(F, P, i, j, pp) = v;
  }
}

// prolon2 stage 2 (even rows in y) and, for cor2, the add into phi with
// the ghost refresh of mudcom.f:540-551 done on write.
__global__ void k_prolong_y(MgDev g, int level, int intpol, int mode) {
  if (*g.alldone) return;
  const LvDev F = g.lv[level - 1], C = g.lv[level - 2];
  const int P = g.P;
  const int nx = F.nx, ny = F.ny, ncy = C.ny;
  const bool ycoarse = ncy < ny;
  const bool cubic_y = !(intpol == 1 || ncy < 4);
  const long n = (long)nx * ny * P;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int pp = (int)(t % P);
    if (g.done[pp]) continue;
    const long q = t / P;
    const int i = 1 + (int)(q % nx), j = 1 + (int)(q / nx);
    auto Q = [&](int jj) -> double {
      return (mode == 0) ? g.scr[((size_t)jj * (nx + 2) + i) * P + pp] : PH(F, P, i, jj, pp);
    };
    double v;
    const bool even = ycoarse && !(j & 1);
    if (even) {
      if (!cubic_y) v = 0.5 * (Q(j - 1) + Q(j + 1));
      else if (j >= 4 && j <= ny - 3) v = (-Q(j - 3) + 9. * (Q(j - 1) + Q(j + 1)) - Q(j + 3)) * .0625;
      else if (j == 2) v = (5. * Q(1) + 15. * Q(3) - 5. * Q(5) + Q(7)) * .0625;
      else v = (5. * Q(ny) + 15. * Q(ny - 2) - 5. * Q(ny - 4) + Q(ny - 6)) * .0625;
    } else {
      v = Q(j);
    }
    if (mode == 1) {
      if (even) PH(F, P, i, j, pp) = v;
    } else {
      double &ph = PH(F, P, i, j, pp);
      const double nv = ph + v;
      ph = nv;
      if (i == nx - 1) PH(F, P, 0, j, pp) = nv;
      if (i == 2) PH(F, P, nx + 1, j, pp) = nv;
    }
  }
}

// Convergence check after a finest-level cycle (mud2cr.f:301-326): per
// problem max|phi| and max|phi - phif|, phif = phi; or, for the residual
// rule, sums of squares of the residual and of the rhs.
__device__ __forceinline__ void atomic_max_pos(double *a, double v) {
  atomicMax(reinterpret_cast<unsigned long long *>(a), (unsigned long long)__double_as_longlong(v));
}
// Thread block = 32 consecutive problems x 8 point slices: a warp reads 32
// problems of one point (coalesced); per-problem partial maxima and sums are
// combined in shared memory and leave the block with one atomic each.
constexpr int kChkY = 8;
__global__ void __launch_bounds__(32 * kChkY) k_check_reduce(MgDev g) {
  if (*g.alldone) return;
  const LvDev L = g.lv[g.ngrid - 1];
  const int P = g.P;
  const int p = blockIdx.x * 32 + threadIdx.x;
  const int ty = threadIdx.y;
  const size_t npt = (size_t)L.nx * L.ny;
  double m0 = 0.0, m1 = 0.0, s2 = 0.0, s3 = 0.0;
  const bool act = (p < P) && !g.done[p];
  if (act) {
    const size_t si = P, sj = (size_t)(L.nx + 2) * P;
    const double kx2 = g.kx2[p];
    for (size_t pt = (size_t)blockIdx.y * kChkY + ty; pt < npt; pt += (size_t)gridDim.y * kChkY) {
      const int i = 1 + (int)(pt % L.nx), j = 1 + (int)(pt / L.nx);
      const double *ph = &PH(L, P, i, j, p);
      const double v = ph[0];
      const double old = g.phif[pt * P + p];
      m0 = fmax(m0, fabs(v));
      m1 = fmax(m1, fabs(v - old));
      if (g.stop_rule == 1) {
        const double *cf = L.cof;
        double s = cf[pt] * ph[si];
        s = s + cf[npt + pt] * ph[si + sj];
        s = s + cf[2 * npt + pt] * ph[sj];
        s = s + cf[3 * npt + pt] * ph[sj - si];
        s = s + cf[4 * npt + pt] * ph[-(long)si];
        s = s + cf[5 * npt + pt] * ph[-(long)(si + sj)];
        s = s + cf[6 * npt + pt] * ph[-(long)sj];
        s = s + cf[7 * npt + pt] * ph[si - sj];
        const double c9v = ((-kx2 * cf[10 * npt + pt]) - cf[8 * npt + pt]) + cf[9 * npt + pt];
        s = s + c9v * v;
        const double b = L.rhs[pt * P + p];
        const double r = b - s;
        s2 += b * b;
        s3 += r * r;
      }
      g.phif[pt * P + p] = v;
    }
  }
  __shared__ double red[4][kChkY][32];
  red[0][ty][threadIdx.x] = m0;
  red[1][ty][threadIdx.x] = m1;
  red[2][ty][threadIdx.x] = s2;
  red[3][ty][threadIdx.x] = s3;
  __syncthreads();
  if (ty == 0 && act) {
    for (int y = 1; y < kChkY; ++y) {
      m0 = fmax(m0, red[0][y][threadIdx.x]);
      m1 = fmax(m1, red[1][y][threadIdx.x]);
      s2 += red[2][y][threadIdx.x];
      s3 += red[3][y][threadIdx.x];
    }
    atomic_max_pos(&g.red[4 * p], m0);
    atomic_max_pos(&g.red[4 * p + 1], m1);
    if (g.stop_rule == 1) {
      atomicAdd(&g.red[4 * p + 2], s2);
      atomicAdd(&g.red[4 * p + 3], s3);
    }
  }
}

// Relative change (MUDPACK) or, for the residual rule, relative residual
// (kx^2 = 0 problems included: their right-hand side was made compatible).
__global__ void k_check_finish(MgDev g, int iter, int last) {
  if (*g.alldone) return;
  __shared__ int active;
  if (threadIdx.x == 0) active = 0;
  __syncthreads();
  for (int p = threadIdx.x; p < g.P; p += blockDim.x) {
    if (g.done[p]) continue;
    g.cycles[p] = iter;
    double relmax = g.red[4 * p + 1];
    const double phmax = g.red[4 * p];
    if (phmax > 0.0) relmax = relmax / phmax;
    bool conv;
    double meas;
    if (g.stop_rule == 0) {
      meas = relmax;
      conv = (g.tol > 0.0) && (relmax <= g.tol);
    } else {
      const double bn = sqrt(g.red[4 * p + 2]);
      meas = (bn > 0.0) ? sqrt(g.red[4 * p + 3]) / bn : 0.0;
      conv = meas <= g.tol;
    }
    g.red[4 * p] = 0.0;
    g.red[4 * p + 1] = 0.0;
    g.red[4 * p + 2] = 0.0;
    g.red[4 * p + 3] = 0.0;
    g.red[4 * g.P + p] = meas;
    if (conv) g.done[p] = 1;
    else atomicAdd(&active, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && (active == 0 || last)) *g.alldone = 1;
}

// --------------------------------------------------------------------------
// Coarse levels 1..lc: one CTA per problem, everything in shared memory.
struct CoarseLv {
  int nx, ny;
  int phi, rhs, inv9, cof;  // offsets (doubles) into shared memory
};
struct CoarseArgs {
  MgDev g;
  const MgOp *ops;
  int nops;
  int intpol;
  int ncof;  // 4 (orthogonal) or 8
  CoarseLv lv[24];
  int scr;   // scratch offset
  int total; // doubles of shared memory
};

__device__ void c_relax(const CoarseArgs &A, double *sm, int level, int count, int &stale) {
  const CoarseLv &L = A.lv[level - 1];
  const int nx = L.nx, ny = L.ny;
  double *phi = sm + L.phi;
  const double *rhs = sm + L.rhs, *inv9 = sm + L.inv9, *cf = sm + L.cof;
  const size_t npt = (size_t)nx * ny;
  const int sj = nx + 2;
  const bool orth = A.g.orth;
  const bool onwrite = orth && (nx % 4 != 2);
  for (int sweep = 0; sweep < count; ++sweep) {
    for (int c = 1; c <= 4; ++c) {
      for (int r = (orth ? 0 : 1); r <= (orth ? 0 : 4); ++r) {
        const int nrow = (r == 0) ? ny : (ny - r) / 4 + 1;
        const int ncol = (nx + 3) / 4 + 1;
        for (int t = threadIdx.x; t < nrow * ncol; t += blockDim.x) {
          const int rowi = t / ncol, coli = t % ncol;
          const int j = (r == 0) ? 1 + rowi : r + 4 * rowi;
          if (j > ny) continue;
          const int i = first_i(c, j) + 4 * coli;
          if (i > nx) continue;
          const size_t pt = (size_t)(j - 1) * nx + (i - 1);
          double *ph = phi + j * sj + i;
          double s;
          if (orth) {
            s = cf[pt] * ph[1];
            s = s + cf[npt + pt] * ph[sj];
            s = s + cf[2 * npt + pt] * ph[-1];
            s = s + cf[3 * npt + pt] * ph[-sj];
          } else {
            s = cf[pt] * ph[1];
            s = s + cf[npt + pt] * ph[1 + sj];
            s = s + cf[2 * npt + pt] * ph[sj];
            s = s + cf[3 * npt + pt] * ph[sj - 1];
            s = s + cf[4 * npt + pt] * ph[-1];
            s = s + cf[5 * npt + pt] * ph[-1 - sj];
            s = s + cf[6 * npt + pt] * ph[-sj];
            s = s + cf[7 * npt + pt] * ph[1 - sj];
          }
          const double v = (rhs[pt] - s) * inv9[pt];
          *ph = v;
          if (onwrite) {
            if (i == nx - 1) phi[j * sj] = v;
            if (i == 2) phi[j * sj + nx + 1] = v;
          }
        }
        __syncthreads();
      }
      if (!onwrite || stale) {
        for (int j = 1 + threadIdx.x; j <= ny; j += blockDim.x) {
          phi[j * sj] = phi[j * sj + nx - 1];
          phi[j * sj + nx + 1] = phi[j * sj + 2];
        }
        stale = 0;
        __syncthreads();
      }
    }
  }
}

__device__ void c_restrict(const CoarseArgs &A, double *sm, int level, int p) {
  const CoarseLv &F = A.lv[level - 1], &C = A.lv[level - 2];
  const int nx = F.nx, ny = F.ny, ncx = C.nx, ncy = C.ny;
  const double *phi = sm + F.phi, *rhs = sm + F.rhs, *cf = sm + F.cof;
  double *scr = sm + A.scr;
  const size_t npt = (size_t)nx * ny;
  const int sj = nx + 2;
  const LvDev &G = A.g.lv[level - 1];
  const size_t gnpt = (size_t)G.nx * G.ny;
  const double kx2 = A.g.kx2[p];
  for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
    const int i = 1 + t % nx, j = 1 + t / nx;
    const double *ph = phi + j * sj + i;
    double s;
    if (A.ncof == 4) {
      s = cf[t] * ph[1];
      s = s + cf[npt + t] * ph[sj];
      s = s + cf[2 * npt + t] * ph[-1];
      s = s + cf[3 * npt + t] * ph[-sj];
    } else {
      s = cf[t] * ph[1];
      s = s + cf[npt + t] * ph[1 + sj];
      s = s + cf[2 * npt + t] * ph[sj];
      s = s + cf[3 * npt + t] * ph[sj - 1];
      s = s + cf[4 * npt + t] * ph[-1];
      s = s + cf[5 * npt + t] * ph[-1 - sj];
      s = s + cf[6 * npt + t] * ph[-sj];
      s = s + cf[7 * npt + t] * ph[1 - sj];
    }
    const double c9v = ((-kx2 * G.cof[10 * gnpt + t]) - G.cof[8 * gnpt + t]) + G.cof[9 * gnpt + t];
    s = s + c9v * ph[0];
    scr[j * sj + i] = rhs[t] - s;
  }
  __syncthreads();
  const int ix = (ncx == nx) ? 0 : 1, jy = (ncy == ny) ? 0 : 1;
  double *phic = sm + C.phi;
  double *rhsc = sm + C.rhs;
  for (int t = threadIdx.x; t < (ncx + 2) * (ncy + 2); t += blockDim.x) phic[t] = 0.0;
  for (int t = threadIdx.x; t < ncx * ncy; t += blockDim.x) {
    const int ic = 1 + t % ncx, jc = 1 + t / ncx;
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
    auto R = [&](int a, int b) { return scr[b * sj + a]; };
    rhsc[t] = (R(im1, jm1) + R(ip1, jm1) + R(im1, jp1) + R(ip1, jp1) +
               2. * (R(im1, j) + R(ip1, j) + R(i, jm1) + R(i, jp1)) + 4. * R(i, j)) * .0625;
  }
  __syncthreads();
}

// mode 0: cor2 (add); mode 1: FMG prolon2 (overwrite, ghosts of the rows
// set by prolon1 only)
__device__ void c_prolong(const CoarseArgs &A, double *sm, int level, int mode, int &stale) {
  const CoarseLv &F = A.lv[level - 1], &C = A.lv[level - 2];
  const int nx = F.nx, ny = F.ny, ncx = C.nx, ncy = C.ny;
  const bool ycoarse = ncy < ny;
  const bool cubic_x = !(A.intpol == 1 || ncx < 4), cubic_y = !(A.intpol == 1 || ncy < 4);
  const int sj = nx + 2, sjc = ncx + 2;
  double *q = (mode == 0) ? sm + A.scr : sm + F.phi;
  const double *pcs = sm + C.phi;
  const int nrows = ycoarse ? (ny + 1) / 2 : ny;
  for (int t = threadIdx.x; t < nrows * (nx + 2); t += blockDim.x) {
    const int i = t % (nx + 2), rr = t / (nx + 2);
    const int j = ycoarse ? 2 * rr + 1 : rr + 1;
    const int jc = ycoarse ? j / 2 + 1 : j;
    auto pc = [&](int ic) { return pcs[jc * sjc + ic]; };
    double v;
    if (i == 0) v = prolon1_at(nx - 1, ncx, nx, cubic_x, pc);
    else if (i == nx + 1) v = prolon1_at(2, ncx, nx, cubic_x, pc);
    else v = prolon1_at(i, ncx, nx, cubic_x, pc);
    q[j * sj + i] = v;
  }
  __syncthreads();
  double *phi = sm + F.phi;
  for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
    const int i = 1 + t % nx, j = 1 + t / nx;
    auto Q = [&](int jj) { return q[jj * sj + i]; };
    const bool even = ycoarse && !(j & 1);
    double v;
    if (even) {
      if (!cubic_y) v = 0.5 * (Q(j - 1) + Q(j + 1));
      else if (j >= 4 && j <= ny - 3) v = (-Q(j - 3) + 9. * (Q(j - 1) + Q(j + 1)) - Q(j + 3)) * .0625;
      else if (j == 2) v = (5. * Q(1) + 15. * Q(3) - 5. * Q(5) + Q(7)) * .0625;
      else v = (5. * Q(ny) + 15. * Q(ny - 2) - 5. * Q(ny - 4) + Q(ny - 6)) * .0625;
    } else {
      v = Q(j);
    }
    if (mode == 1) {
      if (even) phi[j * sj + i] = v;
    } else {
      const double nv = phi[j * sj + i] + v;
      phi[j * sj + i] = nv;
      if (i == nx - 1) phi[j * sj] = nv;
      if (i == 2) phi[j * sj + nx + 1] = nv;
    }
  }
  if (mode == 1 && ycoarse) stale = 1;
  __syncthreads();
}

__global__ void k_coarse(CoarseArgs A) {
  extern __shared__ double sm[];
  const MgDev &g = A.g;
  const int p = blockIdx.x;
  if (*g.alldone || g.done[p]) return;
  const int P = g.P;
  // load every coarse level (phi with ghosts, rhs, 1/c9, coefficients)
  for (int l = 1; l <= g.lc; ++l) {
    const CoarseLv &L = A.lv[l - 1];
    const LvDev &G = g.lv[l - 1];
    const int nph = (L.nx + 2) * (L.ny + 2), npt = L.nx * L.ny;
    for (int t = threadIdx.x; t < nph; t += blockDim.x) sm[L.phi + t] = G.phi[(size_t)t * P + p];
    for (int t = threadIdx.x; t < npt; t += blockDim.x) {
      sm[L.rhs + t] = G.rhs[(size_t)t * P + p];
      sm[L.inv9 + t] = G.inv9[(size_t)t * P + p];
    }
    const int ncof = A.ncof;
    for (int t = threadIdx.x; t < ncof * npt; t += blockDim.x) {
      const int l8 = t / npt, pt = t % npt;
      const int src = (ncof == 4) ? 2 * l8 : l8;  // c1,c3,c5,c7 or c1..c8
      sm[L.cof + t] = G.cof[(size_t)src * npt + pt];
    }
  }
  __syncthreads();
  int stale[24];
  for (int l = 0; l < 24; ++l) stale[l] = 0;
  for (int o = 0; o < A.nops; ++o) {
    const MgOp op = A.ops[o];
    if (op.kind == OP_RELAX) c_relax(A, sm, op.level, op.count, stale[op.level - 1]);
    else if (op.kind == OP_RESTRICT) c_restrict(A, sm, op.level, p);
    else if (op.kind == OP_COR2) c_prolong(A, sm, op.level, 0, stale[op.level - 1]);
    else if (op.kind == OP_PROLONG) c_prolong(A, sm, op.level + 1, 1, stale[op.level]);
  }
  // store phi and rhs of every coarse level
  for (int l = 1; l <= g.lc; ++l) {
    const CoarseLv &L = A.lv[l - 1];
    const LvDev &G = g.lv[l - 1];
    const int nph = (L.nx + 2) * (L.ny + 2), npt = L.nx * L.ny;
    for (int t = threadIdx.x; t < nph; t += blockDim.x) G.phi[(size_t)t * P + p] = sm[L.phi + t];
    for (int t = threadIdx.x; t < npt; t += blockDim.x) G.rhs[(size_t)t * P + p] = sm[L.rhs + t];
  }
}

unsigned nblk(long n, int bs) {
  long b = (n + bs - 1) / bs;
  if (b < 1) b = 1;
  if (b > 65535L * 32) b = 65535L * 32;
  return (unsigned)b;
}

}  // namespace

void mg_work_free(MgWork &w) {
  if (w.pool) cudaFree(w.pool);
  if (w.flags) cudaFree(w.flags);
  w = MgWork{};
}

// Work arrays for up to pmax problems; kx2 is left for the caller to fill.
void mg_work_alloc(Ctx &c, MgWork &w, int pmax) {
  const MgPlan &P = c.mg;
  mg_work_free(w);
  size_t tot = 0;
  std::vector<size_t> ph(P.ngrid), rh(P.ngrid), iv(P.ngrid);
  for (int l = 0; l < P.ngrid; ++l) {
    const MgLevel &L = P.lv[l];
    ph[l] = tot;
    tot += (size_t)(L.nx + 2) * (L.ny + 2) * pmax;
    rh[l] = tot;
    tot += (size_t)L.nx * L.ny * pmax;
    iv[l] = tot;
    tot += (size_t)L.nx * L.ny * pmax;
  }
  const size_t scr_off = tot;
  tot += (size_t)(P.nfx + 2) * (P.nfy + 2) * pmax;
  const size_t phif_off = tot;
  tot += (size_t)P.nfx * P.nfy * pmax;
  const size_t red_off = tot;
  tot += (size_t)6 * pmax + 8;
  const size_t kx_off = tot;
  tot += pmax;
  EK_CUDA(cudaMalloc(&w.pool, tot * sizeof(double)));
  EK_CUDA(cudaMalloc(&w.flags, sizeof(int) * (3 * pmax + 4)));
  w.phi.resize(P.ngrid);
  w.rhs.resize(P.ngrid);
  w.inv9.resize(P.ngrid);
  for (int l = 0; l < P.ngrid; ++l) {
    w.phi[l] = w.pool + ph[l];
    w.rhs[l] = w.pool + rh[l];
    w.inv9[l] = w.pool + iv[l];
  }
  w.scratch = w.pool + scr_off;
  w.phif = w.pool + phif_off;
  w.red = w.pool + red_off;
  w.kx2 = w.pool + kx_off;
  w.done = w.flags;
  w.cycles = w.flags + pmax;
  w.alldone = w.flags + 2 * pmax;
  w.iter = w.flags + 2 * pmax + 1;
  w.idx = w.flags + 2 * pmax + 4;
  w.pmax = pmax;
}

// Coefficients of every level, the main work arrays with the projection
// solves' kx^2 per problem (problem 2I+part is mode I), the operation list.
void mg_alloc(Ctx &c, int pmax) {
  MgPlan &P = c.mg;
  if (c.mg_cof_pool) {
    cudaFree(c.mg_cof_pool);
    c.mg_cof_pool = nullptr;
  }
  size_t tot = 0;
  for (auto &L : P.lv) tot += (size_t)11 * L.nx * L.ny;
  EK_CUDA(cudaMalloc(&c.mg_cof_pool, tot * sizeof(double)));
  tot = 0;
  for (int l = 0; l < P.ngrid; ++l) {
    P.lv[l].cof = c.mg_cof_pool + tot;
    tot += (size_t)11 * P.lv[l].nx * P.lv[l].ny;
    EK_CUDA(cudaMemcpy(P.lv[l].cof, P.cof_host[l].data(), sizeof(double) * P.cof_host[l].size(), cudaMemcpyHostToDevice));
  }
  mg_work_alloc(c, c.mgw, pmax);
  c.mg_kx2_host.assign(pmax, 0.0);
  for (int q = 0; q < pmax; ++q) c.mg_kx2_host[q] = c.kx2_h[std::min(q / 2, c.d.NX2P)];
  EK_CUDA(cudaMemcpy(c.mgw.kx2, c.mg_kx2_host.data(), sizeof(double) * pmax, cudaMemcpyHostToDevice));
  if (P.ops_dev) cudaFree(P.ops_dev);
  EK_CUDA(cudaMalloc(&P.ops_dev, sizeof(MgOp) * P.ops.size()));
  EK_CUDA(cudaMemcpy(P.ops_dev, P.ops.data(), sizeof(MgOp) * P.ops.size(), cudaMemcpyHostToDevice));
  if (c.p.mg_fast) mgfast_alloc(c, pmax);
  if (c.mg_null_part) cudaFree(c.mg_null_part);
  c.mg_null_part = nullptr;
  EK_CUDA(cudaMalloc(&c.mg_null_part, sizeof(double) * (size_t)pmax * kNullChunks));
}

int mg_solve(Ctx &c, int nprob, const double *kx2_dev, const double *kx2_host, ek_mg_stats *st) {
  const int r = c.p.mg_fast ? mgfast_solve(c, nprob, kx2_dev, kx2_host, st)
                            : mg_solve_exact(c, c.mgw, nprob, kx2_dev, st, 0);
  if (c.graph_slot < 0 && (r == EK_OK || r == EK_ERR_NOT_CONVERGED)) {  // a captured solve counts after the step
    c.mg_solved_total += nprob;
    c.mg_nc_total += c.last_stats.n_not_converged;
  }
  return r;
}

// One batched MUDPACK-exact solve in the work arrays w: the finest rhs must
// already be in w.rhs[ngrid-1] (nprob problems, problem fastest); the
// solution is left in w.phif.  max_cycles > 0 stops issuing the schedule
// after that many k-cycles (a batch whose problems all stop by then).
int mg_solve_exact(Ctx &c, MgWork &w, int nprob, const double *kx2_dev, ek_mg_stats *st, int max_cycles) {
  if (nprob > w.pmax) return EK_ERR_ARG;
  const bool wellposed = c.p.mg_stop == EK_MG_STOP_RESIDUAL;
  if (wellposed) mg_null_project(c, w.rhs[c.mg.ngrid - 1], nprob, kx2_dev);
  mg_exact_enqueue(c, w, nprob, kx2_dev, max_cycles, true);
  if (wellposed) mg_null_mean(c, w.phif, nprob, kx2_dev);
  return mg_exact_stats(c, w, nprob, st);
}

namespace {
// Sum over a block of 256 threads (fixed order: deterministic).
__device__ __forceinline__ double block_sum256(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = (threadIdx.x < 8) ? sh[threadIdx.x] : 0.0;
    for (int o = 4; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) sh[8] = v;
  }
  __syncthreads();
  const double r = sh[8];
  __syncthreads();
  return r;
}

// The kx^2 = 0 problems' projections, b <- b - (z.b) z (z of unit norm)
// and phi <- phi - mean(phi), over the npt finest points in two passes:
// kNullChunks blocks per problem form partial sums of their chunks, then
// each block adds the partials in chunk order and updates its chunk.  (One
// block per problem spent 0.24 ms a launch on two problems' 99k points.)
// Grid (kNullChunks, P); problems with kx^2 != 0 return at once.
__device__ __forceinline__ void null_chunk(int npt, int &t0, int &t1) {
  const int per = (npt + kNullChunks - 1) / kNullChunks;
  t0 = (int)blockIdx.x * per;
  t1 = min(npt, t0 + per);
}
__global__ void __launch_bounds__(256) k_null_partial(const double *v, int P, const double *z, int npt,
                                                       const double *kx2, double *part) {
  __shared__ double sh[9];
  const int p = blockIdx.y;
  if (kx2[p] != 0.0) return;
  int t0, t1;
  null_chunk(npt, t0, t1);
  double s = 0.0;
  for (int t = t0 + threadIdx.x; t < t1; t += 256) s += (z ? z[t] : 1.0) * v[(size_t)t * P + p];
  s = block_sum256(s, sh);
  if (threadIdx.x == 0) part[(size_t)p * kNullChunks + blockIdx.x] = s;
}
// mean = 0: v -= (sum) z; mean = 1: v -= sum / npt
__global__ void __launch_bounds__(256) k_null_apply(double *v, int P, const double *z, int npt, const double *kx2,
                                                     const double *part, int mean) {
  const int p = blockIdx.y;
  if (kx2[p] != 0.0) return;
  double s = 0.0;
  for (int q = 0; q < kNullChunks; ++q) s += part[(size_t)p * kNullChunks + q];
  int t0, t1;
  null_chunk(npt, t0, t1);
  if (mean) {
    const double m = s / (double)npt;
    for (int t = t0 + threadIdx.x; t < t1; t += 256) v[(size_t)t * P + p] -= m;
  } else {
    for (int t = t0 + threadIdx.x; t < t1; t += 256) v[(size_t)t * P + p] -= s * z[t];
  }
}
}  // namespace

void mg_null_project(Ctx &c, double *rhs_finest, int nprob, const double *kx2_dev) {
  if (!c.mg_z) throw CudaError("well-posed kx = 0 solve: the left null vector is missing");
  const int npt = c.mg.nfx * c.mg.nfy;
  KScope ks(c, KC_MG_SETUP, 0.0);
  const dim3 grid(kNullChunks, (unsigned)nprob);
  k_null_partial<<<grid, 256, 0, c.stream>>>(rhs_finest, nprob, c.mg_z, npt, kx2_dev, c.mg_null_part);
  after_launch(c);
  k_null_apply<<<grid, 256, 0, c.stream>>>(rhs_finest, nprob, c.mg_z, npt, kx2_dev, c.mg_null_part, 0);
  after_launch(c);
}

void mg_null_mean(Ctx &c, double *phi_finest, int nprob, const double *kx2_dev) {
  const int npt = c.mg.nfx * c.mg.nfy;
  KScope ks(c, KC_MG_SETUP, 0.0);
  const dim3 grid(kNullChunks, (unsigned)nprob);
  k_null_partial<<<grid, 256, 0, c.stream>>>(phi_finest, nprob, nullptr, npt, kx2_dev, c.mg_null_part);
  after_launch(c);
  k_null_apply<<<grid, 256, 0, c.stream>>>(phi_finest, nprob, nullptr, npt, kx2_dev, c.mg_null_part, 1);
  after_launch(c);
}

// k_coarse's shared-memory limit, set once per process (outside any stream
// capture; contexts stepping on several host threads may get here together).
void mg_exact_attributes() {
  static std::once_flag once;
  std::call_once(once, [] {
    EK_CUDA(cudaFuncSetAttribute(k_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  });
}

// The launches of one exact solve on c.stream.  poll: stop issuing cycles
// once every problem is done (the host waits on the stream's progress).
void mg_exact_enqueue(Ctx &c, MgWork &w, int nprob, const double *kx2_dev, int max_cycles, bool poll) {
  MgPlan &PL = c.mg;
  MgDev g{};
  g.P = nprob;
  g.ngrid = PL.ngrid;
  g.lc = PL.lc;
  g.orth = PL.orth ? 1 : 0;
  for (int l = 0; l < PL.ngrid; ++l) g.lv[l] = LvDev{PL.lv[l].nx, PL.lv[l].ny, w.phi[l], w.rhs[l], PL.lv[l].cof, w.inv9[l]};
  g.scr = w.scratch;
  g.kx2 = kx2_dev;
  g.phif = w.phif;
  g.red = w.red;
  g.done = w.done;
  g.cycles = w.cycles;
  g.alldone = w.alldone;
  g.tol = c.p.mg_tol;
  g.stop_rule = c.p.mg_stop;
  const int bs = 256;
  cudaStream_t s = c.stream;
  EK_CUDA(cudaMemsetAsync(w.flags, 0, sizeof(int) * (2 * w.pmax + 4), s));
  EK_CUDA(cudaMemsetAsync(w.red, 0, sizeof(double) * (6 * w.pmax + 8), s));
  for (int l = 1; l <= PL.ngrid; ++l) {
    const long n = (long)PL.lv[l - 1].nx * PL.lv[l - 1].ny * nprob;
    KScope ks(c, KC_MG_SETUP, 8.0 * n);
    k_inv9<<<nblk(n, bs), bs, 0, s>>>(g, l);
    after_launch(c);
  }
  // coarse-kernel shared memory layout
  CoarseArgs A{};
  A.g = g;
  A.intpol = c.p.mg_intpol;
  A.ncof = PL.orth ? 4 : 8;
  int off = 0;
  int maxph = 0;
  for (int l = 1; l <= PL.lc; ++l) {
    const MgLevel &L = PL.lv[l - 1];
    A.lv[l - 1].nx = L.nx;
    A.lv[l - 1].ny = L.ny;
    A.lv[l - 1].phi = off; off += (L.nx + 2) * (L.ny + 2);
    A.lv[l - 1].rhs = off; off += L.nx * L.ny;
    A.lv[l - 1].inv9 = off; off += L.nx * L.ny;
    A.lv[l - 1].cof = off; off += A.ncof * L.nx * L.ny;
    maxph = std::max(maxph, (L.nx + 2) * (L.ny + 2));
  }
  A.scr = off;
  off += maxph;
  A.total = off;
  const size_t smem = sizeof(double) * off;
  mg_exact_attributes();
  const MgOp *ops_dev_cached = PL.ops_dev;
  const int lc = PL.lc;
  auto is_coarse = [&](const MgOp &o) {
    switch (o.kind) {
      case OP_RELAX: return o.level <= lc;
      case OP_RESTRICT: return o.level <= lc;
      case OP_COR2: return o.level <= lc;
      case OP_PROLONG: return o.level + 1 <= lc;
      default: return false;
    }
  };
  std::vector<int> stale(PL.ngrid + 1, 0);
  const int nops = (int)PL.ops.size();
  int o = 0;
  int ncheck = 0, maxcheck = 0;
  for (const MgOp &op : PL.ops) maxcheck += (op.kind == OP_CHECK);
  if (max_cycles > 0) maxcheck = std::min(maxcheck, max_cycles);
  if (poll) {
    c.poll.init();
    c.poll.reset();
  }
  bool stop = false;
  while (o < nops && ncheck < maxcheck && !stop) {
    const MgOp &op = PL.ops[o];
    if (is_coarse(op)) {
      int e = o;
      while (e < nops && is_coarse(PL.ops[e])) ++e;
      A.ops = ops_dev_cached + o;
      A.nops = e - o;
      double cb = 0.0;
      for (int l = 1; l <= lc; ++l) {
        const MgLevel &Lq = PL.lv[l - 1];
        cb += 8.0 * nprob * (2.0 * (Lq.nx + 2) * (Lq.ny + 2) + 3.0 * Lq.nx * Lq.ny);
      }
      KScope ks(c, KC_MG_COARSE, cb);
      k_coarse<<<nprob, 256, smem, s>>>(A);
      after_launch(c);
      o = e;
      continue;
    }
    const MgLevel &L = PL.lv[op.level - 1];
    switch (op.kind) {
      case OP_TRSFC: {
        double tb = 8.0 * PL.nfx * PL.nfy * nprob;
        for (int l = 1; l <= PL.ngrid; ++l) tb += 8.0 * nprob * ((PL.lv[l - 1].nx + 2) * (PL.lv[l - 1].ny + 2) + 2.0 * PL.lv[l - 1].nx * PL.lv[l - 1].ny);
        KScope ks(c, KC_MG_SETUP, tb);
        for (int l = 1; l <= PL.ngrid; ++l) {
          const size_t n = (size_t)(PL.lv[l - 1].nx + 2) * (PL.lv[l - 1].ny + 2) * nprob;
          k_zero<<<nblk((long)n, bs), bs, 0, s>>>(w.phi[l - 1], n);
          after_launch(c);
        }
        {
          const size_t n = (size_t)PL.nfx * PL.nfy * nprob;
          k_zero<<<nblk((long)n, bs), bs, 0, s>>>(w.phif, n);
          after_launch(c);
        }
        for (int l = PL.ngrid; l >= 2; --l) {
          const long n = (long)PL.lv[l - 2].nx * PL.lv[l - 2].ny * nprob;
          k_inject<<<nblk(n, bs), bs, 0, s>>>(g, l);
          after_launch(c);
        }
        break;
      }
      case OP_RELAX: {
        KScope ks(c, KC_MG_RELAX, 32.0 * L.nx * L.ny * nprob * op.count);
        const bool onwrite = PL.orth && (L.nx % 4 != 2);
        const int ncol = (L.nx + 3) / 4 + 1;
        for (int sw = 0; sw < op.count; ++sw)
          for (int col = 1; col <= 4; ++col) {
            for (int r = (PL.orth ? 0 : 1); r <= (PL.orth ? 0 : 4); ++r) {
              const int nrow = (r == 0) ? L.ny : (L.ny - r) / 4 + 1;
              k_relax_phase<<<nblk((long)nrow * ncol * nprob, bs), bs, 0, s>>>(g, op.level, col, r, onwrite ? 1 : 0);
              after_launch(c);
            }
            if (!onwrite || stale[op.level]) {
              k_ghost<<<nblk((long)L.ny * nprob, bs), bs, 0, s>>>(g, op.level);
              after_launch(c);
              stale[op.level] = 0;
            }
          }
        break;
      }
      case OP_RESTRICT: {
        const MgLevel &Cq = PL.lv[op.level - 2];
        KScope ks(c, KC_MG_TRANSFER, 8.0 * nprob * (4.0 * L.nx * L.ny + 2.0 * (Cq.nx + 2) * (Cq.ny + 2)));
        k_resid<<<nblk((long)L.nx * L.ny * nprob, bs), bs, 0, s>>>(g, op.level);
        after_launch(c);
        const MgLevel &C = PL.lv[op.level - 2];
        k_res2<<<nblk((long)(C.nx + 2) * (C.ny + 2) * nprob, bs), bs, 0, s>>>(g, op.level);
        after_launch(c);
        break;
      }
      case OP_COR2:
      case OP_PROLONG: {
        KScope ks(c, KC_MG_TRANSFER, 8.0 * nprob * 4.0 * PL.lv[(op.kind == OP_COR2 ? op.level : op.level + 1) - 1].nx *
                                         PL.lv[(op.kind == OP_COR2 ? op.level : op.level + 1) - 1].ny);
        const int fine = (op.kind == OP_COR2) ? op.level : op.level + 1;
        const int mode = (op.kind == OP_COR2) ? 0 : 1;
        const MgLevel &F = PL.lv[fine - 1];
        k_prolong_x<<<nblk((long)(F.ny + 1) * (F.nx + 2) * nprob, bs), bs, 0, s>>>(g, fine, c.p.mg_intpol, mode);
        after_launch(c);
        k_prolong_y<<<nblk((long)F.nx * F.ny * nprob, bs), bs, 0, s>>>(g, fine, c.p.mg_intpol, mode);
        after_launch(c);
        if (mode == 1 && PL.lv[fine - 2].ny < F.ny) stale[fine] = 1;
        break;
      }
      case OP_CHECK: {
        KScope ks(c, KC_MG_CHECK, 8.0 * nprob * PL.nfx * PL.nfy * (c.p.mg_stop == 1 ? 4.0 : 3.0));
        ++ncheck;
        const MgLevel &F = PL.lv[PL.ngrid - 1];
        const long npt = (long)F.nx * F.ny;
        const int gy = (int)std::min<long>((npt + kChkY - 1) / kChkY, std::max<long>(1, 2048 / ((nprob + 31) / 32)));
        k_check_reduce<<<dim3((nprob + 31) / 32, gy), dim3(32, kChkY), 0, s>>>(g);
        after_launch(c);
        k_check_finish<<<1, 256, 0, s>>>(g, op.count, ncheck == maxcheck ? 1 : 0);
        after_launch(c);
        if (poll && c.poll.after_check(w.alldone, s)) stop = true;
        break;
      }
      default:
        break;
    }
    ++o;
  }
}

// Per-problem results of an exact solve in w (synchronises c.stream).
int mg_exact_stats(Ctx &c, MgWork &w, int nprob, ek_mg_stats *st) {
  cudaStream_t s = c.stream;
  std::vector<int> cyc(nprob), done(nprob);
  std::vector<double> meas(nprob);
  EK_CUDA(cudaMemcpyAsync(cyc.data(), w.cycles, sizeof(int) * nprob, cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaMemcpyAsync(done.data(), w.done, sizeof(int) * nprob, cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaMemcpyAsync(meas.data(), w.red + 4 * nprob, sizeof(double) * nprob, cudaMemcpyDeviceToHost, s));
  EK_CUDA(cudaStreamSynchronize(s));
  ek_mg_stats S{};
  S.nprob = nprob;
  S.min_cycles = nprob ? (1 << 30) : 0;
  for (int p = 0; p < nprob; ++p) {
    S.min_cycles = std::min(S.min_cycles, cyc[p]);
    S.max_cycles = std::max(S.max_cycles, cyc[p]);
    if (done[p] != 1) S.n_not_converged++;
    if (c.p.mg_stop == 0) S.max_relchange = std::max(S.max_relchange, meas[p]);
    else S.max_residual = std::max(S.max_residual, meas[p]);
  }
  c.last_stats = S;
  if (st) *st = S;
  return S.n_not_converged ? EK_ERR_NOT_CONVERGED : EK_OK;
}

}  // namespace ek
