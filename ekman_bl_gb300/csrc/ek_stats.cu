// Plane statistics of SAVE_STATS_CURVI (src/flow_statistics.F90:2-1023):
// averages over the periodic x direction of products of the fluctuations,
// gradients of the mode-0 (x-mean) fields, bulk values, and the state
// round trip through physical space that the routine leaves behind.
//
//   k_stats_lines   one warp per (k,j) line: the x-sums of u'u', u'v', ...
//                   over I = 0..NX-1 (the loops run to MIN(NXP, NXP_L) =
//                   NX-1 on one rank), reading the five physical fields once
//   k_stats_plane   one thread per (k,j): TKE, the mean-gradient planes,
//                   Rig (flow_statistics.F90:165-177, 216-320, 460-552)
//   k_stats_edges   one block: the boundary copies, in the reference's order
//   k_stats_reduce  one block: UBULK, VBULK, THBULK and the INT_JACOB-
//                   weighted rms averages (:80-95, :540-553, :851-879)
//   k_stats_means   mode-0 planes after the transforms back (plot_binary)
//
// The pointwise 2-D formulas use explicitly rounded operations in the
// reference's evaluation order, so they equal a separately rounded CPU
// evaluation bit for bit; the x-sums and the bulk sums are tree reductions.
#include <cmath>

#include "ek_internal.h"

namespace ek {
namespace {

enum {
  S_URMS, S_VRMS, S_WRMS, S_UV, S_UW, S_WV, S_PU, S_PV, S_THRMS, S_THV, S_THW,
  S_TKE, S_DUDY, S_DWDY, S_DUDZ, S_DWDZ, S_OMX, S_DTHDY, S_DTHDZ, S_RIG,
  S_M1, S_M2, S_M3, S_MP, S_MTH, S_N
};
enum { R_UBULK, R_VBULK, R_THBULK, R_AREA, R_URMS, R_VRMS, R_WRMS, R_PROBE3, R_PROBE1, R_N };

struct StatArgs {
  Dims d;
  const cplx_t *CU1, *CU2, *CU3, *CP, *CTH;
  const double *U1, *U2, *U3, *P, *TH;
  const double *jac, *c11, *c12, *c21, *c22, *th_bar;
  double *S;      // S_N planes of (NZ+2)(NY+2)
  double *R;      // R_N scalars
  int th, cont_strat;
  double ri, tke_fac;
  int tke_scaled;
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(256) k_stats_lines(StatArgs a) {
  const Dims &d = a.d;
  const int line = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (line >= d.NZ2 * d.NY2) return;
  const int k = line % d.NZ2, j = line / d.NZ2;
  const size_t c0 = d.ic(0, k, j), p0 = d.ip(0, k, j);
  const double m1 = a.CU1[c0].re, m2 = a.CU2[c0].re, m3 = a.CU3[c0].re;
  // p_mean is filled on K = 1..NZ, J = 1..NY only (flow_statistics.F90:115-120);
  // elsewhere it keeps its fresh allocation, taken as zero
  const bool pin = k >= 1 && k <= d.NZ && j >= 1 && j <= d.NY;
  const double mp = pin ? a.CP[c0].re : 0.0;
  const double mt = a.th ? a.CTH[c0].re : 0.0;
  double s11 = 0, s22 = 0, s33 = 0, s12 = 0, s13 = 0, s32 = 0, s3p = 0, s2p = 0, stt = 0, st2 = 0, st3 = 0;
  for (int i = lane; i < d.NX; i += 32) {
    const double u1 = a.U1[p0 + i] - m1, u2 = a.U2[p0 + i] - m2, u3 = a.U3[p0 + i] - m3;
    const double pp = a.P[p0 + i] - mp;
    s11 += u1 * u1;
    s22 += u2 * u2;
    s33 += u3 * u3;
    s12 += u1 * u2;
    s13 += u1 * u3;
    s32 += u3 * u2;
    s3p += u3 * pp;
    s2p += u2 * pp;
    if (a.th) {
      const double t = a.TH[p0 + i] - mt;
      stt += t * t;
      st2 += t * u2;
      st3 += t * u3;
    }
  }
  s11 = warp_sum(s11); s22 = warp_sum(s22); s33 = warp_sum(s33);
  s12 = warp_sum(s12); s13 = warp_sum(s13); s32 = warp_sum(s32);
  s3p = warp_sum(s3p); s2p = warp_sum(s2p);
  if (a.th) { stt = warp_sum(stt); st2 = warp_sum(st2); st3 = warp_sum(st3); }
  if (lane != 0) return;
  const size_t n2 = (size_t)d.NZ2 * d.NY2, o = (size_t)j * d.NZ2 + k;
  const double nx = (double)d.NX;
  a.S[S_URMS * n2 + o] = __dsqrt_rn(__ddiv_rn(s11, nx));
  a.S[S_VRMS * n2 + o] = __dsqrt_rn(__ddiv_rn(s22, nx));
  a.S[S_WRMS * n2 + o] = __dsqrt_rn(__ddiv_rn(s33, nx));
  // the Reynolds stresses are computed on K = 1..NZ (flow_statistics.F90:181-207)
  const bool kin = k >= 1 && k <= d.NZ;
  a.S[S_UV * n2 + o] = kin ? __ddiv_rn(s12, nx) : 0.0;
  a.S[S_UW * n2 + o] = kin ? __ddiv_rn(s13, nx) : 0.0;
  a.S[S_WV * n2 + o] = kin ? __ddiv_rn(s32, nx) : 0.0;
  a.S[S_PU * n2 + o] = kin ? __ddiv_rn(s3p, nx) : 0.0;
  a.S[S_PV * n2 + o] = kin ? __ddiv_rn(s2p, nx) : 0.0;
  if (a.th) {
    a.S[S_THRMS * n2 + o] = __dsqrt_rn(__ddiv_rn(stt, nx));
    a.S[S_THV * n2 + o] = __ddiv_rn(st2, nx);
    a.S[S_THW * n2 + o] = __ddiv_rn(st3, nx);
  }
}

// 0.125 * (A(K,J,1) + A(K,J+1,1) + A(K,J,2) + A(K+1,J,2)): a metric averaged
// to the cell centre
__device__ __forceinline__ double cavg(const Dims &d, const double *A, int k, int j) {
  const double s = add(add(add(A[d.m3(k, j, 1)], A[d.m3(k, j + 1, 1)]), A[d.m3(k, j, 2)]), A[d.m3(k + 1, j, 2)]);
  return mul(0.125, s);
}

__global__ void __launch_bounds__(256) k_stats_plane(StatArgs a) {
  const Dims &d = a.d;
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= d.NZ2 * d.NY2) return;
  const int k = o % d.NZ2, j = o / d.NZ2;
  const size_t n2 = (size_t)d.NZ2 * d.NY2;
  auto R = [&](const cplx_t *F, int kk, int jj) { return F[d.ic(0, kk, jj)].re; };
  {
    const double v1 = R(a.CU1, k, j), v2 = R(a.CU2, k, j), v3 = R(a.CU3, k, j);
    const double e = add(add(mul(v1, v1), mul(v2, v2)), mul(v3, v3));
    a.S[S_TKE * n2 + o] = a.tke_scaled ? mul(e, a.tke_fac) : e;
  }
  double dudy = 0.0, dwdy = 0.0, dudz = 0.0, dwdz = 0.0, omx = 0.0, dthdy = 0.0, dthdz = 0.0, rig = 0.0;
  const bool inner = k >= 1 && k <= d.NZ && j >= 1 && j <= d.NY;
  if (k >= d.ZS && k <= d.ZE && j >= d.JS && j <= d.JE) {
    const double c12 = cavg(d, a.c12, k, j), c22 = cavg(d, a.c22, k, j), J = a.jac[d.m2(k, j)];
    dudy = __ddiv_rn(add(mul(c12, sub(R(a.CU1, k + 1, j), R(a.CU1, k - 1, j))),
                         mul(c22, sub(R(a.CU1, k, j + 1), R(a.CU1, k, j - 1)))), J);
    dwdy = __ddiv_rn(add(mul(c12, sub(R(a.CU3, k + 1, j), R(a.CU3, k - 1, j))),
                         mul(c22, sub(R(a.CU3, k, j + 1), R(a.CU3, k, j - 1)))), J);
  }
  if (inner) {
    const double c11 = cavg(d, a.c11, k, j), c12 = cavg(d, a.c12, k, j);
    const double c21 = cavg(d, a.c21, k, j), c22 = cavg(d, a.c22, k, j), J = a.jac[d.m2(k, j)];
    dudz = __ddiv_rn(add(mul(c21, sub(R(a.CU1, k, j + 1), R(a.CU1, k, j - 1))),
                         mul(c11, sub(R(a.CU1, k + 1, j), R(a.CU1, k - 1, j)))), J);
    dwdz = __ddiv_rn(add(mul(c21, sub(R(a.CU3, k, j + 1), R(a.CU3, k, j - 1))),
                         mul(c11, sub(R(a.CU3, k + 1, j), R(a.CU3, k - 1, j)))), J);
    const double w = __ddiv_rn(add(mul(c12, sub(R(a.CU3, k + 1, j), R(a.CU3, k - 1, j))),
                                   mul(c22, sub(R(a.CU3, k, j + 1), R(a.CU3, k, j - 1)))), J);
    const double v = __ddiv_rn(add(mul(c21, sub(R(a.CU2, k, j + 1), R(a.CU2, k, j - 1))),
                                   mul(c11, sub(R(a.CU2, k + 1, j), R(a.CU2, k - 1, j)))), J);
    omx = sub(w, v);
    if (a.th) {
      dthdy = __ddiv_rn(add(mul(c12, sub(R(a.CTH, k + 1, j), R(a.CTH, k - 1, j))),
                            mul(c22, sub(R(a.CTH, k, j + 1), R(a.CTH, k, j - 1)))), J);
      if (!a.cont_strat) {
        const double *T = a.th_bar;
        dthdy = add(dthdy, __ddiv_rn(add(mul(c12, sub(T[d.m2(k + 1, j)], T[d.m2(k - 1, j)])),
                                         mul(c22, sub(T[d.m2(k, j + 1)], T[d.m2(k, j - 1)]))), J));
      }
      dthdz = __ddiv_rn(add(mul(c21, sub(R(a.CTH, k, j + 1), R(a.CTH, k, j - 1))),
                            mul(c11, sub(R(a.CTH, k + 1, j), R(a.CTH, k - 1, j)))), J);
      // gradient Richardson number (flow_statistics.F90:528-548)
      const double b = a.cont_strat ? sub(dthdy, 1.0) : dthdy;
      const double nri = -a.ri;
      rig = (dwdy == 0.0) ? mul(mul(nri, b), 1.0e18) : __ddiv_rn(mul(nri, b), add(mul(dwdy, dwdy), mul(dudy, dudy)));
    }
  }
  a.S[S_DUDY * n2 + o] = dudy;
  a.S[S_DWDY * n2 + o] = dwdy;
  a.S[S_DUDZ * n2 + o] = dudz;
  a.S[S_DWDZ * n2 + o] = dwdz;
  a.S[S_OMX * n2 + o] = omx;
  if (a.th) {
    a.S[S_DTHDY * n2 + o] = dthdy;
    a.S[S_DTHDZ * n2 + o] = dthdz;
    a.S[S_RIG * n2 + o] = rig;
  }
}

// Boundary copies (flow_statistics.F90:230-235, 254-264, 322-325, 474-482,
// 512-520): first the copies from the first interior row, then the ones
// that read those copies (dudz(1,J) = dudz(2,J) after dudz(1,0) = dudz(1,1);
// the extrapolation of dthdy(K,0) over K = 0..NZ+1 after dthdy(0,J)).
__global__ void __launch_bounds__(1024) k_stats_edges(StatArgs a) {
  const Dims &d = a.d;
  const size_t n2 = (size_t)d.NZ2 * d.NY2;
  const int NY = d.NY, NZ = d.NZ;
  auto at = [&](int s, int k, int j) -> double & { return a.S[s * n2 + (size_t)j * d.NZ2 + k]; };
  const int vel[5] = {S_DUDY, S_DWDY, S_DUDZ, S_DWDZ, S_OMX};
  const int sca[2] = {S_DTHDY, S_DTHDZ};
  for (int k = 1 + threadIdx.x; k <= NZ; k += blockDim.x) {
    for (int s : vel) {
      at(s, k, 0) = at(s, k, 1);
      at(s, k, NY + 1) = at(s, k, NY);
    }
  }
  if (a.th) {
    for (int j = 1 + threadIdx.x; j <= NY; j += blockDim.x) {
      for (int s : sca) {
        at(s, 0, j) = at(s, 1, j);
        at(s, NZ + 1, j) = at(s, NZ, j);
      }
    }
  }
  __syncthreads();
  for (int j = 1 + threadIdx.x; j <= NY; j += blockDim.x) {
    at(S_DWDZ, 1, j) = at(S_DWDZ, 2, j);
    at(S_DUDZ, 1, j) = at(S_DUDZ, 2, j);
  }
  if (a.th) {
    for (int k = threadIdx.x; k <= NZ + 1; k += blockDim.x) {
      for (int s : sca) {
        at(s, k, 0) = sub(mul(2.0, at(s, k, 1)), at(s, k, 2));
        at(s, k, NY + 1) = sub(mul(2.0, at(s, k, NY)), at(s, k, NY - 1));
      }
    }
  }
}

// Bulk sums over the cells K = 1..NZ, J = 1..NY.
__global__ void __launch_bounds__(1024) k_stats_reduce(StatArgs a) {
  const Dims &d = a.d;
  const size_t n2 = (size_t)d.NZ2 * d.NY2;
  const int nc = d.NZ * d.NY;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  auto m0 = [&](const cplx_t *F, int k, int j) { return F[d.ic(0, k, j)].re; };
  auto corner = [&](const cplx_t *F, int k, int j) {
    return mul(0.25, add(add(add(m0(F, k, j), m0(F, k - 1, j)), m0(F, k - 1, j - 1)), m0(F, k, j - 1)));
  };
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const int k = 1 + c % d.NZ, j = 1 + c / d.NZ;
    acc[0] += corner(a.CU3, k, j);
    acc[1] += corner(a.CU1, k, j);
    if (a.th) acc[2] += corner(a.CTH, k, j);
    const double J = a.jac[d.m2(k, j)];
    acc[3] += J;
    for (int s = 0; s < 3; ++s) {
      const double *q = a.S + (S_URMS + s) * n2;
      auto Q = [&](int kk, int jj) { return q[(size_t)jj * d.NZ2 + kk]; };
      acc[4 + s] += mul(mul(0.25, add(add(add(Q(k, j), Q(k, j - 1)), Q(k - 1, j)), Q(k - 1, j - 1))), J);
    }
  }
  __shared__ double red[32][7];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = 0; q < 7; ++q) {
    const double v = warp_sum(acc[q]);
    if (lane == 0) red[w][q] = v;
  }
  __syncthreads();
  if (w != 0) return;
  const int nw = blockDim.x >> 5;
  for (int q = 0; q < 7; ++q) {
    double v = lane < nw ? red[lane][q] : 0.0;
    v = warp_sum(v);
    if (lane == 0) acc[q] = v;
  }
  if (lane != 0) return;
  // REAL(NY*NZ): the cell count rounded to REAL*4, then widened
  const double ncell = (double)(float)(d.NY * d.NZ);
  a.R[R_UBULK] = __ddiv_rn(acc[0], ncell);
  a.R[R_VBULK] = __ddiv_rn(acc[1], ncell);
  a.R[R_THBULK] = __ddiv_rn(acc[2], ncell);
  a.R[R_AREA] = acc[3];
  a.R[R_URMS] = __ddiv_rn(acc[4], acc[3]);
  a.R[R_VRMS] = __ddiv_rn(acc[5], acc[3]);
  a.R[R_WRMS] = __ddiv_rn(acc[6], acc[3]);
  // U3X(NXP,2,NY), U1X(NXP,2,NY) of the time_bulk.txt line (NXP = NX+1)
  a.R[R_PROBE3] = a.U3[d.ip(d.NX + 1, 2, d.NY)];
  a.R[R_PROBE1] = a.U1[d.ip(d.NX + 1, 2, d.NY)];
}

// Mode-0 planes after the transforms back, and CF1X = CF2X = CF3X = 0
// (flow_statistics.F90:956-963).
__global__ void __launch_bounds__(256) k_stats_means(StatArgs a, cplx_t *cf1, cplx_t *cf2, cplx_t *cf3) {
  const Dims &d = a.d;
  const size_t n2 = (size_t)d.NZ2 * d.NY2;
  const size_t ns = d.nspec();
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < ns; t += (size_t)gridDim.x * blockDim.x) {
    cf1[t] = cplx_t{0.0, 0.0};
    cf2[t] = cplx_t{0.0, 0.0};
    cf3[t] = cplx_t{0.0, 0.0};
    if (t < n2) {
      const int k = (int)(t % d.NZ2), j = (int)(t / d.NZ2);
      const size_t c0 = d.ic(0, k, j);
      a.S[S_M1 * n2 + t] = a.CU1[c0].re;
      a.S[S_M2 * n2 + t] = a.CU2[c0].re;
      a.S[S_M3 * n2 + t] = a.CU3[c0].re;
      a.S[S_MP * n2 + t] = a.CP[c0].re;
      a.S[S_MTH * n2 + t] = a.th ? a.CTH[c0].re : 0.0;
    }
  }
}

}  // namespace

int save_stats(Ctx &c, ek_stats *out) {
  const Dims &d = c.d;
  const ek_params &p = c.p;
  const size_t n2 = (size_t)d.NZ2 * d.NY2;
  if (!c.stats_buf) {
    EK_CUDA(cudaMalloc(&c.stats_buf, sizeof(double) * (S_N * n2 + R_N)));
    c.allocs.push_back(c.stats_buf);
  }
  EK_CUDA(cudaMemsetAsync(c.stats_buf, 0, sizeof(double) * (S_N * n2 + R_N), c.stream));
  const bool th = p.n_th > 0;
  StatArgs a{};
  a.d = d;
  a.CU1 = c.CU1; a.CU2 = c.CU2; a.CU3 = c.CU3; a.CP = c.CP; a.CTH = c.CTH;
  a.U1 = c.U1; a.U2 = c.U2; a.U3 = c.U3; a.P = c.R1; a.TH = c.TH;
  a.jac = c.m.jac; a.c11 = c.m.c11; a.c12 = c.m.c12; a.c21 = c.m.c21; a.c22 = c.m.c22; a.th_bar = c.m.thbar;
  a.S = c.stats_buf;
  a.R = c.stats_buf + S_N * n2;
  a.th = th;
  a.cont_strat = p.cont_strat;
  a.ri = p.ri_tau;
  // TKE * DBLE(AMP_OMEGA0/OMEGA0)**(-2.0) when AMP_OMEGA0 /= 0 (:165-174)
  a.tke_scaled = p.amp_omega0 != 0.0;
  a.tke_fac = a.tke_scaled ? std::pow(p.amp_omega0 / p.omega0, -2.0) : 1.0;
  // to physical space (flow_statistics.F90:156-160, 452); P into scratch R1
  {
    C2rArgs t{};
    t.j0 = 0; t.j1 = d.NY + 1; t.k0 = 0; t.k1 = d.NZ + 1;
    t.src = c.CU1; t.dst = c.U1; launch_c2r(c, t);
    t.src = c.CU2; t.dst = c.U2; launch_c2r(c, t);
    t.src = c.CU3; t.dst = c.U3; launch_c2r(c, t);
    t.src = c.CP; t.dst = c.R1; launch_c2r(c, t);
    if (th) { t.src = c.CTH; t.dst = c.TH; launch_c2r(c, t); }
  }
  const int lines = d.NZ2 * d.NY2;
  k_stats_lines<<<(lines + 7) / 8, 256, 0, c.stream>>>(a);
  after_launch(c);
  k_stats_plane<<<(lines + 255) / 256, 256, 0, c.stream>>>(a);
  after_launch(c);
  k_stats_edges<<<1, 1024, 0, c.stream>>>(a);
  after_launch(c);
  k_stats_reduce<<<1, 1024, 0, c.stream>>>(a);
  after_launch(c);
  // back to Fourier space (flow_statistics.F90:821, 951-954)
  {
    R2cArgs t{};
    t.j0 = 0; t.j1 = d.NY + 1; t.k0 = 0; t.k1 = d.NZ + 1;
    t.pro = PRO_LOAD; t.epi = EPI_STORE;
    t.a = c.U1; t.dst = c.CU1; launch_r2c(c, t);
    t.a = c.U2; t.dst = c.CU2; launch_r2c(c, t);
    t.a = c.U3; t.dst = c.CU3; launch_r2c(c, t);
    t.a = c.R1; t.dst = c.CP; launch_r2c(c, t);
    if (th) { t.a = c.TH; t.dst = c.CTH; launch_r2c(c, t); }
  }
  k_stats_means<<<4 * 152, 256, 0, c.stream>>>(a, c.CF1, c.CF2, c.CF3);
  after_launch(c);
  // results to the caller's planes
  double r[R_N];
  EK_CUDA(cudaMemcpyAsync(r, a.R, sizeof r, cudaMemcpyDeviceToHost, c.stream));
  double *dst[S_N] = {out->urms, out->vrms, out->wrms, out->uv, out->uw, out->wv, out->pu, out->pv,
                      out->thrms, out->thv, out->thw, out->tke, out->dudy, out->dwdy, out->dudz, out->dwdz,
                      out->omega_x, out->dthdy, out->dthdz, out->rig, out->mean_u1, out->mean_u2, out->mean_u3,
                      out->mean_p, out->mean_th};
  for (int s = 0; s < S_N; ++s)
    if (dst[s]) EK_CUDA(cudaMemcpyAsync(dst[s], a.S + s * n2, sizeof(double) * n2, cudaMemcpyDeviceToHost, c.stream));
  EK_CUDA(cudaStreamSynchronize(c.stream));
  out->ubulk = r[R_UBULK];
  out->vbulk = r[R_VBULK];
  out->thbulk = r[R_THBULK];
  out->urms_b = r[R_URMS];
  out->vrms_b = r[R_VRMS];
  out->wrms_b = r[R_WRMS];
  out->u3_probe = r[R_PROBE3];
  out->u1_probe = r[R_PROBE1];
  return EK_OK;
}

}  // namespace ek
