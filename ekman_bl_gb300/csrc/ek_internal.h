// Internal declarations of the GB300 duct substep library (libekgpu.so).
// Host orchestration lives in ek_api.cu, host-side precomputation in
// ek_host.cpp, device kernels in ek_fft.cu, ek_rk.cu and ek_mg.cu.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/ekgpu.h"
#include "ek_ffbits.h"

namespace ek {

struct cplx_t {
  double re, im;
};

// Sizes and index helpers shared by host and device code.
struct Dims {
  int NX, NY, NZ;      // grid_def sizes
  int NKX, NX2P;       // NX/3, NX/2
  int LDX, LDC;        // physical / spectral line lengths: NX+2, NX/2+1
  int NZ2, NY2;        // NZ+2, NY+2
  int LDM;             // metric leading dim NZ+3
  int JS, JE, ZS, ZE;  // velocity ranges (INIT_DUCT)
  int JST, JET, ZST, ZET;  // scalar ranges
  __host__ __device__ size_t ip(int i, int k, int j) const { return ((size_t)j * NZ2 + k) * LDX + i; }
  __host__ __device__ size_t ic(int i, int k, int j) const { return ((size_t)j * NZ2 + k) * LDC + i; }
  __host__ __device__ size_t m2(int k, int j) const { return (size_t)j * LDM + k; }
  __host__ __device__ size_t m3(int k, int j, int f) const {
    return (size_t)(f - 1) * LDM * (NY + 3) + (size_t)j * LDM + k;
  }
  __host__ __device__ size_t nphys() const { return (size_t)LDX * NZ2 * NY2; }
  __host__ __device__ size_t nspec() const { return (size_t)LDC * NZ2 * NY2; }
};

#ifdef __CUDACC__
// Float-float: an unevaluated sum hi + lo of two floats (about 48
// significant bits), with the error-free sum (Knuth's TwoSum) and the
// FMA-based product.  The _rn intrinsics keep the compiler from fusing or
// reassociating the steps.  On GB300 this runs on the FP32 pipe, ~60x
// wider than the FP64 one, at roughly ten FP32 instructions per FP64 one.
struct FF {
  float hi, lo;
  FF() = default;
  __device__ FF(float h, float l) : hi(h), lo(l) {}
  // one FP64 add each way: splitting and joining in 64-bit integer
  // arithmetic costs as much on GB300 (measured), the conversions themselves
  // run on the integer pipes
  __device__ explicit FF(double x) {
    hi = d2f_bits(x);
    lo = d2f_bits(x - f2d_bits(hi));
  }
  __device__ explicit operator double() const { return f2d_bits(hi) + f2d_bits(lo); }
};
__device__ __forceinline__ FF ff_norm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return FF(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ FF operator+(FF a, FF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return ff_norm(s, e);
}
__device__ __forceinline__ FF operator-(FF a) { return FF(-a.hi, -a.lo); }
__device__ __forceinline__ FF operator-(FF a, FF b) { return a + (-b); }
__device__ __forceinline__ FF operator*(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ff_norm(p, e);
}
#endif

// Device copies of the JACOBI_TRANS metric arrays.
struct Metrics {
  double *jac, *g11, *g12, *g22, *c11, *c12, *c21, *c22, *thbar;
  // per-cell coefficient planes (metric-only, built by launch_metric_tables):
  // pg[0..4] the pressure-gradient weights of the CJOB_12/CJOB_22 combination
  // and pg[5..9] of the CJOB_11/CJOB_21 one, for (p0, p(k+1), p(k-1),
  // p(j+1), p(j-1)), each with its 0.5; pg[10] = 1/INT_JACOB; pg[11] and
  // pg[12] the background-stratification terms of the scalar right-hand
  // side that depend on (K, J) only: the coefficient of CU2 and the TH_BAR
  // diffusion bracket that KAPPA/4 multiplies
  double *pg = nullptr;
  // LES variants GMAT_*_y / GMAT_*_z (face layout; null without LES)
  double *g11y = nullptr, *g12y = nullptr, *g22y = nullptr, *g11z = nullptr, *g12z = nullptr, *g22z = nullptr;
};

// Boundary rows of one ADI direction (a row of a tridiagonal line replaced
// by APPLY_BC_*).  Value source: 0 constant, 1 copy of the field at index
// src along the line (lagged periodic), 2 constant times a per-line weight.
struct BcRow {
  int row;
  int kind;
  int src;
  double val;
  double l, dg, u;  // the row's matrix entries (APPLY_BC_*), for solvers that build rows on the device
};
struct BcSet {
  int n;
  BcRow r[4];
  int weight_off;  // offset of per-line weights (kind 2) in the weights buffer
};

// Precomputed Thomas factors of one field/direction/substep: for line l and
// row r: a[l][r] (the -L/B' multiplier), ib[l][r] = 1/B', u[l][r] = U.
struct AdiFactors {
  double *a, *ib, *u;
  int nline, nrow;
  // the same factors split into float-float pairs (hi, lo), for the
  // float-float sweeps of the mixed path (null until ff_arith needs them)
  float2 *a2 = nullptr, *ib2 = nullptr, *u2 = nullptr;
};

// One multigrid level (MUDPACK level k; index k-1).
struct MgLevel {
  int nx, ny;
  double *cof;  // 11 x nx x ny: c1..c8, s4, corr9, jac  (kx-independent)
};

// Work arrays of one batched multigrid solve for up to pmax problems,
// problem fastest: per level phi (0:nx+1, 0:ny+1), rhs (1:nx, 1:ny) and 1/c9
// (nx x ny); the finest-size scratch; the output iterate (finest interior);
// per-problem reductions, kx^2, done flags and cycle counts.
struct MgWork {
  int pmax = 0;
  double *pool = nullptr;
  int *flags = nullptr;
  std::vector<double *> phi, rhs, inv9;
  double *scratch = nullptr, *phif = nullptr, *red = nullptr, *kx2 = nullptr;
  int *done = nullptr, *cycles = nullptr, *alldone = nullptr, *idx = nullptr;
  int *iter = nullptr;        // mixed solver: corrections applied so far (device counter)
  std::vector<int> idx_host;  // host copy of idx (a subset's problem numbers)
};

enum MgOpKind { OP_TRSFC = 0, OP_RELAX = 1, OP_RESTRICT = 2, OP_COR2 = 3, OP_PROLONG = 4, OP_CHECK = 5 };
struct MgOp {
  int kind, level, count;  // level = MUDPACK level (1 coarsest); RESTRICT: from level to level-1;
                           // COR2: level-1 -> level; PROLONG: level -> level+1
};

// FP32 arrays of one level for the mixed-precision multigrid (ek_mgfast.cu).
struct MgLevelF {
  float *e = nullptr, *r = nullptr, *cp = nullptr, *cof = nullptr;
  // the same coefficients packed per point for the level residual's vector
  // loads (planes c[l] of cof): [3 pt] = (c0, c2, c4, c6), the couplings
  // along the axes; [3 pt + 1] = (c8, c9, c10, 0), the diagonal's parts;
  // [3 pt + 2] = (c1, c3, c5, c7), the corner couplings
  float4 *cf4 = nullptr;
};

struct MgPlan {
  int ngrid = 0, nfx = 0, nfy = 0;
  int ixp = 0, jyq = 0, iex = 0, jey = 0;
  int lc = 0;           // levels 1..lc run inside one CTA per problem
  bool orth = false;    // all diagonal couplings zero: 4 colour phases per sweep
  std::vector<MgLevel> lv;
  std::vector<MgOp> ops;
  MgOp *ops_dev = nullptr;
  // host copies of the kx-independent coefficients per level
  std::vector<std::vector<double>> cof_host;
  size_t coarse_smem = 0;
  // mixed solver: layout of the line solves per level (index l = 1..ngrid)
  // and direction -- problems per block and rows per segment; 0 = the
  // default rule (set by ekgpu_mg_autotune)
  std::vector<int> lanes_y, lanes_x, seg_y, seg_x;
};

// Kernel classes for the optional per-kernel timer (ekgpu_set_timing).
enum KClass {
  KC_SPECTRAL = 0, KC_C2R, KC_R2C, KC_FACE, KC_ADI_Y, KC_ADI_Z, KC_MG_RELAX, KC_MG_COARSE,
  KC_MG_TRANSFER, KC_MG_CHECK, KC_MG_SETUP, KC_PROJECTION, KC_DIVERGENCE, KC_GUESS, KC_LES, KC_N
};
struct TimerRec {
  int cls;
  cudaEvent_t a, b;
};

// Early stop of an iteration whose kernels decide on the device when every
// problem is done (they return at once after that).  After each check kernel
// the done flag is copied to pinned host memory; the host then waits for the
// copy made one check earlier, while the GPU still has the latest cycle
// queued, and stops issuing cycles once that copy reads 1.
struct StopPoll {
  int *host = nullptr;  // pinned, kSlots flags
  cudaEvent_t ev[4] = {};
  static constexpr int kSlots = 4;
  int n = 0;
  void init() {
    if (host) return;
    if (cudaHostAlloc(&host, sizeof(int) * kSlots, cudaHostAllocDefault) != cudaSuccess) host = nullptr;
    for (auto &e : ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  }
  void destroy() {
    if (host) cudaFreeHost(host);
    host = nullptr;
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  }
  void reset() { n = 0; }
  // after a check kernel on stream s; returns true when the iteration can stop
  bool after_check(const int *alldone_dev, cudaStream_t s) {
    if (!host) return false;
    const int k = n % kSlots;
    cudaMemcpyAsync(&host[k], alldone_dev, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaEventRecord(ev[k], s);
    ++n;
    if (n < 2) return false;
    const int k1 = (n - 2) % kSlots;
    cudaEventSynchronize(ev[k1]);
    return host[k1] != 0;
  }
};

// Per-substep results of a step run as a CUDA graph, written on the device
// and read once after the step: the projection solve's statistics and the
// divergence check's mean |div|.
struct StepStats {
  int min_cycles, max_cycles, n_not_converged, nprob;
  double max_residual, div;
};
// One RK3 step captured as a CUDA graph (ekgpu_step).  A graph holds every
// launch of the three substeps; the mixed solver's correction cycles sit in
// conditional while-nodes that its check kernel stops.  key: the host-side
// choices a step's launches depend on (see step_graph_key).
struct StepGraph {
  unsigned long long key = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long fixed_launches = 0;  // kernels outside the while bodies
  long long body_launches[3] = {};  // kernels of one correction cycle, per substep
};

class UNet;
// Learned initial guess of the Poisson problems (ek_guess.cu): the network
// (owned by the caller), the image geometry, work buffers, and the optional
// sink that collects (input, target) training pairs after each solve.
struct GuessState {
  UNet *net = nullptr;
  bool use = false;
  int factor = 0, h = 0, w = 0, hv = 0, wv = 0;
  float *x = nullptr, *y = nullptr;
  double *ss = nullptr;
  int *idx = nullptr;
  int cap = 0;
  std::vector<int> idx_host;
  float *alpha = nullptr;
  int alpha_cap = 0;
  float *sink_x = nullptr, *sink_t = nullptr;
  int sink_cap = 0, sink_count = 0;
  long long calls = 0;
  double last_rho = 1.0;  // mean residual ratio |b - A g|/|b| of the last guess
};

// LES (les_chan LES_MODEL_TYPE 2, les_chan_th LES_MODEL_TYPE_TH 1) state
// and work fields (ek_les.cu).  Physical layout unless noted.
struct LesState {
  bool have_metrics = false;
  bool first_time = true;       // FIRST_TIME: recompute C_DYN in every substep
  bool lowp = false;            // stresses in FP32 (fft_fp32 >= 1): the f-suffixed buffers
  bool tab_ok = false;          // delta and tabf match the metrics
  double *nut = nullptr;        // NU_T, zero outside the velocity interior (both precisions)
  double *cdyn = nullptr;       // C_DYN(0:NZ+1, 0:NY+1), K fastest
  double *t[3] = {};            // d(U1,U2,U3)/dx, then tau_11, tau_12, tau_13 in place
  double *t23 = nullptr;        // tau_23
  double *tth = nullptr;        // d(TH)/dx, then the scalar flux -KAPPA_T d(TH)/dx in place
  double *ext[4] = {};          // flux-transform additions of U1, U2, U3, TH
  float *tf[3] = {}, *t23f = nullptr, *tthf = nullptr, *extf[4] = {}, *nutf = nullptr;
  float *tabf = nullptr;        // per-cell FP32 weights of the FP32 kernels
  double *delta = nullptr;      // DELTA_Y(K, J), metric layout
};

struct Ctx {
  ek_params p{};
  Dims d{};
  std::string err;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  long long launches = 0;
  bool have_metrics = false;
  // RKW3
  double H_BAR[4], BETA_BAR[4], ZETA_BAR[4];
  // wavenumbers
  double *kx = nullptr, *kx2 = nullptr;
  std::vector<double> kx_h, kx2_h;
  // FFT twiddles
  double2 *tw_m = nullptr;  // exp(-2 pi i t/M), t < M/2   (M = NX/2)
  double2 *tw_n = nullptr;  // exp(-2 pi i k/NX), k <= M
  float2 *tw_mf = nullptr, *tw_nf = nullptr;  // the same, rounded to FP32
  float4 *tw_mff = nullptr, *tw_nff = nullptr;  // and as float-float pairs
  Metrics m{};
  // spectral fields (complex)
  cplx_t *CU1, *CU2, *CU3, *CP, *CTH, *CF1, *CF2, *CF3, *CFTH, *CR1, *CR2, *CR3, *CRTH, *CS, *CU2b, *CU3b;
  // physical fields
  double *U1, *U2, *U3, *TH, *R1, *R2, *R3, *RTH, *U2b, *U3b, *PHS, *SPH;
  // FP32 copies of the physical fields the nonlinear terms read (fft_fp32)
  float *U1f = nullptr, *U2f = nullptr, *U3f = nullptr, *THf = nullptr, *U2bf = nullptr, *U3bf = nullptr;
  // ADI: [field 0..3][rk 1..3][dir 0 y, 1 z]
  AdiFactors adi[4][4][2];
  BcSet bc[4][2];
  double *bc_weights = nullptr;
  // multigrid
  MgPlan mg;
  double *mg_cof_pool = nullptr;    // the levels' coefficients
  MgWork mgw;                       // the solves' work arrays
  std::vector<double> mg_kx2_host;  // host copy of mgw.kx2
  float *mgf_pool = nullptr;        // mixed-precision multigrid
  float4 *mgf_cf4_pool = nullptr;   // its packed level coefficients
  std::vector<MgLevelF> mgf_levels;
  float *mgf_scratch = nullptr;
  float *mgf_phh = nullptr, *mgf_phl = nullptr;  // float-float finest iterate
  float *mgf_phh2 = nullptr, *mgf_phl2 = nullptr;  // its second buffer (alternate corrections)
  float *mgf_bh = nullptr, *mgf_bl = nullptr;    // float-float finest rhs
  float2 *mgf_cf2 = nullptr;  // float-float finest coefficients, (hi, lo) interleaved
  int mgf_pmax = 0;
  float *mgf_tailfac = nullptr;  // Thomas factors of the coarse levels' lines (k_f_vtail), per problem
  size_t mgf_tailfac_n = 0;
  // residual rule: left null vector of the finest kx = 0 operator (nfx*nfy,
  // unit norm), for the well-posed kx = 0 solve
  double *mg_z = nullptr;
  // per-chunk partial sums of the kx = 0 projections (pmax x kNullChunks)
  double *mg_null_part = nullptr;
  ek_mg_stats last_stats{};
  // problems that missed the residual rule's tolerance, and problems solved,
  // summed over every solve since the context was created
  long long mg_nc_total = 0, mg_solved_total = 0;
  double last_mean_cycles = 0.0;  // mixed solver: mean corrections over the kx^2 != 0 problems
  StopPoll poll;
  // sponge_th: SPONGE_SIGMA(0:NY+1), SPONGE_SIGMA_OUT(0:NZ+1), and the
  // mode-0 mean of CU3X over the upper layer with the dynamic-branch flag
  double *sponge_sig = nullptr, *sponge_sig_out = nullptr, *sponge_red = nullptr;
  // COURANT_CURV_MPI: device minimum of the CFL time steps; host copies of
  // the metrics the dt-dependent ADI factors are built from
  double *cfl_dt = nullptr;
  std::vector<double> h_jac, h_g11, h_g22;
  GuessState guess;
  // SAVE_STATS_CURVI planes and sums (ek_stats.cu)
  double *stats_buf = nullptr;
  // per-cell right-hand-side weights of the two ADI sweeps (k_adi_tab)
  double *adi_tab = nullptr;
  LesState les;
  double *adi_scr = nullptr;      // LES ADI: 1/B and the upper diagonal of the eliminated rows (two fields)
  double *adi_les_tab = nullptr;  // LES ADI: per-cell row weights of the two sweeps (k_adi_les_tab)
  float2 *adi_ff_tab = nullptr;   // LES ADI, float-float: both sweeps' weights as float pairs
  float2 *adi_tab2 = nullptr;     // the weights of adi_tab as float pairs (float-float fields)
  // the increment-form ADI of the four fields runs on four concurrent
  // streams (forked from and joined to the step's stream): each field's own
  // sweep weights and scratch (the y sweep's increment and the copy rows'
  // brackets), allocated in an eager step
  double *adi_tab_f[4] = {nullptr, nullptr, nullptr, nullptr};
  float2 *adi_tab2_f[4] = {nullptr, nullptr, nullptr, nullptr};
  float *inc_scr[4] = {nullptr, nullptr, nullptr, nullptr};  // 2 x nphys floats each
  cudaStream_t field_stream[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t field_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // a captured step runs each substep's divergence check on a side stream
  // (div_ev[0] forks it, div_ev[1] marks its end); div_pending: a check is
  // in flight that the work writing CU1 or the face velocities must wait for
  cudaStream_t div_stream = nullptr;
  cudaEvent_t div_ev[2] = {nullptr, nullptr};
  bool div_pending = false;
  // divergence check
  double *div_part = nullptr;
  double last_div = 0.0;
  std::vector<void *> allocs;
  // whole-step CUDA graphs (ekgpu_step): capture streams, the graphs by
  // variant, a counter of plan changes that invalidate them, whether a step
  // was taken eagerly since (lazy allocations happen there, never inside a
  // capture), and the substep slot being captured (-1: running eagerly)
  bool step_graphs = true;
  unsigned long long epoch = 0;  // process-unique; renewed whenever its step graphs are dropped
  cudaStream_t cap_stream = nullptr, cap_stream2 = nullptr;
  std::vector<StepGraph> graphs;
  bool eager_since_plan = false;
  int graph_slot = -1;
  long long graph_body_launches = 0;  // kernels in the while body of the last captured solve
  StepStats *step_stats_dev = nullptr, *step_stats_host = nullptr;  // 3 slots; host copy pinned
  // per-kernel timer
  bool timing = false;
  std::vector<TimerRec> trec;
  std::vector<cudaEvent_t> evpool;
  double kms[KC_N] = {};
  long long kcnt[KC_N] = {};
  double kbytes[KC_N] = {};
};

// Records CUDA events around the launches in its scope when timing is on.
struct KScope {
  Ctx &c;
  int cls;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEvent_t get() {
    if (!c.evpool.empty()) {
      cudaEvent_t e = c.evpool.back();
      c.evpool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  // bytes: algorithmic HBM bytes the launches in this scope must move
  KScope(Ctx &ctx, int k, double bytes = 0.0) : c(ctx), cls(k) {
    if (!c.timing) return;
    c.kbytes[k] += bytes;
    a = get();
    b = get();
    cudaEventRecord(a, c.stream);
  }
  ~KScope() {
    if (!a) return;
    cudaEventRecord(b, c.stream);
    c.trec.push_back(TimerRec{cls, a, b});
  }
};
void timing_resolve(Ctx &c);
// a captured step's divergence check in flight on the side stream: make the
// step's stream wait for it
void div_join(Ctx &c);
// a captured step's mean |div| into its statistics slot (on c.stream)
void div_final(Ctx &c);

// ---- host helpers (ek_host.cpp) ----
int metrics_from_grid_host(const ek_params *p, const double *xpoint, const double *ypoint, double *int_jacob,
                           double *gmat_11, double *gmat_12, double *gmat_22, double *cjob_11, double *cjob_12,
                           double *cjob_21, double *cjob_22, double *th_bar);
int build_bc_sets(Ctx &c, std::vector<double> &weights, const std::vector<double> &jac,
                  const std::vector<double> &c22);
void adi_factor_host(const Ctx &c, int field, int rk, int dir, const std::vector<double> &jac,
                     const std::vector<double> &g11, const std::vector<double> &g22, std::vector<double> &a,
                     std::vector<double> &ib, std::vector<double> &u);
bool mg_pick_shape(int n, int &p, int &e);
void launch_courant(Ctx &c);
int les_metrics_from_grid_host(const ek_params *p, const double *xpoint, const double *ypoint, double *g11y,
                               double *g12y, double *g22y, double *g11z, double *g12z, double *g22z);
int sponge_profiles_host(const ek_params *p, const double *xpoint, const double *ypoint, double *sig,
                         double *sig_out);
void mg_build_plan_host(Ctx &c, const std::vector<double> &jac, const std::vector<double> &g11,
                        const std::vector<double> &g12, const std::vector<double> &g22);
void mg_build_schedule(MgPlan &plan, int kcycle, int iprer, int ipost, int maxcy);
bool mg_left_null_host(const MgPlan &P, std::vector<double> &z);

// ---- device launch wrappers ----
// FFT (ek_fft.cu)
enum { PRO_LOAD = 0, PRO_PROD = 1, PRO_FLUX = 2 };
enum { EPI_STORE = 0, EPI_ADD = 1, EPI_SUB_IK = 2 };
struct R2cArgs {
  const double *a, *b;    // PRO_LOAD: a; PRO_PROD: jac*a*b; PRO_FLUX: field a
  const double *extra;    // when set: PRO_PROD adds jac*extra, PRO_FLUX adds extra
  const float *extraf;    // the same term in FP32, read by the FP32 kernel instead of extra
  double visc;            // PRO_FLUX viscosity
  cplx_t *dst;
  int epi;
  int pro;
  int j0, j1, k0, k1;
  int lowp;               // a nonlinear-term transform (FP32 arithmetic when fft_fp32 = 1)
  const float *af, *bf;   // FP32 copies of a, b read by the FP32 kernel when given
  // PRO_LOAD of a field held as float-float planes (the float-float kernel
  // reads the pair af + alo and no FP64 a)
  const float *alo;
  // EPI_ADD: also zero the modes above NX/3, as a state's forward transform
  // does (EPI_STORE always does)
  int zero_hi;
  // PRO_PROD with EPI_SUB_IK and fuse_flux = 1: the same launch also
  // transforms the flux term of a2 against b2 (PRO_FLUX with visc2, plus
  // extra2/extraf2) and adds it, dst = dst - i kx X + X2, as the two
  // launches would in turn
  int fuse_flux;
  const double *a2, *b2, *extra2;
  const float *a2f, *b2f, *extraf2;
  double visc2;
};
void launch_r2c(Ctx &c, const R2cArgs &a);
struct C2rArgs {
  const cplx_t *src, *src2;  // x = src (+ scale2*src2)
  double scale2;
  int ik;                    // 1: x = i kx src (the x derivative)
  double *dst;
  int j0, j1, k0, k1;
  int lowp;                  // as R2cArgs::lowp
  float *dstf;               // also write an FP32 copy of dst when given (dst may then be null)
  // the float-float kernel with dstlo set writes its result as two float
  // planes, high part to dstf and low part to dstlo, and no FP64 dst
  float *dstlo;
};
void launch_c2r(Ctx &c, const C2rArgs &a);

// RK pieces (ek_rk.cu)
void launch_spectral_rhs(Ctx &c, int rk);
void launch_metric_tables(Ctx &c);
void launch_face_velocity(Ctx &c);
void launch_adi(Ctx &c, int field, int rk);
void mg_exact_attributes();

// LES (ek_les.cu)
bool les_active(const Ctx &c);
// The mixed path's explicit-increment form (fft_fp32 >= 1): CR keeps only
// CR - J CU, its inverse transform S = R - J phi_old runs in FP32 into R's
// slots, and the ADI right-hand sides fold the J phi_old halves into their
// weights.  The same terms as RK_DUCT's R = c2r(CR + beta h CF) and
// S = R - J phi_old (duct.F90:1127-1161, 1334-2392), without transforming
// the large J CU part: the FP32 rounding then falls on the O(h) increment.
inline bool explicit_increment_form(const Ctx &c) { return c.p.fft_fp32 >= 1; }
// The mixed path's float-float physical fields: with ff_arith and the
// nonlinear-term transforms in FP32 (and no LES in the substep), the
// physical U1, U2, U3, TH live as float-float pairs -- the high part is the
// FP32 copy the nonlinear terms read (U1f ...), the low part sits in the
// first half of the FP64 buffer (U1 ...) -- from the inverse transform at
// the substep's start, through the float-float ADI, to the forward transform
// at its end, so none of those kernels splits or joins an FP64 value per
// physical point.
bool ff_fields(const Ctx &c);
// the spectral kernels' sizes: NX2P lowered to NKX on the mixed path
Dims spec_dims(const Ctx &c);
inline float *ff_lo(double *field) { return reinterpret_cast<float *>(field); }
// The increment form of the state path (ff_arith = 2, nonlinear-term
// transforms in FP32, no LES in the substep): the inverse transforms of the
// state are FP32 (the fields' FP32 copies), each ADI sweep solves in FP32 for
// the increment of its field over the field it starts from, and the forward
// transform of the total increment (in the second half of the field's R
// buffer) is added to the FP64 spectral state.  Every FP32 rounding then
// falls on an O(h) increment or on an O(h) viscous term, never on the state.
bool inc_fields(const Ctx &c);
// the total ADI increment of a field: the second float half of its R buffer
inline float *inc_plane(Ctx &c, double *R) { return reinterpret_cast<float *>(R) + c.d.nphys(); }
void split_ff(Ctx &c, const double *in, float2 *out, size_t n);
void les_alloc(Ctx &c);
void launch_les(Ctx &c, int rk);
void launch_th_corners(Ctx &c);
void launch_divergence_rhs(Ctx &c, double *rhs_finest, int nprob);
void launch_projection(Ctx &c, const double *phif, int nprob, double temp4, bool update_p);
int finish_divergence(Ctx &c, double *div_out);
void step_graphs_clear(Ctx &c);

// multigrid (ek_mg.cu).  mg_solve: nprob problems whose finest rhs is in
// c.mgw.rhs[ngrid-1]; the solution is left in c.mgw.phif.  kx2_host may be
// null (it is then read back from kx2_dev when the mixed-precision solver
// needs it).
int mg_solve(Ctx &c, int nprob, const double *kx2_dev, const double *kx2_host, ek_mg_stats *st);
int mg_solve_exact(Ctx &c, MgWork &w, int nprob, const double *kx2_dev, ek_mg_stats *st, int max_cycles);
void mg_exact_enqueue(Ctx &c, MgWork &w, int nprob, const double *kx2_dev, int max_cycles, bool poll);
int mg_exact_stats(Ctx &c, MgWork &w, int nprob, ek_mg_stats *st);
// The residual rule's well-posed kx^2 = 0 problems (finest level, problem
// fastest): b <- b - (z.b) z before the solve, phi <- phi - mean(phi) after.
void mg_null_project(Ctx &c, double *rhs_finest, int nprob, const double *kx2_dev);
void mg_null_mean(Ctx &c, double *phi_finest, int nprob, const double *kx2_dev);
constexpr int kNullChunks = 64;  // blocks per kx = 0 problem of the null-space projections
void mg_alloc(Ctx &c, int pmax);
void mg_work_alloc(Ctx &c, MgWork &w, int pmax);
void mg_work_free(MgWork &w);
int mgfast_solve(Ctx &c, int nprob, const double *kx2_dev, const double *kx2_host, ek_mg_stats *st);
void mgfast_alloc(Ctx &c, int pmax);
// the coarse levels 1..ltop the mixed solver runs in one launch per cycle
int mgfast_tail_levels(const Ctx &c);
int mgfast_autotune(Ctx &c, int reps, std::string &report);

// restart files (ek_io.cpp): SAVE_FLOW / READ_FLOW records from and into the state
int save_flow(Ctx &c, const char *flow_path, const char *th_path);
int read_flow(Ctx &c, const char *flow_path, const char *th_path);
// plane statistics (ek_stats.cu): SAVE_STATS_CURVI's reductions and its state round trip
int save_stats(Ctx &c, ek_stats *out);
// learned guess (ek_guess.cu)
void guess_geometry(const Ctx &c, int f, int &h, int &w, int &hv, int &wv);
void guess_predict(Ctx &c, int P, const double *rhs, const double *kx2_dev, const std::vector<int> &nonsing,
                   float *phh, cudaStream_t s);
void guess_collect(Ctx &c, int P, const double *rhs, const double *phi, const double *kx2_dev,
                   const std::vector<double> &kx2_host, cudaStream_t s);
void guess_free(Ctx &c);

#define EK_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) throw ek::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct CudaError {
  std::string msg;
  explicit CudaError(std::string m) : msg(std::move(m)) {}
};

inline void after_launch(Ctx &c) {
  c.launches++;
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) throw CudaError(std::string("kernel launch: ") + cudaGetErrorString(e));
}

}  // namespace ek
