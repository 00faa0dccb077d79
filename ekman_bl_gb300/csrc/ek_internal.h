// Internal declarations of the GB300 duct substep library (libekgpu.so).
// Host orchestration lives in ek_api.cu, host-side precomputation in
// ek_host.cpp, device kernels in ek_fft.cu, ek_rk.cu and ek_mg.cu.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/ekgpu.h"

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

// Device copies of the JACOBI_TRANS metric arrays.
struct Metrics {
  double *jac, *g11, *g12, *g22, *c11, *c12, *c21, *c22, *thbar;
};

// Boundary rows of one ADI direction (a row of a tridiagonal line replaced
// by APPLY_BC_*).  Value source: 0 constant, 1 copy of the field at index
// src along the line (lagged periodic), 2 constant times a per-line weight.
struct BcRow {
  int row;
  int kind;
  int src;
  double val;
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
};

// One multigrid level (MUDPACK level k; index k-1).
struct MgLevel {
  int nx, ny;
  double *phi;   // (0:nx+1, 0:ny+1) x P, problem fastest
  double *rhs;   // (1:nx, 1:ny) x P
  double *cof;   // 11 x nx x ny: c1..c8, s4, corr9, jac  (kx-independent)
  double *inv9;  // nx x ny x P: 1/c9 for the current problems
  size_t phi_off, rhs_off, cof_off;
};

enum MgOpKind { OP_TRSFC = 0, OP_RELAX = 1, OP_RESTRICT = 2, OP_COR2 = 3, OP_PROLONG = 4, OP_CHECK = 5 };
struct MgOp {
  int kind, level, count;  // level = MUDPACK level (1 coarsest); RESTRICT: from level to level-1;
                           // COR2: level-1 -> level; PROLONG: level -> level+1
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
};

// Kernel classes for the optional per-kernel timer (ekgpu_set_timing).
enum KClass {
  KC_SPECTRAL = 0, KC_C2R, KC_R2C, KC_FACE, KC_ADI_Y, KC_ADI_Z, KC_MG_RELAX, KC_MG_COARSE,
  KC_MG_TRANSFER, KC_MG_CHECK, KC_MG_SETUP, KC_PROJECTION, KC_DIVERGENCE, KC_N
};
struct TimerRec {
  int cls;
  cudaEvent_t a, b;
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
  Metrics m{};
  // spectral fields (complex)
  cplx_t *CU1, *CU2, *CU3, *CP, *CTH, *CF1, *CF2, *CF3, *CFTH, *CR1, *CR2, *CR3, *CRTH, *CS, *CU2b, *CU3b;
  // physical fields
  double *U1, *U2, *U3, *TH, *R1, *R2, *R3, *RTH, *U2b, *U3b, *PHS, *SPH;
  // ADI: [field 0..3][rk 1..3][dir 0 y, 1 z]
  AdiFactors adi[4][4][2];
  BcSet bc[4][2];
  double *bc_weights = nullptr;
  // multigrid
  MgPlan mg;
  double *mg_pool = nullptr;
  double *mg_kx2 = nullptr;         // per problem
  double *mg_scratch = nullptr;     // finest-size scratch x P
  double *mg_phif = nullptr;        // output iterate per problem (finest interior)
  double *mg_red = nullptr;         // per-problem reductions
  int *mg_done = nullptr;           // per problem: 0 active, 1 converged
  int *mg_cycles = nullptr;         // per problem cycle count
  int *mg_alldone = nullptr;
  int mg_pmax = 0;                  // problem capacity
  ek_mg_stats last_stats{};
  // divergence check
  double *div_part = nullptr;
  double last_div = 0.0;
  std::vector<void *> allocs;
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
void mg_build_plan_host(Ctx &c, const std::vector<double> &jac, const std::vector<double> &g11,
                        const std::vector<double> &g12, const std::vector<double> &g22);
void mg_build_schedule(MgPlan &plan, int kcycle, int iprer, int ipost, int maxcy);

// ---- device launch wrappers ----
// FFT (ek_fft.cu)
enum { PRO_LOAD = 0, PRO_PROD = 1, PRO_FLUX = 2 };
enum { EPI_STORE = 0, EPI_ADD = 1, EPI_SUB_IK = 2 };
struct R2cArgs {
  const double *a, *b;    // PRO_LOAD: a; PRO_PROD: jac*a*b; PRO_FLUX: field a
  double visc;            // PRO_FLUX viscosity
  cplx_t *dst;
  int epi;
  int pro;
  int j0, j1, k0, k1;
};
void launch_r2c(Ctx &c, const R2cArgs &a);
struct C2rArgs {
  const cplx_t *src, *src2;  // x = src (+ scale2*src2)
  double scale2;
  double *dst;
  int j0, j1, k0, k1;
};
void launch_c2r(Ctx &c, const C2rArgs &a);

// RK pieces (ek_rk.cu)
void launch_spectral_rhs(Ctx &c, int rk);
void launch_face_velocity(Ctx &c);
void launch_adi(Ctx &c, int field, int rk);
void launch_th_corners(Ctx &c);
void launch_divergence_rhs(Ctx &c, double *rhs_finest, int nprob);
void launch_projection(Ctx &c, const double *phif, int nprob, double temp4, bool update_p);
int finish_divergence(Ctx &c, double *div_out);

// multigrid (ek_mg.cu)
int mg_solve(Ctx &c, int nprob, const double *kx2_dev, ek_mg_stats *st);
void mg_alloc(Ctx &c, int pmax);

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
