// C ABI of the GB300 duct substep (include/ekgpu.h) and the host-side
// orchestration of one RK substep: the same order of operations as
// RK_DUCT (src/duct.F90:237-2469), with every transform, stencil and solve
// running on the GPU and the state resident in HBM.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include "ek_internal.h"
#include "ek_unet.h"

using namespace ek;

struct ek_ctx {
  Ctx c;
};

struct ek_unet {
  std::unique_ptr<ek::UNet> net;
  std::string err;
};

namespace ek {
void rk_init_attributes();
void fft_init_attributes();
void les_init_attributes();
const char *last_global_error();
}  // namespace ek

namespace {

int fail(Ctx &c, int code, const std::string &m) {
  c.err = m;
  return code;
}

template <typename F>
int guarded(ek_ctx *h, F &&f) {
  if (!h) return EK_ERR_ARG;
  try {
    return f(h->c);
  } catch (const CudaError &e) {
    h->c.err = e.msg;
    return EK_ERR_CUDA;
  } catch (const std::bad_alloc &) {
    h->c.err = "host allocation failed";
    return EK_ERR_CUDA;
  }
}

template <typename T>
T *dalloc(Ctx &c, size_t n) {
  void *p = nullptr;
  EK_CUDA(cudaMalloc(&p, n * sizeof(T)));
  EK_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), c.stream));
  c.allocs.push_back(p);
  return static_cast<T *>(p);
}

bool supported_bc(const ek_params &p, std::string &why) {
  auto in = [](int v, std::initializer_list<int> s) { return std::find(s.begin(), s.end(), v) != s.end(); };
  for (int f = 0; f < 3; ++f) {
    const int *b = (f == 0) ? p.u_bc : (f == 1) ? p.v_bc : p.w_bc;
    if (!in(b[EK_YMIN], {0, 1, 6}) || !in(b[EK_YMAX], {0, 1, 6})) { why = "velocity y BC must be 0, 1 or 6"; return false; }
    if (!in(b[EK_ZMIN], {0, 1, 6}) || !in(b[EK_ZMAX], {0, 1, 6})) { why = "velocity z BC must be 0, 1 or 6"; return false; }
    if ((f == 1 || f == 2) && b[EK_ZMIN] == 0) { why = "U2/U3 Dirichlet z-min needs the background profiles"; return false; }
  }
  if (!in(p.th_bc[EK_YMIN], {0, 1, 5, 6}) || !in(p.th_bc[EK_YMAX], {0, 1, 6}) || !in(p.th_bc[EK_ZMIN], {0, 1, 6}) ||
      !in(p.th_bc[EK_ZMAX], {0, 1, 6})) {
    why = "unsupported TH BC";
    return false;
  }
  return true;
}

// Thomas factors of every field, substep and direction for the current
// DELTA_T (they depend on it through TEMP1 = NU*H_BAR(RK_STEP)/2).
void build_adi_factors(Ctx &c) {
  for (int f = 0; f < 4; ++f)
    for (int rk = 1; rk <= 3; ++rk)
      for (int dir = 0; dir < 2; ++dir) {
        std::vector<double> a, ib, u;
        adi_factor_host(c, f, rk, dir, c.h_jac, c.h_g11, c.h_g22, a, ib, u);
        AdiFactors &F = c.adi[f][rk][dir];
        if (!F.a) {
          F.a = dalloc<double>(c, a.size());
          F.ib = dalloc<double>(c, ib.size());
          F.u = dalloc<double>(c, u.size());
          if (c.p.ff_arith) {
            F.a2 = dalloc<float2>(c, a.size());
            F.ib2 = dalloc<float2>(c, ib.size());
            F.u2 = dalloc<float2>(c, u.size());
          }
        }
        EK_CUDA(cudaMemcpyAsync(F.a, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice, c.stream));
        EK_CUDA(cudaMemcpyAsync(F.ib, ib.data(), sizeof(double) * ib.size(), cudaMemcpyHostToDevice, c.stream));
        EK_CUDA(cudaMemcpyAsync(F.u, u.data(), sizeof(double) * u.size(), cudaMemcpyHostToDevice, c.stream));
        if (F.a2) {
          split_ff(c, F.a, F.a2, a.size());
          split_ff(c, F.ib, F.ib2, ib.size());
          split_ff(c, F.u, F.u2, u.size());
        }
        EK_CUDA(cudaStreamSynchronize(c.stream));
      }
}

// DELTA_T and the H_BAR of COURANT_CURV_MPI (duct.F90:3655-3668)
void set_delta_t(Ctx &c, double dt) {
  c.p.delta_t = dt;
  c.H_BAR[1] = dt * (8.0 / 15.0);
  c.H_BAR[2] = dt * (2.0 / 15.0);
  c.H_BAR[3] = dt * (5.0 / 15.0);
  build_adi_factors(c);
}

// What a substep reports for its projection solve.  Under the residual rule
// a problem that reached mg_maxcy above the tolerance makes it
// EK_ERR_NOT_CONVERGED (the substep is complete and its state valid).  Under
// MUDPACK's relative-change rule the count stays in the statistics only, as
// MULTIGRID_MUDPACK ignores mud2cr's ierror = -1 (mg_solver2d.F90:195-199,
// mud2cr.f:204-207).
int projection_status(const Ctx &c, int mg) {
  // REM_DIV_CURV ends with IF (DELTA_T .LT. 1.0E-4) STOP 'DELTA_T is zero'
  // (duct.F90:2812): the bound is the REAL*4 literal 1.0E-4
  if (c.p.delta_t < static_cast<double>(1.0e-4f)) return EK_ERR_DT;
  if (mg == EK_OK) return EK_OK;
  if (mg == EK_ERR_NOT_CONVERGED) return c.p.mg_stop == EK_MG_STOP_RESIDUAL ? EK_ERR_NOT_CONVERGED : EK_OK;
  return mg;
}

void run_rem_div(Ctx &c, double temp4, bool update_p, int *mg_status) {
  const int P = 2 * (c.d.NKX + 1);
  launch_divergence_rhs(c, c.mgw.rhs[c.mg.ngrid - 1], P);
  *mg_status = mg_solve(c, P, c.mgw.kx2, c.mg_kx2_host.data(), nullptr);
  if (c.guess.sink_x)
    guess_collect(c, P, c.mgw.rhs[c.mg.ngrid - 1], c.mgw.phif, c.mgw.kx2, c.mg_kx2_host, c.stream);
  launch_projection(c, c.mgw.phif, P, temp4, update_p);
}

int substep(Ctx &c, int rk) {
  const Dims &d = c.d;
  const ek_params &p = c.p;
  if (p.les && !c.les.have_metrics) return fail(c, EK_ERR_STATE, "LES metrics not set (ekgpu_set_les_metrics)");
  const bool th = p.n_th > 0;
  const double TEMP4 = c.H_BAR[rk];
  const double TEMP5 = c.BETA_BAR[rk] * c.H_BAR[rk];
  // FP32 copies of the physical fields for the nonlinear terms (fft_fp32)
  const bool f32 = p.fft_fp32 != 0;
  // float-float physical fields: the FP32 copy is the high part, the low
  // part goes to the FP64 buffer's first half, no FP64 field is written
  const bool ffp = ff_fields(c);
  // increment form: the state's inverse transforms are FP32, into the FP32
  // copies only
  const bool inc = inc_fields(c);
  launch_spectral_rhs(c, rk);
  // to physical space (duct.F90:656-673)
  {
    C2rArgs a{};
    a.j0 = 0; a.j1 = d.NY + 1; a.k0 = 0; a.k1 = d.NZ + 1;
    a.lowp = inc ? 1 : 0;
    auto to_phys = [&](const cplx_t *src, double *dst, float *dstf) {
      a.src = src;
      a.dst = (ffp || inc) ? nullptr : dst;
      a.dstf = f32 ? dstf : nullptr;
      a.dstlo = ffp ? ff_lo(dst) : nullptr;
      launch_c2r(c, a);
    };
    to_phys(c.CU1, c.U1, c.U1f);
    to_phys(c.CU2, c.U2, c.U2f);
    to_phys(c.CU3, c.U3, c.U3f);
    if (th) to_phys(c.CTH, c.TH, c.THf);
  }
  // les_chan / les_chan_th (duct.F90:641-654): NU_T and the stress terms
  // that the transforms below add to CF1..CF3 and CFTH
  const bool les = les_active(c);
  if (les) launch_les(c, rk);
  launch_face_velocity(c);
  // nonlinear and cross-diffusion terms of velocity component f (0..2),
  // fused with their forward FFTs (duct.F90:683-1121)
  auto nl_velocity = [&](int f) {
    R2cArgs a{};
    a.j0 = d.JS; a.j1 = d.JE; a.k0 = d.ZS; a.k1 = d.ZE;
    const double *uu[3] = {c.U1, c.U2, c.U3};
    const float *uf[3] = {c.U1f, c.U2f, c.U3f};
    cplx_t *cf[3] = {c.CF1, c.CF2, c.CF3};
    a.lowp = 1;
    // the component's product and flux terms in one launch
    a.fuse_flux = 1;
    a.pro = PRO_PROD; a.a = c.U1; a.b = uu[f]; a.epi = EPI_SUB_IK; a.dst = cf[f];
    a.af = f32 ? c.U1f : nullptr; a.bf = f32 ? uf[f] : nullptr;
    a.extra = les ? c.les.t[f] : nullptr;  // + J tau_1f
    a.extraf = les ? c.les.tf[f] : nullptr;
    a.a2 = uu[f]; a.b2 = c.U2b; a.visc2 = p.nu;
    a.a2f = f32 ? uf[f] : nullptr; a.b2f = f32 ? c.U2bf : nullptr;
    a.extra2 = les ? c.les.ext[f] : nullptr;  // + NU_T cross term - stress divergence
    a.extraf2 = les ? c.les.extf[f] : nullptr;
    launch_r2c(c, a);
  };
  // R = c2r(CR + beta h CF) (duct.F90:1127-1161); in the explicit-increment
  // form S = R - J phi_old, in FP32, into R's slots
  const bool sform = explicit_increment_form(c);
  auto rdst = [&](C2rArgs &a, double *r) {
    a.dst = sform ? nullptr : r;
    a.dstf = sform ? reinterpret_cast<float *>(r) : nullptr;
    a.lowp = sform ? 1 : 0;
  };
  auto r_velocity = [&](int f) {
    const cplx_t *cr[3] = {c.CR1, c.CR2, c.CR3}, *cf[3] = {c.CF1, c.CF2, c.CF3};
    double *rr[3] = {c.R1, c.R2, c.R3};
    C2rArgs a{};
    a.j0 = d.JS; a.j1 = d.JE; a.k0 = d.ZS; a.k1 = d.ZE;
    a.scale2 = TEMP5;
    a.src = cr[f]; a.src2 = cf[f]; rdst(a, rr[f]); launch_c2r(c, a);
  };
  // scalar nonlinear terms (duct.F90:1165-1252) and RTH (1304-1326)
  auto th_explicit = [&]() {
    R2cArgs a{};
    a.j0 = d.JST; a.j1 = d.JET; a.k0 = d.ZST; a.k1 = d.ZET;
    a.lowp = 1;
    a.pro = PRO_PROD; a.a = c.TH; a.b = c.U1; a.epi = EPI_SUB_IK; a.dst = c.CFTH;
    a.af = f32 ? c.THf : nullptr; a.bf = f32 ? c.U1f : nullptr;
    a.extra = les ? c.les.tth : nullptr;  // + J (-KAPPA_T dTH/dx)
    a.extraf = les ? c.les.tthf : nullptr;
    a.fuse_flux = 1;
    a.a2 = c.TH; a.b2 = c.U2b; a.visc2 = p.nu / p.pr;
    a.a2f = f32 ? c.THf : nullptr; a.b2f = f32 ? c.U2bf : nullptr;
    a.extra2 = les ? c.les.ext[3] : nullptr;  // + KAPPA_T cross term
    a.extraf2 = les ? c.les.extf[3] : nullptr;
    launch_r2c(c, a);
    C2rArgs b{};
    b.j0 = d.JST; b.j1 = d.JET; b.k0 = d.ZST; b.k1 = d.ZET;
    b.scale2 = TEMP5; b.src = c.CRTH; b.src2 = c.CFTH; rdst(b, c.RTH);
    launch_c2r(c, b);
  };
  // back to Fourier space (duct.F90:2421-2451), one field
  auto to_fourier = [&](int f) {
    double *src = (f == 0) ? c.TH : (f == 1) ? c.U1 : (f == 2) ? c.U2 : c.U3;
    const float *srcf = (f == 0) ? c.THf : (f == 1) ? c.U1f : (f == 2) ? c.U2f : c.U3f;
    cplx_t *dst = (f == 0) ? c.CTH : (f == 1) ? c.CU1 : (f == 2) ? c.CU2 : c.CU3;
    double *R = (f == 0) ? c.RTH : (f == 1) ? c.R1 : (f == 2) ? c.R2 : c.R3;
    R2cArgs a{};
    a.j0 = 0; a.j1 = d.NY + 1; a.k0 = 0; a.k1 = d.NZ + 1;
    a.pro = PRO_LOAD; a.epi = EPI_STORE;
    if (inc) {
      // CU += the FP32 transform of the ADI's total increment
      a.lowp = 1;
      a.epi = EPI_ADD;
      a.zero_hi = 1;
      a.a = nullptr;
      a.af = inc_plane(c, R);
      a.alo = nullptr;
    } else {
      a.a = ffp ? nullptr : src;
      a.af = ffp ? srcf : nullptr;
      a.alo = ffp ? ff_lo(src) : nullptr;
    }
    a.dst = dst;
    launch_r2c(c, a);
  };
  // COURANT_CURV_MPI (duct.F90:2417-2419) reads every field after its ADI
  const bool courant = p.variable_dt && rk == 3 && p.update_dt > 0 && p.time_step % p.update_dt == 0;
  // In the increment form each field's chain -- its explicit terms, ADI
  // (with TH's corner copies) and forward transform -- runs on a stream of
  // its own, forked from and joined back to the step's stream: the chains
  // share no array (every one reads the FP32 physical fields and face
  // velocities, none writes them), and the transforms of one fill the
  // latency-bound line solves of another.  (Not under the per-kernel timer,
  // whose events need one stream, nor when COURANT_CURV_MPI sits between the
  // ADI and the transforms.)
  const bool fork = inc && !c.timing && !courant;
  const int f0 = th ? 0 : 1;
  // the previous substep's divergence check reads CU1 and the face
  // velocities, which the chains below and the projection write
  div_join(c);
  if (fork) {
    const cudaStream_t main = c.stream;
    EK_CUDA(cudaEventRecord(c.field_ev[4], main));
    try {
      for (int f = f0; f < 4; ++f) {
        EK_CUDA(cudaStreamWaitEvent(c.field_stream[f], c.field_ev[4], 0));
        c.stream = c.field_stream[f];
        if (f == 0) th_explicit();
        else {
          nl_velocity(f - 1);
          r_velocity(f - 1);
        }
        launch_adi(c, f, rk);
        if (f == 0) launch_th_corners(c);
        to_fourier(f);
        EK_CUDA(cudaEventRecord(c.field_ev[f], c.stream));
        c.stream = main;
      }
    } catch (...) {
      c.stream = main;
      throw;
    }
    for (int f = f0; f < 4; ++f) EK_CUDA(cudaStreamWaitEvent(main, c.field_ev[f], 0));
  } else {
    for (int f = 0; f < 3; ++f) nl_velocity(f);
    for (int f = 0; f < 3; ++f) r_velocity(f);
    if (th) {
      th_explicit();
      launch_adi(c, 0, rk);
      launch_th_corners(c);
    }
    launch_adi(c, 1, rk);
    launch_adi(c, 2, rk);
    launch_adi(c, 3, rk);
    // the new DELTA_T applies from the next substep; this one's projection
    // keeps TEMP4
    if (courant) {
      launch_courant(c);
      double dt = 0.0;
      EK_CUDA(cudaMemcpyAsync(&dt, c.cfl_dt, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      EK_CUDA(cudaStreamSynchronize(c.stream));
      if (dt > 0.0) {
        const double nd = (dt >= p.delta_t_set) ? p.delta_t_set : dt;
        if (nd != p.delta_t) set_delta_t(c, nd);
      }
    }
    to_fourier(1);
    to_fourier(2);
    to_fourier(3);
    if (th) to_fourier(0);
  }
  int mg = EK_OK;
  run_rem_div(c, TEMP4, true, &mg);
  const int dv = finish_divergence(c, nullptr);
  return dv != EK_OK ? dv : projection_status(c, mg);
}

// ---- whole-step CUDA graphs ------------------------------------------------
// ekgpu_step runs each RK3 step as one CUDA graph when the step's launches
// depend on nothing but the context's plan and a few host-side choices (the
// key below): the mixed solver (its correction cycles loop in conditional
// while-nodes), a fixed time step, constant mean-pressure forcing, no learned
// guess or pair collection, the per-kernel timer off.  Statistics and the
// divergence of each substep are read once, after the step.
bool step_graph_eligible(const Ctx &c) {
  const ek_params &p = c.p;
  // a time step below the reference's bound stops the run after the first
  // substep's projection, which the eager path reports
  return c.step_graphs && !c.timing && p.mg_fast && !p.variable_dt && p.f_type == 1 &&
         p.delta_t >= static_cast<double>(1.0e-4f) &&
         !(c.guess.net && c.guess.use) && !c.guess.sink_x;
}

// The host-side choices a step's launches depend on: LES active, FIRST_TIME,
// C_DYN due at RK_STEP 1 (MOD(TIME_STEP, 5) = 0), sponge_th's CU2X reset.
unsigned long long step_graph_key(const Ctx &c) {
  const ek_params &p = c.p;
  const bool reset = p.sponge_type != 0 && p.save_stats_int > 0 && (2 * p.time_step) % p.save_stats_int == 0;
  return (les_active(c) ? 1ull : 0ull) | (c.les.first_time ? 2ull : 0ull) | (p.time_step % 5 == 0 ? 4ull : 0ull) |
         (reset ? 8ull : 0ull);
}

// The three substeps of one step, captured on stream s (which is capturing);
// fills the launch counts of sg.
void capture_substeps(Ctx &c, cudaStream_t s, StepGraph &sg) {
  const cudaStream_t saved = c.stream;
  const long long l0 = c.launches;
  long long body = 0;
  c.stream = s;
  try {
    for (int rk = 1; rk <= 3; ++rk) {
      c.graph_slot = rk - 1;
      c.graph_body_launches = 0;
      const int st = substep(c, rk);
      if (st != EK_OK) throw CudaError("step graph: substep " + std::to_string(rk) + " returned " + std::to_string(st));
      sg.body_launches[rk - 1] = c.graph_body_launches;
      body += c.graph_body_launches;
    }
    div_join(c);  // the last substep's check ends inside the graph
  } catch (...) {
    c.graph_slot = -1;
    c.stream = saved;
    c.launches = l0;
    c.div_pending = false;
    throw;
  }
  c.graph_slot = -1;
  c.stream = saved;
  sg.fixed_launches = c.launches - l0 - body;
  c.launches = l0;
}

StepGraph &step_graph_capture(Ctx &c, unsigned long long key) {
  StepGraph sg;
  sg.key = key;
  EK_CUDA(cudaStreamBeginCapture(c.cap_stream, cudaStreamCaptureModeThreadLocal));
  try {
    capture_substeps(c, c.cap_stream, sg);
  } catch (...) {
    cudaGraph_t junk = nullptr;
    cudaStreamEndCapture(c.cap_stream, &junk);
    if (junk) cudaGraphDestroy(junk);
    throw;
  }
  EK_CUDA(cudaStreamEndCapture(c.cap_stream, &sg.graph));
  if (cudaGraphInstantiate(&sg.exec, sg.graph, 0) != cudaSuccess) {
    cudaGraphDestroy(sg.graph);
    throw CudaError("step graph: cudaGraphInstantiate failed");
  }
  c.graphs.push_back(sg);
  return c.graphs.back();
}

int step_stats_apply(Ctx &c, const StepGraph &sg, int &late);

// One step from its graph; late becomes EK_ERR_NOT_CONVERGED when a solve
// of the step missed the residual rule's tolerance.
int step_graph_run(Ctx &c, const StepGraph &sg, int &late) {
  EK_CUDA(cudaGraphLaunch(sg.exec, c.stream));
  EK_CUDA(cudaMemcpyAsync(c.step_stats_host, c.step_stats_dev, 3 * sizeof(StepStats), cudaMemcpyDeviceToHost,
                          c.stream));
  EK_CUDA(cudaStreamSynchronize(c.stream));
  return step_stats_apply(c, sg, late);
}

// The statistics a graph-run step left in the context's pinned slots: launch
// count, multigrid totals and last stats, divergence, status.
int step_stats_apply(Ctx &c, const StepGraph &sg, int &late) {
  long long n = sg.fixed_launches;
  bool nan = false;
  for (int k = 0; k < 3; ++k) {
    const StepStats &S = c.step_stats_host[k];
    n += (long long)S.max_cycles * sg.body_launches[k];
    c.mg_solved_total += S.nprob;
    c.mg_nc_total += S.n_not_converged;
    if (S.n_not_converged && c.p.mg_stop == EK_MG_STOP_RESIDUAL) late = EK_ERR_NOT_CONVERGED;
    if (S.div != S.div) nan = true;
  }
  c.launches += n;
  const StepStats &L = c.step_stats_host[2];
  ek_mg_stats st{};
  st.nprob = L.nprob;
  st.min_cycles = L.min_cycles;
  st.max_cycles = L.max_cycles;
  st.n_not_converged = L.n_not_converged;
  st.max_residual = L.max_residual;
  c.last_stats = st;
  c.last_div = L.div;
  return nan ? EK_ERR_NAN : EK_OK;
}

// ---- ensembles in one graph launch -------------------------------------------
// Members that all take the graph path step together from one CUDA graph
// per ensemble step: each member's three substeps are a branch of its own,
// forked from and joined to the graph's root, so one cudaGraphLaunch runs
// every member's kernels side by side.  Graphs are cached process-wide by
// the members' (epoch, key) pairs; an epoch is never reused, so a graph of
// a destroyed or re-planned member is never launched again.
struct EnsembleGraph {
  std::vector<unsigned long long> sig;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<StepGraph> parts;  // per member: its launch counts
  std::vector<cudaEvent_t> ev;   // ordering against the members' own streams
  ~EnsembleGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
};
std::mutex g_ens_mu;
// most recent last; never destroyed at exit (the CUDA runtime may be gone by then)
std::vector<std::unique_ptr<EnsembleGraph>> &g_ens = *new std::vector<std::unique_ptr<EnsembleGraph>>();
constexpr size_t kEnsembleGraphsKept = 8;

EnsembleGraph &ensemble_graph(const std::vector<ek_ctx *> &m, const std::vector<unsigned long long> &sig) {
  for (auto &e : g_ens)
    if (e->sig == sig) return *e;
  const int n = (int)m.size();
  auto eg = std::make_unique<EnsembleGraph>();
  eg->sig = sig;
  eg->parts.resize(n);
  eg->ev.resize(n + 1);
  for (cudaEvent_t &e : eg->ev) EK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  Ctx &c0 = m[0]->c;
  const cudaStream_t root = c0.cap_stream;
  EK_CUDA(cudaStreamBeginCapture(root, cudaStreamCaptureModeThreadLocal));
  try {
    EK_CUDA(cudaEventRecord(eg->ev[n], root));  // the fork
    for (int i = 0; i < n; ++i) {
      Ctx &c = m[i]->c;
      if (i > 0) EK_CUDA(cudaStreamWaitEvent(c.cap_stream, eg->ev[n], 0));
      capture_substeps(c, c.cap_stream, eg->parts[i]);
      if (i > 0) {
        EK_CUDA(cudaEventRecord(eg->ev[i], c.cap_stream));
        EK_CUDA(cudaStreamWaitEvent(root, eg->ev[i], 0));
      }
    }
  } catch (...) {
    cudaGraph_t junk = nullptr;
    cudaStreamEndCapture(root, &junk);
    if (junk) cudaGraphDestroy(junk);
    throw;
  }
  EK_CUDA(cudaStreamEndCapture(root, &eg->graph));
  if (cudaGraphInstantiate(&eg->exec, eg->graph, 0) != cudaSuccess) throw CudaError("ensemble graph: instantiate failed");
  if (g_ens.size() >= kEnsembleGraphsKept) g_ens.erase(g_ens.begin());
  g_ens.push_back(std::move(eg));
  return *g_ens.back();
}

// One step of every member from one graph launch; st[i] receives member i's
// status.  Throws CudaError when the graph cannot be captured (nothing has
// run then, and TIME_STEP is left as it was).
void ensemble_graph_step(const std::vector<ek_ctx *> &m, std::vector<int> &st, std::vector<int> &late) {
  const int n = (int)m.size();
  std::lock_guard<std::mutex> lk(g_ens_mu);
  for (ek_ctx *h : m) h->c.p.time_step += 1;
  std::vector<unsigned long long> sig;
  for (ek_ctx *h : m) {
    sig.push_back(h->c.epoch);
    sig.push_back(step_graph_key(h->c));
  }
  EnsembleGraph *eg = nullptr;
  try {
    eg = &ensemble_graph(m, sig);
  } catch (...) {
    for (ek_ctx *h : m) h->c.p.time_step -= 1;
    throw;
  }
  Ctx &c0 = m[0]->c;
  // after the work already queued on every member's stream
  for (int i = 1; i < n; ++i) {
    EK_CUDA(cudaEventRecord(eg->ev[i], m[i]->c.stream));
    EK_CUDA(cudaStreamWaitEvent(c0.stream, eg->ev[i], 0));
  }
  EK_CUDA(cudaGraphLaunch(eg->exec, c0.stream));
  for (ek_ctx *h : m)
    EK_CUDA(cudaMemcpyAsync(h->c.step_stats_host, h->c.step_stats_dev, 3 * sizeof(StepStats), cudaMemcpyDeviceToHost,
                            c0.stream));
  EK_CUDA(cudaEventRecord(eg->ev[n], c0.stream));
  for (int i = 1; i < n; ++i) EK_CUDA(cudaStreamWaitEvent(m[i]->c.stream, eg->ev[n], 0));
  EK_CUDA(cudaStreamSynchronize(c0.stream));
  for (int i = 0; i < n; ++i) {
    Ctx &c = m[i]->c;
    const int r = step_stats_apply(c, eg->parts[i], late[i]);
    if (r == EK_ERR_NAN) st[i] = fail(c, EK_ERR_NAN, "DIV is a NaN");
    c.p.time += c.p.delta_t;
    c.les.first_time = false;
  }
}

__global__ void k_transpose(const double *in, double *out, int P, long npt, int to_inner) {
  const long n = (long)P * npt;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    if (to_inner) {  // in [p][pt] -> out [pt][p]
      const int p = (int)(t % P);
      const long pt = t / P;
      out[t] = in[(size_t)p * npt + pt];
    } else {         // in [pt][p] -> out [p][pt]
      const long pt = t % npt;
      const int p = (int)(t / npt);
      out[t] = in[(size_t)pt * P + p];
    }
  }
}

}  // namespace

namespace ek {
// Drop every captured step graph (the plan they were captured from changed).
// The new epoch also retires every ensemble graph that holds this context.
void step_graphs_clear(Ctx &c) {
  static std::atomic<unsigned long long> next_epoch{1};
  for (StepGraph &g : c.graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  c.graphs.clear();
  c.eager_since_plan = false;
  c.epoch = next_epoch.fetch_add(1);
}

// Sum the recorded per-kernel-class event pairs into kms/kcnt.
void timing_resolve(Ctx &c) {
  if (c.trec.empty()) return;
  EK_CUDA(cudaStreamSynchronize(c.stream));
  for (const TimerRec &r : c.trec) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    c.kms[r.cls] += ms;
    c.kcnt[r.cls] += 1;
    c.evpool.push_back(r.a);
    c.evpool.push_back(r.b);
  }
  c.trec.clear();
}
}  // namespace ek

namespace {

int poisson_dev(Ctx &c, const double *rhs_dev, double *phi_dev, const double *kx2_dev, const double *kx2_host,
                int nprob, ek_mg_stats *st) {
  if (!c.have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
  if (nprob <= 0) return fail(c, EK_ERR_ARG, "nprob must be positive");
  if (nprob > c.mgw.pmax) mg_alloc(c, nprob);
  const long npt = (long)c.mg.nfx * c.mg.nfy;
  long n = npt * nprob;
  unsigned blocks = (unsigned)std::min<long>((n + 255) / 256, 65535L * 16);
  k_transpose<<<blocks, 256, 0, c.stream>>>(rhs_dev, c.mgw.rhs[c.mg.ngrid - 1], nprob, npt, 1);
  after_launch(c);
  const int r = mg_solve(c, nprob, kx2_dev, kx2_host, st);
  k_transpose<<<blocks, 256, 0, c.stream>>>(c.mgw.phif, phi_dev, nprob, npt, 0);
  after_launch(c);
  EK_CUDA(cudaStreamSynchronize(c.stream));
  return r;
}

}  // namespace

extern "C" {

int ekgpu_default_params(ek_params *p) {
  if (!p) return EK_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  p->lx = 4.0 * M_PI;
  p->nu = 1.0e-3;
  p->delta_t = 1.0e-3;
  p->f0 = 1.0e-4;
  p->wbulk0 = 5.0e-2;
  p->f_type = 1;
  p->n_th = 1;
  p->pr = 1.0;
  p->ic_type = 7;
  for (int *b : {p->u_bc, p->v_bc, p->w_bc, p->th_bc}) {
    b[EK_YMIN] = 0; b[EK_YMAX] = 1; b[EK_ZMIN] = 6; b[EK_ZMAX] = 6;
  }
  p->mudpack_bc[0] = 0; p->mudpack_bc[1] = 0; p->mudpack_bc[2] = 2; p->mudpack_bc[3] = 2;
  p->mg_maxcy = 6; p->mg_kcycle = 2; p->mg_iprer = 2; p->mg_ipost = 1; p->mg_intpol = 3;
  p->mg_stop = EK_MG_STOP_RELCHANGE;
  p->mg_tol = (double)powf(10.0f, -6.0f);
  p->ny_s_t = 0;
  p->nz_s_r = 0;
  p->nz_s_l = 0;
  p->save_stats_int = 100;
  p->les_model_type = 2;
  p->les_model_type_th = 1;
  p->create_new_flow = 1;
  return EK_OK;
}

int ekgpu_create(const ek_params *pp, ek_ctx **out) {
  if (!pp || !out) return EK_ERR_ARG;
  *out = nullptr;
  auto h = std::unique_ptr<ek_ctx>(new (std::nothrow) ek_ctx());
  if (!h) return EK_ERR_ARG;
  Ctx &c = h->c;
  c.p = *pp;
  const ek_params &p = c.p;
  std::string why;
  auto reject = [&](const std::string &m) {
    c.err = m;
    *out = h.release();
    return (int)EK_ERR_ARG;
  };
  if (p.nx < 8 || p.nx > 1024 || (p.nx & (p.nx - 1))) return reject("NX must be a power of two in [8, 1024]");
  if (p.ny < 4 || p.nz < 4) return reject("NY and NZ must be >= 4");
  if (p.ic_type != 7) return reject("only IC_TYPE = 7 boundary rows are supported");
  if (p.mudpack_bc[0] != 0 || p.mudpack_bc[1] != 0 || p.mudpack_bc[2] != 2 || p.mudpack_bc[3] != 2)
    return reject("only MUDPACK_BC = 0 0 2 2 is supported");
  if (p.sponge_type < 0 || p.sponge_type > 2) return reject("SPONGE_TYPE must be 0, 1 or 2");
  if (p.sponge_type != 0 && p.save_stats_int < 1) return reject("SAVE_STATS_INT must be >= 1 with a sponge");
  if (p.fft_fp32 < 0 || p.fft_fp32 > 2) return reject("fft_fp32 must be 0, 1 or 2");
  if (p.ff_arith < 0 || p.ff_arith > 2) return reject("ff_arith must be 0, 1 or 2");
  if (p.variable_dt && (p.update_dt < 1 || !(p.cfl > 0.0) || !(p.delta_t_set > 0.0)))
    return reject("VARIABLE_DT needs UPDATE_DT >= 1, CFL > 0 and DELTA_T_SET > 0");
  if (p.sponge_type != 0 && p.ny_s_t <= p.ny && p.ny_s_t < 0) return reject("NY_S_T must be >= 0");
  if (p.les != 0) {
    if (p.les_model_type != 2) return reject("LES: only LES_MODEL_TYPE = 2 (dynamic Smagorinsky) is supported");
    if (p.n_th > 0 && p.les_model_type_th != 1) return reject("LES: only LES_MODEL_TYPE_TH = 1 is supported");
  }
  if (p.f_type != 1 && p.f_type != 2) return reject("F_TYPE must be 1 or 2");
  if (p.n_th < 0 || p.n_th > 1) return reject("N_TH must be 0 or 1");
  if (p.mg_kcycle < 1 || p.mg_iprer < 1 || p.mg_ipost < 1 || (p.mg_intpol != 1 && p.mg_intpol != 3) || p.mg_maxcy < 1)
    return reject("bad multigrid options");
  if (p.mg_stop != EK_MG_STOP_RELCHANGE && p.mg_stop != EK_MG_STOP_RESIDUAL) return reject("bad mg_stop");
  if (p.mg_fast && p.mg_stop != EK_MG_STOP_RESIDUAL) return reject("mg_fast needs mg_stop = EK_MG_STOP_RESIDUAL");
  if (!supported_bc(p, why)) return reject(why);
  MgPlan &P = c.mg;
  if (p.mg_ixp > 0) {
    P.ixp = p.mg_ixp; P.jyq = p.mg_jyq; P.iex = p.mg_iex; P.jey = p.mg_jey;
  } else if (!mg_pick_shape(p.nz + 2, P.ixp, P.iex) || !mg_pick_shape(p.ny + 2, P.jyq, P.jey)) {
    return reject("NZ+2 and NY+2 must have the form p*2^k+1 (MUDPACK)");
  }
  if (P.ixp < 2 || P.jyq < 2 || P.ixp * (1 << (P.iex - 1)) + 1 != p.nz + 2 || P.jyq * (1 << (P.jey - 1)) + 1 != p.ny + 2)
    return reject("Mudpack Multigrid Parameters are not Matching Grid Dimensions.");
  try {
    EK_CUDA(cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking));
    c.stream = c.own_stream;
    EK_CUDA(cudaStreamCreateWithFlags(&c.cap_stream, cudaStreamNonBlocking));
    EK_CUDA(cudaStreamCreateWithFlags(&c.cap_stream2, cudaStreamNonBlocking));
    for (int f = 0; f < 4; ++f) EK_CUDA(cudaStreamCreateWithFlags(&c.field_stream[f], cudaStreamNonBlocking));
    for (int f = 0; f < 5; ++f) EK_CUDA(cudaEventCreateWithFlags(&c.field_ev[f], cudaEventDisableTiming));
    EK_CUDA(cudaStreamCreateWithFlags(&c.div_stream, cudaStreamNonBlocking));
    for (int f = 0; f < 2; ++f) EK_CUDA(cudaEventCreateWithFlags(&c.div_ev[f], cudaEventDisableTiming));
    EK_CUDA(cudaHostAlloc(&c.step_stats_host, 3 * sizeof(StepStats), cudaHostAllocDefault));
    step_graphs_clear(c);  // a fresh epoch
    rk_init_attributes();
    fft_init_attributes();
    if (p.les) les_init_attributes();
    Dims &d = c.d;
    d.NX = p.nx; d.NY = p.ny; d.NZ = p.nz;
    d.NKX = p.nx / 3; d.NX2P = p.nx / 2;
    d.LDX = p.nx + 2; d.LDC = p.nx / 2 + 1;
    d.NZ2 = p.nz + 2; d.NY2 = p.ny + 2; d.LDM = p.nz + 3;
    // INIT_DUCT (duct.F90:7-232), IC_TYPE = 7 branches
    const int *ub = p.u_bc, *wb = p.w_bc, *tb = p.th_bc;
    d.JS = (wb[EK_YMIN] == 0 || wb[EK_YMIN] == 1 || wb[EK_YMIN] == 6) ? 1 : 2;
    d.ZS = (ub[EK_ZMIN] == 1 || ub[EK_ZMIN] == 6) ? 1 : 2;
    d.JE = (wb[EK_YMAX] == 0 || wb[EK_YMAX] == 1 || wb[EK_YMAX] == 6) ? p.ny : p.ny - 1;
    d.ZE = (ub[EK_ZMAX] == 0 || ub[EK_ZMAX] == 1 || ub[EK_ZMAX] == 6) ? p.nz : p.nz - 1;
    d.JST = (tb[EK_YMIN] == 0 || tb[EK_YMIN] == 1 || tb[EK_YMIN] == 5 || tb[EK_YMIN] == 6) ? 1 : 2;
    d.ZST = (tb[EK_ZMIN] == 0 || tb[EK_ZMIN] == 1 || tb[EK_ZMIN] == 6) ? 1 : 2;
    d.JET = (tb[EK_YMAX] == 0 || tb[EK_YMAX] == 1 || tb[EK_YMAX] == 6) ? p.ny : p.ny - 1;
    d.ZET = (tb[EK_ZMAX] == 0 || tb[EK_ZMAX] == 1 || tb[EK_ZMAX] == 6) ? p.nz : p.nz - 1;
    // RKW3 (diablo.F90:568-576)
    const double dt = p.delta_t;
    c.H_BAR[1] = dt * (8.0 / 15.0); c.H_BAR[2] = dt * (2.0 / 15.0); c.H_BAR[3] = dt * (5.0 / 15.0);
    c.BETA_BAR[1] = 1.0; c.BETA_BAR[2] = 25.0 / 8.0; c.BETA_BAR[3] = 9.0 / 4.0;
    c.ZETA_BAR[1] = 0.0; c.ZETA_BAR[2] = -17.0 / 8.0; c.ZETA_BAR[3] = -5.0 / 4.0;
    // wavenumbers KX = 2 pi i / LX, KX2 = KX^2
    c.kx_h.resize(d.NX2P + 1);
    c.kx2_h.resize(d.NX2P + 1);
    for (int i = 0; i <= d.NX2P; ++i) {
      c.kx_h[i] = i * (2.0 * M_PI) / p.lx;
      c.kx2_h[i] = c.kx_h[i] * c.kx_h[i];
    }
    c.kx = dalloc<double>(c, d.NX2P + 1);
    c.kx2 = dalloc<double>(c, d.NX2P + 1);
    EK_CUDA(cudaMemcpy(c.kx, c.kx_h.data(), sizeof(double) * (d.NX2P + 1), cudaMemcpyHostToDevice));
    EK_CUDA(cudaMemcpy(c.kx2, c.kx2_h.data(), sizeof(double) * (d.NX2P + 1), cudaMemcpyHostToDevice));
    // twiddles
    const int M = d.NX / 2;
    std::vector<double2> twm(M / 2 > 0 ? M / 2 : 1), twn(M + 1);
    for (int t = 0; t < M / 2; ++t) twm[t] = make_double2(cos(-2.0 * M_PI * t / M), sin(-2.0 * M_PI * t / M));
    for (int k = 0; k <= M; ++k) twn[k] = make_double2(cos(-2.0 * M_PI * k / d.NX), sin(-2.0 * M_PI * k / d.NX));
    c.tw_m = dalloc<double2>(c, twm.size());
    c.tw_n = dalloc<double2>(c, twn.size());
    EK_CUDA(cudaMemcpy(c.tw_m, twm.data(), sizeof(double2) * twm.size(), cudaMemcpyHostToDevice));
    EK_CUDA(cudaMemcpy(c.tw_n, twn.data(), sizeof(double2) * twn.size(), cudaMemcpyHostToDevice));
    {
      std::vector<float2> fm(twm.size()), fn(twn.size());
      for (size_t t = 0; t < twm.size(); ++t) fm[t] = make_float2((float)twm[t].x, (float)twm[t].y);
      for (size_t t = 0; t < twn.size(); ++t) fn[t] = make_float2((float)twn[t].x, (float)twn[t].y);
      c.tw_mf = dalloc<float2>(c, fm.size());
      c.tw_nf = dalloc<float2>(c, fn.size());
      EK_CUDA(cudaMemcpy(c.tw_mf, fm.data(), sizeof(float2) * fm.size(), cudaMemcpyHostToDevice));
      EK_CUDA(cudaMemcpy(c.tw_nf, fn.data(), sizeof(float2) * fn.size(), cudaMemcpyHostToDevice));
      auto split = [](double x) {
        const float h = (float)x;
        return std::make_pair(h, (float)(x - (double)h));
      };
      std::vector<float4> gm(twm.size()), gn(twn.size());
      for (size_t t = 0; t < twm.size(); ++t) {
        const auto a = split(twm[t].x), b = split(twm[t].y);
        gm[t] = make_float4(a.first, a.second, b.first, b.second);
      }
      for (size_t t = 0; t < twn.size(); ++t) {
        const auto a = split(twn[t].x), b = split(twn[t].y);
        gn[t] = make_float4(a.first, a.second, b.first, b.second);
      }
      c.tw_mff = dalloc<float4>(c, gm.size());
      c.tw_nff = dalloc<float4>(c, gn.size());
      EK_CUDA(cudaMemcpy(c.tw_mff, gm.data(), sizeof(float4) * gm.size(), cudaMemcpyHostToDevice));
      EK_CUDA(cudaMemcpy(c.tw_nff, gn.data(), sizeof(float4) * gn.size(), cudaMemcpyHostToDevice));
    }
    // fields
    const size_t nc = d.nspec(), np = d.nphys();
    for (cplx_t **f : {&c.CU1, &c.CU2, &c.CU3, &c.CP, &c.CTH, &c.CF1, &c.CF2, &c.CF3, &c.CFTH, &c.CR1, &c.CR2, &c.CR3,
                       &c.CRTH, &c.CS})
      *f = dalloc<cplx_t>(c, nc);
    c.CU2b = dalloc<cplx_t>(c, 2 * nc);
    c.CU3b = c.CU2b + nc;
    for (double **f : {&c.U1, &c.U2, &c.U3, &c.TH, &c.R1, &c.R2, &c.R3, &c.RTH, &c.PHS, &c.SPH}) *f = dalloc<double>(c, np);
    c.U2b = dalloc<double>(c, 2 * np);
    c.U3b = c.U2b + np;
    if (p.les) les_alloc(c);
    if (p.fft_fp32) {
      for (float **f : {&c.U1f, &c.U2f, &c.U3f, &c.THf}) *f = dalloc<float>(c, np);
      c.U2bf = dalloc<float>(c, 2 * np);
      c.U3bf = c.U2bf + np;
    }
    c.div_part = dalloc<double>(c, d.NY2);
    c.step_stats_dev = dalloc<StepStats>(c, 3);
    c.cfl_dt = dalloc<double>(c, 1);
    c.sponge_sig = dalloc<double>(c, d.NY2 + d.NZ2 + 4);
    c.sponge_sig_out = c.sponge_sig + d.NY2;
    c.sponge_red = c.sponge_sig_out + d.NZ2;
    EK_CUDA(cudaMemsetAsync(c.sponge_sig, 0, sizeof(double) * (d.NY2 + d.NZ2 + 4), c.stream));
    EK_CUDA(cudaStreamSynchronize(c.stream));
  } catch (const CudaError &e) {
    c.err = e.msg;
    *out = h.release();
    return EK_ERR_CUDA;
  }
  *out = h.release();
  return EK_OK;
}

void ekgpu_destroy(ek_ctx *h) {
  if (!h) return;
  Ctx &c = h->c;
  if (c.stream) cudaStreamSynchronize(c.stream);
  for (void *p : c.allocs) cudaFree(p);
  if (c.mg_cof_pool) cudaFree(c.mg_cof_pool);
  mg_work_free(c.mgw);
  guess_free(c);
  if (c.mgf_pool) cudaFree(c.mgf_pool);
  if (c.mgf_cf4_pool) cudaFree(c.mgf_cf4_pool);
  if (c.mg_null_part) cudaFree(c.mg_null_part);
  if (c.mg.ops_dev) cudaFree(c.mg.ops_dev);
  c.poll.destroy();
  step_graphs_clear(c);
  if (c.cap_stream) cudaStreamDestroy(c.cap_stream);
  if (c.cap_stream2) cudaStreamDestroy(c.cap_stream2);
  for (int f = 0; f < 4; ++f)
    if (c.field_stream[f]) cudaStreamDestroy(c.field_stream[f]);
  for (int f = 0; f < 5; ++f)
    if (c.field_ev[f]) cudaEventDestroy(c.field_ev[f]);
  if (c.div_stream) cudaStreamDestroy(c.div_stream);
  for (int f = 0; f < 2; ++f)
    if (c.div_ev[f]) cudaEventDestroy(c.div_ev[f]);
  if (c.step_stats_host) cudaFreeHost(c.step_stats_host);
  for (auto &r : c.trec) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (auto e : c.evpool) cudaEventDestroy(e);
  if (c.own_stream) cudaStreamDestroy(c.own_stream);
  delete h;
}

const char *ekgpu_last_error(const ek_ctx *h) { return h ? h->c.err.c_str() : ek::last_global_error(); }

int ekgpu_set_stream(ek_ctx *h, void *stream) {
  return guarded(h, [&](Ctx &c) {
    EK_CUDA(cudaStreamSynchronize(c.stream));
    c.stream = stream ? static_cast<cudaStream_t>(stream) : c.own_stream;
    return (int)EK_OK;
  });
}

int ekgpu_sponge_profiles(const ek_params *p, const double *xpoint, const double *ypoint, double *sponge_sigma,
                          double *sponge_sigma_out) {
  if (!p || !xpoint || !ypoint || !sponge_sigma || !sponge_sigma_out) return EK_ERR_ARG;
  return sponge_profiles_host(p, xpoint, ypoint, sponge_sigma, sponge_sigma_out);
}

int ekgpu_set_sponge(ek_ctx *h, const double *sponge_sigma, const double *sponge_sigma_out) {
  return guarded(h, [&](Ctx &c) {
    if (!sponge_sigma || !sponge_sigma_out) return fail(c, EK_ERR_ARG, "sponge profile is NULL");
    EK_CUDA(cudaMemcpyAsync(c.sponge_sig, sponge_sigma, sizeof(double) * c.d.NY2, cudaMemcpyHostToDevice, c.stream));
    EK_CUDA(cudaMemcpyAsync(c.sponge_sig_out, sponge_sigma_out, sizeof(double) * c.d.NZ2, cudaMemcpyHostToDevice,
                            c.stream));
    EK_CUDA(cudaStreamSynchronize(c.stream));
    return (int)EK_OK;
  });
}

int ekgpu_set_time(ek_ctx *h, double time, int time_step) {
  return guarded(h, [&](Ctx &c) {
    c.p.time = time;
    c.p.time_step = time_step;
    return (int)EK_OK;
  });
}

int ekgpu_get_time(ek_ctx *h, double *time, int *time_step, double *delta_t) {
  return guarded(h, [&](Ctx &c) {
    if (time) *time = c.p.time;
    if (time_step) *time_step = c.p.time_step;
    if (delta_t) *delta_t = c.p.delta_t;
    return (int)EK_OK;
  });
}

int ekgpu_metrics_from_grid(const ek_params *p, const double *xpoint, const double *ypoint, double *int_jacob,
                            double *gmat_11, double *gmat_12, double *gmat_22, double *cjob_11, double *cjob_12,
                            double *cjob_21, double *cjob_22, double *th_bar) {
  if (!p || !int_jacob || !gmat_11 || !gmat_12 || !gmat_22 || !cjob_11 || !cjob_12 || !cjob_21 || !cjob_22)
    return EK_ERR_ARG;
  return metrics_from_grid_host(p, xpoint, ypoint, int_jacob, gmat_11, gmat_12, gmat_22, cjob_11, cjob_12, cjob_21,
                                cjob_22, th_bar);
}

int ekgpu_les_metrics_from_grid(const ek_params *p, const double *xpoint, const double *ypoint, double *gmat_11_y,
                                double *gmat_12_y, double *gmat_22_y, double *gmat_11_z, double *gmat_12_z,
                                double *gmat_22_z) {
  if (!p) return EK_ERR_ARG;
  return les_metrics_from_grid_host(p, xpoint, ypoint, gmat_11_y, gmat_12_y, gmat_22_y, gmat_11_z, gmat_12_z, gmat_22_z);
}

int ekgpu_set_les_metrics(ek_ctx *h, const double *gmat_11_y, const double *gmat_12_y, const double *gmat_22_y,
                          const double *gmat_11_z, const double *gmat_12_z, const double *gmat_22_z) {
  return guarded(h, [&](Ctx &c) {
    if (!c.p.les) return fail(c, EK_ERR_STATE, "LES is off (ek_params.les = 0)");
    if (!gmat_11_y || !gmat_12_y || !gmat_22_y || !gmat_11_z || !gmat_12_z || !gmat_22_z)
      return fail(c, EK_ERR_ARG, "LES metric pointer is NULL");
    const size_t n3 = 2 * (size_t)c.d.LDM * (c.d.NY + 3);
    auto up = [&](double *&dst, const double *src) {
      if (!dst) dst = dalloc<double>(c, n3);
      EK_CUDA(cudaMemcpy(dst, src, n3 * sizeof(double), cudaMemcpyHostToDevice));
    };
    up(c.m.g11y, gmat_11_y); up(c.m.g12y, gmat_12_y); up(c.m.g22y, gmat_22_y);
    up(c.m.g11z, gmat_11_z); up(c.m.g12z, gmat_12_z); up(c.m.g22z, gmat_22_z);
    c.les.have_metrics = true;
    c.les.tab_ok = false;
    return (int)EK_OK;
  });
}

int ekgpu_les_set_first_time(ek_ctx *h, int first_time) {
  return guarded(h, [&](Ctx &c) {
    if (!c.p.les) return fail(c, EK_ERR_STATE, "LES is off (ek_params.les = 0)");
    c.les.first_time = first_time != 0;
    return (int)EK_OK;
  });
}

int ekgpu_les_get(ek_ctx *h, double *nu_t, double *c_dyn) {
  return guarded(h, [&](Ctx &c) {
    if (!c.p.les) return fail(c, EK_ERR_STATE, "LES is off (ek_params.les = 0)");
    EK_CUDA(cudaStreamSynchronize(c.stream));
    if (nu_t) EK_CUDA(cudaMemcpy(nu_t, c.les.nut, sizeof(double) * c.d.nphys(), cudaMemcpyDeviceToHost));
    if (c_dyn)
      EK_CUDA(cudaMemcpy(c_dyn, c.les.cdyn, sizeof(double) * (size_t)c.d.NZ2 * c.d.NY2, cudaMemcpyDeviceToHost));
    return (int)EK_OK;
  });
}

int ekgpu_set_metrics(ek_ctx *h, const ek_metrics *m) {
  return guarded(h, [&](Ctx &c) {
    if (!m || !m->int_jacob || !m->gmat_11 || !m->gmat_12 || !m->gmat_22 || !m->cjob_11 || !m->cjob_12 ||
        !m->cjob_21 || !m->cjob_22)
      return fail(c, EK_ERR_ARG, "metric pointer is NULL");
    if (c.p.n_th > 0 && !c.p.cont_strat && !m->th_bar) return fail(c, EK_ERR_ARG, "th_bar is required");
    const Dims &d = c.d;
    const size_t n2 = (size_t)d.LDM * (d.NY + 3);
    auto up = [&](double *&dst, const double *src, size_t n) {
      if (!dst) dst = dalloc<double>(c, n);
      if (src) EK_CUDA(cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyHostToDevice));
      else EK_CUDA(cudaMemset(dst, 0, n * sizeof(double)));
    };
    up(c.m.jac, m->int_jacob, n2);
    up(c.m.g11, m->gmat_11, 2 * n2); up(c.m.g12, m->gmat_12, 2 * n2); up(c.m.g22, m->gmat_22, 2 * n2);
    up(c.m.c11, m->cjob_11, 2 * n2); up(c.m.c12, m->cjob_12, 2 * n2);
    up(c.m.c21, m->cjob_21, 2 * n2); up(c.m.c22, m->cjob_22, 2 * n2);
    up(c.m.thbar, m->th_bar, n2);
    step_graphs_clear(c);  // the plan they were captured from is rebuilt below
    if (!c.m.pg) c.m.pg = dalloc<double>(c, 13 * n2);
    launch_metric_tables(c);
    c.les.tab_ok = false;
    std::vector<double> jac(m->int_jacob, m->int_jacob + n2), g11(m->gmat_11, m->gmat_11 + 2 * n2),
        g12(m->gmat_12, m->gmat_12 + 2 * n2), g22(m->gmat_22, m->gmat_22 + 2 * n2), c22(m->cjob_22, m->cjob_22 + 2 * n2);
    // boundary rows and Thomas factors of every field, substep and direction
    std::vector<double> w;
    if (build_bc_sets(c, w, jac, c22) != EK_OK) return fail(c, EK_ERR_ARG, "unsupported boundary condition");
    if (!w.empty()) {
      if (c.bc_weights == nullptr) c.bc_weights = dalloc<double>(c, w.size());
      EK_CUDA(cudaMemcpy(c.bc_weights, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice));
    }
    c.h_jac = jac;
    c.h_g11 = g11;
    c.h_g22 = g22;
    build_adi_factors(c);
    // multigrid plan
    MgPlan &P = c.mg;
    mg_build_plan_host(c, jac, g11, g12, g22);
    mg_build_schedule(P, c.p.mg_kcycle, c.p.mg_iprer, c.p.mg_ipost, c.p.mg_maxcy);
    if (c.p.mg_stop == EK_MG_STOP_RESIDUAL) {
      // left null vector of the kx = 0 operator (the well-posed kx = 0 solve)
      std::vector<double> z;
      if (!mg_left_null_host(P, z)) return fail(c, EK_ERR_ARG, "kx = 0 operator: zero pivot while finding its null vector");
      if (!c.mg_z) c.mg_z = dalloc<double>(c, z.size());
      EK_CUDA(cudaMemcpy(c.mg_z, z.data(), sizeof(double) * z.size(), cudaMemcpyHostToDevice));
    }
    const int ncof = P.orth ? 4 : 8;
    P.lc = 1;
    for (int l = 1; l <= P.ngrid; ++l) {
      size_t tot = 0, maxph = 0;
      for (int k = 1; k <= l; ++k) {
        const MgLevel &L = P.lv[k - 1];
        tot += (size_t)(L.nx + 2) * (L.ny + 2) + (size_t)(2 + ncof) * L.nx * L.ny;
        maxph = std::max(maxph, (size_t)(L.nx + 2) * (L.ny + 2));
      }
      if ((tot + maxph) * sizeof(double) <= 96 * 1024) P.lc = l;
    }
    const int pmax = std::max(c.mgw.pmax, d.NX + 2);
    mg_alloc(c, pmax);
    c.have_metrics = true;
    return (int)EK_OK;
  });
}

int ekgpu_upload_state(ek_ctx *h, const double *cu1, const double *cu2, const double *cu3, const double *cp,
                       const double *cth) {
  return guarded(h, [&](Ctx &c) {
    if (!cu1 || !cu2 || !cu3 || !cp || (c.p.n_th > 0 && !cth)) return fail(c, EK_ERR_ARG, "state pointer is NULL");
    const size_t bytes = c.d.nspec() * sizeof(cplx_t);
    EK_CUDA(cudaMemcpyAsync(c.CU1, cu1, bytes, cudaMemcpyHostToDevice, c.stream));
    EK_CUDA(cudaMemcpyAsync(c.CU2, cu2, bytes, cudaMemcpyHostToDevice, c.stream));
    EK_CUDA(cudaMemcpyAsync(c.CU3, cu3, bytes, cudaMemcpyHostToDevice, c.stream));
    EK_CUDA(cudaMemcpyAsync(c.CP, cp, bytes, cudaMemcpyHostToDevice, c.stream));
    if (cth) EK_CUDA(cudaMemcpyAsync(c.CTH, cth, bytes, cudaMemcpyHostToDevice, c.stream));
    for (cplx_t *f : {c.CF1, c.CF2, c.CF3, c.CFTH}) EK_CUDA(cudaMemsetAsync(f, 0, bytes, c.stream));
    EK_CUDA(cudaStreamSynchronize(c.stream));
    return (int)EK_OK;
  });
}

int ekgpu_download_state(ek_ctx *h, double *cu1, double *cu2, double *cu3, double *cp, double *cth) {
  return guarded(h, [&](Ctx &c) {
    const size_t bytes = c.d.nspec() * sizeof(cplx_t);
    if (cu1) EK_CUDA(cudaMemcpyAsync(cu1, c.CU1, bytes, cudaMemcpyDeviceToHost, c.stream));
    if (cu2) EK_CUDA(cudaMemcpyAsync(cu2, c.CU2, bytes, cudaMemcpyDeviceToHost, c.stream));
    if (cu3) EK_CUDA(cudaMemcpyAsync(cu3, c.CU3, bytes, cudaMemcpyDeviceToHost, c.stream));
    if (cp) EK_CUDA(cudaMemcpyAsync(cp, c.CP, bytes, cudaMemcpyDeviceToHost, c.stream));
    if (cth) EK_CUDA(cudaMemcpyAsync(cth, c.CTH, bytes, cudaMemcpyDeviceToHost, c.stream));
    EK_CUDA(cudaStreamSynchronize(c.stream));
    return (int)EK_OK;
  });
}

int ekgpu_save_flow(ek_ctx *h, const char *flow_path, const char *th_path) {
  return guarded(h, [&](Ctx &c) {
    if (!flow_path) return fail(c, EK_ERR_ARG, "flow_path is NULL");
    if (th_path && c.p.n_th < 1) return fail(c, EK_ERR_ARG, "th_path given but n_th == 0");
    return save_flow(c, flow_path, th_path);
  });
}

int ekgpu_read_flow(ek_ctx *h, const char *flow_path, const char *th_path) {
  return guarded(h, [&](Ctx &c) {
    if (!flow_path) return fail(c, EK_ERR_ARG, "flow_path is NULL");
    if (th_path && c.p.n_th < 1) return fail(c, EK_ERR_ARG, "th_path given but n_th == 0");
    return read_flow(c, flow_path, th_path);
  });
}

int ekgpu_save_stats(ek_ctx *h, ek_stats *st) {
  return guarded(h, [&](Ctx &c) {
    if (!st) return fail(c, EK_ERR_ARG, "stats is NULL");
    if (!c.have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
    return save_stats(c, st);
  });
}

static cplx_t *field_of(Ctx &c, int f) {
  switch (f) {
    case EK_F_CU1: return c.CU1; case EK_F_CU2: return c.CU2; case EK_F_CU3: return c.CU3;
    case EK_F_CP: return c.CP; case EK_F_CTH: return c.CTH; case EK_F_CF1: return c.CF1;
    case EK_F_CF2: return c.CF2; case EK_F_CF3: return c.CF3; case EK_F_CFTH: return c.CFTH;
    case EK_F_CR1: return c.CR1;
    default: return nullptr;
  }
}

int ekgpu_get_field(ek_ctx *h, int f, double *out) {
  return guarded(h, [&](Ctx &c) {
    cplx_t *src = field_of(c, f);
    if (!src || !out) return fail(c, EK_ERR_ARG, "bad field");
    EK_CUDA(cudaMemcpyAsync(out, src, c.d.nspec() * sizeof(cplx_t), cudaMemcpyDeviceToHost, c.stream));
    EK_CUDA(cudaStreamSynchronize(c.stream));
    return (int)EK_OK;
  });
}

int ekgpu_put_field(ek_ctx *h, int f, const double *in) {
  return guarded(h, [&](Ctx &c) {
    cplx_t *dst = field_of(c, f);
    if (!dst || !in) return fail(c, EK_ERR_ARG, "bad field");
    EK_CUDA(cudaMemcpyAsync(dst, in, c.d.nspec() * sizeof(cplx_t), cudaMemcpyHostToDevice, c.stream));
    EK_CUDA(cudaStreamSynchronize(c.stream));
    return (int)EK_OK;
  });
}

int ekgpu_rk_substep(ek_ctx *h, int rk) {
  return guarded(h, [&](Ctx &c) {
    if (!c.have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
    if (rk < 1 || rk > 3) return fail(c, EK_ERR_ARG, "rk_step must be 1, 2 or 3");
    const int st = substep(c, rk);
    if (st == EK_ERR_NAN) return fail(c, EK_ERR_NAN, "DIV is a NaN");
    if (st == EK_ERR_DT) return fail(c, EK_ERR_DT, "DELTA_T is zero");
    if (st == EK_ERR_NOT_CONVERGED) return fail(c, st, "a Poisson problem reached mg_maxcy above the tolerance");
    return st;
  });
}

int ekgpu_step(ek_ctx *h, int nsteps) {
  return guarded(h, [&](Ctx &c) {
    if (!c.have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
    if (nsteps < 0) return fail(c, EK_ERR_ARG, "nsteps must be >= 0");
    // a solve that misses its tolerance does not stop the run (the state
    // stays valid); the call reports it once all steps are done
    int late = EK_OK;
    for (int n = 0; n < nsteps; ++n) {
      c.p.time_step += 1;
      const bool graph = step_graph_eligible(c) && c.eager_since_plan;
      if (graph) {
        const unsigned long long key = step_graph_key(c);
        const StepGraph *sg = nullptr;
        for (const StepGraph &g : c.graphs)
          if (g.key == key) sg = &g;
        if (!sg) sg = &step_graph_capture(c, key);
        const int st = step_graph_run(c, *sg, late);
        if (st == EK_ERR_NAN) return fail(c, EK_ERR_NAN, "DIV is a NaN");
        if (st != EK_OK) return st;
      } else {
        for (int rk = 1; rk <= 3; ++rk) {
          const int st = substep(c, rk);
          if (st == EK_ERR_NAN) return fail(c, EK_ERR_NAN, "DIV is a NaN");
          if (st == EK_ERR_DT) return fail(c, EK_ERR_DT, "DELTA_T is zero");
          if (st == EK_ERR_NOT_CONVERGED) late = st;
          else if (st != EK_OK) return st;
        }
        // lazily allocated buffers exist now, outside any capture
        c.eager_since_plan = true;
      }
      c.p.time += c.p.delta_t;
      c.les.first_time = false;  // FIRST_TIME = .FALSE. after the first step (diablo.F90:157)
    }
    if (late != EK_OK) return fail(c, late, "a Poisson problem reached mg_maxcy above the tolerance");
    return (int)EK_OK;
  });
}

int ekgpu_ensemble_step(ek_ctx *const *members, int n, int nsteps, int *status) {
  if (!members || n < 1 || nsteps < 0) return EK_ERR_ARG;
  std::vector<ek_ctx *> m(members, members + n);
  for (int i = 0; i < n; ++i)
    if (!m[i]) return EK_ERR_ARG;
  std::vector<ek_ctx *> sorted(m);
  std::sort(sorted.begin(), sorted.end());
  if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) return EK_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return EK_ERR_CUDA;
  std::vector<int> st(n, EK_OK);
  // every member on the graph path: one graph launch per ensemble step
  bool graph = n >= 2;
  for (ek_ctx *h : m) graph = graph && step_graph_eligible(h->c) && h->c.have_metrics && h->c.eager_since_plan;
  int done = 0;
  if (graph) {
    std::vector<int> late(n, EK_OK);
    try {
      for (; done < nsteps; ++done) {
        ensemble_graph_step(m, st, late);
        if (std::any_of(st.begin(), st.end(), [](int v) { return v != EK_OK; })) {
          ++done;
          break;
        }
      }
    } catch (const CudaError &e) {
      m[0]->c.err = e.msg;  // capture failed: the remaining steps run as below
    }
    for (int i = 0; i < n; ++i)
      if (st[i] == EK_OK && late[i] != EK_OK) st[i] = fail(m[i]->c, late[i], "a Poisson problem reached mg_maxcy above the tolerance");
    if (done == nsteps) {
      int r = EK_OK;
      for (int i = 0; i < n; ++i) {
        if (status) status[i] = st[i];
        if (r == EK_OK && st[i] != EK_OK) r = st[i];
      }
      return r;
    }
  }
  // the remaining steps (all of them off the graph path) member by member;
  // a member that failed above does not step again
  std::vector<int> prior(st);
  const int rest = nsteps - done;
  // member 0 on the calling thread, the others on their own threads (every
  // context owns its stream, buffers and pinned stop flags, so the members
  // share nothing but the device)
  std::vector<std::thread> th;
  th.reserve(n - 1);
  for (int i = 1; i < n; ++i) {
    try {
      th.emplace_back([&, i] {
        if (cudaSetDevice(dev) != cudaSuccess) {
          st[i] = fail(m[i]->c, EK_ERR_CUDA, "ensemble: cudaSetDevice failed");
          return;
        }
        if (prior[i] == EK_OK || prior[i] == EK_ERR_NOT_CONVERGED) st[i] = ekgpu_step(m[i], rest);
      });
    } catch (const std::system_error &) {
      // no thread to spare: step it here
      if (prior[i] == EK_OK || prior[i] == EK_ERR_NOT_CONVERGED) st[i] = ekgpu_step(m[i], rest);
    }
  }
  if (prior[0] == EK_OK || prior[0] == EK_ERR_NOT_CONVERGED) st[0] = ekgpu_step(m[0], rest);
  for (auto &t : th) t.join();
  for (int i = 0; i < n; ++i)
    if (prior[i] != EK_OK && st[i] == EK_OK) st[i] = prior[i];
  int r = EK_OK;
  for (int i = 0; i < n; ++i) {
    if (status) status[i] = st[i];
    if (r == EK_OK && st[i] != EK_OK) r = st[i];
  }
  return r;
}

int ekgpu_rem_div(ek_ctx *h) {
  return guarded(h, [&](Ctx &c) {
    if (!c.have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
    int mg = EK_OK;
    run_rem_div(c, 1.0, false, &mg);
    const int st = finish_divergence(c, nullptr);
    if (st == EK_ERR_NAN) return fail(c, EK_ERR_NAN, "DIV is a NaN");
    if (st != EK_OK) return st;
    const int ps = projection_status(c, mg);
    if (ps == EK_ERR_DT) return fail(c, ps, "DELTA_T is zero");
    if (ps == EK_ERR_NOT_CONVERGED) return fail(c, ps, "a Poisson problem reached mg_maxcy above the tolerance");
    return ps;
  });
}

int ekgpu_poisson_batch(ek_ctx *h, const double *rhs, double *phi, const double *kx2, int nprob, ek_mg_stats *stats) {
  return guarded(h, [&](Ctx &c) {
    if (!rhs || !phi || !kx2 || nprob <= 0) return fail(c, EK_ERR_ARG, "bad poisson arguments");
    const size_t n = (size_t)c.mg.nfx * c.mg.nfy * nprob;
    double *buf = nullptr;
    EK_CUDA(cudaMalloc(&buf, sizeof(double) * (2 * n + nprob)));
    int r = EK_OK;
    try {
      EK_CUDA(cudaMemcpyAsync(buf, rhs, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
      EK_CUDA(cudaMemcpyAsync(buf + 2 * n, kx2, sizeof(double) * nprob, cudaMemcpyHostToDevice, c.stream));
      r = poisson_dev(c, buf, buf + n, buf + 2 * n, kx2, nprob, stats);
      EK_CUDA(cudaMemcpyAsync(phi, buf + n, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
      EK_CUDA(cudaStreamSynchronize(c.stream));
    } catch (...) {
      cudaFree(buf);
      throw;
    }
    cudaFree(buf);
    return r;
  });
}

int ekgpu_poisson_batch_device(ek_ctx *h, const double *rhs_dev, double *phi_dev, const double *kx2_dev, int nprob,
                               ek_mg_stats *stats) {
  return guarded(h, [&](Ctx &c) {
    if (!rhs_dev || !phi_dev || !kx2_dev || nprob <= 0) return fail(c, EK_ERR_ARG, "bad poisson arguments");
    return poisson_dev(c, rhs_dev, phi_dev, kx2_dev, nullptr, nprob, stats);
  });
}

int ekgpu_last_divergence(ek_ctx *h, double *div) {
  return guarded(h, [&](Ctx &c) {
    if (!div) return fail(c, EK_ERR_ARG, "div is NULL");
    *div = c.last_div;
    return (int)EK_OK;
  });
}

int ekgpu_set_step_graph(ek_ctx *h, int on) {
  return guarded(h, [&](Ctx &c) {
    c.step_graphs = on != 0;
    return (int)EK_OK;
  });
}

int ekgpu_mg_counters(ek_ctx *h, long long *solved, long long *not_converged) {
  return guarded(h, [&](Ctx &c) {
    if (solved) *solved = c.mg_solved_total;
    if (not_converged) *not_converged = c.mg_nc_total;
    return (int)EK_OK;
  });
}

int ekgpu_last_mg_stats(ek_ctx *h, ek_mg_stats *s) {
  return guarded(h, [&](Ctx &c) {
    if (!s) return fail(c, EK_ERR_ARG, "stats is NULL");
    *s = c.last_stats;
    return (int)EK_OK;
  });
}

long long ekgpu_launch_count(const ek_ctx *h) { return h ? h->c.launches : -1; }

static const char *kKClassNames[KC_N] = {"spectral_rhs", "fft_c2r", "fft_r2c", "face_velocity", "adi_y", "adi_z",
                                         "mg_relax", "mg_coarse", "mg_transfer", "mg_check", "mg_setup",
                                         "projection", "divergence", "guess", "les"};

const char *ekgpu_timing_class_name(int k) { return (k >= 0 && k < KC_N) ? kKClassNames[k] : ""; }

int ekgpu_set_timing(ek_ctx *h, int on) {
  return guarded(h, [&](Ctx &c) {
    timing_resolve(c);
    for (int k = 0; k < KC_N; ++k) { c.kms[k] = 0.0; c.kcnt[k] = 0; c.kbytes[k] = 0.0; }
    c.timing = on != 0;
    return (int)EK_OK;
  });
}

int ekgpu_get_timing(ek_ctx *h, double *ms, long long *count, double *bytes, int n) {
  return guarded(h, [&](Ctx &c) {
    timing_resolve(c);
    for (int k = 0; k < n && k < KC_N; ++k) {
      if (ms) ms[k] = c.kms[k];
      if (count) count[k] = c.kcnt[k];
      if (bytes) bytes[k] = c.kbytes[k];
    }
    return (int)KC_N;
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Learned Poisson initial guess: the network object and its use in the solves.
namespace {
template <typename F>
int unet_guarded(ek_unet *u, F &&f) {
  if (!u || !u->net) return EK_ERR_ARG;
  try {
    return f(*u->net);
  } catch (const CudaError &e) {
    u->err = e.msg;
    return EK_ERR_CUDA;
  } catch (const std::bad_alloc &) {
    u->err = "host allocation failed";
    return EK_ERR_CUDA;
  }
}
}  // namespace

int ekgpu_unet_create(int cin, int channels, int max_batch, int h, int w, ek_unet **out) {
  if (!out) return EK_ERR_ARG;
  *out = nullptr;
  if (cin < 1 || channels < 1 || channels > 64 || max_batch < 1 || h < 8 || w < 8 || h % 8 || w % 8)
    return EK_ERR_ARG;
  ek_unet *u = new (std::nothrow) ek_unet;
  if (!u) return EK_ERR_CUDA;
  try {
    u->net.reset(new ek::UNet(cin, channels, max_batch, h, w));
  } catch (const CudaError &) {
    delete u;
    return EK_ERR_CUDA;
  }
  *out = u;
  return EK_OK;
}

void ekgpu_unet_destroy(ek_unet *u) { delete u; }

const char *ekgpu_unet_last_error(const ek_unet *u) { return u ? u->err.c_str() : "null network"; }

long ekgpu_unet_num_params(const ek_unet *u) { return (u && u->net) ? u->net->nparams() : -1; }

int ekgpu_unet_set_params(ek_unet *u, const float *params) {
  return unet_guarded(u, [&](ek::UNet &n) {
    if (!params) return (int)EK_ERR_ARG;
    n.set_params(params);
    return (int)EK_OK;
  });
}

int ekgpu_unet_get_params(ek_unet *u, float *params) {
  return unet_guarded(u, [&](ek::UNet &n) {
    if (!params) return (int)EK_ERR_ARG;
    n.get_params(params);
    return (int)EK_OK;
  });
}

int ekgpu_unet_forward(ek_unet *u, const float *x_dev, int n, float *y_dev, void *stream) {
  return unet_guarded(u, [&](ek::UNet &net) {
    if (!x_dev || !y_dev || n < 1 || n > net.max_n) return (int)EK_ERR_ARG;
    net.forward(x_dev, n, y_dev, (cudaStream_t)stream);
    EK_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    if (net.tcgen05() && net.tc_error((cudaStream_t)stream)) return (int)EK_ERR_TIMEOUT;
    return (int)EK_OK;
  });
}

int ekgpu_unet_set_tcgen05(ek_unet *u, int on) {
  return unet_guarded(u, [&](ek::UNet &net) {
    net.set_tcgen05(on != 0);
    return (int)EK_OK;
  });
}

int ekgpu_unet_train_step(ek_unet *u, const float *x_dev, const float *t_dev, int n, int hv, int wv, double lr,
                          double *loss, void *stream) {
  return unet_guarded(u, [&](ek::UNet &net) {
    if (!x_dev || !t_dev || n < 1 || n > net.max_n || hv < 1 || hv > net.h || wv < 1 || wv > net.w)
      return (int)EK_ERR_ARG;
    const double l = net.train_step(x_dev, t_dev, n, hv, wv, lr, (cudaStream_t)stream);
    if (loss) *loss = l;
    return (int)EK_OK;
  });
}

int ekgpu_unet_gradient(ek_unet *u, const float *x_dev, const float *t_dev, int n, int hv, int wv, double *loss,
                        float *y_dev, float *grad_host, void *stream) {
  return unet_guarded(u, [&](ek::UNet &net) {
    if (!x_dev || !t_dev || n < 1 || n > net.max_n || hv < 1 || hv > net.h || wv < 1 || wv > net.w)
      return (int)EK_ERR_ARG;
    const double l = net.forward_backward(x_dev, t_dev, n, hv, wv, y_dev, (cudaStream_t)stream);
    if (loss) *loss = l;
    if (grad_host)
      EK_CUDA(cudaMemcpy(grad_host, net.grads(), sizeof(float) * net.nparams(), cudaMemcpyDeviceToHost));
    return (int)EK_OK;
  });
}

int ekgpu_guess_geometry(ek_ctx *h, int factor, int *hh, int *ww, int *hv, int *wv) {
  return guarded(h, [&](Ctx &c) {
    if (factor < 1 || !hh || !ww || !hv || !wv) return fail(c, EK_ERR_ARG, "bad guess geometry arguments");
    guess_geometry(c, factor, *hh, *ww, *hv, *wv);
    return (int)EK_OK;
  });
}

static int set_guess_factor(Ctx &c, int factor) {
  GuessState &G = c.guess;
  if (G.factor != 0 && G.factor != factor && ((G.sink_x && G.sink_count > 0) || (G.use && G.net)))
    return fail(c, EK_ERR_STATE, "the guess and the pair sink need the same factor");
  int h, w, hv, wv;
  guess_geometry(c, factor, h, w, hv, wv);
  if (G.factor != factor) G.cap = 0;  // buffers are sized per image
  G.factor = factor;
  G.h = h;
  G.w = w;
  G.hv = hv;
  G.wv = wv;
  return EK_OK;
}

int ekgpu_set_poisson_guess(ek_ctx *h, ek_unet *net, int factor) {
  return guarded(h, [&](Ctx &c) {
    GuessState &G = c.guess;
    if (!net) {
      G.use = false;
      G.net = nullptr;
      return (int)EK_OK;
    }
    if (!net->net || factor < 1) return fail(c, EK_ERR_ARG, "bad network or factor");
    if (!c.p.mg_fast) return fail(c, EK_ERR_STATE, "the learned guess needs mg_fast = 1");
    G.use = false;
    G.net = nullptr;
    const int st = set_guess_factor(c, factor);
    if (st != EK_OK) return st;
    if (net->net->h != G.h || net->net->w != G.w || net->net->cin != 2)
      return fail(c, EK_ERR_ARG, "network image size or input channels do not match the guess geometry");
    G.net = net->net.get();
    G.use = true;
    return (int)EK_OK;
  });
}

int ekgpu_set_pair_sink(ek_ctx *h, float *x_dev, float *t_dev, int capacity, int factor) {
  return guarded(h, [&](Ctx &c) {
    GuessState &G = c.guess;
    if (!x_dev || !t_dev || capacity < 1) {
      G.sink_x = G.sink_t = nullptr;
      G.sink_cap = G.sink_count = 0;
      return (int)EK_OK;
    }
    if (factor < 1) return fail(c, EK_ERR_ARG, "factor < 1");
    G.sink_x = nullptr;
    G.sink_count = 0;
    const int st = set_guess_factor(c, factor);
    if (st != EK_OK) return st;
    G.sink_x = x_dev;
    G.sink_t = t_dev;
    G.sink_cap = capacity;
    return (int)EK_OK;
  });
}

int ekgpu_pair_count(ek_ctx *h, int *count) {
  return guarded(h, [&](Ctx &c) {
    if (!count) return fail(c, EK_ERR_ARG, "count is NULL");
    *count = c.guess.sink_count;
    return (int)EK_OK;
  });
}

int ekgpu_last_guess_stats(ek_ctx *h, double *mean_rho, double *mean_cycles) {
  return guarded(h, [&](Ctx &c) {
    if (mean_rho) *mean_rho = c.guess.last_rho;
    if (mean_cycles) *mean_cycles = c.last_mean_cycles;
    return (int)EK_OK;
  });
}

// ---------------------------------------------------------------------------
// Tile-shape autotuner of the mixed solver's line solves.
int ekgpu_mg_autotune(ek_ctx *h, int reps, char *report, int report_len) {
  return guarded(h, [&](Ctx &c) {
    if (!c.p.mg_fast) return fail(c, EK_ERR_STATE, "the autotuner tunes the mixed solver (mg_fast = 1)");
    if (!c.have_metrics) return fail(c, EK_ERR_STATE, "metrics not set");
    std::string rep;
    step_graphs_clear(c);  // captured with the old layouts
    const int st = mgfast_autotune(c, reps < 1 ? 1 : reps, rep);
    if (st != EK_OK) return fail(c, st, "autotune failed");
    if (report && report_len > 0) {
      const size_t n = std::min(rep.size(), (size_t)report_len - 1);
      std::memcpy(report, rep.data(), n);
      report[n] = 0;
    }
    return (int)EK_OK;
  });
}

int ekgpu_mg_set_layout(ek_ctx *h, int level, int dir, int lanes, int seg) {
  return guarded(h, [&](Ctx &c) {
    MgPlan &PL = c.mg;
    if (level < 2 || level > PL.ngrid || dir < 0 || dir > 1 || !(lanes == 0 || lanes == 8 || lanes == 16 || lanes == 32) ||
        !(seg == 0 || seg == 4 || seg == 8))
      return fail(c, EK_ERR_ARG, "level in 2..ngrid, dir 0 (y-lines) or 1 (x-lines), lanes 0/8/16/32, seg 0/4/8");
    std::vector<int> &t = dir ? PL.lanes_x : PL.lanes_y;
    std::vector<int> &u = dir ? PL.seg_x : PL.seg_y;
    if ((int)t.size() < PL.ngrid + 1) t.resize(PL.ngrid + 1, 0);
    if ((int)u.size() < PL.ngrid + 1) u.resize(PL.ngrid + 1, 0);
    t[level] = lanes;
    u[level] = seg;
    step_graphs_clear(c);  // captured with the old layouts
    return (int)EK_OK;
  });
}

int ekgpu_mg_tail_levels(ek_ctx *h, int *ltop) {
  return guarded(h, [&](Ctx &c) {
    if (!ltop) return fail(c, EK_ERR_ARG, "ltop is NULL");
    *ltop = mgfast_tail_levels(c);
    return (int)EK_OK;
  });
}

int ekgpu_mg_levels(ek_ctx *h, int *ngrid, int *nx, int *ny, int cap) {
  return guarded(h, [&](Ctx &c) {
    const MgPlan &PL = c.mg;
    if (ngrid) *ngrid = PL.ngrid;
    for (int l = 0; l < PL.ngrid && l < cap; ++l) {
      if (nx) nx[l] = PL.lv[l].nx;
      if (ny) ny[l] = PL.lv[l].ny;
    }
    return (int)EK_OK;
  });
}
