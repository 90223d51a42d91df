// Batching and serving engine (include/bolt_gb300.h: bolt_engine_*,
// bolt_request_run).
//
// A request is one cosmology with its own k grid, hierarchy and outputs:
// P_lin(k) (Bolt.jl src/spectra.jl:163-198) or C_l (source_grid + cltt /
// clte / clee, spectra.jl:6-160), optionally with the Jacobian with respect
// to theta = (h, omega_b, omega_c, n, A, Sigma m_nu).
//
//   submit ──> host worker threads: Background + RECFAST tables
//              (7 table sets for a gradient: the cosmology and theta_j + d_j)
//          ──> ready FIFO ──> scheduler thread: admits ready requests while
//              the in-flight device footprint fits the budget, forms a batch
//              and enqueues it on an idle lane (stream):
//                upload ─ solver graph (all modes of all requests, one
//                persistent launch) ─ solver graph (replay modes of the
//                gradient sets) ─ line-of-sight kernels per request ─
//                download ─ done event
//          ──> on the done event: outputs, central differences, release.
//
// Lanes overlap on the device: the CTAs of a new batch fill the SMs that the
// tail of the previous batch leaves idle, so requests that arrive while
// others are on the GPU are admitted as memory and lanes free up.
//
// Gradients are forward differences of the discrete pipeline with every
// discretisation choice frozen: the perturbed modes replay the accepted
// steps of the unperturbed mode (MODE_RECORD / MODE_REPLAY), RECFAST replays
// its steps, step sizes, switch redshifts and right-hand-side branches
// (RecfastFreeze), and the k grids and the Bessel grid are those of the
// unperturbed cosmology, as the reference's ForwardDiff gradient holds them
// (spectra.jl:46-66, recfast.jl:451-456).  The pipeline is then a smooth,
// deterministic function of theta, so one-sided differences with the
// relative step 1e-6 carry truncation and round-off errors of ~1e-6
// (relative): 7 parameter sets per gradient request.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bolt_gb300.h"
#include "bolt_dev.cuh"
#include "host_cosmo.hpp"
#include "tuner.hpp"

namespace bolt {
int rodas_grid_warps(int nmodes, int maxN, int maxnq, int maxL, int wpm, int* blocks);
int rodas_grid_warps(int nmodes, int maxN, int maxnq, int maxL, int wpm, int kind, int* blocks);
int rodas_node_params(int wpm, int kind, const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos,
                      const SolverCfg& cfg, int* d_queue, int maxN, int maxnq, int maxL, int blocks, double* d_scratch,
                      RodasNodeArgs* args, cudaKernelNodeParams* p);
size_t rodas_scratch_per_warp(int maxN, int kind);
int rodas_node_params(int wpm, const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const SolverCfg& cfg,
                      int* d_queue, int maxN, int maxnq, int maxL, int blocks, double* d_scratch, RodasNodeArgs* args,
                      cudaKernelNodeParams* p);
size_t rodas_smem_per_mode(int maxN, int maxnq, int maxL, int wpm);
size_t rodas_scratch_per_warp(int maxN);
int launch_jl_raw(int nb, const double* d_dgs, int ncz, int Lmax, const int* d_slot_of_l, int nslots, double* d_raw,
                  double* d_norm, int* d_flags, cudaStream_t st);
int launch_jl_prefilter(int nb, int nslots, int ncz, const double* d_raw, const double* d_norm, const double* d_w,
                        double* d_coef, cudaStream_t st);
int launch_sdense(int nx, int i0, int nrow, int nk, const double* d_kgrid, const double* d_ST, const double* d_SE, int nm,
                  const double* d_kmid, const double* d_dx, double* d_SdT, double* d_SdE, cudaStream_t st);
int launch_los_cl(const LosArgs& a, int ncz, cudaStream_t st);
int launch_sdense_diff(int nx, int i0, int nrow, int nk, const double* d_kgrid, const double* d_Sa, const double* d_Sb,
                       double scale, int nm, const double* d_kmid, const double* d_dx, double* d_out, cudaStream_t st);
int launch_los_tt_grad(const LosGradArgs& a, cudaStream_t st);
int launch_los_adjoint(const LosAdjArgs& a, cudaStream_t st);
void fill_cosmo_dev(const CosmoTables& T, double* d_tab, double* h_tab, CosmoDev& d);
size_t cosmo_table_doubles(const CosmoTables& T);
}  // namespace bolt

using namespace bolt;

namespace {

constexpr int kTheta = 6;
constexpr int kRecCapMax = 65536;   // recorded steps per mode (gradient requests): min(max_steps, this)
constexpr double kRelStep = 1e-6;   // forward-difference step, relative to |theta_j|
constexpr int kNb = 5001;           // Bessel grid points (spectra.jl:52)
constexpr int kNkd = 5000;          // dense LOS k grid (spectra.jl:133)
constexpr double kFillModes = 24.0;  // modes per SM that make a launch worth starting while others run
constexpr int kThetaN = 3, kThetaA = 4;  // n_s and A_s in theta

// n_s and A_s enter only the primordial spectrum A (k/0.05)^(n-1) of the
// C_l sum and of P_lin (spectra.jl:92, 195-196), not the tables or the
// perturbation solve: their parameter sets of a gradient request reuse the
// unperturbed set's solver outputs and launch no modes.
bool solve_free(int j) { return j == kThetaN || j == kThetaA; }
// Parameter set s of request r takes no solver modes.
bool skips_solve(int nsets, int s) { return nsets > 1 && s >= 1 && solve_free(s - 1); }

struct EngErr : std::runtime_error {
  int code;
  EngErr(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw EngErr(-3, std::string(what) + ": " + cudaGetErrorString(e));
}

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

struct GrowDev {  // grow-only device buffer, resized only while its lane is idle
  void* p = nullptr;
  size_t cap = 0;
  void* get(size_t bytes) {
    if (bytes > cap) {
      if (p) cudaFree(p);
      p = nullptr;
      cap = 0;
      size_t want = std::max<size_t>(bytes + bytes / 4, 4096);
      ck(cudaMalloc(&p, want), "cudaMalloc lane scratch");
      cap = want;
    }
    return p;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct GrowHost {  // grow-only pinned host buffer
  void* p = nullptr;
  size_t cap = 0;
  void* get(size_t bytes) {
    if (bytes > cap) {
      if (p) cudaFreeHost(p);
      p = nullptr;
      cap = 0;
      size_t want = std::max<size_t>(bytes + bytes / 4, 4096);
      ck(cudaMallocHost(&p, want), "cudaMallocHost lane staging");
      cap = want;
    }
    return p;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

// theta = (h, omega_b, omega_c, n, A, Sigma m_nu [eV]) <-> CosmoParams.
void theta_of(const CosmoParamsH& p, double* th) {
  const double me = units_mass_eV();
  th[0] = p.h;
  th[1] = p.Omega_b * p.h * p.h;
  th[2] = p.Omega_c * p.h * p.h;
  th[3] = p.n;
  th[4] = p.A;
  th[5] = p.Sigma_m_nu / me;
}
CosmoParamsH params_of(const CosmoParamsH& base, const double* th) {
  const double me = units_mass_eV();
  CosmoParamsH p = base;
  p.h = th[0];
  p.Omega_b = th[1] / (th[0] * th[0]);
  p.Omega_c = th[2] / (th[0] * th[0]);
  p.n = th[3];
  p.A = th[4];
  p.Sigma_m_nu = th[5] * me;
  return p;
}

struct Req {
  int64_t ticket = 0;
  bolt_request r{};
  std::vector<double> k;
  std::vector<int> ells;
  GridSpec grid{};
  int nsets = 1;
  std::vector<CosmoParamsH> pars;  // [nsets]
  double step[kTheta] = {0, 0, 0, 0, 0, 0};
  std::vector<CosmoTables> T;      // [nsets]
  RecfastFreeze fz;
  int tables_left = 0;
  int state = 0;  // 0 building, 1 ready, 2 on the GPU, 3 done
  int rc = 0;
  std::string err;
  double t[4] = {0, 0, 0, 0};
  double steps = 0.0;  // accepted + rejected steps of all its modes (every parameter set)
  size_t bytes = 0;  // device footprint of the request in a batch
  int N = 0;
  // LOS (C_l): sorted unique multipoles
  std::vector<int> uniq;
  // offsets into the batch's device block and the lane's download area
  size_t o_xout = 0, o_src = 0, o_plin = 0, o_stat = 0, o_cnt = 0, o_rec = 0, o_cl = 0, o_los = 0;
  size_t h_stat = 0, h_plin = 0, h_cl = 0, h_cnt = 0;
  int cos0 = 0;  // first CosmoDev index of the request in the batch
  bool wantE = false;
  bool wantP = false;        // P_lin at x = grid end (BOLT_REQ_PLIN, or a C_l request with plin set)
  int rec_cap = 0;           // recorded steps per mode (gradient requests)
  int src_from = 0;          // C_l: first x node with sources, findfirst(x_grid .> -8) (spectra.jl:86)
  bool los_tangent = false;  // C_l^TT gradient from the tangent of the LOS integral
  bool tangent = false;      // gradient from tangent-linear modes (sets 1..6 hold derivatives, not perturbed results)
  // a pullback by the discrete adjoint (bolt_cl_vjp of C_l^TT, bolt_plin_vjp):
  // the cotangent (C_l: per unique multipole; P_lin: per k) and where the
  // parameter cotangent goes
  bool adjoint = false;
  std::vector<double> ybar;
  double* vjp_grad = nullptr;
  size_t o_ckpt = 0, o_sbar = 0, o_tbar = 0, o_ybar = 0, h_tbar = 0;
};

// The four parameters whose derivatives need a solve (theta indices), in the
// order of the tangent directions of a tangent mode.
constexpr int kSolvedTheta[kTD] = {0, 1, 2, 5};
// Whether parameter set s of request r has modes of its own: the perturbed
// sets of n_s and A_s never do, and those of a tangent request are filled by
// the base modes' tangents.
bool set_has_modes(const Req* r, int s) {
  return !skips_solve(r->nsets, s) && !((r->tangent || r->adjoint) && s > 0);
}
// The kind of a gradient request's second solver phase: 0 frozen-step
// replays, 1 tangent-linear modes, 2 adjoint modes (rodas_kernel's KIND).
int grad_kind(const Req* r) { return r->adjoint ? 2 : (r->tangent ? 1 : 0); }

struct Graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t knode = nullptr;
};

struct Lane {
  cudaStream_t st = nullptr;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // start, phase 1, phase 2, LOS, done
  int* d_queue = nullptr;  // [2] work-queue counters of the two solver phases
  Graph graph[5][2];       // [kernel variant: warps per mode 1, 2, 4; tangent; adjoint][phase]
  GrowDev scr, los_raw, los_norm, los_coef, los_SdT, los_SdE, los_dSd, los_cbar, los_ulo;
  GrowHost up, down;
  bool busy = false;
  std::vector<Req*> batch;
  void* d_block = nullptr;
  size_t block_bytes = 0;
  int wpm[2] = {4, 4};
  int kind[2] = {0, 0};  // rodas_kernel KIND of each phase (0 plain, 1 tangent, 2 adjoint)
  int nmodes[2] = {0, 0};
  int waiting = 0;       // modes of the requests still waiting when the batch was taken
  int key[2] = {0, 0};   // tuner key of each phase (own modes, or the whole load when shared)
  bool shared[2] = {false, false};
  int nlaunch = 0;
};

}  // namespace

struct bolt_engine {
  bolt_engine_cfg cfg{};
  int device = 0, nsm = 0;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_sched, cv_done, cv_pool;
  bool stop = false;
  std::string err;
  int64_t next_ticket = 1;
  std::map<int64_t, std::unique_ptr<Req>> reqs;
  std::deque<Req*> ready;
  std::deque<std::function<void()>> tasks;
  std::vector<std::thread> pool;
  std::thread sched;
  std::vector<Lane> lanes;
  size_t inflight_bytes = 0;
  size_t budget = 0;
  Tuner tuner;
  int64_t stats[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  double* d_w = nullptr;  // Bessel prefilter pivots (constant)
  int* d_flags = nullptr;
};

namespace {

// --------------------------------------------------------------- validation
// Whether a hierarchy's chains pack into one warp, as build_pack does for
// 32 threads (at most 24 elements per lane, one lane kept spare): the
// tangent-linear and adjoint kernels run one warp per mode.
bool fits_one_warp(const bolt_hier& h) {
  for (int E = 2; E <= 24; ++E)
    if (2 * ((h.lg + E) / E) + (h.lnu + E) / E + h.nq * ((h.lmnu + E) / E) <= 31) return true;
  return false;
}

// need_jac = false: a pullback, whose Jacobian stays inside the library.
void check_request(const bolt_request* q, bool need_jac = true) {
  if (!q) throw EngErr(-1, "request is null");
  if (q->kind != BOLT_REQ_PLIN && q->kind != BOLT_REQ_CL) throw EngErr(-1, "request kind must be PLIN or CL");
  const bolt_hier& h = q->hier;
  if (h.lg < 3 || h.lnu < 3 || h.lmnu < 3) throw EngErr(-1, "hierarchy truncations must be >= 3");
  if (h.nq < 1 || h.nq > 27) throw EngErr(-1, "nq must be in 1..27");
  if (h.lg > 1000 || h.lnu > 1000 || h.lmnu > 1000) throw EngErr(-1, "hierarchy truncation too large");
  if (q->nq != h.nq) throw EngErr(-1, "hierarchy nq must equal the Background nq");
  if (!(q->reltol > 0) || !(q->abstol > 0)) throw EngErr(-1, "tolerances must be positive");
  if (!q->k || q->nk < 1) throw EngErr(-1, "no wavenumbers");
  if (q->nk > 1000000) throw EngErr(-1, "too many wavenumbers");
  for (int i = 0; i < q->nk; ++i) {
    if (!(q->k[i] > 0) || !std::isfinite(q->k[i])) throw EngErr(-1, "wavenumbers must be positive and finite");
    if (i > 0 && !(q->k[i] > q->k[i - 1])) throw EngErr(-1, "wavenumbers must be strictly ascending");
  }
  const bolt_params& p = q->par;
  if (!(p.h > 0) || !(p.Omega_b > 0) || !(p.Omega_c >= 0) || !(p.Omega_r > 0) || !(p.A > 0) || !(p.N_nu > 0) ||
      !(p.Sigma_m_nu >= 0) || !std::isfinite(p.n))
    throw EngErr(-1, "invalid cosmological parameters");
  if (!(q->grid.step > 0) || !(q->grid.stop > q->grid.start)) throw EngErr(-1, "invalid x grid");
  if (q->kind == BOLT_REQ_PLIN) {
    if (!q->plin) throw EngErr(-1, "plin output is null");
    if (q->grad && need_jac && !q->dplin) throw EngErr(-1, "dplin output is null");
    if (!(q->plin_x > q->grid.start) || !(q->plin_x <= q->grid.stop)) throw EngErr(-1, "plin_x outside the x grid");
  } else {
    if (q->nk < 2) throw EngErr(-1, "C_l needs at least two source-grid wavenumbers");
    if (!q->ells || q->nell < 1) throw EngErr(-1, "no multipoles");
    for (int i = 0; i < q->nell; ++i)
      if (q->ells[i] < 2 || q->ells[i] > 20000) throw EngErr(-1, "multipoles must be in 2..20000");
    const int w = q->cl_want;
    if (w <= 0 || w > 7) throw EngErr(-1, "cl_want must name TT, TE and/or EE");
    if (q->plin && q->grad && need_jac && !q->dplin) throw EngErr(-1, "dplin output is null");
    if (((w & BOLT_CL_TT) && !q->tt) || ((w & BOLT_CL_TE) && !q->te) || ((w & BOLT_CL_EE) && !q->ee))
      throw EngErr(-1, "C_l output is null");
    if (q->grad && need_jac &&
        (((w & BOLT_CL_TT) && !q->dtt) || ((w & BOLT_CL_TE) && !q->dte) || ((w & BOLT_CL_EE) && !q->dee)))
      throw EngErr(-1, "C_l gradient output is null");
  }
}

// ------------------------------------------------------------ host tables
void build_set(Req* r, int s) {
  RecfastOpts ro;
  const CosmoParamsH& p = r->pars[s];
  ro.Yp = p.Y_p;
  ro.OmegaB = p.Omega_b;
  ro.OmegaG = p.Omega_r;
  ro.Tnow = -1.0;
  ro.tol = 1e-8;
  build_cosmo_tables(p, r->grid, r->r.nq, ro, r->T[s], r->nsets > 1 ? &r->fz : nullptr);
}

size_t align_up(size_t v) { return (v + 255) & ~size_t(255); }

// Device footprint of a request inside a batch (its share of the batch block).
void layout_request(Req* r, size_t& off) {
  const int nk = r->r.nk, n = r->grid.n, ns = r->nsets;
  const size_t tabd = cosmo_table_doubles(r->T[0]);
  size_t start = off;
  off = align_up(off + size_t(ns) * tabd * 8);  // tables of every set
  r->o_xout = off;
  off = align_up(off + size_t(r->r.kind == BOLT_REQ_CL ? n - r->src_from : 1) * 8);
  r->o_stat = off;
  off = align_up(off + size_t(ns) * nk * 4);
  r->o_cnt = off;
  off = align_up(off + size_t(ns) * nk * 16);
  r->o_rec = off;
  if (r->nsets > 1 && !r->tangent) off = align_up(off + size_t(nk) * r->rec_cap * 8);
  if (r->adjoint) {  // checkpoints, output cotangents, per-mode parameter cotangents, C_l cotangent
    r->o_ckpt = off;
    off = align_up(off + size_t(nk) * (r->rec_cap / kCkptEvery + 1) * r->N * 8);
    r->o_sbar = off;
    off = align_up(off + size_t(nk) * (r->r.kind == BOLT_REQ_CL ? r->grid.n - r->src_from : 1) * 8);
    r->o_tbar = off;
    off = align_up(off + size_t(nk) * kTD * 8);
    r->o_ybar = off;
    off = align_up(off + std::max<size_t>(r->ybar.size(), 1) * 8);
  }
  if (r->r.kind == BOLT_REQ_CL) {
    r->o_src = off;
    off = align_up(off + size_t(ns) * nk * (n - r->src_from) * 8 * (r->wantE ? 2 : 1));
    r->o_cl = off;
    off = align_up(off + size_t(ns) * 3 * r->uniq.size() * 8);
    r->o_los = off;  // k grid, kmid, dx, slots, ells, inv_dg, per-set wts and y
    const int nm = kNkd - 1;
    off = align_up(off + size_t(nk + nm + n + 8) * 8 + size_t(r->uniq.back() + 1 + r->uniq.size()) * 4 +
                   size_t(ns) * (nm + n) * 8 + 1024);
  }
  if (r->wantP) {
    r->o_plin = off;
    off = align_up(off + size_t(ns) * nk * 8);
  }
  r->bytes = off - start;
}

}  // namespace

// ------------------------------------------------------------------ engine
namespace {

void pool_worker(bolt_engine* E) {
  cudaSetDevice(E->device);
  std::unique_lock<std::mutex> lk(E->mu);
  while (true) {
    E->cv_pool.wait(lk, [&] { return E->stop || !E->tasks.empty(); });
    if (E->tasks.empty()) {
      if (E->stop) return;
      continue;
    }
    auto f = std::move(E->tasks.front());
    E->tasks.pop_front();
    lk.unlock();
    f();
    lk.lock();
  }
}

// Called with the lock held when a table set of r finished (ok or not).
void set_done(bolt_engine* E, Req* r, int s, const std::string& err) {
  if (!err.empty() && r->rc == 0) {
    r->rc = -1;
    r->err = "table construction: " + err;
  }
  if (s == 0 && r->rc == 0 && r->nsets > 1) {
    for (int j = 1; j < r->nsets; ++j)
      E->tasks.push_back([E, r, j] {
        std::string e;
        try { build_set(r, j); } catch (const std::exception& x) { e = x.what(); }
        std::lock_guard<std::mutex> g(E->mu);
        set_done(E, r, j, e);
      });
    E->cv_pool.notify_all();
  }
  if (s == 0 && r->rc != 0) r->tables_left = 1;  // skip the perturbed sets
  if (--r->tables_left == 0) {
    r->t[1] = now_s(E->t0);
    if (r->rc != 0) {
      r->state = 3;
      r->t[3] = r->t[1];
      E->cv_done.notify_all();
    } else {
      r->state = 1;
      E->ready.push_back(r);
      E->cv_sched.notify_all();
    }
  }
}

Graph& lane_graph(Lane& L, int wpm, int kind, int phase, const cudaKernelNodeParams& kp) {
  const int v = kind ? 2 + kind : (wpm == 1 ? 0 : (wpm == 2 ? 1 : 2));
  Graph& G = L.graph[v][phase];
  if (!G.exec) {
    ck(cudaGraphCreate(&G.g, 0), "cudaGraphCreate");
    cudaMemsetParams mp;
    std::memset(&mp, 0, sizeof(mp));
    mp.dst = L.d_queue + phase;
    mp.value = 0;
    mp.elementSize = 4;
    mp.width = 1;
    mp.height = 1;
    mp.pitch = 0;
    cudaGraphNode_t mnode;
    ck(cudaGraphAddMemsetNode(&mnode, G.g, nullptr, 0, &mp), "cudaGraphAddMemsetNode");
    ck(cudaGraphAddKernelNode(&G.knode, G.g, &mnode, 1, &kp), "cudaGraphAddKernelNode");
    ck(cudaGraphInstantiate(&G.exec, G.g, 0), "cudaGraphInstantiate");
  } else {
    ck(cudaGraphExecKernelNodeSetParams(G.exec, G.knode, &kp), "cudaGraphExecKernelNodeSetParams");
  }
  return G;
}

// Enqueues one batch on an idle lane.  Runs without the engine lock.  Every
// lane buffer is sized before the first enqueue (a reallocation later would
// free memory that enqueued work still uses).
void launch_batch(bolt_engine* E, Lane& L, std::vector<Req*>& batch) {
  cudaStream_t st = L.st;
  // ---- device layout of the batch block (inputs and outputs)
  size_t off = 0;
  int ncos = 0, m1 = 0, m2 = 0, mt = 0, ma = 0, maxN = 0, maxnq = 1, maxL = 3;
  size_t max_sd = 0;
  int max_slots = 0;
  bool anyE = false, anyTangent = false;
  for (Req* r : batch) {
    layout_request(r, off);
    anyTangent |= r->los_tangent;
    r->cos0 = ncos;
    ncos += r->nsets;
    if (r->tangent) {
      mt += r->r.nk;
    } else if (r->adjoint) {
      m1 += r->r.nk;
      ma += r->r.nk;
    } else {
      m1 += r->r.nk;
      for (int s = 1; s < r->nsets; ++s) m2 += skips_solve(r->nsets, s) ? 0 : r->r.nk;
    }
    maxN = std::max(maxN, r->N);
    maxnq = std::max(maxnq, r->r.hier.nq);
    maxL = std::max(maxL, std::max(r->r.hier.lg, std::max(r->r.hier.lnu, r->r.hier.lmnu)));
    if (r->r.kind == BOLT_REQ_CL) {
      max_slots = std::max(max_slots, int(r->uniq.size()));
      int n = r->grid.n, i0 = 0;
      while (i0 < n && !(r->grid.at(i0) > -8.0)) ++i0;
      max_sd = std::max(max_sd, size_t(std::max(n - 1 - i0, 1)) * (kNkd - 1));
      anyE |= r->wantE;
    }
  }
  const size_t o_cos = off;
  off = align_up(off + size_t(ncos) * sizeof(CosmoDev));
  const size_t o_modes = off;
  off = align_up(off + size_t(m1 + m2 + mt + ma) * sizeof(ModeDev));
  const size_t total = off;
  // ---- solver configurations of both phases (autotuned) and lane buffers
  // phase 0: plain modes (and recorded, checkpointed ones); phase 1: their
  // frozen-step replays, the tangent modes or the adjoint modes (a batch
  // holds one kind, see scheduler)
  int wpm[2] = {4, 4}, blocks[2] = {0, 0};
  const int kind1 = mt > 0 ? 1 : (ma > 0 ? 2 : 0);
  const int nph = (m2 > 0 || mt > 0 || ma > 0) ? 2 : 1;
  const int nmodes[2] = {m1, mt > 0 ? mt : (ma > 0 ? ma : m2)};
  L.kind[0] = 0;
  L.kind[1] = kind1;
  int other = 0;  // lanes are launched and finished on this (the scheduler) thread
  for (Lane& o : E->lanes)
    if (&o != &L && o.busy) other += o.nmodes[0] + o.nmodes[1];
  for (int ph = 0; ph < nph; ++ph) {
    L.shared[ph] = other > 0 || L.waiting > 0 || E->cfg.objective == 1;
    L.key[ph] = L.shared[ph] ? nmodes[ph] + other + L.waiting : nmodes[ph];
    int w = E->cfg.warps_per_mode;
    if (L.kind[ph]) {
      w = 1;  // the tangent-linear and adjoint kernels run one warp per mode
    } else if (w != 1 && w != 2 && w != 4) {
      std::lock_guard<std::mutex> g(E->mu);
      w = E->tuner.pick(L.shared[ph], L.key[ph], E->nsm);
    }
    if (nmodes[ph] == 0) {  // a batch of tangent requests alone has no plain modes
      blocks[ph] = 0;
      wpm[ph] = w;
      continue;
    }
    int rc = rodas_grid_warps(nmodes[ph], maxN, maxnq, maxL, w, L.kind[ph], &blocks[ph]);
    if (rc != 0) throw EngErr(-3, std::string("solver configuration: ") + cudaGetErrorString(cudaError_t(-rc)));
    wpm[ph] = w;
  }
  double* d_scr = static_cast<double*>(
      L.scr.get(std::max(size_t(blocks[0]) * rodas_scratch_per_warp(maxN, 0),
                         size_t(blocks[1]) * rodas_scratch_per_warp(maxN, kind1))));
  double *raw = nullptr, *norm = nullptr, *coef = nullptr, *SdT = nullptr, *SdE = nullptr;
  if (max_slots > 0) {
    raw = static_cast<double*>(L.los_raw.get(size_t(max_slots) * kNb * 8));
    norm = static_cast<double*>(L.los_norm.get(size_t(kNb) * 8));
    coef = static_cast<double*>(L.los_coef.get(size_t(max_slots) * (kNb + 2) * 8));
    SdT = static_cast<double*>(L.los_SdT.get(max_sd * 8));
    if (anyE) SdE = static_cast<double*>(L.los_SdE.get(max_sd * 8));
  }
  double* dSd = anyTangent ? static_cast<double*>(L.los_dSd.get(size_t(kTheta) * max_sd * 8)) : nullptr;
  // adjoint C_l requests: 2 w Delta per slot and midpoint, the slots' skip
  // bounds, and the resampled sources' cotangent (a batch of them holds no
  // tangent-LOS request, so dSd's buffer serves)
  double *cbar = nullptr, *ulo = nullptr, *Sbd = nullptr;
  if (kind1 == 2 && max_slots > 0) {
    cbar = static_cast<double*>(L.los_cbar.get(size_t(max_slots) * (kNkd - 1) * 8));
    ulo = static_cast<double*>(L.los_ulo.get(size_t(max_slots) * 8));
    Sbd = static_cast<double*>(L.los_dSd.get(max_sd * 8));
  }
  // ---- host staging (pinned, compact): input segments only
  struct Seg {
    size_t dev, host, bytes;
  };
  std::vector<Seg> segs;
  size_t hoff = 0;
  auto seg = [&](size_t dev_off, size_t bytes) {
    segs.push_back({dev_off, hoff, bytes});
    hoff = align_up(hoff + bytes);
    return segs.size() - 1;
  };
  std::vector<size_t> seg_tab(batch.size()), seg_x(batch.size()), seg_los(batch.size()), seg_yb(batch.size());
  size_t req_start = 0;
  std::vector<size_t> starts(batch.size());
  for (size_t b = 0; b < batch.size(); ++b) {
    Req* r = batch[b];
    starts[b] = req_start;
    seg_tab[b] = seg(req_start, size_t(r->nsets) * cosmo_table_doubles(r->T[0]) * 8);
    seg_x[b] = seg(r->o_xout, size_t(r->r.kind == BOLT_REQ_CL ? r->grid.n - r->src_from : 1) * 8);
    if (r->r.kind == BOLT_REQ_CL) {
      const int nm = kNkd - 1, n = r->grid.n, ns = int(r->uniq.size());
      size_t head = align_up(size_t(r->r.nk + nm + n + 8) * 8 + size_t(r->uniq.back() + 1 + ns) * 4);
      seg_los[b] = seg(r->o_los, head + size_t(r->nsets) * (nm + n) * 8);
    }
    if (r->adjoint)  // the cotangent: C_l per slot, or P_lin per k (the reverse modes' seeds)
      seg_yb[b] = r->r.kind == BOLT_REQ_CL ? seg(r->o_ybar, r->ybar.size() * 8) : seg(r->o_sbar, r->ybar.size() * 8);
    req_start += r->bytes;
  }
  const size_t seg_cos = seg(o_cos, size_t(ncos) * sizeof(CosmoDev));
  const size_t seg_modes = seg(o_modes, size_t(m1 + m2 + mt + ma) * sizeof(ModeDev));
  char* up = static_cast<char*>(L.up.get(std::max<size_t>(hoff, 8)));
  // downloads: status + counters + results per request
  size_t doff = 0;
  for (Req* r : batch) {
    const int nk = r->r.nk, ns = r->nsets;
    r->h_stat = doff;
    doff = align_up(doff + size_t(ns) * nk * 4);
    r->h_cnt = doff;
    doff = align_up(doff + size_t(ns) * nk * 16);
    if (r->r.kind == BOLT_REQ_CL) {
      r->h_cl = doff;
      doff = align_up(doff + size_t(ns) * 3 * r->uniq.size() * 8);
    }
    if (r->wantP) {
      r->h_plin = doff;
      doff = align_up(doff + size_t(ns) * nk * 8);
    }
    if (r->adjoint) {
      r->h_tbar = doff;
      doff = align_up(doff + size_t(nk) * kTD * 8);
    }
  }
  char* down = static_cast<char*>(L.down.get(std::max<size_t>(doff, 8)));
  ck(cudaMallocAsync(&L.d_block, total, st), "cudaMallocAsync batch");
  char* dev = static_cast<char*>(L.d_block);
  // ---- host images: tables, x nodes, modes
  std::vector<CosmoDev> cos(ncos);
  std::vector<ModeDev> modes, modes2;
  modes.reserve(m1);
  modes2.reserve(m2 + mt + ma);
  for (size_t b = 0; b < batch.size(); ++b) {
    Req* r = batch[b];
    const int nk = r->r.nk, ns = r->nsets, nsrc = r->grid.n - r->src_from;
    const size_t tabd = cosmo_table_doubles(r->T[0]);
    for (int s = 0; s < ns; ++s) {
      double* h_tab = reinterpret_cast<double*>(up + segs[seg_tab[b]].host + size_t(s) * tabd * 8);
      double* d_tab = reinterpret_cast<double*>(dev + starts[b] + size_t(s) * tabd * 8);
      fill_cosmo_dev(r->T[s], d_tab, h_tab, cos[r->cos0 + s]);
    }
    double* hx = reinterpret_cast<double*>(up + segs[seg_x[b]].host);
    const double* dx = reinterpret_cast<const double*>(dev + r->o_xout);
    int nout;
    if (r->r.kind == BOLT_REQ_CL) {  // the nodes the line of sight reads, x > -8
      for (int j = 0; j < nsrc; ++j) hx[j] = r->grid.at(r->src_from + j);
      nout = nsrc;
    } else {
      hx[0] = r->r.plin_x;
      nout = 1;
    }
    int32_t* dstat = reinterpret_cast<int32_t*>(dev + r->o_stat);
    int64_t* dcnt = reinterpret_cast<int64_t*>(dev + r->o_cnt);
    double* drec = reinterpret_cast<double*>(dev + r->o_rec);
    if (r->adjoint)
      std::memcpy(up + segs[seg_yb[b]].host, r->ybar.data(), r->ybar.size() * 8);
    for (int s = 0; s < ns; ++s)
      for (int i = 0; i < nk && set_has_modes(r, s); ++i) {
        ModeDev m;
        std::memset(&m, 0, sizeof(m));
        m.k = r->k[i];
        m.cosmo = r->cos0 + s;
        m.lg = r->r.hier.lg; m.lnu = r->r.hier.lnu; m.lmnu = r->r.hier.lmnu; m.nq = r->r.hier.nq;
        m.nout = nout;
        m.xout = dx;
        if (r->r.kind == BOLT_REQ_CL) {
          double* src = reinterpret_cast<double*>(dev + r->o_src);
          m.flags = MODE_SOURCES;
          m.src_T = src + (size_t(s) * nk + i) * nsrc;
          m.src_E = r->wantE ? src + size_t(ns) * nk * nsrc + (size_t(s) * nk + i) * nsrc : nullptr;
        }
        if (r->wantP) {  // at the last node: plin_x, or the end of the x grid for a C_l request
          m.flags |= MODE_PLIN;
          m.plin = reinterpret_cast<double*>(dev + r->o_plin) + size_t(s) * nk + i;
        }
        m.status = dstat + size_t(s) * nk + i;
        m.counters = dcnt + 2 * (size_t(s) * nk + i);
        if (r->tangent) {  // derivatives into the slots of the perturbed sets of theta 0, 1, 2, 5
          m.flags |= MODE_TANGENT;
          for (int d = 0; d < kTD; ++d) {
            const int sj = 1 + kSolvedTheta[d];
            m.tcos[d] = r->cos0 + sj;
            m.tinv[d] = 1.0 / r->step[kSolvedTheta[d]];
            if (r->r.kind == BOLT_REQ_CL) {
              double* src = reinterpret_cast<double*>(dev + r->o_src);
              m.tsrc_T[d] = src + (size_t(sj) * nk + i) * nsrc;
              m.tsrc_E[d] = r->wantE ? src + size_t(ns) * nk * nsrc + (size_t(sj) * nk + i) * nsrc : nullptr;
            }
            if (r->wantP) m.tplin[d] = reinterpret_cast<double*>(dev + r->o_plin) + size_t(sj) * nk + i;
          }
          modes2.push_back(m);
          continue;
        }
        if (ns > 1) {
          m.flags |= s == 0 ? MODE_RECORD : MODE_REPLAY;
          m.rec = drec + size_t(i) * r->rec_cap;
          m.rec_cap = r->rec_cap;
        }
        if (r->adjoint) {  // checkpointed forward mode, and its reverse sweep in phase 1
          m.flags |= MODE_CKPT;
          m.ckpt = reinterpret_cast<double*>(dev + r->o_ckpt) + size_t(i) * (r->rec_cap / kCkptEvery + 1) * r->N;
          modes.push_back(m);
          ModeDev a = m;
          a.flags = MODE_ADJOINT | (r->r.kind == BOLT_REQ_CL ? MODE_SOURCES : MODE_PLIN);
          a.src_T = a.src_E = nullptr;
          a.plin = nullptr;
          a.nfwd = dcnt + 2 * size_t(i);
          a.sbar = reinterpret_cast<const double*>(dev + r->o_sbar) + (r->r.kind == BOLT_REQ_CL ? size_t(i) * nsrc : i);
          a.tbar = reinterpret_cast<double*>(dev + r->o_tbar) + size_t(i) * kTD;
          for (int d = 0; d < kTD; ++d) {
            a.tcos[d] = r->cos0 + 1 + kSolvedTheta[d];
            a.tinv[d] = 1.0 / r->step[kSolvedTheta[d]];
          }
          a.status = dstat + size_t(nk) + i;  // the slots of parameter set 1
          a.counters = dcnt + 2 * (size_t(nk) + i);
          modes2.push_back(a);
          continue;
        }
        if (s == 0) modes.push_back(m);
        else modes2.push_back(m);
      }
  }
  // longest modes first: the cost grows with k and with the state length
  auto cost_order = [](std::vector<ModeDev>& v) {
    std::stable_sort(v.begin(), v.end(), [](const ModeDev& a, const ModeDev& b) {
      double ca = a.k * (2 * (a.lg + 1) + (a.lnu + 1) + (a.lmnu + 1) * a.nq);
      double cb = b.k * (2 * (b.lg + 1) + (b.lnu + 1) + (b.lmnu + 1) * b.nq);
      return ca > cb;
    });
  };
  cost_order(modes);
  cost_order(modes2);
  std::memcpy(up + segs[seg_cos].host, cos.data(), cos.size() * sizeof(CosmoDev));
  std::memcpy(up + segs[seg_modes].host, modes.data(), modes.size() * sizeof(ModeDev));
  if (!modes2.empty())
    std::memcpy(up + segs[seg_modes].host + modes.size() * sizeof(ModeDev), modes2.data(),
                modes2.size() * sizeof(ModeDev));
  // ---- LOS inputs per C_l request (grids frozen to the unperturbed set)
  struct LosPlan {
    Req* r;
    int i0, nrow, nm, ns, Lmax;
    size_t head;
  };
  std::vector<LosPlan> plans;
  for (size_t b = 0; b < batch.size(); ++b) {
    Req* r = batch[b];
    if (r->r.kind != BOLT_REQ_CL) continue;
    const CosmoTables& T0 = r->T[0];
    const GridSpec& g = r->grid;
    const int n = g.n, nm = kNkd - 1, ns = int(r->uniq.size());
    int i0 = 0;
    while (i0 < n && !(g.at(i0) > -8.0)) ++i0;
    const int nrow = n - 1 - i0;
    char* lb = up + segs[seg_los[b]].host;
    double* kg = reinterpret_cast<double*>(lb);
    double* kmid = kg + r->r.nk;
    double* dxs = kmid + nm;
    double* misc = dxs + n;  // [0] Bessel grid step, [1] its inverse
    int* slot = reinterpret_cast<int*>(misc + 8);
    int* ells = slot + (r->uniq.back() + 1);
    const size_t head = align_up(size_t(r->r.nk + nm + n + 8) * 8 + size_t(r->uniq.back() + 1 + ns) * 4);
    double* per = reinterpret_cast<double*>(lb + head);
    std::copy(r->k.begin(), r->k.end(), kg);
    std::vector<double> kd(kNkd), dk(nm);
    for (int i = 1; i <= kNkd; ++i) {  // quadratic_k(0.01 H0, 1000 H0, 5000), spectra.jl:60-63,133
      double t = double(i) / double(kNkd);
      kd[i - 1] = 0.01 * T0.H0 + (1000.0 * T0.H0 - 0.01 * T0.H0) * (t * t);
    }
    for (int m = 0; m < nm; ++m) {
      kmid[m] = (kd[m] + kd[m + 1]) / 2.0;
      dk[m] = kd[m + 1] - kd[m];
    }
    for (int i = 0; i < nrow; ++i) dxs[i] = g.at(i0 + i + 1) - g.at(i0 + i);
    misc[0] = kd[kNkd - 1] * T0.eta0 / 5000.0;  // bessel_interpolator grid (spectra.jl:49-58)
    misc[1] = 1.0 / misc[0];
    for (int l = 0; l <= r->uniq.back(); ++l) slot[l] = -1;
    for (int q = 0; q < ns; ++q) {
      slot[r->uniq[q]] = q;
      ells[q] = r->uniq[q];
    }
    for (int s = 0; s < r->nsets; ++s) {
      const CosmoTables& T = r->T[s];
      double* wts = per + size_t(s) * (nm + n);
      double* yv = wts + nm;
      for (int m = 0; m < nm; ++m) wts[m] = T.par.A * std::pow(kmid[m] / 0.05, T.par.n - 1.0) * dk[m] / kmid[m];
      for (int i = 0; i < nrow; ++i) yv[i] = T.eta0 - spline_eval(T.coef[T_ETA].data(), n, g.x0, g.h, g.at(i0 + i));
    }
    if (r->los_tangent || r->adjoint)  // sets 1..6 -> derivatives of the weights and of y along theta_j
      for (int j = 0; j < kTheta; ++j) {
        double* d = per + size_t(1 + j) * (nm + n);
        if (solve_free(j)) {  // exact: dw/dn = w ln(k/0.05), dw/dA = w/A; y does not depend on them
          for (int m = 0; m < nm; ++m)
            d[m] = j == kThetaN ? per[m] * std::log(kmid[m] / 0.05) : per[m] / T0.par.A;
          for (int i = 0; i < nrow; ++i) d[nm + i] = 0.0;
          continue;
        }
        const double inv = 1.0 / r->step[j];
        for (int q = 0; q < nm + nrow; ++q) d[q] = (d[q] - per[q]) * inv;
      }
    plans.push_back({r, i0, nrow, nm, ns, r->uniq.back(), head});
  }
  // ---- enqueue
  int launches = 0;
  ck(cudaEventRecord(L.ev[0], st), "event");
  for (const Seg& sg : segs)
    if (sg.bytes) ck(cudaMemcpyAsync(dev + sg.dev, up + sg.host, sg.bytes, cudaMemcpyHostToDevice, st), "upload");
  const ModeDev* d_modes = reinterpret_cast<const ModeDev*>(dev + o_modes);
  const CosmoDev* d_cos = reinterpret_cast<const CosmoDev*>(dev + o_cos);
  SolverCfg cfg;
  cfg.reltol = batch[0]->r.reltol;  // a batch groups requests of equal tolerances
  cfg.abstol = batch[0]->r.abstol;
  cfg.h0 = 1e-3;
  cfg.x_dense = -8.5;
  cfg.max_steps = E->cfg.max_steps > 0 ? E->cfg.max_steps : 100000;
  cfg.land_stride = E->cfg.land_stride > 1 ? E->cfg.land_stride : 1;
  auto run_phase = [&](int ph) {
    L.wpm[ph] = wpm[ph];
    L.nmodes[ph] = nmodes[ph];
    if (nmodes[ph] > 0) {
      RodasNodeArgs args;
      cudaKernelNodeParams kp;
      rodas_node_params(wpm[ph], L.kind[ph], d_modes + (ph ? m1 : 0), nmodes[ph], d_cos, cfg, L.d_queue + ph, maxN,
                        maxnq, maxL, blocks[ph], d_scr, &args, &kp);
      Graph& G = lane_graph(L, wpm[ph], L.kind[ph], ph, kp);
      ck(cudaGraphLaunch(G.exec, st), "cudaGraphLaunch");
      ++launches;
    }
    ck(cudaEventRecord(L.ev[1 + ph], st), "event");
  };
  run_phase(0);
  // adjoint C_l^TT requests: the projection and its adjoint between the
  // phases -- the reverse modes start from the sources' cotangent
  for (auto& P : plans) {
    Req* r = P.r;
    if (!r->adjoint) continue;
    const int n = r->grid.n, nk = r->r.nk, nsrc = n - r->src_from, i0s = P.i0 - r->src_from;
    char* lb = dev + r->o_los;
    const double* kg = reinterpret_cast<const double*>(lb);
    const double* kmid = kg + nk;
    const double* dxs = kmid + P.nm;
    const double* misc = dxs + n;
    const int* slot = reinterpret_cast<const int*>(misc + 8);
    const int* ells = slot + (P.Lmax + 1);
    const double* per = reinterpret_cast<const double*>(lb + P.head);
    int rc = launch_jl_raw(kNb, misc, 1, P.Lmax, slot, P.ns, raw, norm, E->d_flags, st);
    if (rc == 0) rc = launch_jl_prefilter(kNb, P.ns, 1, raw, norm, E->d_w, coef, st);
    const double* src = reinterpret_cast<const double*>(dev + r->o_src);
    double* cl = reinterpret_cast<double*>(dev + r->o_cl);
    if (rc == 0) rc = launch_sdense(nsrc, i0s, P.nrow, nk, kg, src, nullptr, P.nm, kmid, dxs, SdT, nullptr, st);
    if (rc == 0) {
      LosGradArgs a;
      a.nb = kNb; a.nslots = P.ns; a.nrow = P.nrow; a.nm = P.nm;
      a.ells = ells; a.coef = coef; a.inv_dg = misc + 1;
      a.wts = per; a.yv = per + P.nm; a.dwts = per + (P.nm + n); a.dyv = per + (P.nm + n) + P.nm; a.dstride = P.nm + n;
      a.kmid = kmid; a.Sd = SdT; a.dSd = nullptr; a.tt = cl; a.dtt = cl + P.ns;
      a.terms = nullptr;
      a.cbar = cbar;
      a.ulo = ulo;
      rc = launch_los_tt_grad(a, st);
    }
    if (rc == 0) {
      LosAdjArgs b;
      b.nb = kNb; b.nslots = P.ns; b.nrow = P.nrow; b.nm = P.nm; b.nk = nk; b.nx = nsrc; b.i0 = i0s;
      b.coef = coef; b.inv_dg = misc + 1; b.yv = per + P.nm; b.kmid = kmid; b.kgrid = kg; b.dxs = dxs;
      b.ybar = reinterpret_cast<const double*>(dev + r->o_ybar);
      b.cbar = cbar; b.ulo = ulo; b.Sbd = Sbd;
      b.Sbar = reinterpret_cast<double*>(dev + r->o_sbar);
      rc = launch_los_adjoint(b, st);
    }
    if (rc != 0) throw EngErr(-3, std::string("line of sight (adjoint): ") + cudaGetErrorString(cudaError_t(rc)));
    launches += 6;
  }
  if (nph == 2) {
    run_phase(1);
  } else {
    L.nmodes[1] = 0;
    ck(cudaEventRecord(L.ev[2], st), "event");
  }
  for (auto& P : plans) {
    Req* r = P.r;
    if (r->adjoint) continue;
    const int n = r->grid.n, nk = r->r.nk, nsrc = n - r->src_from, i0s = P.i0 - r->src_from;
    char* lb = dev + r->o_los;
    const double* kg = reinterpret_cast<const double*>(lb);
    const double* kmid = kg + nk;
    const double* dxs = kmid + P.nm;
    const double* misc = dxs + n;
    const int* slot = reinterpret_cast<const int*>(misc + 8);
    const int* ells = slot + (P.Lmax + 1);
    const double* per = reinterpret_cast<const double*>(lb + P.head);
    int rc = launch_jl_raw(kNb, misc, 1, P.Lmax, slot, P.ns, raw, norm, E->d_flags, st);
    if (rc == 0) rc = launch_jl_prefilter(kNb, P.ns, 1, raw, norm, E->d_w, coef, st);
    if (rc != 0) throw EngErr(-3, std::string("Bessel tables: ") + cudaGetErrorString(cudaError_t(rc)));
    launches += 2;
    const double* src = reinterpret_cast<const double*>(dev + r->o_src);
    double* cl = reinterpret_cast<double*>(dev + r->o_cl);
    if (r->los_tangent) {
      rc = launch_sdense(nsrc, i0s, P.nrow, nk, kg, src, nullptr, P.nm, kmid, dxs, SdT, nullptr, st);
      for (int j = 0; j < kTheta && rc == 0; ++j) {
        if (solve_free(j)) {  // the sources do not depend on theta_j
          rc = int(cudaMemsetAsync(dSd + size_t(j) * P.nrow * P.nm, 0, size_t(P.nrow) * P.nm * 8, st));
          continue;
        }
        if (r->tangent)  // the tangent modes stored dS/dtheta_j in set 1 + j
          rc = launch_sdense(nsrc, i0s, P.nrow, nk, kg, src + size_t(1 + j) * nk * nsrc, nullptr, P.nm, kmid, dxs,
                             dSd + size_t(j) * P.nrow * P.nm, nullptr, st);
        else
          rc = launch_sdense_diff(nsrc, i0s, P.nrow, nk, kg, src + size_t(1 + j) * nk * nsrc, src,
                                  1.0 / r->step[j], P.nm, kmid, dxs, dSd + size_t(j) * P.nrow * P.nm, st);
      }
      if (rc != 0) throw EngErr(-3, std::string("source resampling: ") + cudaGetErrorString(cudaError_t(rc)));
      LosGradArgs a;
      a.nb = kNb; a.nslots = P.ns; a.nrow = P.nrow; a.nm = P.nm;
      a.ells = ells; a.coef = coef; a.inv_dg = misc + 1;
      a.wts = per; a.yv = per + P.nm; a.dwts = per + (P.nm + n); a.dyv = per + (P.nm + n) + P.nm; a.dstride = P.nm + n;
      a.kmid = kmid; a.Sd = SdT; a.dSd = dSd; a.tt = cl; a.dtt = cl + P.ns;
      a.terms = nullptr;
      a.cbar = nullptr;
      a.ulo = nullptr;
      rc = launch_los_tt_grad(a, st);
      if (rc != 0) throw EngErr(-3, std::string("line of sight (tangent): ") + cudaGetErrorString(cudaError_t(rc)));
      launches += 2 + kTheta;
      continue;
    }
    for (int s = 0; s < r->nsets; ++s) {
      const int ss = skips_solve(r->nsets, s) ? 0 : s;  // parameter set whose sources hold for set s
      const double* ST = src + size_t(ss) * nk * nsrc;
      const double* SE = r->wantE ? src + size_t(r->nsets) * nk * nsrc + size_t(ss) * nk * nsrc : nullptr;
      rc = launch_sdense(nsrc, i0s, P.nrow, nk, kg, ST, SE, P.nm, kmid, dxs, SdT, SE ? SdE : nullptr, st);
      if (rc != 0) throw EngErr(-3, std::string("source resampling: ") + cudaGetErrorString(cudaError_t(rc)));
      const double* wts = per + size_t(s) * (P.nm + n);
      LosArgs a;
      a.nb = kNb; a.nslots = P.ns; a.nrow = P.nrow; a.nm = P.nm;
      a.ells = ells; a.coef = coef; a.inv_dg = misc + 1; a.yv = wts + P.nm; a.kmid = kmid; a.wts = wts;
      a.SdT = SdT; a.SdE = SE ? SdE : nullptr;
      double* out = cl + size_t(s) * 3 * P.ns;
      a.tt = out; a.te = SE ? out + P.ns : nullptr; a.ee = SE ? out + 2 * P.ns : nullptr;
      a.terms = nullptr;
      rc = launch_los_cl(a, 1, st);
      if (rc != 0) throw EngErr(-3, std::string("line of sight: ") + cudaGetErrorString(cudaError_t(rc)));
      launches += 2;
    }
  }
  ck(cudaEventRecord(L.ev[3], st), "event");
  for (Req* r : batch) {
    const int nk = r->r.nk, ns = r->nsets;
    ck(cudaMemcpyAsync(down + r->h_stat, dev + r->o_stat, size_t(ns) * nk * 4, cudaMemcpyDeviceToHost, st), "status");
    ck(cudaMemcpyAsync(down + r->h_cnt, dev + r->o_cnt, size_t(ns) * nk * 16, cudaMemcpyDeviceToHost, st), "counters");
    if (r->r.kind == BOLT_REQ_CL)
      ck(cudaMemcpyAsync(down + r->h_cl, dev + r->o_cl, size_t(ns) * 3 * r->uniq.size() * 8, cudaMemcpyDeviceToHost,
                         st), "C_l");
    if (r->wantP)
      ck(cudaMemcpyAsync(down + r->h_plin, dev + r->o_plin, size_t(ns) * nk * 8, cudaMemcpyDeviceToHost, st), "P_lin");
    if (r->adjoint)
      ck(cudaMemcpyAsync(down + r->h_tbar, dev + r->o_tbar, size_t(nk) * kTD * 8, cudaMemcpyDeviceToHost, st),
         "parameter cotangents");
  }
  ck(cudaFreeAsync(L.d_block, st), "cudaFreeAsync batch");
  L.d_block = nullptr;
  ck(cudaEventRecord(L.ev[4], st), "event");
  L.nlaunch = launches;
}

// Outputs of one request from the lane's download area (lock held).
void finalize_request(Lane& L, Req* r) {
  const char* down = static_cast<const char*>(L.down.p);
  const int nk = r->r.nk, ns = r->nsets;
  const int32_t* st = reinterpret_cast<const int32_t*>(down + r->h_stat);
  if (r->r.status) std::copy(st, st + nk, r->r.status);
  for (int s = 0; s < ns && r->rc == 0; ++s)
    for (int i = 0; i < nk && set_has_modes(r, s); ++i) {
      int v = st[size_t(s) * nk + i];
      if ((v & 0xFF) != 0 || (s == 0 && ns > 1 && !r->tangent && (v & ST_REC_OVERFLOW))) {
        r->rc = -4;
        char buf[192];
        if ((v & 0xFF) == 0)
          std::snprintf(buf, sizeof(buf), "mode k=%.6g took more than %d accepted steps, the step record of a "
                        "gradient request (raise max_steps)", r->k[i], r->rec_cap);
        else
          std::snprintf(buf, sizeof(buf), "mode k=%.6g (parameter set %d) ended with status %d", r->k[i], s, v);
        r->err = buf;
        break;
      }
    }
  if (r->adjoint) {
    for (int i = 0; i < nk && r->rc == 0; ++i) {  // the reverse sweeps
      int v = st[size_t(nk) + i];
      if ((v & 0xFF) != 0) {
        r->rc = -4;
        char buf[160];
        std::snprintf(buf, sizeof(buf), "adjoint of mode k=%.6g ended with status %d", r->k[i], v);
        r->err = buf;
      }
    }
    if (r->rc != 0) return;
    const double* tb = reinterpret_cast<const double*>(down + r->h_tbar);
    double g[kTheta] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < nk; ++i)
      for (int d = 0; d < kTD; ++d) g[kSolvedTheta[d]] += tb[size_t(i) * kTD + d];
    if (r->r.kind == BOLT_REQ_CL) {  // [0, nsl): C_l^TT, then [6][nsl] its derivatives at fixed sources
      const double* cl = reinterpret_cast<const double*>(down + r->h_cl);
      const int nsl = int(r->uniq.size());
      for (int j = 0; j < kTheta; ++j)
        for (int sl = 0; sl < nsl; ++sl) g[j] += r->ybar[sl] * cl[size_t(1 + j) * nsl + sl];
      if (r->r.tt)
        for (int e = 0; e < r->r.nell; ++e) {
          int sl = int(std::lower_bound(r->uniq.begin(), r->uniq.end(), r->ells[e]) - r->uniq.begin());
          r->r.tt[e] = cl[sl];
        }
    } else {  // n_s and A_s enter only A (k/0.05)^(n-1) (spectra.jl:195-197)
      const double* P = reinterpret_cast<const double*>(down + r->h_plin);
      for (int i = 0; i < nk; ++i) {
        g[kThetaN] += r->ybar[i] * P[i] * std::log(r->k[i] / 0.05);
        g[kThetaA] += r->ybar[i] * P[i] / r->T[0].par.A;
      }
      if (r->r.plin) std::copy(P, P + nk, r->r.plin);
    }
    if (r->vjp_grad) std::copy(g, g + kTheta, r->vjp_grad);
    return;
  }
  auto deriv = [&](const double* f, size_t stride, int j, size_t i) -> double {  // set 1 + j: theta_j + h
    if (r->tangent) return f[size_t(1 + j) * stride + i];  // the tangent itself
    return (f[size_t(1 + j) * stride + i] - f[i]) / r->step[j];
  };
  if (r->wantP) {
    const double* P = reinterpret_cast<const double*>(down + r->h_plin);
    std::copy(P, P + nk, r->r.plin);
    if (ns > 1)
      for (int j = 0; j < kTheta; ++j)
        for (int i = 0; i < nk; ++i)  // P = (2 pi^2 / k^3) delta_m^2 A (k/0.05)^(n-1) (spectra.jl:195-197)
          r->r.dplin[size_t(j) * nk + i] = j == kThetaN   ? P[i] * std::log(r->k[i] / 0.05)
                                           : j == kThetaA ? P[i] / r->T[0].par.A
                                                          : deriv(P, nk, j, i);
  }
  if (r->r.kind == BOLT_REQ_CL) {
    const double* cl = reinterpret_cast<const double*>(down + r->h_cl);
    const int nsl = int(r->uniq.size());
    const size_t stride = size_t(3) * nsl;
    double* outs[3] = {r->r.tt, r->r.te, r->r.ee};
    double* douts[3] = {r->r.dtt, r->r.dte, r->r.dee};
    const int bits[3] = {BOLT_CL_TT, BOLT_CL_TE, BOLT_CL_EE};
    if (r->los_tangent) {  // [0, nsl): C_l^TT, then [6][nsl] its derivatives
      for (int e = 0; e < r->r.nell; ++e) {
        int sl = int(std::lower_bound(r->uniq.begin(), r->uniq.end(), r->ells[e]) - r->uniq.begin());
        r->r.tt[e] = cl[sl];
        for (int j = 0; j < kTheta; ++j) r->r.dtt[size_t(j) * r->r.nell + e] = cl[size_t(1 + j) * nsl + sl];
      }
      return;
    }
    for (int q = 0; q < 3; ++q) {
      if (!(r->r.cl_want & bits[q])) continue;
      for (int e = 0; e < r->r.nell; ++e) {
        int sl = int(std::lower_bound(r->uniq.begin(), r->uniq.end(), r->ells[e]) - r->uniq.begin());
        outs[q][e] = cl[size_t(q) * nsl + sl];
        if (ns > 1)
          for (int j = 0; j < kTheta; ++j) douts[q][size_t(j) * r->r.nell + e] = deriv(cl, stride, j, size_t(q) * nsl + sl);
      }
    }
  }
}

void finish_lane(bolt_engine* E, Lane& L) {
  float ms1 = 0, ms2 = 0, ms3 = 0;
  cudaEventElapsedTime(&ms1, L.ev[0], L.ev[1]);
  cudaEventElapsedTime(&ms2, L.ev[1], L.ev[2]);
  cudaEventElapsedTime(&ms3, L.ev[2], L.ev[3]);
  const char* down = static_cast<const char*>(L.down.p);
  double steps[2] = {0, 0};
  int64_t modes = 0;
  for (Req* r : L.batch) {
    const int64_t* cnt = reinterpret_cast<const int64_t*>(down + r->h_cnt);
    for (int s = 0; s < r->nsets; ++s)
      for (int i = 0; i < r->r.nk && set_has_modes(r, s); ++i) {
        size_t q = 2 * (size_t(s) * r->r.nk + i);
        steps[(s == 0 && !r->tangent) ? 0 : 1] += double(cnt[q] + cnt[q + 1]);
        r->steps += double(cnt[q] + cnt[q + 1]);
      }
    for (int s = 0; s < r->nsets; ++s) modes += set_has_modes(r, s) ? r->r.nk : 0;
    if (r->adjoint)  // the reverse sweeps (their accepted steps, in the slots of set 1)
      for (int i = 0; i < r->r.nk; ++i) {
        size_t q = 2 * (size_t(r->r.nk) + i);
        steps[1] += double(cnt[q]);
        r->steps += double(cnt[q]);
        ++modes;
      }
  }
  if (L.nmodes[0] > 0) E->tuner.update(L.shared[0], L.key[0], L.wpm[0], ms1 * 1e-3, steps[0]);
  if (L.nmodes[1] > 0 && L.kind[1] == 0) E->tuner.update(L.shared[1], L.key[1], L.wpm[1], ms2 * 1e-3, steps[1]);
  const double t = now_s(E->t0);
  for (Req* r : L.batch) {
    finalize_request(L, r);
    r->state = 3;
    r->t[3] = t;
    E->inflight_bytes -= r->bytes;
  }
  E->stats[0] += 1;
  E->stats[1] += int64_t(L.batch.size());
  E->stats[2] += modes;
  E->stats[3] += int64_t((ms1 + ms2) * 1000.0);
  E->stats[4] += int64_t(ms3 * 1000.0);
  E->stats[5] += int64_t(steps[0] + steps[1]);
  E->stats[6] += L.nlaunch;
  E->stats[7] += L.nmodes[1] > 0 ? 2 : 1;
  E->stats[8 + (L.wpm[0] == 1 ? 0 : (L.wpm[0] == 2 ? 1 : 2))] += 1;
  L.batch.clear();
  L.busy = false;
  E->cv_done.notify_all();
}

void fail_batch(bolt_engine* E, Lane& L, const std::string& msg, int code) {
  const double t = now_s(E->t0);
  for (Req* r : L.batch) {
    if (r->rc == 0) { r->rc = code; r->err = msg; }
    r->state = 3;
    r->t[3] = t;
    E->inflight_bytes -= r->bytes;
  }
  L.batch.clear();
  L.busy = false;
  E->cv_done.notify_all();
}

void scheduler(bolt_engine* E) {
  cudaSetDevice(E->device);
  std::unique_lock<std::mutex> lk(E->mu);
  while (true) {
    // completions
    bool any_busy = false;
    for (Lane& L : E->lanes) {
      if (!L.busy) continue;
      cudaError_t q = cudaEventQuery(L.ev[4]);
      if (q == cudaSuccess) finish_lane(E, L);
      else if (q != cudaErrorNotReady) fail_batch(E, L, std::string("device error: ") + cudaGetErrorString(q), -3);
      else any_busy = true;
    }
    if (E->stop && !any_busy) break;
    // new batches on idle lanes.  With a batching window, while another lane
    // keeps the GPU busy a batch waits until its ready requests hold at
    // least kFillModes modes per SM or the oldest has waited the window:
    // fewer, larger launches; an idle GPU takes whatever is ready at once.
    if (!E->stop && !E->ready.empty() && E->cfg.batch_window_s > 0) {
      bool busy_other = false;
      for (Lane& L : E->lanes) busy_other |= L.busy;
      double ready_modes = 0.0;
      for (Req* r : E->ready) ready_modes += double(r->r.nk) * r->nsets;
      const double waited = now_s(E->t0) - E->ready.front()->t[1];
      if (busy_other && ready_modes < kFillModes * E->nsm && waited < E->cfg.batch_window_s) {
        E->cv_sched.wait_for(lk, std::chrono::microseconds(200));
        continue;
      }
    }
    if (!E->stop) {
      for (Lane& L : E->lanes) {
        if (L.busy || E->ready.empty()) continue;
        std::vector<Req*> batch;
        size_t bytes = 0;
        const int maxb = E->cfg.max_batch > 0 ? E->cfg.max_batch : 1 << 30;
        const double rt = E->ready.front()->r.reltol, at = E->ready.front()->r.abstol;
        int gkind = -1;  // gradient requests of one batch: one kind (replays, tangent or adjoint)
        for (auto it = E->ready.begin(); it != E->ready.end() && int(batch.size()) < maxb;) {
          Req* r = *it;
          if (r->r.reltol != rt || r->r.abstol != at) { ++it; continue; }
          if (r->nsets > 1) {
            const int kind = grad_kind(r);
            if (gkind >= 0 && kind != gkind) { ++it; continue; }
            gkind = kind;
          }
          size_t off = 0;
          layout_request(r, off);
          if (r->bytes > E->budget) {
            r->rc = -5;
            r->err = "request exceeds the device memory budget";
            r->state = 3;
            r->t[3] = now_s(E->t0);
            it = E->ready.erase(it);
            E->cv_done.notify_all();
            continue;
          }
          if (E->inflight_bytes + bytes + r->bytes > E->budget) break;  // FIFO admission
          bytes += r->bytes;
          batch.push_back(r);
          it = E->ready.erase(it);
        }
        if (batch.empty()) continue;
        E->inflight_bytes += bytes;
        E->stats[11] = std::max<int64_t>(E->stats[11], int64_t(E->inflight_bytes));
        const double t = now_s(E->t0);
        for (Req* r : batch) { r->state = 2; r->t[2] = t; }
        L.busy = true;
        L.batch = batch;
        L.waiting = 0;
        for (auto& kv : E->reqs) {
          const Req* q = kv.second.get();
          if (q->state <= 1) L.waiting += q->r.nk * q->nsets;
        }
        lk.unlock();
        std::string msg;
        try {
          launch_batch(E, L, L.batch);
        } catch (const std::exception& x) {
          msg = x.what();
        }
        lk.lock();
        if (!msg.empty()) {
          if (L.d_block) { cudaStreamSynchronize(L.st); cudaFree(L.d_block); L.d_block = nullptr; }
          fail_batch(E, L, msg, -3);
        }
      }
    }
    E->cv_sched.wait_for(lk, std::chrono::microseconds(200));
  }
}

}  // namespace

namespace bolt {
// Per-cosmology device table image (capi.cu's upload layout): hot[n+2][4],
// cold[C_COUNT][n+2], GL nodes and weights.
size_t cosmo_table_doubles(const CosmoTables& T) {
  const size_t n2 = size_t(T.grid.n) + 2;
  return n2 * 4 + size_t(C_COUNT) * n2 + 2 * size_t(T.nq);
}

void fill_cosmo_dev(const CosmoTables& T, double* d_tab, double* h, CosmoDev& d) {
  const int n = T.grid.n, n2 = n + 2, nq = T.nq;
  const int hot_ids[4] = {T_H, T_ETA, T_TAUP, T_CSB2};
  for (int j = 0; j < n2; ++j)
    for (int t = 0; t < 4; ++t) h[size_t(j) * 4 + t] = T.coef[hot_ids[t]][j];
  const int cold_ids[C_COUNT] = {T_H, T_HP, T_HPP, T_ETA, T_TAU, T_TAUP, T_TAUPP, T_G, T_GP, T_GPP, T_CSB2, T_RHO0M};
  double* cold = h + size_t(n2) * 4;
  for (int t = 0; t < C_COUNT; ++t) std::copy(T.coef[cold_ids[t]].begin(), T.coef[cold_ids[t]].end(), cold + size_t(t) * n2);
  double* qx = cold + size_t(C_COUNT) * n2;
  std::copy(T.quad_pts.begin(), T.quad_pts.end(), qx);
  std::copy(T.quad_wts.begin(), T.quad_wts.end(), qx + nq);
  const CosmoParamsH& p = T.par;
  d.h = p.h; d.Omega_r = p.Omega_r; d.Omega_b = p.Omega_b; d.Omega_c = p.Omega_c; d.A = p.A; d.n_s = p.n;
  d.Y_p = p.Y_p; d.N_nu = p.N_nu; d.Sigma_m_nu = p.Sigma_m_nu;
  d.H0 = T.H0; d.eta0 = T.eta0; d.rho_crit = T.rho_crit;
  d.eta_last = spline_eval(T.coef[T_ETA].data(), n, T.grid.x0, T.grid.h, T.grid.at(n - 1));
  d.x_last = T.grid.at(n - 1);
  d.Tnu = T.Tnu; d.logqmin = T.logqmin; d.logqmax = T.logqmax;
  d.Omega_nu = 7.0 * (2.0 / 3.0) * p.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * p.Omega_r;
  d.x0 = T.grid.x0; d.hx = T.grid.h; d.inv_hx = 1.0 / T.grid.h;
  d.n = n; d.nq = nq;
  d.hot = d_tab;
  d.cold = d_tab + size_t(n2) * 4;
  d.qx = d.cold + size_t(C_COUNT) * n2;
  d.qw = d.qx + nq;
}
}  // namespace bolt

// ------------------------------------------------------------------- C ABI
extern "C" {

int bolt_engine_create(const bolt_engine_cfg* cfg, bolt_engine** out) {
  if (!out) return -1;
  *out = nullptr;
  std::unique_ptr<bolt_engine> E(new bolt_engine());
  if (cfg) E->cfg = *cfg;
  if (E->cfg.objective != 0 && E->cfg.objective != 1) return -1;
  if (E->cfg.land_stride < 0 || E->cfg.land_stride > 64) return -1;
  if (E->cfg.grad_scheme < 0 || E->cfg.grad_scheme > 2) return -1;
  E->device = E->cfg.device;
  if (E->cfg.lanes <= 0) E->cfg.lanes = 6;
  if (E->cfg.lanes > 8) E->cfg.lanes = 8;
  if (E->cfg.max_steps <= 0) E->cfg.max_steps = 100000;  // OrdinaryDiffEq's default maxiters
  E->budget = size_t((E->cfg.mem_budget_gb > 0 ? E->cfg.mem_budget_gb : 150.0) * 1073741824.0);
  E->t0 = std::chrono::steady_clock::now();
  try {
    ck(cudaSetDevice(E->device), "cudaSetDevice");
    ck(cudaDeviceGetAttribute(&E->nsm, cudaDevAttrMultiProcessorCount, E->device), "device attribute");
    cudaMemPool_t pool;
    ck(cudaDeviceGetDefaultMemPool(&pool, E->device), "memory pool");
    uint64_t thr = ~uint64_t(0);
    ck(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr), "memory pool threshold");
    E->lanes.resize(E->cfg.lanes);
    for (Lane& L : E->lanes) {
      ck(cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking), "stream");
      for (auto& e : L.ev) ck(cudaEventCreate(&e), "event");
      ck(cudaMalloc(&L.d_queue, 2 * sizeof(int)), "queue");
    }
    // Bessel prefilter pivots of the constant (1, 4, 1) system (natural ends)
    std::vector<double> w(kNb - 2);
    w[0] = 0.25;
    for (int r = 1; r < kNb - 2; ++r) w[r] = 1.0 / (4.0 - w[r - 1]);
    ck(cudaMalloc(&E->d_w, w.size() * sizeof(double)), "pivots");
    ck(cudaMemcpy(E->d_w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice), "pivots");
    ck(cudaMalloc(&E->d_flags, sizeof(int)), "flags");
    ck(cudaMemset(E->d_flags, 0, sizeof(int)), "flags");
  } catch (const std::exception& x) {
    for (Lane& L : E->lanes) {
      if (L.st) cudaStreamDestroy(L.st);
      for (auto& e : L.ev) if (e) cudaEventDestroy(e);
      if (L.d_queue) cudaFree(L.d_queue);
    }
    return -3;
  }
  int nt = E->cfg.host_threads > 0 ? E->cfg.host_threads : int(std::thread::hardware_concurrency());
  nt = std::max(1, std::min(nt, 64));
  bolt_engine* raw = E.get();
  for (int i = 0; i < nt; ++i) E->pool.emplace_back(pool_worker, raw);
  E->sched = std::thread(scheduler, raw);
  *out = E.release();
  return 0;
}

void bolt_engine_destroy(bolt_engine* E) {
  if (!E) return;
  {
    std::lock_guard<std::mutex> g(E->mu);
    E->stop = true;
  }
  E->cv_pool.notify_all();
  E->cv_sched.notify_all();
  for (auto& t : E->pool) t.join();
  E->sched.join();
  cudaSetDevice(E->device);
  for (Lane& L : E->lanes) {
    cudaStreamSynchronize(L.st);
    for (auto& row : L.graph)
      for (auto& G : row) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        if (G.g) cudaGraphDestroy(G.g);
      }
    L.scr.release(); L.los_raw.release(); L.los_norm.release(); L.los_coef.release(); L.los_SdT.release();
    L.los_dSd.release();
    L.los_SdE.release(); L.up.release(); L.down.release();
    cudaFree(L.d_queue);
    for (auto& e : L.ev) cudaEventDestroy(e);
    cudaStreamDestroy(L.st);
  }
  cudaFree(E->d_w);
  cudaFree(E->d_flags);
  delete E;
}

const char* bolt_engine_last_error(const bolt_engine* E) { return E ? E->err.c_str() : "null engine"; }

// Submission; with ybar set, a pullback by the discrete adjoint (q->grad is
// 1; C_l: TT only, ybar per entry of q->ells; P_lin: ybar per k) whose
// parameter cotangent goes to vjp_grad[6] when the request completes.
static int submit_impl(bolt_engine* E, const bolt_request* q, const double* ybar, double* vjp_grad, int64_t* ticket) {
  if (!E || !ticket) return -1;
  std::unique_ptr<Req> r(new Req());
  try {
    check_request(q, ybar == nullptr);
    r->r = *q;
    r->k.assign(q->k, q->k + q->nk);
    r->r.k = r->k.data();
    if (q->kind == BOLT_REQ_CL) {
      r->ells.assign(q->ells, q->ells + q->nell);
      r->r.ells = r->ells.data();
      r->uniq = r->ells;
      std::sort(r->uniq.begin(), r->uniq.end());
      r->uniq.erase(std::unique(r->uniq.begin(), r->uniq.end()), r->uniq.end());
      r->wantE = (q->cl_want & (BOLT_CL_TE | BOLT_CL_EE)) != 0;
      r->los_tangent = q->grad && q->cl_want == BOLT_CL_TT;
      r->wantP = q->plin != nullptr;
    } else {
      r->wantP = true;
      r->r.ells = nullptr;
      r->r.nell = 0;
    }
    // P_lin and C_l^TT Jacobians come from tangent-linear modes when the
    // engine is set to them; otherwise (and for TE / EE) from replays
    r->tangent = q->grad && E->cfg.grad_scheme == 1 && (q->kind == BOLT_REQ_PLIN || r->los_tangent) &&
                 fits_one_warp(q->hier);
    if (ybar) {
      if (!fits_one_warp(q->hier)) throw EngErr(-1, "hierarchy does not fit the adjoint kernel's one warp");
      if (!q->grad || (q->kind == BOLT_REQ_CL && (q->cl_want != BOLT_CL_TT || q->plin)))
        throw EngErr(-1, "an adjoint pullback takes C_l^TT alone or P_lin");
      r->adjoint = true;
      r->tangent = false;
      r->los_tangent = false;
      r->wantE = false;
      r->vjp_grad = vjp_grad;
      if (q->kind == BOLT_REQ_CL) {
        r->ybar.assign(r->uniq.size(), 0.0);
        for (int e = 0; e < q->nell; ++e) {
          int sl = int(std::lower_bound(r->uniq.begin(), r->uniq.end(), q->ells[e]) - r->uniq.begin());
          r->ybar[sl] += ybar[e];
        }
      } else {
        r->ybar.assign(ybar, ybar + q->nk);
      }
    }
    r->grid = make_grid(q->grid.start, q->grid.step, q->grid.stop);
    if (r->grid.n < 4 || r->grid.n > 100000) throw EngErr(-1, "x grid needs 4..100000 nodes");
    if (q->kind == BOLT_REQ_CL) {
      if (!(r->grid.at(r->grid.n - 2) > -8.0)) throw EngErr(-1, "x grid needs two nodes at x > -8");
      while (!(r->grid.at(r->src_from) > -8.0)) ++r->src_from;
    }
    const bolt_hier& h = q->hier;
    r->N = 2 * (h.lg + 1) + (h.lnu + 1) + (h.lmnu + 1) * h.nq + 5;
    const size_t smem = rodas_smem_per_mode(r->N, h.nq, std::max(h.lg, std::max(h.lnu, h.lmnu)), 4);
    if (smem > 227 * 1024) throw EngErr(-1, "hierarchy too large for shared memory");
    CosmoParamsH base{q->par.h, q->par.Omega_r, q->par.Omega_b, q->par.Omega_c, q->par.A, q->par.n, q->par.Y_p,
                      q->par.N_nu, q->par.Sigma_m_nu};
    r->pars.push_back(base);
    if (q->grad) {
      r->nsets = 1 + kTheta;
      r->rec_cap = int(std::min<long long>(E->cfg.max_steps, kRecCapMax));
      double th[kTheta];
      theta_of(base, th);
      for (int j = 0; j < kTheta; ++j) {
        // step = 1e-6 |theta_j| (Sigma m_nu: at least 1e-7 eV, so it works at 0)
        double hstep = kRelStep * std::max(std::fabs(th[j]), j == 5 ? 0.1 : 1e-30);
        r->step[j] = hstep;
        double a[kTheta];
        std::copy(th, th + kTheta, a);
        a[j] += hstep;
        r->pars.push_back(params_of(base, a));
      }
    }
    r->T.resize(r->nsets);
    r->tables_left = r->nsets;
  } catch (const EngErr& x) {
    std::lock_guard<std::mutex> g(E->mu);
    E->err = x.what();
    return x.code;
  } catch (const std::exception& x) {
    std::lock_guard<std::mutex> g(E->mu);
    E->err = x.what();
    return -1;
  }
  std::lock_guard<std::mutex> g(E->mu);
  if (E->stop) { E->err = "engine is shutting down"; return -6; }
  r->ticket = E->next_ticket++;
  r->t[0] = now_s(E->t0);
  Req* rp = r.get();
  E->reqs[r->ticket] = std::move(r);
  E->tasks.push_back([E, rp] {
    std::string e;
    try { build_set(rp, 0); } catch (const std::exception& x) { e = x.what(); }
    std::lock_guard<std::mutex> g2(E->mu);
    set_done(E, rp, 0, e);
  });
  E->cv_pool.notify_one();
  *ticket = rp->ticket;
  return 0;
}

int bolt_engine_submit(bolt_engine* E, const bolt_request* q, int64_t* ticket) {
  return submit_impl(E, q, nullptr, nullptr, ticket);
}

int bolt_engine_wait(bolt_engine* E, int64_t ticket, double timeout_s, int* rc_out, double* times_out, char* errbuf,
                     int errlen) {
  if (!E) return -1;
  std::unique_lock<std::mutex> lk(E->mu);
  auto it = E->reqs.find(ticket);
  if (it == E->reqs.end()) { E->err = "unknown ticket"; return -2; }
  Req* r = it->second.get();
  auto pred = [&] { return r->state == 3; };
  if (timeout_s < 0) E->cv_done.wait(lk, pred);
  else if (!E->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return 0;
  if (rc_out) *rc_out = r->rc;
  if (times_out) {
    std::copy(r->t, r->t + 4, times_out);
    times_out[4] = r->steps;
  }
  if (errbuf && errlen > 0) {
    std::strncpy(errbuf, r->err.c_str(), size_t(errlen) - 1);
    errbuf[errlen - 1] = 0;
  }
  E->reqs.erase(it);
  return 1;
}

int bolt_request_run(bolt_engine* E, const bolt_request* q, char* errbuf, int errlen) {
  int64_t t = 0;
  int rc = bolt_engine_submit(E, q, &t);
  if (rc != 0) {
    if (errbuf && errlen > 0) {
      std::lock_guard<std::mutex> g(E->mu);
      std::strncpy(errbuf, E->err.c_str(), size_t(errlen) - 1);
      errbuf[errlen - 1] = 0;
    }
    return rc;
  }
  int out = 0;
  rc = bolt_engine_wait(E, t, -1.0, &out, nullptr, errbuf, errlen);
  return rc == 1 ? out : rc;
}

// Reverse-mode products: run the request with its Jacobian (library-owned
// [6][n] buffers), then contract with the caller's cotangents.
static int run_vjp(bolt_engine* E, const bolt_request* q, int kind, const double* const ybar[3], double* grad,
                   char* errbuf, int errlen) {
  auto fail = [&](const char* m) {
    if (errbuf && errlen > 0) {
      std::strncpy(errbuf, m, size_t(errlen) - 1);
      errbuf[errlen - 1] = 0;
    }
    return -1;
  };
  if (!E || !q || !grad) return fail("null argument");
  if (q->kind != kind) return fail(kind == BOLT_REQ_CL ? "bolt_cl_vjp needs a C_l request" : "bolt_plin_vjp needs a P_lin request");
  bolt_request r = *q;
  r.grad = 1;
  const bool adjoint = E->cfg.grad_scheme == 2 && ybar[0] && fits_one_warp(q->hier) &&
                       (kind == BOLT_REQ_PLIN || (q->cl_want == BOLT_CL_TT && !q->plin && !ybar[1] && !ybar[2]));
  if (adjoint) {  // one forward and one reverse sweep (csrc/adjoint.cuh)
    r.dtt = r.dte = r.dee = r.dplin = nullptr;
    std::vector<double> prim;
    if (kind == BOLT_REQ_CL && !r.tt && r.nell > 0) { prim.assign(size_t(r.nell), 0.0); r.tt = prim.data(); }
    if (kind == BOLT_REQ_PLIN && !r.plin && r.nk > 0) { prim.assign(size_t(r.nk), 0.0); r.plin = prim.data(); }
    int64_t t = 0;
    int rc = submit_impl(E, &r, ybar[0], grad, &t);
    if (rc != 0) {
      std::lock_guard<std::mutex> g(E->mu);
      return fail(E->err.c_str());
    }
    int out = 0;
    rc = bolt_engine_wait(E, t, -1.0, &out, nullptr, errbuf, errlen);
    return rc == 1 ? out : rc;
  }
  const int n = kind == BOLT_REQ_CL ? r.nell : r.nk;
  if (n <= 0) return fail(kind == BOLT_REQ_CL ? "no multipoles" : "no wavenumbers");
  std::vector<double> prim[3], jac[3], jac_p;
  double** outs[3] = {&r.tt, &r.te, &r.ee};
  double** douts[3] = {&r.dtt, &r.dte, &r.dee};
  if (kind == BOLT_REQ_CL) {
    if (r.plin) {  // P_lin asked for alongside: its Jacobian is computed but not contracted
      jac_p.assign(size_t(kTheta) * r.nk, 0.0);
      r.dplin = jac_p.data();
    }
    for (int c = 0; c < 3; ++c) {
      *douts[c] = nullptr;
      if (!(r.cl_want & (1 << c))) continue;
      if (!*outs[c]) { prim[c].assign(size_t(n), 0.0); *outs[c] = prim[c].data(); }
      jac[c].assign(size_t(kTheta) * n, 0.0);
      *douts[c] = jac[c].data();
    }
  } else {
    if (!r.plin) { prim[0].assign(size_t(n), 0.0); r.plin = prim[0].data(); }
    jac[0].assign(size_t(kTheta) * n, 0.0);
    r.dplin = jac[0].data();
  }
  int rc = bolt_request_run(E, &r, errbuf, errlen);
  if (rc != 0) return rc;
  for (int j = 0; j < kTheta; ++j) {
    double acc = 0.0;
    for (int c = 0; c < 3; ++c) {
      if (jac[c].empty() || !ybar[c]) continue;
      for (int i = 0; i < n; ++i) acc += ybar[c][i] * jac[c][size_t(j) * n + i];
    }
    grad[j] = acc;
  }
  return 0;
}

int bolt_cl_vjp(bolt_engine* E, const bolt_request* q, const double* ybar_tt, const double* ybar_te,
                const double* ybar_ee, double* grad, char* errbuf, int errlen) {
  const double* yb[3] = {ybar_tt, ybar_te, ybar_ee};
  return run_vjp(E, q, BOLT_REQ_CL, yb, grad, errbuf, errlen);
}

int bolt_plin_vjp(bolt_engine* E, const bolt_request* q, const double* ybar, double* grad, char* errbuf,
                  int errlen) {
  const double* yb[3] = {ybar, nullptr, nullptr};
  return run_vjp(E, q, BOLT_REQ_PLIN, yb, grad, errbuf, errlen);
}

int bolt_engine_stats(bolt_engine* E, int64_t* out) {
  if (!E || !out) return -1;
  std::lock_guard<std::mutex> g(E->mu);
  std::copy(E->stats, E->stats + 12, out);
  return 0;
}

}  // extern "C"
