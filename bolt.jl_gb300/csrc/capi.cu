// C ABI (include/bolt_gb300.h): context, cosmology registry in HBM and the
// drop-in entry points for boltsolve / source_grid / cltt / clte / clee /
// plin.  Host arrays in, host arrays out; device memory, the stream and the
// kernel launches are owned by the context.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/bolt_gb300.h"
#include "bolt_dev.cuh"
#include "host_cosmo.hpp"

namespace bolt {
int rodas_grid_warps(int nmodes, int maxN, int maxnq, int maxL, int warps_per_block, int* blocks);
int launch_rodas(const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const SolverCfg& cfg, int* d_queue,
                 int maxN, int maxnq, int maxL, int warps_per_block, int blocks, double* d_scratch, cudaStream_t stream);
size_t rodas_smem_per_warp(int maxN, int maxnq, int maxL);
size_t rodas_smem_per_mode(int maxN, int maxnq, int maxL, int wpm);
size_t rodas_scratch_per_warp(int maxN);
int launch_rsa_post(const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const int* d_first, int nout,
                    cudaStream_t stream);
int launch_jl_raw(int nb, const double* d_dgs, int ncz, int Lmax, const int* d_slot_of_l, int nslots, double* d_raw,
                  double* d_norm, int* d_flags, cudaStream_t st);
int launch_jl_prefilter(int nb, int nslots, int ncz, const double* d_raw, const double* d_norm, const double* d_w,
                        double* d_coef, cudaStream_t st);
int launch_sdense(int nx, int i0, int nrow, int nk, const double* d_kgrid, const double* d_ST, const double* d_SE, int nm,
                  const double* d_kmid, const double* d_dx, double* d_SdT, double* d_SdE, cudaStream_t st);
int launch_los_cl(const LosArgs& a, int ncz, cudaStream_t st);
int launch_moment_direct(int n, double m, const double* d_x, int nx, double* d_out, const GL8& g, cudaStream_t st);
int launch_moment_table(const MomTabDev& T, double* d_y, double* d_seg, const double* d_w, double* d_work,
                        cudaStream_t st);
int launch_moment_eval(const MomTabDev& T, const double* d_x, int nx, double* d_out, cudaStream_t st);
int launch_filon(const MomTabDev& T, int n, const double* f, const double* fp, const double* fpp, const double* k,
                 const double* a, const double* b, double* out, cudaStream_t st);
int launch_filon_piecewise(const MomTabDev& T, int nt, const double* t, const double* f, const double* fp,
                           const double* fpp, double* D, int nk, const double* k, double* out, int nblocks,
                           cudaStream_t st);
int launch_filon_batched(const MomTabDev& T, int nt, const double* t, const double* f, const double* fp,
                         const double* fpp, int nk, const double* k, double* out, int nblocks, cudaStream_t st);
int launch_adjoint_check(const CosmoDev* d_cos, int id, double k, int lg, int lnu, int lmnu, int nq, double x,
                         double hs, double* d_scr, double* d_out, cudaStream_t st);
size_t adjoint_check_scratch_bytes(int N);
}  // namespace bolt

using namespace bolt;

namespace {

struct Err : std::runtime_error {
  int code;
  Err(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Err(-3, std::string(what) + ": " + cudaGetErrorString(e));
}

struct DBuf {
  void* p = nullptr;
  size_t cap = 0;
  void* get(size_t bytes) {
    if (bytes > cap) {
      if (p) cudaFree(p);
      p = nullptr;
      cap = 0;
      size_t want = std::max<size_t>(bytes, 256);
      ck(cudaMalloc(&p, want), "cudaMalloc");
      cap = want;
    }
    return p;
  }
  template <class T> T* as(size_t n) { return static_cast<T*>(get(n * sizeof(T))); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct CosmoEntry {
  bool live = false;
  CosmoTables T;
  double* d_tab = nullptr;  // hot + cold + qx + qw
  CosmoDev dev;
};

}  // namespace

struct MomEntry {
  bool live = false;
  MomTabDev T{};
  DBuf coef;
};

struct bolt_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4];
  int wpb = 0;
  long long max_steps = 100000;  // OrdinaryDiffEq's default maxiters
  double x_dense = -8.5;
  int land_stride = 1;
  std::vector<CosmoEntry> cos;
  DBuf d_cos;
  DBuf modes, xout, srcT, srcE, traj, plin, status, counters, queue, flags, scratch;
  DBuf kgrid, raw, norm, coef, w, slot_of_l, ells, SdT, SdE, kmid, wts, yv, dx, dgs, idg, out, terms;
  std::vector<MomEntry> mtab;
  DBuf m0, m1, m2, m3, m4, m5, m6, m7, m8;  // Bessel-moment and Filon arguments
  std::string err;
  int64_t stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

namespace {

int fail(bolt_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  return code;
}

void upload_cosmo(bolt_ctx* c, CosmoEntry& e) {
  const CosmoTables& T = e.T;
  const int n = T.grid.n, n2 = n + 2, nq = T.nq;
  size_t count = size_t(n2) * 4 + size_t(C_COUNT) * n2 + 2 * nq;
  std::vector<double> h(count);
  const int hot_ids[4] = {T_H, T_ETA, T_TAUP, T_CSB2};
  for (int j = 0; j < n2; ++j)
    for (int t = 0; t < 4; ++t) h[size_t(j) * 4 + t] = T.coef[hot_ids[t]][j];
  const int cold_ids[C_COUNT] = {T_H, T_HP, T_HPP, T_ETA, T_TAU, T_TAUP, T_TAUPP, T_G, T_GP, T_GPP, T_CSB2, T_RHO0M};
  double* cold = h.data() + size_t(n2) * 4;
  for (int t = 0; t < C_COUNT; ++t) std::copy(T.coef[cold_ids[t]].begin(), T.coef[cold_ids[t]].end(), cold + size_t(t) * n2);
  double* qx = cold + size_t(C_COUNT) * n2;
  std::copy(T.quad_pts.begin(), T.quad_pts.end(), qx);
  std::copy(T.quad_wts.begin(), T.quad_wts.end(), qx + nq);
  ck(cudaMalloc(&e.d_tab, count * sizeof(double)), "cudaMalloc tables");
  ck(cudaMemcpyAsync(e.d_tab, h.data(), count * sizeof(double), cudaMemcpyHostToDevice, c->stream), "upload tables");
  ck(cudaStreamSynchronize(c->stream), "sync");
  CosmoDev& d = e.dev;
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
  d.hot = e.d_tab;
  d.cold = e.d_tab + size_t(n2) * 4;
  d.qx = qx - h.data() + e.d_tab;
  d.qw = d.qx + nq;
}

void sync_cosmo_array(bolt_ctx* c) {
  std::vector<CosmoDev> v(c->cos.size());
  for (size_t i = 0; i < c->cos.size(); ++i) v[i] = c->cos[i].dev;
  CosmoDev* d = c->d_cos.as<CosmoDev>(std::max<size_t>(v.size(), 1));
  if (!v.empty()) ck(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(CosmoDev), cudaMemcpyHostToDevice, c->stream), "cosmo array");
}

CosmoEntry& get_cosmo(bolt_ctx* c, int id) {
  if (id < 0 || id >= int(c->cos.size()) || !c->cos[id].live) throw Err(-2, "unknown cosmology id");
  return c->cos[id];
}

int add_cosmo(bolt_ctx* c, CosmoEntry&& e) {
  int id = -1;
  for (size_t i = 0; i < c->cos.size(); ++i)
    if (!c->cos[i].live) { id = int(i); break; }
  if (id < 0) { c->cos.emplace_back(); id = int(c->cos.size()) - 1; }
  c->cos[id] = std::move(e);
  c->cos[id].live = true;
  upload_cosmo(c, c->cos[id]);
  sync_cosmo_array(c);
  return id;
}

CosmoParamsH to_h(const bolt_params* p) {
  CosmoParamsH q{p->h, p->Omega_r, p->Omega_b, p->Omega_c, p->A, p->n, p->Y_p, p->N_nu, p->Sigma_m_nu};
  return q;
}

void check_hier(const bolt_hier* h) {
  if (!h) throw Err(-1, "hierarchy is null");
  if (h->lg < 3 || h->lnu < 3 || h->lmnu < 3) throw Err(-1, "hierarchy truncations must be >= 3");
  if (h->nq < 1 || h->nq > 27) throw Err(-1, "nq must be in 1..27 (one warp lane per chain)");
  if (h->lg > 1000 || h->lnu > 1000 || h->lmnu > 1000) throw Err(-1, "hierarchy truncation too large");
}

int state_len(const bolt_hier* h) { return 2 * (h->lg + 1) + (h->lnu + 1) + (h->lmnu + 1) * h->nq + 5; }

// Runs the solver over nk modes of one cosmology; all device outputs are
// laid out per mode.  Returns the device mode array for callers that need it.
void run_solver(bolt_ctx* c, int id, const double* k, int nk, const bolt_hier* h, double reltol, double abstol,
                const double* d_x, int nx, int flags, double* d_srcT, double* d_srcE, double* d_traj, double* d_plin,
                int32_t* status_host) {
  CosmoEntry& e = get_cosmo(c, id);
  check_hier(h);
  if (h->nq != e.T.nq) throw Err(-1, "hierarchy nq must equal the Background nq");
  if (!(reltol > 0) || !(abstol > 0)) throw Err(-1, "tolerances must be positive");
  if (nk <= 0) throw Err(-1, "no wavenumbers");
  for (int i = 0; i < nk; ++i)
    if (!(k[i] > 0) || !std::isfinite(k[i])) throw Err(-1, "wavenumbers must be positive and finite");
  const int N = state_len(h);
  ModeDev* d_modes = c->modes.as<ModeDev>(nk);
  int32_t* d_status = c->status.as<int32_t>(nk);
  int64_t* d_cnt = c->counters.as<int64_t>(2 * size_t(nk));
  int* d_queue = c->queue.as<int>(1);
  std::vector<ModeDev> hm(nk);
  // longest modes first (cost grows with k)
  std::vector<int> order(nk);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return k[a] > k[b]; });
  for (int r = 0; r < nk; ++r) {
    int i = order[r];
    ModeDev& m = hm[r];
    m.k = k[i];
    m.cosmo = id;
    m.lg = h->lg; m.lnu = h->lnu; m.lmnu = h->lmnu; m.nq = h->nq;
    m.flags = flags;
    m.nout = nx;
    m.xout = d_x;
    m.src_T = d_srcT ? d_srcT + size_t(i) * nx : nullptr;
    m.src_E = d_srcE ? d_srcE + size_t(i) * nx : nullptr;
    m.traj = d_traj ? d_traj + size_t(i) * nx * N : nullptr;
    m.plin = d_plin ? d_plin + i : nullptr;
    m.status = d_status + i;
    m.counters = d_cnt + 2 * size_t(i);
  }
  ck(cudaMemcpyAsync(d_modes, hm.data(), nk * sizeof(ModeDev), cudaMemcpyHostToDevice, c->stream), "modes");
  SolverCfg cfg;
  cfg.reltol = reltol;
  cfg.abstol = abstol;
  cfg.h0 = 1e-3;
  cfg.x_dense = c->x_dense;
  cfg.max_steps = c->max_steps;
  cfg.land_stride = c->land_stride;
  int Lmax = std::max(h->lg, std::max(h->lnu, h->lmnu));
  // warps per mode: 0 chooses by the launch size alone, one warp per mode
  // from about 20 modes per SM (where the FP64 issue rate, not the longest
  // mode's chain of dependent steps, bounds a launch; measured at N = 473),
  // else four
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
  const int wpb = c->wpb != 0 ? c->wpb : (nk >= 20 * std::max(nsm, 1) ? 1 : 4);
  size_t pw = rodas_smem_per_mode(N, h->nq, Lmax, wpb);  // shared memory of one mode (one CTA)
  if (pw > 227 * 1024) throw Err(-1, "hierarchy too large for shared memory");
  int blocks = 0;
  int rc = rodas_grid_warps(nk, N, h->nq, Lmax, wpb, &blocks);
  if (rc != 0) throw Err(-3, std::string("solver configuration: ") + cudaGetErrorString(cudaError_t(-rc)));
  double* d_scr = c->scratch.as<double>(size_t(blocks) * rodas_scratch_per_warp(N) / sizeof(double));
  ck(cudaEventRecord(c->ev[0], c->stream), "event");
  rc = launch_rodas(d_modes, nk, c->d_cos.as<CosmoDev>(c->cos.size()), cfg, d_queue, N, h->nq, Lmax, wpb, blocks,
                    d_scr, c->stream);
  if (rc != 0) throw Err(-3, std::string("solver launch: ") + cudaGetErrorString(cudaError_t(rc)));
  ck(cudaEventRecord(c->ev[1], c->stream), "event");
  std::vector<int32_t> st(nk);
  std::vector<int64_t> cnt(2 * size_t(nk));
  ck(cudaMemcpyAsync(st.data(), d_status, nk * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "status");
  ck(cudaMemcpyAsync(cnt.data(), d_cnt, 2 * nk * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream), "counters");
  ck(cudaStreamSynchronize(c->stream), "solver");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
  int64_t acc = 0, rej = 0;
  for (int i = 0; i < nk; ++i) { acc += cnt[2 * i]; rej += cnt[2 * i + 1]; }
  c->stats[0] += acc;
  c->stats[1] += rej;
  c->stats[2] += int64_t(ms * 1000.0);
  c->stats[4] += nk;
  c->stats[5] += 1;
  c->stats[6] += 1;
  if (status_host) std::copy(st.begin(), st.end(), status_host);
}

std::vector<double> quadratic_k(double kmin, double kmax, int nk) {  // spectra.jl:60-63
  std::vector<double> out(nk);
  for (int i = 1; i <= nk; ++i) {
    double t = double(i) / double(nk);
    out[i - 1] = kmin + (kmax - kmin) * (t * t);
  }
  return out;
}

// First x node the line-of-sight sums use: findfirst(x_grid .> -8)
// (spectra.jl:86).
int los_first_node(const GridSpec& g) {
  int i0 = 0;
  while (i0 < g.n && !(g.at(i0) > -8.0)) ++i0;
  return i0;
}

// LOS on device source grids (d_ST, d_SE: [nk][nx - src_from], x nodes
// src_from .. nx-1; src_from <= los_first_node).
void run_los(bolt_ctx* c, int id, const double* d_ST, const double* d_SE, int src_from, const double* k, int nk,
             const int* ells, int nell, double* tt, double* te, double* ee) {
  CosmoEntry& e = get_cosmo(c, id);
  const CosmoTables& T = e.T;
  const GridSpec& g = T.grid;
  const int nx = g.n;
  if (nk < 2) throw Err(-1, "need at least two source-grid wavenumbers");
  for (int i = 1; i < nk; ++i)
    if (!(k[i] > k[i - 1])) throw Err(-1, "source-grid wavenumbers must be strictly ascending");
  if (nell <= 0) throw Err(-1, "no multipoles");
  if ((te || ee) && !d_SE) throw Err(-1, "TE / EE need the polarization source grid");
  std::vector<int> uniq(ells, ells + nell);
  for (int l : uniq)
    if (l < 0 || l > 20000) throw Err(-1, "multipole out of range");
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  const int ns = int(uniq.size()), Lmax = uniq.back();
  std::vector<int> slot_of_l(Lmax + 1, -1);
  for (int s = 0; s < ns; ++s) slot_of_l[uniq[s]] = s;
  // dense k grid and weights (spectra.jl:84-96, 132-135)
  const int nkd = 5000, nm = nkd - 1, nb = 5001;
  std::vector<double> kd = quadratic_k(0.01 * T.H0, 1000.0 * T.H0, nkd);
  std::vector<double> kmid(nm), wts(nm);
  for (int m = 0; m < nm; ++m) {
    double km = (kd[m] + kd[m + 1]) / 2.0, dk = kd[m + 1] - kd[m];
    kmid[m] = km;
    wts[m] = T.par.A * std::pow(km / 0.05, T.par.n - 1.0) * dk / km;
  }
  double argmax = kd[nkd - 1] * T.eta0;
  double dg = argmax / 5000.0;
  double inv_dg = 1.0 / dg;
  const int i0 = los_first_node(g);
  const int nrow = nx - 1 - i0;
  if (nrow <= 0) throw Err(-1, "x grid does not reach x > -8");
  if (src_from < 0 || src_from > i0) throw Err(-1, "source grid starts past the first x > -8");
  std::vector<double> yv(nrow), dxs(nrow);
  for (int i = 0; i < nrow; ++i) {
    double x = g.at(i0 + i);
    yv[i] = T.eta0 - spline_eval(T.coef[T_ETA].data(), nx, g.x0, g.h, x);
    dxs[i] = g.at(i0 + i + 1) - x;
  }
  std::vector<double> w(nb - 2);
  w[0] = 0.25;
  for (int r = 1; r < nb - 2; ++r) w[r] = 1.0 / (4.0 - w[r - 1]);
  cudaStream_t st = c->stream;
  double* d_kg = c->kgrid.as<double>(nk);
  double* d_kmid = c->kmid.as<double>(nm);
  double* d_wts = c->wts.as<double>(nm);
  double* d_yv = c->yv.as<double>(nrow);
  double* d_dx = c->dx.as<double>(nrow);
  double* d_w = c->w.as<double>(nb - 2);
  int* d_sl = c->slot_of_l.as<int>(Lmax + 1);
  int* d_ells = c->ells.as<int>(ns);
  double* d_dg = c->dgs.as<double>(2);
  double* d_raw = c->raw.as<double>(size_t(ns) * nb);
  double* d_norm = c->norm.as<double>(nb);
  double* d_coef = c->coef.as<double>(size_t(ns) * (nb + 2));
  double* d_SdT = c->SdT.as<double>(size_t(nrow) * nm);
  double* d_SdE = d_SE ? c->SdE.as<double>(size_t(nrow) * nm) : nullptr;
  double* d_out = c->out.as<double>(3 * size_t(ns));
  int* d_flags = c->flags.as<int>(1);
  double dgv[2] = {dg, inv_dg};
  ck(cudaMemcpyAsync(d_kg, k, nk * sizeof(double), cudaMemcpyHostToDevice, st), "kgrid");
  ck(cudaMemcpyAsync(d_kmid, kmid.data(), nm * sizeof(double), cudaMemcpyHostToDevice, st), "kmid");
  ck(cudaMemcpyAsync(d_wts, wts.data(), nm * sizeof(double), cudaMemcpyHostToDevice, st), "wts");
  ck(cudaMemcpyAsync(d_yv, yv.data(), nrow * sizeof(double), cudaMemcpyHostToDevice, st), "yv");
  ck(cudaMemcpyAsync(d_dx, dxs.data(), nrow * sizeof(double), cudaMemcpyHostToDevice, st), "dx");
  ck(cudaMemcpyAsync(d_w, w.data(), (nb - 2) * sizeof(double), cudaMemcpyHostToDevice, st), "w");
  ck(cudaMemcpyAsync(d_sl, slot_of_l.data(), (Lmax + 1) * sizeof(int), cudaMemcpyHostToDevice, st), "slots");
  ck(cudaMemcpyAsync(d_ells, uniq.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st), "ells");
  ck(cudaMemcpyAsync(d_dg, dgv, 2 * sizeof(double), cudaMemcpyHostToDevice, st), "dg");
  ck(cudaMemsetAsync(d_flags, 0, sizeof(int), st), "flags");
  unsigned long long* d_terms = c->terms.as<unsigned long long>(1);
  ck(cudaMemsetAsync(d_terms, 0, sizeof(unsigned long long), st), "terms");
  ck(cudaEventRecord(c->ev[2], st), "event");
  int rc = launch_jl_raw(nb, d_dg, 1, Lmax, d_sl, ns, d_raw, d_norm, d_flags, st);
  if (!rc) rc = launch_jl_prefilter(nb, ns, 1, d_raw, d_norm, d_w, d_coef, st);
  if (!rc)
    rc = launch_sdense(nx - src_from, i0 - src_from, nrow, nk, d_kg, d_ST, d_SE, nm, d_kmid, d_dx, d_SdT, d_SdE, st);
  if (rc) throw Err(-3, std::string("LOS launch: ") + cudaGetErrorString(cudaError_t(rc)));
  LosArgs a;
  a.nb = nb; a.nslots = ns; a.nrow = nrow; a.nm = nm;
  a.ells = d_ells; a.coef = d_coef; a.inv_dg = d_dg + 1; a.yv = d_yv; a.kmid = d_kmid; a.wts = d_wts;
  a.SdT = d_SdT; a.SdE = d_SdE;
  a.tt = d_out; a.te = d_SE ? d_out + ns : nullptr; a.ee = d_SE ? d_out + 2 * ns : nullptr;
  a.terms = d_terms;
  rc = launch_los_cl(a, 1, st);
  if (rc) throw Err(-3, std::string("LOS launch: ") + cudaGetErrorString(cudaError_t(rc)));
  ck(cudaEventRecord(c->ev[3], st), "event");
  std::vector<double> out(3 * size_t(ns));
  unsigned long long terms = 0;
  ck(cudaMemcpyAsync(out.data(), d_out, 3 * ns * sizeof(double), cudaMemcpyDeviceToHost, st), "cl out");
  ck(cudaMemcpyAsync(&terms, d_terms, sizeof(terms), cudaMemcpyDeviceToHost, st), "terms");
  ck(cudaStreamSynchronize(st), "los");
  c->stats[7] += int64_t(terms);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
  c->stats[3] += int64_t(ms * 1000.0);
  c->stats[6] += 4;
  for (int i = 0; i < nell; ++i) {
    int s = slot_of_l[ells[i]];
    if (tt) tt[i] = out[s];
    if (te) te[i] = out[ns + s];
    if (ee) ee[i] = out[2 * ns + s];
  }
}

template <class F>
int guard(bolt_ctx* c, F&& f) {
  if (!c) return -1;
  try {
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return fail(c, -3, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    std::fill(c->stats, c->stats + 8, 0);
    f();
    c->err.clear();
    return 0;
  } catch (const Err& e) {
    return fail(c, e.code, e.what());
  } catch (const std::exception& e) {
    return fail(c, -4, e.what());
  }
}

}  // namespace

extern "C" {

int bolt_version(void) { return 1; }
double bolt_mass_natural(void) { return units_mass_eV(); }
double bolt_km_s_Mpc_100(void) { return units_km_s_Mpc_100(); }

int bolt_host_tables(const bolt_params* par, const bolt_grid* grid, int nq, const bolt_recfast* rf, double* nodes,
                     double* scalars, char* errbuf, int errlen) {
  try {
    if (!par || !grid || !rf || !nodes || !scalars) throw Err(-1, "null argument");
    if (!(grid->step > 0) || !(grid->stop > grid->start)) throw Err(-1, "bad x grid");
    CosmoTables T;
    RecfastOpts ro{rf->Yp, rf->OmegaB, rf->OmegaG, rf->Tnow, rf->tol > 0 ? rf->tol : 1e-8, rf->ionization};
    if (ro.ionization != 0 && ro.ionization != 1) throw Err(-1, "ionization must be 0 (RECFAST) or 1 (Saha-Peebles)");
    build_cosmo_tables(to_h(par), make_grid(grid->start, grid->step, grid->stop), nq, ro, T);
    const int n = T.grid.n;
    for (int t = 0; t < T_COUNT; ++t) std::copy(T.nodes[t].begin(), T.nodes[t].end(), nodes + size_t(t) * n);
    scalars[0] = T.H0; scalars[1] = T.eta0; scalars[2] = T.rho_crit; scalars[3] = T.Omega_Lambda;
    scalars[4] = T.z_He_evo_start; scalars[5] = T.z_H_He_evo_start; scalars[6] = T.Tnow; scalars[7] = T.Tnu;
    scalars[8] = spline_eval(T.coef[T_ETA].data(), n, T.grid.x0, T.grid.h, T.grid.at(n - 1));
    scalars[9] = n;
    return 0;
  } catch (const Err& e) {
    if (errbuf && errlen > 0) { std::snprintf(errbuf, errlen, "%s", e.what()); }
    return e.code;
  } catch (const std::exception& e) {
    if (errbuf && errlen > 0) { std::snprintf(errbuf, errlen, "%s", e.what()); }
    return -4;
  }
}

int bolt_host_tables_frozen(const bolt_params* base, const bolt_params* par, const bolt_grid* grid, int nq,
                            const bolt_recfast* rf_base, const bolt_recfast* rf, double* nodes, char* errbuf,
                            int errlen) {
  try {
    if (!base || !par || !grid || !rf_base || !rf || !nodes) throw Err(-1, "null argument");
    if (!(grid->step > 0) || !(grid->stop > grid->start)) throw Err(-1, "bad x grid");
    const GridSpec g = make_grid(grid->start, grid->step, grid->stop);
    RecfastFreeze fz;
    CosmoTables T0, T;
    RecfastOpts r0{rf_base->Yp, rf_base->OmegaB, rf_base->OmegaG, rf_base->Tnow, rf_base->tol > 0 ? rf_base->tol : 1e-8};
    build_cosmo_tables(to_h(base), g, nq, r0, T0, &fz);  // records
    RecfastOpts ro{rf->Yp, rf->OmegaB, rf->OmegaG, rf->Tnow, rf->tol > 0 ? rf->tol : 1e-8, rf->ionization};
    if (ro.ionization != 0 && ro.ionization != 1) throw Err(-1, "ionization must be 0 (RECFAST) or 1 (Saha-Peebles)");
    build_cosmo_tables(to_h(par), g, nq, ro, T, &fz);    // replays
    const int n = T.grid.n;
    for (int t = 0; t < T_COUNT; ++t) std::copy(T.nodes[t].begin(), T.nodes[t].end(), nodes + size_t(t) * n);
    return 0;
  } catch (const Err& e) {
    if (errbuf && errlen > 0) { std::snprintf(errbuf, errlen, "%s", e.what()); }
    return e.code;
  } catch (const std::exception& e) {
    if (errbuf && errlen > 0) { std::snprintf(errbuf, errlen, "%s", e.what()); }
    return -4;
  }
}

int bolt_ctx_create(const bolt_opts* opts, bolt_ctx** out) {
  if (!out) return -1;
  *out = nullptr;
  bolt_ctx* c = new bolt_ctx();
  if (opts) {
    c->device = opts->device;
    c->wpb = opts->warps_per_block;
    if (opts->max_steps > 0) c->max_steps = opts->max_steps;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= c->device) {
    delete c;
    return -3;
  }
  if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return -3;
  }
  for (int i = 0; i < 4; ++i) cudaEventCreate(&c->ev[i]);
  *out = c;
  return 0;
}

void bolt_ctx_destroy(bolt_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& e : c->cos)
    if (e.d_tab) cudaFree(e.d_tab);
  DBuf* bufs[] = {&c->d_cos, &c->modes, &c->xout, &c->srcT, &c->srcE, &c->traj, &c->plin, &c->status, &c->counters,
                  &c->queue, &c->flags, &c->scratch, &c->kgrid, &c->raw, &c->norm, &c->coef, &c->w, &c->slot_of_l, &c->ells,
                  &c->SdT, &c->SdE, &c->kmid, &c->wts, &c->yv, &c->dx, &c->dgs, &c->idg, &c->out, &c->terms,
                  &c->m0, &c->m1, &c->m2, &c->m3, &c->m4, &c->m5, &c->m6, &c->m7, &c->m8};
  for (auto& e : c->mtab) e.coef.release();
  for (DBuf* b : bufs) b->release();
  for (int i = 0; i < 4; ++i) cudaEventDestroy(c->ev[i]);
  cudaStreamDestroy(c->stream);
  delete c;
}

const char* bolt_last_error(const bolt_ctx* c) { return c ? c->err.c_str() : "null context"; }

int bolt_cosmo_build(bolt_ctx* c, const bolt_params* par, const bolt_grid* grid, int nq, const bolt_recfast* rf,
                     int* cosmo_id) {
  return guard(c, [&] {
    if (!par || !grid || !rf || !cosmo_id) throw Err(-1, "null argument");
    if (!(grid->step > 0) || !(grid->stop > grid->start)) throw Err(-1, "bad x grid");
    CosmoEntry e;
    RecfastOpts ro{rf->Yp, rf->OmegaB, rf->OmegaG, rf->Tnow, rf->tol > 0 ? rf->tol : 1e-8, rf->ionization};
    if (ro.ionization != 0 && ro.ionization != 1) throw Err(-1, "ionization must be 0 (RECFAST) or 1 (Saha-Peebles)");
    build_cosmo_tables(to_h(par), make_grid(grid->start, grid->step, grid->stop), nq, ro, e.T);
    *cosmo_id = add_cosmo(c, std::move(e));
  });
}

int bolt_cosmo_upload(bolt_ctx* c, const bolt_params* par, const bolt_grid* grid, int nq, const double* nodes,
                      const double* scalars, int* cosmo_id) {
  return guard(c, [&] {
    if (!par || !grid || !nodes || !scalars || !cosmo_id) throw Err(-1, "null argument");
    if (nq < 1) throw Err(-1, "nq must be positive");
    CosmoEntry e;
    CosmoTables& T = e.T;
    T.par = to_h(par);
    T.grid = make_grid(grid->start, grid->step, grid->stop);
    T.nq = nq;
    const int n = T.grid.n;
    const int order[8] = {T_H, T_ETA, T_RHO0M, T_XE, T_TAU, T_G, T_TMAT, T_CSB2};
    for (int s = 0; s < 8; ++s) T.nodes[order[s]].assign(nodes + size_t(s) * n, nodes + size_t(s + 1) * n);
    T.H0 = scalars[0];
    T.eta0 = scalars[1];
    T.rho_crit = scalars[2];
    T.Omega_Lambda = 0.0;
    T.z_He_evo_start = T.z_H_He_evo_start = 0.0;
    T.Tnow = 0.0;
    const CosmoParamsH& p = T.par;
    T.Tnu = std::pow(p.N_nu / 3.0, 0.25) * std::pow(4.0 / 11.0, 1.0 / 3.0) *
            std::pow(15.0 / (M_PI * M_PI) * T.rho_crit * p.Omega_r, 0.25);
    T.logqmin = std::log10(T.Tnu / 30.0);
    T.logqmax = std::log10(T.Tnu * 30.0);
    // Gauss-Legendre nodes (FastGaussQuadrature.gausslegendre)
    T.quad_pts.assign(nq, 0.0);
    T.quad_wts.assign(nq, 0.0);
    {
      int half = (nq + 1) / 2;
      for (int i = 0; i < half; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (nq + 0.5)), dp = 1.0;
        for (int it = 0; it < 64; ++it) {
          double p0 = 1.0, p1 = z;
          for (int kk = 2; kk <= nq; ++kk) { double p2 = ((2.0 * kk - 1.0) * z * p1 - (kk - 1.0) * p0) / kk; p0 = p1; p1 = p2; }
          dp = nq * (z * p1 - p0) / (z * z - 1.0);
          double dz = p1 / dp;
          z -= dz;
          if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int kk = 2; kk <= nq; ++kk) { double p2 = ((2.0 * kk - 1.0) * z * p1 - (kk - 1.0) * p0) / kk; p0 = p1; p1 = p2; }
        dp = nq * (z * p1 - p0) / (z * z - 1.0);
        double wt = 2.0 / ((1.0 - z * z) * dp * dp);
        T.quad_pts[nq - 1 - i] = z; T.quad_wts[nq - 1 - i] = wt;
        T.quad_pts[i] = -z; T.quad_wts[i] = wt;
      }
      if (nq % 2 == 1) T.quad_pts[nq / 2] = 0.0;
    }
    finish_uploaded_tables(T);
    *cosmo_id = add_cosmo(c, std::move(e));
  });
}

int bolt_cosmo_info(bolt_ctx* c, int id, double* s) {
  return guard(c, [&] {
    CosmoEntry& e = get_cosmo(c, id);
    const CosmoTables& T = e.T;
    s[0] = T.H0; s[1] = T.eta0; s[2] = T.rho_crit; s[3] = T.Omega_Lambda; s[4] = T.z_He_evo_start;
    s[5] = T.z_H_He_evo_start; s[6] = T.Tnow; s[7] = T.Tnu; s[8] = e.dev.eta_last; s[9] = T.grid.n;
  });
}

int bolt_cosmo_table(bolt_ctx* c, int id, int which, double* out) {
  return guard(c, [&] {
    CosmoEntry& e = get_cosmo(c, id);
    if (which < 0 || which >= T_COUNT) throw Err(-1, "bad table id");
    std::copy(e.T.nodes[which].begin(), e.T.nodes[which].end(), out);
  });
}

int bolt_cosmo_free(bolt_ctx* c, int id) {
  return guard(c, [&] {
    CosmoEntry& e = get_cosmo(c, id);
    ck(cudaStreamSynchronize(c->stream), "sync");
    if (e.d_tab) cudaFree(e.d_tab);
    e = CosmoEntry();
  });
}

int bolt_boltsolve(bolt_ctx* c, int id, const double* k, int nk, const bolt_hier* h, double reltol, double abstol,
                   const double* x_out, int nx, double* u_out, int32_t* status) {
  return guard(c, [&] {
    if (!k || !x_out || !u_out || nx <= 0) throw Err(-1, "null or empty argument");
    CosmoEntry& e = get_cosmo(c, id);
    check_hier(h);
    const GridSpec& g = e.T.grid;
    for (int i = 0; i < nx; ++i) {
      if (!(x_out[i] >= g.at(0)) || !(x_out[i] <= g.at(g.n - 1))) throw Err(-1, "x_out outside the x grid");
      if (i > 0 && !(x_out[i] > x_out[i - 1])) throw Err(-1, "x_out must be strictly ascending");
    }
    const int N = state_len(h);
    double* d_x = c->xout.as<double>(nx);
    double* d_traj = c->traj.as<double>(size_t(nk) * nx * N);
    ck(cudaMemcpyAsync(d_x, x_out, nx * sizeof(double), cudaMemcpyHostToDevice, c->stream), "x_out");
    run_solver(c, id, k, nk, h, reltol, abstol, d_x, nx, MODE_TRAJ, nullptr, nullptr, d_traj, nullptr, status);
    ck(cudaMemcpyAsync(u_out, d_traj, size_t(nk) * nx * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "u_out");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_boltsolve_rsa(bolt_ctx* c, int id, const double* k, int nk, const bolt_hier* h, double reltol, double abstol,
                       double* u_out, int32_t* status) {
  return guard(c, [&] {
    if (!k || !u_out || nk <= 0) throw Err(-1, "null or empty argument");
    CosmoEntry& e = get_cosmo(c, id);
    check_hier(h);
    const CosmoTables& T = e.T;
    const GridSpec& g = T.grid;
    const int n = g.n, N = state_len(h);
    // the switch (perturbations.jl:95-103): first node with k eta > 240,
    // first node with -tau' H / eta > 100 (evaluated on the node values as the
    // reference's broadcasts are), the later of the two; later nodes switch
    int jo = -1;
    std::vector<double> eta(n);
    for (int j = 0; j < n; ++j) {
      const double x = g.at(j);
      eta[j] = spline_eval(T.coef[T_ETA].data(), n, g.x0, g.h, x);
      const double od = -spline_eval(T.coef[T_TAUP].data(), n, g.x0, g.h, x) *
                        spline_eval(T.coef[T_H].data(), n, g.x0, g.h, x) / eta[j];
      if (jo < 0 && od > 100.0) jo = j;
    }
    if (jo < 0) throw Err(-1, "RSA switch undefined: the opacity condition never holds on the x grid");
    std::vector<int> first(nk);
    for (int i = 0; i < nk; ++i) {
      int jh = n - 1;
      for (int j = 0; j < n; ++j)
        if (k[i] * eta[j] > 240.0) { jh = j; break; }
      first[i] = std::max(jh, jo) + 1;
    }
    std::vector<double> xs(n);
    for (int j = 0; j < n; ++j) xs[j] = g.at(j);
    double* d_x = c->xout.as<double>(n);
    double* d_traj = c->traj.as<double>(size_t(nk) * n * N);
    ck(cudaMemcpyAsync(d_x, xs.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "x grid");
    run_solver(c, id, k, nk, h, reltol, abstol, d_x, n, MODE_TRAJ, nullptr, nullptr, d_traj, nullptr, status);
    // the solver's mode array is in decreasing-k order (run_solver)
    std::vector<int> order(nk);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return k[a] > k[b]; });
    std::vector<int> first_sorted(nk);
    for (int r = 0; r < nk; ++r) first_sorted[r] = first[order[r]];
    int* d_first = c->slot_of_l.as<int>(nk);
    ck(cudaMemcpyAsync(d_first, first_sorted.data(), nk * sizeof(int), cudaMemcpyHostToDevice, c->stream), "switch");
    int rc = launch_rsa_post(c->modes.as<ModeDev>(nk), nk, c->d_cos.as<CosmoDev>(c->cos.size()), d_first, n, c->stream);
    if (rc != 0) throw Err(-3, std::string("RSA post-processing: ") + cudaGetErrorString(cudaError_t(rc)));
    ck(cudaMemcpyAsync(u_out, d_traj, size_t(nk) * n * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "u_out");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

// Sources on the x nodes from .. n-1 ([nk][n - from]).  The polarization
// source is emitted only when want_E is set (*d_SE is null otherwise):
// TT-only calls skip its stores and the E half of the projection.
static void source_grid_device(bolt_ctx* c, int id, const double* k, int nk, const bolt_hier* h, double reltol,
                               double abstol, bool want_E, int from, double** d_ST, double** d_SE, int32_t* status) {
  CosmoEntry& e = get_cosmo(c, id);
  const GridSpec& g = e.T.grid;
  const int nout = g.n - from;
  std::vector<double> xs(nout);
  for (int j = 0; j < nout; ++j) xs[j] = g.at(from + j);
  double* d_x = c->xout.as<double>(nout);
  *d_ST = c->srcT.as<double>(size_t(nk) * nout);
  *d_SE = want_E ? c->srcE.as<double>(size_t(nk) * nout) : nullptr;
  ck(cudaMemcpyAsync(d_x, xs.data(), nout * sizeof(double), cudaMemcpyHostToDevice, c->stream), "x grid");
  run_solver(c, id, k, nk, h, reltol, abstol, d_x, nout, MODE_SOURCES, *d_ST, *d_SE, nullptr, nullptr, status);
}

int bolt_source_grid(bolt_ctx* c, int id, const double* k, int nk, const bolt_hier* h, double reltol, double abstol,
                     double* S_T, double* S_E, int32_t* status) {
  return guard(c, [&] {
    if (!k || !S_T) throw Err(-1, "null argument");
    double *d_ST, *d_SE;
    source_grid_device(c, id, k, nk, h, reltol, abstol, S_E != nullptr, 0, &d_ST, &d_SE, status);
    const int n = get_cosmo(c, id).T.grid.n;
    ck(cudaMemcpyAsync(S_T, d_ST, size_t(nk) * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "S_T");
    if (S_E) ck(cudaMemcpyAsync(S_E, d_SE, size_t(nk) * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "S_E");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_cl(bolt_ctx* c, int id, const double* S_T, const double* S_E, const double* k, int nk, const int* ells,
            int nell, double* tt, double* te, double* ee) {
  return guard(c, [&] {
    if (!S_T || !k || !ells) throw Err(-1, "null argument");
    const int n = get_cosmo(c, id).T.grid.n;
    double* d_ST = c->srcT.as<double>(size_t(nk) * n);
    double* d_SE = S_E ? c->srcE.as<double>(size_t(nk) * n) : nullptr;
    ck(cudaMemcpyAsync(d_ST, S_T, size_t(nk) * n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "S_T");
    if (S_E) ck(cudaMemcpyAsync(d_SE, S_E, size_t(nk) * n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "S_E");
    run_los(c, id, d_ST, d_SE, 0, k, nk, ells, nell, tt, te, ee);
  });
}

int bolt_cl_pipeline(bolt_ctx* c, int id, const double* k, int nk, const bolt_hier* h, double reltol, double abstol,
                     const int* ells, int nell, double* tt, double* te, double* ee, int32_t* status) {
  return guard(c, [&] {
    if (!k || !ells) throw Err(-1, "null argument");
    double *d_ST, *d_SE;
    // the projection reads the sources at x > -8 only: the solve emits no
    // others (no dense output below, no landing on the nodes in between)
    const int from = los_first_node(get_cosmo(c, id).T.grid);
    source_grid_device(c, id, k, nk, h, reltol, abstol, te || ee, from, &d_ST, &d_SE, status);
    run_los(c, id, d_ST, d_SE, from, k, nk, ells, nell, tt, te, ee);
  });
}

int bolt_plin(bolt_ctx* c, int id, const double* k, int nk, const bolt_hier* h, double x, double reltol,
              double abstol, double* P, int32_t* status) {
  return guard(c, [&] {
    if (!k || !P) throw Err(-1, "null argument");
    CosmoEntry& e = get_cosmo(c, id);
    const GridSpec& g = e.T.grid;
    if (!(x > g.at(0)) || !(x <= g.at(g.n - 1))) throw Err(-1, "x outside the x grid");
    double* d_x = c->xout.as<double>(1);
    double* d_p = c->plin.as<double>(nk);
    ck(cudaMemcpyAsync(d_x, &x, sizeof(double), cudaMemcpyHostToDevice, c->stream), "x");
    run_solver(c, id, k, nk, h, reltol, abstol, d_x, 1, MODE_PLIN, nullptr, nullptr, nullptr, d_p, status);
    ck(cudaMemcpyAsync(P, d_p, nk * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "P");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_set_dense_x(bolt_ctx* c, double x) {
  if (!c) return -1;
  c->x_dense = x;
  return 0;
}

int bolt_set_land_stride(bolt_ctx* c, int stride) {
  if (!c) return -1;
  if (stride < 0 || stride > 64) return fail(c, -1, "land stride must be in 0..64");
  c->land_stride = stride > 1 ? stride : 1;
  return 0;
}

int bolt_adjoint_check(bolt_ctx* c, int id, double k, const bolt_hier* h, double x, double hstep, double* out) {
  return guard(c, [&] {
    if (!out || !(k > 0.0) || !(hstep > 0.0)) throw Err(-1, "null argument, k <= 0 or hstep <= 0");
    CosmoEntry& e = get_cosmo(c, id);
    check_hier(h);
    const GridSpec& g = e.T.grid;
    if (!(x >= g.at(0)) || !(x + hstep <= g.at(g.n - 1))) throw Err(-1, "step outside the x grid");
    const int N = state_len(h);
    double* d_scr = c->scratch.as<double>(adjoint_check_scratch_bytes(N) / sizeof(double));
    double* d_out = c->out.as<double>(16);
    ck(cudaMemsetAsync(d_out, 0, 16 * sizeof(double), c->stream), "out");
    int rc = launch_adjoint_check(c->d_cos.as<CosmoDev>(c->cos.size()), id, k, h->lg, h->lnu, h->lmnu, h->nq, x,
                                  hstep, d_scr, d_out, c->stream);
    if (rc != 0) throw Err(-3, std::string("adjoint check: ") + cudaGetErrorString(cudaError_t(rc)));
    double o[16];
    ck(cudaMemcpyAsync(o, d_out, 16 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "out");
    ck(cudaStreamSynchronize(c->stream), "sync");
    if (o[15] < 0.0) throw Err(-1, "hierarchy does not fit the solver's lane packing");
    std::copy(o, o + 14, out);
  });
}

}  // extern "C"

// ------------------------------------------- Bessel moments and Filon ---
namespace {

// 8-point Gauss-Legendre nodes and weights (Newton on the Legendre
// recurrence), computed once.
const GL8& gl8() {
  static const GL8 g = [] {
    GL8 r;
    const int n = 8;
    for (int i = 0; i < n; ++i) {
      double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
          double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        double dz = p1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-17) break;
      }
      r.x[n - 1 - i] = z;
      r.w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    return r;
  }();
  return g;
}

MomEntry& get_mtab(bolt_ctx* c, int id) {
  if (id < 0 || id >= int(c->mtab.size()) || !c->mtab[id].live) throw Err(-1, "no such moment table");
  return c->mtab[id];
}

template <class T>
T* upload(bolt_ctx* c, DBuf& b, const T* h, size_t n, const char* what) {
  T* d = b.as<T>(std::max<size_t>(n, 1));
  ck(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, c->stream), what);
  return d;
}

void time_kernels(bolt_ctx* c, int launches) {
  ck(cudaEventRecord(c->ev[1], c->stream), "event");
  ck(cudaEventSynchronize(c->ev[1]), "sync");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
  c->stats[3] += int64_t(ms * 1000.0);
  c->stats[6] += launches;
}

}  // namespace

extern "C" {

int bolt_sph_j_moment(bolt_ctx* c, int nu, double m, const double* x, int nx, double* out) {
  return guard(c, [&] {
    if (!x || !out || nx < 0) throw Err(-1, "null argument or nx < 0");
    if (nu < 0 || nu > 100000 || !(m + nu > -1.0) || !std::isfinite(m)) throw Err(-1, "need 0 <= nu, m + nu > -1");
    for (int i = 0; i < nx; ++i)
      if (!(x[i] >= 0.0) || !std::isfinite(x[i])) throw Err(-1, "x must be finite and >= 0");
    if (nx == 0) return;
    const double* dx = upload(c, c->m0, x, nx, "x");
    double* d_out = c->m1.as<double>(nx);
    ck(cudaEventRecord(c->ev[0], c->stream), "event");
    int rc = launch_moment_direct(nu, m, dx, nx, d_out, gl8(), c->stream);
    if (rc != 0) throw Err(-3, std::string("moment launch: ") + cudaGetErrorString(cudaError_t(rc)));
    time_kernels(c, 1);
    ck(cudaMemcpyAsync(out, d_out, nx * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "out");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_moment_table_build(bolt_ctx* c, int nu, int order, double kmin, double kmax, int N, int* table_id) {
  return guard(c, [&] {
    if (!table_id) throw Err(-1, "null argument");
    *table_id = -1;
    if (nu < 0 || nu > 100000) throw Err(-1, "nu must be in 0..100000");
    if (order < 1 || order > 4) throw Err(-1, "order must be 1..4");
    if (N < 2 || N > (1 << 28)) throw Err(-1, "N must be in 2..2^28");
    if (!(kmin >= 0.0) || !(kmax > kmin) || !std::isfinite(kmax)) throw Err(-1, "need 0 <= kmin < kmax");
    int id = -1;
    for (int i = 0; i < int(c->mtab.size()); ++i)
      if (!c->mtab[i].live) { id = i; break; }
    if (id < 0) { id = int(c->mtab.size()); c->mtab.emplace_back(); }
    MomEntry& e = c->mtab[id];
    MomTabDev& T = e.T;
    T.n = nu;
    T.order = order;
    T.N = N;
    T.kmin = kmin;
    T.kmax = kmax;
    T.h = (kmax - kmin) / (N - 1);
    T.g = gl8();
    T.coef = e.coef.as<double>(size_t(N + 2) * order);
    const double r = 2.0 - std::sqrt(3.0);
    double w[33];
    for (int d = 0; d <= 32; ++d) w[d] = std::sqrt(3.0) * std::pow(-r, d);
    const double* d_w = upload(c, c->m2, w, 33, "weights");
    double* d_y = c->m3.as<double>(size_t(N) * order);
    double* d_seg = c->m4.as<double>(size_t(N) * order);
    double* d_work = c->m5.as<double>(size_t(4) * 70);
    ck(cudaEventRecord(c->ev[0], c->stream), "event");
    int rc = launch_moment_table(T, d_y, d_seg, d_w, d_work, c->stream);
    if (rc != 0) throw Err(-3, std::string("moment table launch: ") + cudaGetErrorString(cudaError_t(rc)));
    time_kernels(c, 4);
    e.live = true;
    *table_id = id;
  });
}

int bolt_moment_table_eval(bolt_ctx* c, int id, const double* x, int nx, double* out) {
  return guard(c, [&] {
    if (!x || !out || nx < 0) throw Err(-1, "null argument or nx < 0");
    MomEntry& e = get_mtab(c, id);
    for (int i = 0; i < nx; ++i)
      if (!(x[i] >= 0.0) || !std::isfinite(x[i])) throw Err(-1, "x must be finite and >= 0");
    if (nx == 0) return;
    const double* dx = upload(c, c->m0, x, nx, "x");
    double* d_out = c->m1.as<double>(size_t(nx) * e.T.order);
    ck(cudaEventRecord(c->ev[0], c->stream), "event");
    int rc = launch_moment_eval(e.T, dx, nx, d_out, c->stream);
    if (rc != 0) throw Err(-3, std::string("moment eval launch: ") + cudaGetErrorString(cudaError_t(rc)));
    time_kernels(c, 1);
    ck(cudaMemcpyAsync(out, d_out, size_t(nx) * e.T.order * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
       "out");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_moment_table_free(bolt_ctx* c, int id) {
  return guard(c, [&] {
    MomEntry& e = get_mtab(c, id);
    ck(cudaStreamSynchronize(c->stream), "sync");
    e.coef.release();
    e.live = false;
  });
}

int bolt_filon(bolt_ctx* c, int id, int n, const double* f, const double* fp, const double* fpp, const double* k,
               const double* a, const double* b, double* out) {
  return guard(c, [&] {
    if (!f || !fp || !fpp || !k || !a || !b || !out || n < 0) throw Err(-1, "null argument or n < 0");
    MomEntry& e = get_mtab(c, id);
    if (e.T.order < 3) throw Err(-1, "the Filon integral needs a table of order >= 3");
    for (int i = 0; i < n; ++i)
      if (!(k[i] > 0.0) || !(a[i] >= 0.0) || !(b[i] >= 0.0) || !std::isfinite(k[i] * a[i]) ||
          !std::isfinite(k[i] * b[i]))
        throw Err(-1, "need k > 0 and finite a, b >= 0");
    if (n == 0) return;
    const double* df = upload(c, c->m0, f, n, "f");
    const double* dfp = upload(c, c->m1, fp, n, "fp");
    const double* dfpp = upload(c, c->m2, fpp, n, "fpp");
    const double* dk = upload(c, c->m3, k, n, "k");
    const double* da = upload(c, c->m4, a, n, "a");
    const double* db = upload(c, c->m5, b, n, "b");
    double* d_out = c->m6.as<double>(n);
    ck(cudaEventRecord(c->ev[0], c->stream), "event");
    int rc = launch_filon(e.T, n, df, dfp, dfpp, dk, da, db, d_out, c->stream);
    if (rc != 0) throw Err(-3, std::string("filon launch: ") + cudaGetErrorString(cudaError_t(rc)));
    time_kernels(c, 1);
    ck(cudaMemcpyAsync(out, d_out, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "out");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_filon_piecewise(bolt_ctx* c, int id, int nt, const double* t, const double* f, const double* fp,
                         const double* fpp, int nk, const double* k, double* out) {
  return guard(c, [&] {
    if (!t || !f || !fp || !fpp || !k || !out || nt < 0 || nk < 0) throw Err(-1, "null argument or negative size");
    MomEntry& e = get_mtab(c, id);
    if (e.T.order < 3) throw Err(-1, "the Filon integral needs a table of order >= 3");
    double kmax = 0.0, tmax = 0.0;
    for (int i = 0; i < nk; ++i) {
      if (!(k[i] > 0.0) || !std::isfinite(k[i])) throw Err(-1, "need finite k > 0");
      kmax = std::max(kmax, k[i]);
    }
    for (int i = 0; i < nt; ++i) {
      if (!(t[i] >= 0.0) || !std::isfinite(t[i])) throw Err(-1, "need finite t >= 0");
      tmax = std::max(tmax, t[i]);
    }
    if (!std::isfinite(kmax * tmax)) throw Err(-1, "k t overflows");
    if (nk == 0) return;
    if (nt < 2) {
      std::fill(out, out + nk, 0.0);
      return;
    }
    const double* dt = upload(c, c->m0, t, nt, "t");
    const double* df = upload(c, c->m1, f, nt, "f");
    const double* dfp = upload(c, c->m2, fp, nt, "fp");
    const double* dfpp = upload(c, c->m3, fpp, nt, "fpp");
    const double* dk = upload(c, c->m4, k, nk, "k");
    double* dD = c->m5.as<double>(size_t(nt) * 4);
    double* d_out = c->m6.as<double>(nk);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    const int nblocks = std::min(nk, std::max(nsm, 1) * 8);
    ck(cudaEventRecord(c->ev[0], c->stream), "event");
    int rc = launch_filon_piecewise(e.T, nt, dt, df, dfp, dfpp, dD, nk, dk, d_out, nblocks, c->stream);
    if (rc != 0) throw Err(-3, std::string("filon launch: ") + cudaGetErrorString(cudaError_t(rc)));
    time_kernels(c, 2);
    ck(cudaMemcpyAsync(out, d_out, nk * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "out");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_filon_batched(bolt_ctx* c, int id, int nt, const double* t, const double* f, const double* fp,
                       const double* fpp, int nk, const double* k, double* out) {
  return guard(c, [&] {
    if (!t || !f || !fp || !fpp || !k || !out || nt < 0 || nk < 0) throw Err(-1, "null argument or negative size");
    MomEntry& e = get_mtab(c, id);
    if (e.T.order < 3) throw Err(-1, "the Filon integral needs a table of order >= 3");
    double kmax = 0.0, tmax = 0.0;
    for (int i = 0; i < nk; ++i) {
      if (!(k[i] > 0.0) || !std::isfinite(k[i])) throw Err(-1, "need finite k > 0");
      kmax = std::max(kmax, k[i]);
    }
    for (int i = 0; i < nt; ++i) {
      if (!(t[i] >= 0.0) || !std::isfinite(t[i])) throw Err(-1, "need finite t >= 0");
      tmax = std::max(tmax, t[i]);
    }
    if (!std::isfinite(kmax * tmax)) throw Err(-1, "k t overflows");
    if (nk == 0) return;
    if (nt < 2) {
      std::fill(out, out + nk, 0.0);
      return;
    }
    const size_t nf = size_t(nk) * nt;
    const double* dt = upload(c, c->m0, t, nt, "t");
    const double* df = upload(c, c->m1, f, nf, "f");
    const double* dfp = upload(c, c->m2, fp, nf, "fp");
    const double* dfpp = upload(c, c->m3, fpp, nf, "fpp");
    const double* dk = upload(c, c->m4, k, nk, "k");
    double* d_out = c->m6.as<double>(nk);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
    const int nblocks = std::min(nk, std::max(nsm, 1) * 8);
    ck(cudaEventRecord(c->ev[0], c->stream), "event");
    int rc = launch_filon_batched(e.T, nt, dt, df, dfp, dfpp, nk, dk, d_out, nblocks, c->stream);
    if (rc != 0) throw Err(-3, std::string("filon launch: ") + cudaGetErrorString(cudaError_t(rc)));
    time_kernels(c, 1);
    ck(cudaMemcpyAsync(out, d_out, nk * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "out");
    ck(cudaStreamSynchronize(c->stream), "sync");
  });
}

int bolt_last_stats(bolt_ctx* c, int64_t* out) {
  if (!c || !out) return -1;
  std::copy(c->stats, c->stats + 8, out);
  return 0;
}

}  // extern "C"

#ifdef BOLT_PHASE_TIMERS
namespace bolt {
int rodas_phase_cycles(unsigned long long* out, bool reset);
}
extern "C" int bolt_debug_phase_cycles(unsigned long long* out, int reset) {
  return bolt::rodas_phase_cycles(out, reset != 0);
}
#endif
