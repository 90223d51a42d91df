// Allocation-free source grid: bolt_source_grid_static().
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's memory pool or allocator hooks, hosts that forbid device
// allocation after start-up, or pipelines that hand the library only the
// buffers they own.  For them this entry point runs the same perturbation
// solver as bolt_source_grid(), but every piece of device memory it needs
// beyond the caller's inputs and outputs -- the cosmology's spline tables,
// the per-mode records, the work-queue counter and the solver's per-CTA
// scratch slabs -- lives in one file-scope __device__ array of fixed size
// (kStaticBytes below).  The array exists on every GPU that loads the library
// until the process exits.
//
// Limits (calls beyond them are rejected with a message): state length
// N <= 512, at most 2048 wavenumbers per call, at most 4097 x-grid nodes and
// nq <= 27.
//
// The first call on a device (the current device) looks up the array's
// device address with cudaGetSymbolAddress; make that first call before any
// stream capture.  The address is kept per device for the life of the
// process: after a reset of the device's primary context (cudaDeviceReset)
// the library must be reloaded.  Every call shares the array, so calls whose
// work overlaps on the GPU race with each other; serialise them (one stream,
// or wait for the previous call).  The work-queue counter is cleared at the
// start of every call; everything else in the array is overwritten before
// use.  Each mode stops after 10^5 steps (OrdinaryDiffEq's default maxiters),
// as in bolt_source_grid with default options.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/bolt_gb300.h"
#include "bolt_dev.cuh"
#include "host_cosmo.hpp"

namespace bolt {
int rodas_grid_warps(int nmodes, int maxN, int maxnq, int maxL, int warps_per_block, int* blocks);
int launch_rodas(const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const SolverCfg& cfg, int* d_queue,
                 int maxN, int maxnq, int maxL, int warps_per_block, int blocks, double* d_scratch, cudaStream_t stream);
size_t rodas_scratch_per_warp(int maxN);
}  // namespace bolt

namespace {

using namespace bolt;

constexpr int kMaxN = 512;
constexpr int kMaxModes = 2048;
constexpr int kMaxGrid = 4097;
constexpr int kMaxNq = 27;
constexpr int kMaxCTAs = 320;

// Layout of the static array (byte offsets, each 256-byte aligned).
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kOffCosmo = 0;
constexpr size_t kOffTables = align256(kOffCosmo + sizeof(CosmoDev));
constexpr size_t kTableDoubles = size_t(kMaxGrid + 2) * (4 + C_COUNT) + 2 * kMaxNq;
constexpr size_t kOffModes = align256(kOffTables + kTableDoubles * sizeof(double));
constexpr size_t kOffX = align256(kOffModes + kMaxModes * sizeof(ModeDev));
constexpr size_t kOffCounters = align256(kOffX + kMaxGrid * sizeof(double));
constexpr size_t kOffQueue = align256(kOffCounters + 2 * kMaxModes * sizeof(int64_t));
constexpr size_t kOffSlabs = align256(kOffQueue + 256);
constexpr size_t kSlabDoubles = size_t(10) * kMaxN;  // the solver's per-CTA global scratch
constexpr size_t kStaticBytes = align256(kOffSlabs + kMaxCTAs * kSlabDoubles * sizeof(double));
constexpr long long kMaxSteps = 100000;  // per mode, OrdinaryDiffEq's default maxiters

// The regions hold their largest cases: every table of a 4097-node grid with
// nq = 27 Gauss-Legendre nodes and weights, 2048 mode records and counters,
// and kMaxCTAs solver slabs of 10 N doubles at N = 512 (the kernel's per-CTA
// scratch, checked again against rodas_scratch_per_warp at run time).
static_assert(kOffTables + kTableDoubles * sizeof(double) <= kOffModes, "table region overlaps the mode records");
static_assert(kOffModes + kMaxModes * sizeof(ModeDev) <= kOffX, "mode records overlap the x nodes");
static_assert(kOffX + kMaxGrid * sizeof(double) <= kOffCounters, "x nodes overlap the counters");
static_assert(kOffCounters + 2 * kMaxModes * sizeof(int64_t) <= kOffQueue, "counters overlap the queue");
static_assert(kOffSlabs + size_t(kMaxCTAs) * kSlabDoubles * sizeof(double) <= kStaticBytes, "slabs overrun the array");
static_assert(kOffTables % 256 == 0 && kOffModes % 256 == 0 && kOffSlabs % 256 == 0, "regions are 256-byte aligned");

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// Device address of g_static_scratch, per device (host code must not use the
// symbol itself as a pointer: on the host it names a stand-in object).  Two
// host threads making their first call at once may both look it up; they
// store the same address.
constexpr int kMaxDevices = 64;
std::atomic<unsigned char*> g_addr[kMaxDevices] = {};

int fail(char* errbuf, int errlen, int code, const char* msg) {
  if (errbuf && errlen > 0) std::snprintf(errbuf, errlen, "%s", msg);
  return code;
}

}  // namespace

extern "C" int bolt_source_grid_static(const bolt_params* par, const bolt_grid* grid, int nq, const double* nodes,
                                       const double* scalars, const double* k, int nk, const bolt_hier* hier,
                                       double reltol, double abstol, double* d_S_T, double* d_S_E,
                                       int32_t* d_status, void* stream, char* errbuf, int errlen) {
  if (!par || !grid || !nodes || !scalars || !k || !hier || !d_S_T || !d_S_E || !d_status)
    return fail(errbuf, errlen, -1, "null argument");
  if (!(grid->step > 0) || !(grid->stop > grid->start)) return fail(errbuf, errlen, -1, "bad x grid");
  if (hier->lg < 3 || hier->lnu < 3 || hier->lmnu < 3) return fail(errbuf, errlen, -1, "hierarchy truncations must be >= 3");
  if (nq < 1 || nq > kMaxNq || hier->nq != nq) return fail(errbuf, errlen, -1, "nq must be 1..27 and equal hier->nq");
  const int N = 2 * (hier->lg + 1) + (hier->lnu + 1) + (hier->lmnu + 1) * nq + 5;
  if (N > kMaxN) return fail(errbuf, errlen, -1, "state length exceeds the static limit N <= 512");
  if (nk < 1 || nk > kMaxModes) return fail(errbuf, errlen, -1, "number of wavenumbers must be 1..2048");
  if (!(reltol > 0) || !(abstol > 0)) return fail(errbuf, errlen, -1, "tolerances must be positive");
  for (int i = 0; i < nk; ++i)
    if (!(k[i] > 0) || !std::isfinite(k[i])) return fail(errbuf, errlen, -1, "wavenumbers must be positive and finite");
  GridSpec g = make_grid(grid->start, grid->step, grid->stop);
  if (g.n < 4 || g.n > kMaxGrid) return fail(errbuf, errlen, -1, "x grid must have 4..4097 nodes");

  // set-up, once per device, with that device current
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(errbuf, errlen, -3, "no current CUDA device");
  unsigned char* base = g_addr[dev].load(std::memory_order_acquire);
  if (!base) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) return fail(errbuf, errlen, -3, cudaGetErrorString(e));
    base = static_cast<unsigned char*>(p);
    g_addr[dev].store(base, std::memory_order_release);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // host side: spline tables from the caller's node values (as bolt_cosmo_upload)
  CosmoTables T;
  try {
    T.par = CosmoParamsH{par->h, par->Omega_r, par->Omega_b, par->Omega_c, par->A, par->n, par->Y_p, par->N_nu,
                         par->Sigma_m_nu};
    T.grid = g;
    T.nq = nq;
    const int order[8] = {T_H, T_ETA, T_RHO0M, T_XE, T_TAU, T_G, T_TMAT, T_CSB2};
    for (int s = 0; s < 8; ++s) T.nodes[order[s]].assign(nodes + size_t(s) * g.n, nodes + size_t(s + 1) * g.n);
    T.H0 = scalars[0];
    T.eta0 = scalars[1];
    T.rho_crit = scalars[2];
    const CosmoParamsH& p = T.par;
    T.Tnu = std::pow(p.N_nu / 3.0, 0.25) * std::pow(4.0 / 11.0, 1.0 / 3.0) *
            std::pow(15.0 / (M_PI * M_PI) * T.rho_crit * p.Omega_r, 0.25);
    T.logqmin = std::log10(T.Tnu / 30.0);
    T.logqmax = std::log10(T.Tnu * 30.0);
    gauss_legendre(nq, T.quad_pts, T.quad_wts);
    finish_uploaded_tables(T);
  } catch (const std::exception& ex) {
    return fail(errbuf, errlen, -4, ex.what());
  }
  const int n2 = g.n + 2;
  std::vector<double> tab(size_t(n2) * (4 + C_COUNT) + 2 * nq);
  const int hot_ids[4] = {T_H, T_ETA, T_TAUP, T_CSB2};
  for (int j = 0; j < n2; ++j)
    for (int t = 0; t < 4; ++t) tab[size_t(j) * 4 + t] = T.coef[hot_ids[t]][j];
  const int cold_ids[C_COUNT] = {T_H, T_HP, T_HPP, T_ETA, T_TAU, T_TAUP, T_TAUPP, T_G, T_GP, T_GPP, T_CSB2, T_RHO0M};
  for (int t = 0; t < C_COUNT; ++t)
    std::copy(T.coef[cold_ids[t]].begin(), T.coef[cold_ids[t]].end(), tab.begin() + size_t(n2) * 4 + size_t(t) * n2);
  double* qx_h = tab.data() + size_t(n2) * (4 + C_COUNT);
  std::copy(T.quad_pts.begin(), T.quad_pts.end(), qx_h);
  std::copy(T.quad_wts.begin(), T.quad_wts.end(), qx_h + nq);

  double* d_tab = reinterpret_cast<double*>(base + kOffTables);
  CosmoDev cd;
  std::memset(&cd, 0, sizeof(cd));
  cd.h = T.par.h;
  cd.Omega_r = T.par.Omega_r; cd.Omega_b = T.par.Omega_b; cd.Omega_c = T.par.Omega_c; cd.A = T.par.A;
  cd.n_s = T.par.n; cd.Y_p = T.par.Y_p; cd.N_nu = T.par.N_nu; cd.Sigma_m_nu = T.par.Sigma_m_nu;
  cd.H0 = T.H0; cd.eta0 = T.eta0; cd.rho_crit = T.rho_crit;
  cd.eta_last = spline_eval(T.coef[T_ETA].data(), g.n, g.x0, g.h, g.at(g.n - 1));
  cd.x_last = g.at(g.n - 1);
  cd.Tnu = T.Tnu; cd.logqmin = T.logqmin; cd.logqmax = T.logqmax;
  cd.Omega_nu = 7.0 * (2.0 / 3.0) * T.par.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * T.par.Omega_r;
  cd.x0 = g.x0; cd.hx = g.h; cd.inv_hx = 1.0 / g.h;
  cd.n = g.n; cd.nq = nq;
  cd.hot = d_tab;
  cd.cold = d_tab + size_t(n2) * 4;
  cd.qx = d_tab + size_t(n2) * (4 + C_COUNT);
  cd.qw = cd.qx + nq;

  std::vector<double> xs(g.n);
  for (int j = 0; j < g.n; ++j) xs[j] = g.at(j);
  double* d_x = reinterpret_cast<double*>(base + kOffX);
  int64_t* d_cnt = reinterpret_cast<int64_t*>(base + kOffCounters);
  std::vector<ModeDev> hm(nk);
  std::vector<int> ord(nk);
  for (int i = 0; i < nk; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return k[a] > k[b]; });
  for (int r = 0; r < nk; ++r) {
    int i = ord[r];
    ModeDev& m = hm[r];
    std::memset(&m, 0, sizeof(m));
    m.k = k[i];
    m.cosmo = 0;
    m.lg = hier->lg; m.lnu = hier->lnu; m.lmnu = hier->lmnu; m.nq = nq;
    m.flags = MODE_SOURCES;
    m.nout = g.n;
    m.xout = d_x;
    m.src_T = d_S_T + size_t(i) * g.n;
    m.src_E = d_S_E + size_t(i) * g.n;
    m.status = d_status + i;
    m.counters = d_cnt + 2 * size_t(i);
  }
  cudaError_t e = cudaMemcpyAsync(base + kOffCosmo, &cd, sizeof(cd), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_x, xs.data(), xs.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(base + kOffModes, hm.data(), hm.size() * sizeof(ModeDev), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return fail(errbuf, errlen, -3, cudaGetErrorString(e));

  SolverCfg cfg;
  cfg.reltol = reltol;
  cfg.abstol = abstol;
  cfg.h0 = 1e-3;
  cfg.x_dense = -8.5;
  cfg.max_steps = kMaxSteps;
  cfg.land_stride = 1;
  const int Lmax = hier->lg > hier->lnu ? (hier->lg > hier->lmnu ? hier->lg : hier->lmnu)
                                        : (hier->lnu > hier->lmnu ? hier->lnu : hier->lmnu);
  int blocks = 0;
  int rc = rodas_grid_warps(nk, N, nq, Lmax, 0, &blocks);
  if (rc != 0) return fail(errbuf, errlen, -3, cudaGetErrorString(cudaError_t(-rc)));
  if (blocks > kMaxCTAs) blocks = kMaxCTAs;
  double* slabs = reinterpret_cast<double*>(base + kOffSlabs);
  // the slab stride is the kernel's per-CTA scratch for this N (<= kSlabDoubles)
  if (rodas_scratch_per_warp(N) > kSlabDoubles * sizeof(double))
    return fail(errbuf, errlen, -1, "state length exceeds the static scratch slab");
  rc = launch_rodas(reinterpret_cast<const ModeDev*>(base + kOffModes), nk,
                    reinterpret_cast<const CosmoDev*>(base + kOffCosmo), cfg, reinterpret_cast<int*>(base + kOffQueue),
                    N, nq, Lmax, 0, blocks, slabs, st);
  if (rc != 0) return fail(errbuf, errlen, -3, cudaGetErrorString(cudaError_t(rc)));
  return 0;
}
