/* C ABI of the GB300 Boltzmann library (libbolt_gb300.so).
 *
 * Drop-in boundary for Bolt.jl's hot path.  Each entry point replaces one
 * reference function; the Julia side binds them with ccall (see
 * INTEGRATION.md).  Conventions:
 *   - every function returns 0 on success, a negative code on error; the
 *     message is available from bolt_last_error(ctx);
 *   - all arrays are caller-owned host memory (Julia arrays are column
 *     major; the layouts below are given as [slow][fast]);
 *   - a context is not thread safe; use one per host thread.
 *   - per-mode status codes: 0 ok, 1 max iterations, 2 step underflow,
 *     3 non-finite state, 4 singular step matrix, 5 bad input; bit 8 (256)
 *     is OR-ed in when the radiation-streaming switch fired.
 */
#ifndef BOLT_GB300_H
#define BOLT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bolt_ctx bolt_ctx;

/* CosmoParams (src/Bolt.jl:56-66).  Sigma_m_nu in Mpc^-1 as in the
 * reference (eV * bolt_mass_natural()). */
typedef struct {
  double h, Omega_r, Omega_b, Omega_c, A, n, Y_p, N_nu, Sigma_m_nu;
} bolt_params;

/* Uniform x = ln(a) grid, Background(par; x_grid = start:step:stop). */
typedef struct {
  double start, step, stop;
} bolt_grid;

/* RECFAST(bg; Yp, OmegaB, OmegaG, Tnow, tol) (src/ionization/recfast.jl:22-121).
 * Tnow <= 0 derives the CMB temperature from OmegaG (recfast.jl:108). */
typedef struct {
  double Yp, OmegaB, OmegaG, Tnow, tol;
} bolt_recfast;

/* Hierarchy truncation (src/perturbations.jl:7-21). */
typedef struct {
  int lg, lnu, lmnu, nq;
} bolt_hier;

typedef struct {
  int device;          /* CUDA device ordinal */
  int warps_per_block; /* solver CTA size in warps (0 = autotune) */
  long long max_steps; /* per mode (0 = 10^7) */
} bolt_opts;

/* Table slots for bolt_cosmo_table (nodes on the x grid). */
enum {
  BOLT_T_H = 0, BOLT_T_HP, BOLT_T_HPP, BOLT_T_ETA, BOLT_T_ETAP, BOLT_T_ETAPP, BOLT_T_RHO0M,
  BOLT_T_XE, BOLT_T_TAU, BOLT_T_TAUP, BOLT_T_TAUPP, BOLT_T_G, BOLT_T_GP, BOLT_T_GPP,
  BOLT_T_TMAT, BOLT_T_CSB2, BOLT_T_COUNT
};

int bolt_version(void);
double bolt_mass_natural(void);   /* 1 eV in Mpc^-1 (src/Bolt.jl:51) */
double bolt_km_s_Mpc_100(void);   /* 100 km/s/Mpc in Mpc^-1 (src/Bolt.jl:49) */

/* Host-only table construction (no GPU needed): Background + RECFAST
 * IonizationHistory node values nodes[BOLT_T_COUNT][n_grid] and
 * scalars[10] as in bolt_cosmo_info.  n_grid = round((stop-start)/step)+1. */
int bolt_host_tables(const bolt_params* par, const bolt_grid* grid, int nq, const bolt_recfast* rf,
                     double* nodes, double* scalars, char* errbuf, int errlen);

/* Creates a context bound to one GPU. */
int bolt_ctx_create(const bolt_opts* opts, bolt_ctx** out);
void bolt_ctx_destroy(bolt_ctx* ctx);
const char* bolt_last_error(const bolt_ctx* ctx);

/* Background(par; x_grid, nq) (src/background.jl:104-128) followed by
 * IonizationHistory(RECFAST(bg; ...), par, bg) (src/ionization/recfast.jl:674-726),
 * built on the host and made resident in HBM.  Returns a cosmology id. */
int bolt_cosmo_build(bolt_ctx* ctx, const bolt_params* par, const bolt_grid* grid, int nq,
                     const bolt_recfast* rf, int* cosmo_id);

/* Drop-in variant: the caller (Julia) passes the node values of its own
 * Background / IonizationHistory splines on the grid: nodes[8][n] in the
 * order H, eta, rho0M, Xe, tau, g, Tmat, csb2, plus scalars[3] = H0, eta0,
 * rho_crit.  The re-splined derivative tables are rebuilt the reference way
 * (util.jl:12-13). */
int bolt_cosmo_upload(bolt_ctx* ctx, const bolt_params* par, const bolt_grid* grid, int nq,
                      const double* nodes, const double* scalars, int* cosmo_id);

/* scalars[10] = H0, eta0, rho_crit, Omega_Lambda, z_He_evo_start,
 * z_H_He_evo_start, Tnow, Tnu, eta_last, n_grid */
int bolt_cosmo_info(bolt_ctx* ctx, int cosmo_id, double* scalars);
/* Node values of one table (BOLT_T_*), n_grid doubles. */
int bolt_cosmo_table(bolt_ctx* ctx, int cosmo_id, int which, double* out);
int bolt_cosmo_free(bolt_ctx* ctx, int cosmo_id);

/* boltsolve (src/perturbations.jl:25-33) for nk modes, sampled at the
 * ascending x_out (x_out[0] >= first grid node, x_out[nx-1] <= last).
 * u_out[ik][ix][N], N = 2(lg+1)+(lnu+1)+(lmnu+1)nq+5 in the reference's
 * unpack order (perturbations.jl:114-125).  status[nk]. */
int bolt_boltsolve(bolt_ctx* ctx, int cosmo_id, const double* k, int nk, const bolt_hier* hier,
                   double reltol, double abstol, const double* x_out, int nx, double* u_out,
                   int32_t* status);

/* source_grid + source_grid_P (src/spectra.jl:6-42): S_T[ik][ix] and
 * S_E[ik][ix] on every x-grid node (S_E may be NULL). */
int bolt_source_grid(bolt_ctx* ctx, int cosmo_id, const double* k, int nk, const bolt_hier* hier,
                     double reltol, double abstol, double* S_T, double* S_E, int32_t* status);

/* cltt / clte / clee (src/spectra.jl:84-160) for the l in ells, from a source
 * grid on the k grid k[nk].  The dense k grid is quadratic_k(0.01 H0,
 * 1000 H0, 5000) as in spectra.jl:133.  Any of tt / te / ee may be NULL;
 * te and ee need S_E. */
int bolt_cl(bolt_ctx* ctx, int cosmo_id, const double* S_T, const double* S_E, const double* k, int nk,
            const int* ells, int nell, double* tt, double* te, double* ee);

/* Fused source_grid + cltt/clte/clee: the source grids stay in HBM. */
int bolt_cl_pipeline(bolt_ctx* ctx, int cosmo_id, const double* k, int nk, const bolt_hier* hier,
                     double reltol, double abstol, const int* ells, int nell, double* tt, double* te,
                     double* ee, int32_t* status);

/* plin (src/spectra.jl:163-198) for nk wavenumbers, evaluated at x. */
int bolt_plin(bolt_ctx* ctx, int cosmo_id, const double* k, int nk, const bolt_hier* hier, double x,
              double reltol, double abstol, double* P, int32_t* status);

/* Source-grid nodes with x below x_dense (default -8.5, before
 * recombination; the line-of-sight integral starts at x > -8) are produced by
 * cubic Hermite dense output between accepted steps instead of landing the
 * integrator on every node.  Pass -INFINITY to land on every node. */
int bolt_set_dense_x(bolt_ctx* ctx, double x_dense);

/* Counters of the last call: [0] accepted steps, [1] rejected steps,
 * [2] solver kernel microseconds, [3] LOS kernels microseconds,
 * [4] modes, [5] solver kernel launches, [6] total kernel launches. */
int bolt_last_stats(bolt_ctx* ctx, int64_t* out);

/* Allocation-free source grid (no counterpart in the reference; added for
 * callers that cannot allocate device memory themselves, e.g. code running
 * under another framework's allocator or a host that forbids cudaMalloc after
 * start-up).  Same solver as bolt_source_grid, no context: inputs are host
 * arrays (parameters, the grid, nodes[8][n] and scalars[3] as for
 * bolt_cosmo_upload, k[nk]); outputs are caller-owned DEVICE buffers
 * d_S_T[nk][n], d_S_E[nk][n], d_status[nk], written asynchronously on
 * `stream` (a cudaStream_t, NULL = legacy default stream).  All other device
 * memory comes from one fixed, file-scope device array (~14 MB, held by every
 * GPU that loads the library until exit): N <= 512, nk <= 2048, n <= 4097,
 * nq <= 27; larger calls are rejected with an error.  No cudaMalloc or cudaFree
 * is called.  The first call on a device looks up the array's address (make
 * it before any stream capture); calls that overlap on the GPU share the
 * array and race, so serialise them.  Returns 0, or a negative code with the
 * message in errbuf. */
int bolt_source_grid_static(const bolt_params* par, const bolt_grid* grid, int nq, const double* nodes,
                            const double* scalars, const double* k, int nk, const bolt_hier* hier, double reltol,
                            double abstol, double* d_S_T, double* d_S_E, int32_t* d_status, void* stream,
                            char* errbuf, int errlen);

/* Measured FP64 FMA throughput of the device (TFLOP/s): the roofline
 * denominator for the FP64-pipe-bound kernels. */
int bolt_fp64_peak(int device, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* BOLT_GB300_H */
