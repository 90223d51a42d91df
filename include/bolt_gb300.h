/* C ABI of the GB300 Boltzmann library (libbolt_gb300.so).
 *
 * Drop-in boundary for Bolt.jl's hot path.  Each entry point replaces one
 * reference function; the Julia side binds them with ccall.  Conventions:
 *   - every function returns 0 on success, a negative code on error; the
 *     message is available from bolt_last_error(ctx);
 *   - all arrays are caller-owned host memory (Julia arrays are column
 *     major; the layouts below are given as [slow][fast]);
 *   - a context is not thread safe; use one per host thread.
 *   - per-mode status codes: 0 ok, 1 max iterations, 2 step underflow,
 *     3 non-finite state, 4 singular step matrix, 5 bad input, 6 a replayed
 *     mode ran past its recorded steps; bit 8 (256) is OR-ed in when the
 *     radiation-streaming switch fired, bit 9 (512) when a recorded mode
 *     outgrew its step record (gradient requests).
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
  int ionization; /* 0 = RECFAST (src/ionization/recfast.jl:674-726); 1 = Saha until z = 1587.4, then the
                     Peebles equation (saha_peebles_recombination, src/ionization/ionization.jl:83-93) through
                     customion (ionization.jl:141-164) with T_mat = 2.725 K (1 + z) and RECFAST's sound-speed
                     formula on it; OmegaG, Tnow and tol then apply to that formula only */
} bolt_recfast;

/* Hierarchy truncation (src/perturbations.jl:7-21). */
typedef struct {
  int lg, lnu, lmnu, nq;
} bolt_hier;

typedef struct {
  int device;          /* CUDA device ordinal */
  int warps_per_block; /* warps per k-mode in the solver, 1, 2 or 4 (0 = by launch size: one from
                          about 20 modes per SM, else four) */
  long long max_steps; /* per mode (0 = 10^5, OrdinaryDiffEq's default maxiters) */
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

/* Host-only: the tables of `par` built on the RECFAST discretisation of
 * `base` (its Saha switch redshifts and the accepted steps of its three
 * Tsit5 integrations, replayed without error control), as the engine builds
 * the parameter sets of a gradient.  The tables are then a smooth function
 * of par near base; par == base gives bolt_host_tables' nodes exactly.
 * No counterpart in the reference (its ForwardDiff gradient differentiates
 * through one discretisation in the same way).  nodes[BOLT_T_COUNT][n]. */
int bolt_host_tables_frozen(const bolt_params* base, const bolt_params* par, const bolt_grid* grid, int nq,
                            const bolt_recfast* rf_base, const bolt_recfast* rf, double* nodes, char* errbuf,
                            int errlen);

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

/* boltsolve_rsa (src/perturbations.jl:90-111): boltsolve sampled on every
 * x-grid node, then on the nodes past the radiation-streaming switch (the
 * later of the first node with k eta > 240 and the first node with
 * -tau' H / eta > 100) the photon and massless-neutrino multipoles replaced
 * by rsa_perts! (perturbations.jl:35-88).  u_out[ik][ix][N] on all n_grid
 * nodes; status[nk]. */
int bolt_boltsolve_rsa(bolt_ctx* ctx, int cosmo_id, const double* k, int nk, const bolt_hier* hier,
                       double reltol, double abstol, double* u_out, int32_t* status);

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

/* Fused source_grid + cltt/clte/clee: the source grids stay in HBM.  Any of
 * tt / te / ee may be NULL; with te and ee both NULL the polarization source
 * is neither computed nor projected. */
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

/* Source grids at x >= x_dense: the integrator lands on every stride-th node
 * (and the last) and takes the others from the same cubic Hermite dense
 * output (0 or 1, the default: lands on every node; at most 64).  The
 * reference samples its integrator's interpolant at every node
 * (src/spectra.jl:6-42); stride 2 moves C_l by below 1e-5 relative at the
 * served tolerances (the engine's land_stride is the same option). */
int bolt_set_land_stride(bolt_ctx* ctx, int stride);

/* Self-check of the discrete adjoint's building blocks (no counterpart in
 * the reference; the test suite's probe of the reverse sweep's pieces) on
 * one mode of cosmology id, wavenumber k and hierarchy h, at the Rosenbrock
 * step from x of size hstep, with pseudo-random vectors u, lam, du:
 *   [0..4] |lam.(A u) - (A^T lam).u| / sum |lam_i (A u)_i| at the five
 *          stage abscissae (A: hierarchy!'s linear map, src/perturbations.jl:196-270;
 *          A^T: its column form);
 *   [5]    the same for dA/dx;
 *   [6]    max |M^T z - lam| / max |lam| for z from the transposed solve
 *          (M = I/(h gamma) - A, the step matrix);
 *   [7]    max |M x - u| / max |u| for x from the forward solve;
 *   [8]    source_function (src/perturbations.jl:343-389) against its
 *          gradient: |S_T(u, du) - (g_u.u + g_du.du)| / sum of the terms;
 *   [9]    plin (src/spectra.jl:163-198) against its gradient: relative error
 *          of a central difference (exact for the quadratic P_lin);
 *   [10]   1 if the radiation-streaming switch is on at x, else 0;
 *   [11]   |lam.(M^-1 u) - (M^-T lam).u| / sum |lam_i (M^-1 u)_i|: the two
 *          solves are each other's transposes;
 *   [12]   the parameter cotangent lam.(dA/dtheta u) from the coefficients'
 *          cotangents against tangent-number arithmetic, on pseudo-random
 *          coefficient tangents (largest relative difference);
 *   [13]   the same for lam.(d(dA/dx)/dtheta u).
 * (14 doubles.)  Returns 0 or a negative code. */
int bolt_adjoint_check(bolt_ctx* ctx, int id, double k, const bolt_hier* h, double x, double hstep, double* out);

/* ---------------------------------------------------------------------
 * Moments of spherical Bessel functions and the Filon-type integrator
 * (src/bessel/).  I_m(x) = int_0^x t^m j_nu(t) dt.
 * --------------------------------------------------------------------- */

/* sph_j_moment_maclaurin_1F2 / sph_j_moment_asymp / sph_j_moment_weniger_1F2
 * (src/bessel/moments.jl:56-92; each returns I_m(x), by its own method):
 * out[i] = I_m(x[i]) for integer 0 <= nu <= 100000, real m with m + nu > -1,
 * x[i] >= 0, evaluated on the device (series below x = 2, quadrature up to
 * max(50, 4 nu), the Lommel-function form above).  J_moment_* of
 * half-integer order nu + 1/2 and power alpha is sqrt(2/pi) times this
 * with m = alpha + 1/2. */
int bolt_sph_j_moment(bolt_ctx* ctx, int nu, double m, const double* x, int nx, double* out);

/* sph_bessel_interpolator(nu, order, kmin, kmax, N)
 * (src/bessel/interpolator.jl:81-94): the moments m = 0..order-1
 * (order 1..4) on N uniform nodes of [kmin, kmax] (0 <= kmin < kmax,
 * 2 <= N <= 2^28), one cubic B-spline per order (Cubic(Line(OnGrid()))),
 * built and kept on the device; *table_id names the table in this
 * context. */
int bolt_moment_table_build(bolt_ctx* ctx, int nu, int order, double kmin, double kmax, int N, int* table_id);

/* The table's call (src/bessel/interpolator.jl:67-75): out[i][m] = I_m(x[i])
 * from the splines inside [kmin, kmax], the Lommel form above, the
 * Maclaurin series below.  out[nx][order]. */
int bolt_moment_table_eval(bolt_ctx* ctx, int table_id, const double* x, int nx, double* out);
int bolt_moment_table_free(bolt_ctx* ctx, int table_id);

/* integrate_sph_bessel_filon(f, f', f'', k, a, b, itp)
 * (src/bessel/integrator.jl:7-19), n independent segments:
 * out[i] = int_{a_i}^{b_i} p_i(t) j_nu(k_i t) dt, p_i the quadratic with
 * p(a_i) = f_i, p'(a_i) = fp_i, p'' = fpp_i.  Table order >= 3; k > 0,
 * a, b >= 0. */
int bolt_filon(bolt_ctx* ctx, int table_id, int n, const double* f, const double* fp, const double* fpp,
               const double* k, const double* a, const double* b, double* out);

/* The piecewise integrator that _loop_integrate_sph_bessel_filon
 * (src/bessel/integrator.jl:25-38) serves: for every k,
 * out[ik] = sum_{i < nt-1} int_{t_i}^{t_{i+1}} p_i(t) j_nu(k t) dt with the
 * quadratic p_i at t_i (f, fp, fpp sampled on the nodes t[nt] >= 0), each
 * node's moments evaluated once.  Device time in bolt_last_stats [3]. */
int bolt_filon_piecewise(bolt_ctx* ctx, int table_id, int nt, const double* t, const double* f, const double* fp,
                         const double* fpp, int nk, const double* k, double* out);

/* The line-of-sight shape: one integrand per k on shared nodes t[nt],
 * f, fp, fpp [nk][nt]; out[ik] = sum_{i < nt-1} int_{t_i}^{t_{i+1}}
 * p_{ik,i}(t) j_nu(k_ik t) dt (Tl's sum over x with j_nu taken exactly
 * through the moments and the integrand quadratic per segment). */
int bolt_filon_batched(bolt_ctx* ctx, int table_id, int nt, const double* t, const double* f, const double* fp,
                       const double* fpp, int nk, const double* k, double* out);

/* Counters of the last call: [0] accepted steps, [1] rejected steps,
 * [2] solver kernel microseconds, [3] LOS kernels microseconds (the
 * Bessel-moment and Filon calls: their kernels' microseconds),
 * [4] modes, [5] solver kernel launches, [6] total kernel launches,
 * [7] (l, k, x) terms the line-of-sight reduction evaluated (those below
 * the Bessel turning point are skipped).  out[8]. */
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

/* ------------------------------------------------------------------------
 * Batched and served requests (the serving side of plin / cltt / clte /
 * clee, with gradients for the rrule of the Julia binding).
 *
 * A request is one cosmology with its own k grid, hierarchy, tolerances and
 * outputs: P_lin(k) at x (plin, spectra.jl:163-198) or C_l^TT/TE/EE for its
 * multipoles (source_grid + cltt/clte/clee, spectra.jl:6-160; source grid
 * on the request's k grid, dense k grid quadratic_k(0.01 H0, 1000 H0, 5000)).
 * Background and RECFAST are built on the host (worker threads) from the
 * parameters (RECFAST's Yp/OmegaB/OmegaG from the parameters, tol 1e-8).
 *
 * Gradients (grad = 1) are with respect to
 *   theta = (h, omega_b = Omega_b h^2, omega_c = Omega_c h^2, n, A, Sigma m_nu [eV])
 * with Omega_r, Y_p and N_nu held fixed: d/dtheta of the discrete pipeline
 * by forward differences (relative step 1e-6, accurate to ~1e-6) with every
 * discretisation choice frozen -- the perturbed modes replay the accepted
 * steps of the unperturbed solve, RECFAST replays its steps, switch
 * redshifts and right-hand-side branches, and the k grids and the Bessel
 * grid stay those of the unperturbed cosmology (the reference's
 * assume_nondual points, spectra.jl:46-66, recfast.jl:451-456).  Layout
 * d*[6][n].
 *
 * Output arrays are caller-owned host memory that must stay valid (and
 * untouched) until the request has completed.
 * ---------------------------------------------------------------------- */
enum { BOLT_REQ_PLIN = 1, BOLT_REQ_CL = 2 };
enum { BOLT_CL_TT = 1, BOLT_CL_TE = 2, BOLT_CL_EE = 4 };

typedef struct {
  int kind;              /* BOLT_REQ_PLIN or BOLT_REQ_CL */
  int grad;              /* 1: also the Jacobian with respect to theta */
  bolt_params par;
  bolt_grid grid;        /* Background x grid (e.g. -20:0.01:0) */
  int nq;                /* massive-neutrino momentum bins (Background nq) */
  bolt_hier hier;        /* hier.nq must equal nq */
  double reltol, abstol;
  const double* k;       /* [nk] ascending wavenumbers, Mpc^-1 (copied at submit) */
  int nk;
  double plin_x;         /* BOLT_REQ_PLIN: x at which P_lin is evaluated */
  const int* ells;       /* BOLT_REQ_CL: [nell] multipoles (copied at submit) */
  int nell;
  int cl_want;           /* BOLT_CL_* bits */
  /* outputs */
  double* plin;          /* [nk]: BOLT_REQ_PLIN, P_lin at plin_x; BOLT_REQ_CL, optional (NULL = none),
                            P_lin at the end of the x grid from the source-grid solve (same modes) */
  double* dplin;         /* [6][nk] (grad) */
  double *tt, *te, *ee;  /* [nell] each, per cl_want */
  double *dtt, *dte, *dee; /* [6][nell] each (grad), per cl_want */
  int32_t* status;       /* [nk] status of the unperturbed modes, or NULL */
} bolt_request;

typedef struct {
  int device;
  int lanes;             /* batches in flight on separate streams (0 = 6; at most 8) */
  int host_threads;      /* table-building threads (0 = hardware threads) */
  int max_batch;         /* requests per batch (0 = unlimited; 1 = one request per batch) */
  double mem_budget_gb;  /* device memory admitted to in-flight requests (0 = 150) */
  int warps_per_mode;    /* 0 = autotuned per launch (see objective), else 1, 2 or 4 */
  long long max_steps;   /* per mode (0 = 10^5, OrdinaryDiffEq's default maxiters) */
  double batch_window_s; /* > 0: while another batch runs, hold ready requests up to this long
                            until they fill the GPU (24 modes per SM); 0 = launch at once */
  int objective;         /* autotuner: 0 = latency-aware (a launch onto an idle GPU with nothing
                            waiting gets the variant fastest for that launch alone), 1 = throughput
                            (every launch is costed as part of a full GPU) */
  int land_stride;       /* source grids: the solver lands on every land_stride-th x node at x >= -8.5
                            (and the last) and takes the others from cubic Hermite dense output, as it
                            does below -8.5 (0 or 1 = lands on every node there; at most 64) */
  int grad_scheme;       /* derivatives of P_lin and C_l^TT: 0 = forward differences of four frozen-step
                            replays (the default: the fastest measured); 1 = the tangent-linear solver
                            (one solve carries the state and its derivatives along h, omega_b, omega_c
                            and Sigma m_nu, sharing each step's factorisation); 2 = as 0 for Jacobian
                            requests, and bolt_cl_vjp (C_l^TT cotangents only) / bolt_plin_vjp by the
                            discrete adjoint (a checkpointed reverse sweep of the solve and of the line
                            of sight); C_l requests with TE or EE Jacobians always replay */
} bolt_engine_cfg;

typedef struct bolt_engine bolt_engine;

/* Creates an engine bound to one GPU: a scheduler thread forms batches from
 * the requests whose tables are ready (admitted while the in-flight device
 * footprint stays within the budget), runs every k-mode of a batch in one
 * persistent solver launch (a CUDA graph whose kernel node is updated per
 * batch; warps per mode autotuned by the load), then the line-of-sight
 * projections, on one of `lanes` streams, so a batch starts while earlier
 * ones are still on the GPU. */
int bolt_engine_create(const bolt_engine_cfg* cfg, bolt_engine** out);
void bolt_engine_destroy(bolt_engine* eng);
const char* bolt_engine_last_error(const bolt_engine* eng);

/* Queues a request (validated and copied; outputs written on completion).
 * Returns 0 and a ticket, or a negative code (message in last_error). */
int bolt_engine_submit(bolt_engine* eng, const bolt_request* req, int64_t* ticket);

/* Waits up to timeout_s (< 0: forever) for a ticket.  Returns 1 when done
 * (the ticket is then released; rc_out = 0 or the request's negative error
 * code, message in errbuf), 0 on timeout, negative on an unknown ticket.
 * times_out (optional, 5 doubles): seconds since engine creation [0]
 * submitted, [1] tables ready, [2] batch launched, [3] completed; [4] the
 * request's Rodas4 steps (accepted + rejected, every parameter set). */
int bolt_engine_wait(bolt_engine* eng, int64_t ticket, double timeout_s, int* rc_out, double* times_out,
                     char* errbuf, int errlen);

/* One request, alone: submit + wait (the one-request-per-call path). */
int bolt_request_run(bolt_engine* eng, const bolt_request* req, char* errbuf, int errlen);

/* Reverse-mode products, the pullback of an rrule over cltt / clte / clee
 * (src/spectra.jl:132-160) and plin (src/spectra.jl:163-198): the request runs
 * alone with its Jacobian (req->grad is taken as 1; its d* pointers are
 * ignored, the Jacobian stays in library memory) and
 *   bolt_cl_vjp:   grad[j] = sum over the spectra X in req->cl_want of
 *                  sum_l ybar_X[l] dC_l^X/dtheta_j  (ybar_X [nell]; NULL = 0)
 *   bolt_plin_vjp: grad[j] = sum_k ybar[k] dP_lin(k)/dtheta_j  (ybar [nk])
 * for theta = (h, omega_b, omega_c, n_s, A_s, Sigma m_nu [eV]), grad[6].  The
 * primal outputs named in req are written too (NULL ones are not).  Returns
 * 0 or a negative code with the message in errbuf. */
int bolt_cl_vjp(bolt_engine* eng, const bolt_request* req, const double* ybar_tt, const double* ybar_te,
                const double* ybar_ee, double* grad, char* errbuf, int errlen);
int bolt_plin_vjp(bolt_engine* eng, const bolt_request* req, const double* ybar, double* grad, char* errbuf,
                  int errlen);

/* Engine counters: [0] batches, [1] requests completed, [2] modes solved,
 * [3] solver microseconds (sum over batches), [4] LOS microseconds,
 * [5] accepted + rejected steps, [6] kernel launches, [7] graph launches,
 * [8..10] batches run with 1 / 2 / 4 warps per mode, [11] the largest
 * device footprint of the batches in flight at once (bytes).  out[12]. */
int bolt_engine_stats(bolt_engine* eng, int64_t* out);

#ifdef __cplusplus
}
#endif
#endif /* BOLT_GB300_H */
