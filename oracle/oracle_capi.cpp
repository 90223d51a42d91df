// Oracle (test infrastructure only): C entry points over the CPU
// restatement, loaded by tests/ and by bench.py's CPU-baseline leg through
// oracle/oracle.py.  Never linked into the product library.
#include <omp.h>

#include <cstdio>
#include <memory>

#include "oracle_bessel.hpp"
#include "oracle_grad.hpp"

using namespace orc;

extern "C" {

struct oracle_params {
  double h, Omega_r, Omega_b, Omega_c, A, n, Y_p, N_nu, Sigma_m_nu;
};

struct OCosmo {
  Cosmo C;
  std::unique_ptr<Background> bg;
  std::unique_ptr<Recfast> rf;
  std::unique_ptr<SahaPeebles> sp;
  std::unique_ptr<Ionization> ih;
};

static Params to_params(const oracle_params* p) {
  Params q;
  q.h = p->h; q.Omega_r = p->Omega_r; q.Omega_b = p->Omega_b; q.Omega_c = p->Omega_c;
  q.A = p->A; q.n = p->n; q.Y_p = p->Y_p; q.N_nu = p->N_nu; q.Sigma_m_nu = p->Sigma_m_nu;
  return q;
}

double oracle_mass_natural() { return units().mass_natural; }
double oracle_km_s_Mpc_100() { return units().km_s_Mpc_100; }

// Background(par; x_grid, nq) + RECFAST(bg; Yp, OmegaB, OmegaG[, Tnow]) +
// IonizationHistory(recfast, par, bg).  Tnow <= 0 derives it from OmegaG.
void* oracle_cosmo_new(const oracle_params* p, double x_start, double x_step, double x_stop, int nq, double Yp,
                       double OmegaB, double OmegaG, double Tnow, double recfast_tol) {
  try {
    OCosmo* o = new OCosmo();
    o->C.par = to_params(p);
    o->bg.reset(new Background(o->C.par, Grid::range(x_start, x_step, x_stop), nq));
    o->rf.reset(new Recfast(o->bg.get(), Yp, OmegaB, OmegaG, Tnow, recfast_tol));
    o->ih.reset(new Ionization(*o->rf, o->C.par, *o->bg));
    o->C.bg = o->bg.get();
    o->C.ih = o->ih.get();
    return o;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_cosmo_new: %s\n", e.what());
    return nullptr;
  }
}

// As oracle_cosmo_new with RECFAST's absolute tolerance set too (tight
// tables for finite-difference gradient checks).
void* oracle_cosmo_new_atol(const oracle_params* p, double x_start, double x_step, double x_stop, int nq, double Yp,
                            double OmegaB, double OmegaG, double Tnow, double recfast_tol, double recfast_atol) {
  try {
    OCosmo* o = new OCosmo();
    o->C.par = to_params(p);
    o->bg.reset(new Background(o->C.par, Grid::range(x_start, x_step, x_stop), nq));
    o->rf.reset(new Recfast(o->bg.get(), Yp, OmegaB, OmegaG, Tnow, recfast_tol));
    o->rf->atol = recfast_atol;
    o->ih.reset(new Ionization(*o->rf, o->C.par, *o->bg));
    o->C.bg = o->bg.get();
    o->C.ih = o->ih.get();
    return o;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_cosmo_new_atol: %s\n", e.what());
    return nullptr;
  }
}

// Background + the Saha-Peebles ionization history (saha_peebles_recombination
// through customion, ionization.jl:83-93, 141-164; T_mat = 2.725 K (1 + z),
// the sound speed by RECFAST's formula with Yp, OmegaB, OmegaG).
void* oracle_cosmo_new_peebles(const oracle_params* p, double x_start, double x_step, double x_stop, int nq,
                               double Yp, double OmegaB, double OmegaG) {
  try {
    OCosmo* o = new OCosmo();
    o->C.par = to_params(p);
    o->bg.reset(new Background(o->C.par, Grid::range(x_start, x_step, x_stop), nq));
    o->rf.reset(new Recfast(o->bg.get(), Yp, OmegaB, OmegaG, -1.0, 1e-8));
    std::vector<double> xs(o->bg->xg.n);
    for (int j = 0; j < o->bg->xg.n; ++j) xs[j] = o->bg->xg.at(j);
    o->sp.reset(new SahaPeebles(o->bg.get(), xs));
    o->ih.reset(new Ionization(*o->sp, *o->rf, o->C.par, *o->bg));
    o->C.bg = o->bg.get();
    o->C.ih = o->ih.get();
    return o;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_cosmo_new_peebles: %s\n", e.what());
    return nullptr;
  }
}

void oracle_cosmo_free(void* h) { delete static_cast<OCosmo*>(h); }

int oracle_cosmo_ngrid(void* h) { return static_cast<OCosmo*>(h)->bg->xg.n; }

void oracle_grid_nodes(void* h, double* out) {
  const Grid& g = static_cast<OCosmo*>(h)->bg->xg;
  for (int j = 0; j < g.n; ++j) out[j] = g.at(j);
}

// H0, eta0, rho_crit, Omega_Lambda, z_He_evo_start, z_H_He_evo_start, tau0, Tnow
void oracle_cosmo_scalars(void* h, double* out) {
  OCosmo* o = static_cast<OCosmo*>(h);
  out[0] = o->bg->H0; out[1] = o->bg->eta0; out[2] = o->bg->rho_crit; out[3] = o->bg->Omega_Lambda;
  out[4] = o->ih->z_He_evo_start; out[5] = o->ih->z_H_He_evo_start; out[6] = o->ih->tau0; out[7] = o->rf->Tnow;
}

static const Spline* table(OCosmo* o, int which) {
  switch (which) {
    case 0: return &o->bg->H;
    case 1: return &o->bg->Hp;
    case 2: return &o->bg->Hpp;
    case 3: return &o->bg->eta;
    case 4: return &o->bg->etap;
    case 5: return &o->bg->etapp;
    case 6: return &o->bg->rho0M;
    case 7: return &o->ih->Xe;
    case 8: return &o->ih->tau;
    case 9: return &o->ih->taup;
    case 10: return &o->ih->taupp;
    case 11: return &o->ih->g;
    case 12: return &o->ih->gp;
    case 13: return &o->ih->gpp;
    case 14: return &o->ih->Tmat;
    case 15: return &o->ih->csb2;
  }
  return nullptr;
}

int oracle_table_eval(void* h, int which, const double* x, int n, double* out) {
  const Spline* s = table(static_cast<OCosmo*>(h), which);
  if (!s) return -1;
  for (int i = 0; i < n; ++i) out[i] = (*s)(x[i]);
  return 0;
}

int oracle_table_coefs(void* h, int which, double* out) {
  const Spline* s = table(static_cast<OCosmo*>(h), which);
  if (!s) return -1;
  for (size_t i = 0; i < s->c.size(); ++i) out[i] = s->c[i];
  return int(s->c.size());
}

// Xe_RECFAST(recfastsolve(RECFAST(bg; ...)), z) at the given redshifts
// (recfast.jl:413-475), as the reference's RECFAST test calls it.
int oracle_recfast_xe(const oracle_params* p, double x_start, double x_step, double x_stop, int nq, double Yp,
                      double OmegaB, double OmegaG, double Tnow, double tol, const double* z, int nz, double* xe) {
  try {
    Params q = to_params(p);
    Background bg(q, Grid::range(x_start, x_step, x_stop), nq);
    Recfast rf(&bg, Yp, OmegaB, OmegaG, Tnow, tol);
    std::vector<double> zs(z, z + nz);
    RecfastHistory rh(&rf, zs);
    for (int i = 0; i < nz; ++i) xe[i] = rh.Xe_RECFAST(z[i]);
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_recfast_xe: %s\n", e.what());
    return -1;
  }
}

void oracle_rhs(void* h, double k, int lg, int lnu, int lmnu, int nq, double x, const double* u, double* du,
                double* dudx) {
  OCosmo* o = static_cast<OCosmo*>(h);
  Mode md(&o->C, k, lg, lnu, lmnu, nq);
  std::vector<D1> d(md.N);
  hierarchy_rhs<D1>(md, D1(x, 1.0), u, d.data());
  for (int i = 0; i < md.N; ++i) { du[i] = d[i].v; if (dudx) dudx[i] = d[i].d; }
}

// Jacobian split J = L + sum_r U_r W_r^T as a dense N x N matrix (row-major).
void oracle_jacobian(void* h, double k, int lg, int lnu, int lmnu, int nq, double x, double* J) {
  OCosmo* o = static_cast<OCosmo*>(h);
  Mode md(&o->C, k, lg, lnu, lmnu, nq);
  JacSplit S;
  jacobian_split(md, x, S);
  int N = md.N;
  std::fill(J, J + size_t(N) * N, 0.0);
  for (auto& e : S.L) J[size_t(e.r) * N + e.c] += e.v;
  for (int r = 0; r < 3; ++r)
    for (int i = 0; i < N; ++i)
      if (S.U[r][i] != 0.0)
        for (int j = 0; j < N; ++j) J[size_t(i) * N + j] += S.U[r][i] * S.W[r][j];
}

void oracle_initial_conditions(void* h, double k, int lg, int lnu, int lmnu, int nq, double* u) {
  OCosmo* o = static_cast<OCosmo*>(h);
  Mode md(&o->C, k, lg, lnu, lmnu, nq);
  initial_conditions(md, o->bg->xg.at(0), u);
}

// boltsolve (perturbations.jl:25-33) sampled at ascending xout: u_out[j*N + i]
// rsa_perts! (perturbations.jl:35-88) applied in place to one state u at x.
void oracle_rsa_perts(void* h, double k, int lg, int lnu, int lmnu, int nq, double x, double* u) {
  OCosmo* o = static_cast<OCosmo*>(h);
  Mode md(&o->C, k, lg, lnu, lmnu, nq);
  const Params& p = o->C.par;
  const Background& bg = *o->bg;
  const Ionization& ih = *o->ih;
  const double H0sq = bg.H0 * bg.H0;
  const double Hc = bg.H(x), tp = ih.taup(x), tpp = ih.taupp(x), cs2 = ih.csb2(x);
  const double a = std::exp(x);
  const double Omega_nu = 7.0 * (2.0 / 3.0) * p.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * p.Omega_r;
  double* Th = u;
  double* Nn = u + md.iN;
  const double* M = u + md.iM;
  double rhoM, sigM;
  rho_sigma(md, a, M, M + 2 * nq, rhoM, sigM);
  const double Phi = u[md.iPhi], del = u[md.iPhi + 1], delb = u[md.iPhi + 3], vb = u[md.iPhi + 4];
  const double Psi = -Phi - 12.0 * H0sq / (k * k) / (a * a) * (p.Omega_r * Th[2] + Omega_nu * Nn[2] + sigM / bg.rho_crit / 4.0);
  const double Phip = Psi - k * k / (3.0 * Hc * Hc) * Phi +
                      H0sq / (2.0 * Hc * Hc) *
                          (p.Omega_c / a * del + p.Omega_b / a * delb + 4.0 * p.Omega_r / (a * a) * Th[0] +
                           4.0 * Omega_nu / (a * a) * Nn[0] + rhoM / (a * a) / bg.rho_crit);
  Th[0] = Phi - Hc / k * tp * vb;
  Th[1] = Hc / k * (-2.0 * Phip + tp * (Phi - cs2 * delb) + Hc / k * (tpp - tp) * vb);
  Th[2] = 0.0;
  Nn[0] = Phi;
  Nn[1] = -2.0 * Hc / k * Phip;
  Nn[2] = 0.0;
  for (int l = 3; l <= lg; ++l) {  // Julia u[l], u[(lg+1)+l] for l = 3..lg (1-based)
    u[l - 1] = 0.0;
    u[(lg + 1) + l - 1] = 0.0;
  }
  for (int l = 3; l <= lnu; ++l) u[2 * (lg + 1) + l - 1] = 0.0;
}

int oracle_boltsolve(void* h, double k, int lg, int lnu, int lmnu, int nq, double reltol, double abstol,
                     const double* xout, int nx, double* u_out, long* stats) {
  OCosmo* o = static_cast<OCosmo*>(h);
  Mode md(&o->C, k, lg, lnu, lmnu, nq);
  std::vector<double> xo(xout, xout + nx);
  int N = md.N;
  SolveStats s = solve_mode(md, reltol, abstol, xo, [&](int j, double, const double* y) {
    std::copy(y, y + N, u_out + size_t(j) * N);
  });
  if (stats) { stats[0] = s.steps; stats[1] = s.rejects; stats[2] = s.rsa; }
  return s.status;
}

// source_grid / source_grid_P (spectra.jl:6-42): S_T and S_E on every x-grid
// node for every k; layout S[ik * nx + ix].
int oracle_source_grid(void* h, const double* kg, int nk, int lg, int lnu, int lmnu, int nq, double reltol,
                       double abstol, double* ST, double* SE, long* steps, int nthreads) {
  OCosmo* o = static_cast<OCosmo*>(h);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return source_grid_of(o->C, kg, nk, lg, lnu, lmnu, nq, reltol, abstol, ST, SE, steps);
}

int oracle_cl_frozen(void* h, const double* ST, const double* SE, const double* kg, int nk, const int* ells, int nell,
                     double kd_min, double kd_max, int nkd, double argmax_in, double* tt, double* te, double* ee,
                     int nthreads);

int oracle_cl(void* h, const double* ST, const double* SE, const double* kg, int nk, const int* ells, int nell,
              double kd_min, double kd_max, int nkd, double* tt, double* te, double* ee, int nthreads) {
  return oracle_cl_frozen(h, ST, SE, kg, nk, ells, nell, kd_min, kd_max, nkd, -1.0, tt, te, ee, nthreads);
}

// quadratic_k (spectra.jl:60-63)
void oracle_quadratic_k(double kmin, double kmax, int nk, double* out) {
  for (int i = 1; i <= nk; ++i) {
    double t = double(i) / double(nk);
    out[i - 1] = kmin + (kmax - kmin) * (t * t);
  }
}

// log10_k (spectra.jl:65-68)
void oracle_log10_k(double kmin, double kmax, int nk, double* out) {
  for (int i = 1; i <= nk; ++i)
    out[i - 1] = std::pow(10.0, std::log10(kmin) + (std::log10(kmax / kmin)) * double(i - 1) / double(nk - 1));
}

void oracle_sph_bessel(int L, double x, double* out) { sph_bessel_all(L, x, out); }

// cltt / clte / clee (spectra.jl:49-160) on a precomputed source grid.
// The dense k grid is quadratic_k(kd_min, kd_max, nkd); the reference uses
// (0.01 H0, 1000 H0, 5000).  Any of tt/te/ee may be null.
// argmax_in > 0 fixes the Bessel grid's upper end (spectra.jl:49-52 with the
// argument held constant, as assume_nondual does under ForwardDiff); <= 0
// takes kd_max * eta0 of this cosmology.
int oracle_cl_frozen(void* h, const double* ST, const double* SE, const double* kg, int nk, const int* ells, int nell,
                     double kd_min, double kd_max, int nkd, double argmax_in, double* tt, double* te, double* ee,
                     int nthreads) {
  OCosmo* o = static_cast<OCosmo*>(h);
  std::vector<double> kd(nkd);
  oracle_quadratic_k(kd_min, kd_max, nkd, kd.data());
  double argmax = argmax_in > 0 ? argmax_in : kd[nkd - 1] * o->bg->eta0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  cl_of(o->C, ST, SE, kg, nk, ells, nell, kd, argmax, tt, te, ee);
  return 0;
}

// plin (spectra.jl:163-198)
double oracle_plin(void* h, double k, int nq, int lg, int lnu, int lmnu, double x, double reltol, double abstol,
                   int* status) {
  OCosmo* o = static_cast<OCosmo*>(h);
  return plin_of(o->C, k, nq, lg, lnu, lmnu, x, reltol, abstol, status);
}

// ------------------------------------------------------- gradient oracle ---
// Background + RECFAST + IonizationHistory with every quantity carrying its
// partial derivatives (G6): the reference's ForwardDiff gradient restated.
struct ODual {
  CosmoT<G6> C;
  std::unique_ptr<BackgroundT<G6>> bg;
  std::unique_ptr<RecfastT<G6>> rf;
  std::unique_ptr<IonizationT<G6>> ih;
};

static void* dual_build(const ParamsT<G6>& par, double x_start, double x_step, double x_stop, int nq,
                        double recfast_tol, double recfast_atol) {
  ODual* o = new ODual();
  o->C.par = par;
  o->bg.reset(new BackgroundT<G6>(o->C.par, Grid::range(x_start, x_step, x_stop), nq));
  o->rf.reset(new RecfastT<G6>(o->bg.get(), par.Y_p, par.Omega_b, par.Omega_r, -1.0, recfast_tol));
  if (recfast_atol > 0) o->rf->atol = recfast_atol;
  o->ih.reset(new IonizationT<G6>(*o->rf, o->C.par, *o->bg));
  o->C.bg = o->bg.get();
  o->C.ih = o->ih.get();
  return o;
}

// theta = (h, omega_b, omega_c, n_s, A_s, Sigma m_nu [eV]), partial j along
// theta_j; Omega_b = omega_b / h^2, Omega_c = omega_c / h^2; Omega_r, Y_p and
// N_nu from `fixed` (constants).  recfast_atol <= 0 keeps RECFAST's default.
void* oracle_dual_cosmo_theta(const double* th, const oracle_params* fixed, double x_start, double x_step,
                              double x_stop, int nq, double recfast_tol, double recfast_atol) {
  try {
    ParamsT<G6> q;
    G6 h = G6::seed(th[0], 0), wb = G6::seed(th[1], 1), wc = G6::seed(th[2], 2);
    q.h = h;
    q.Omega_b = wb / (h * h);
    q.Omega_c = wc / (h * h);
    q.n = G6::seed(th[3], 3);
    q.A = G6::seed(th[4], 4);
    q.Sigma_m_nu = G6::seed(th[5], 5) * units().mass_natural;
    q.Omega_r = fixed->Omega_r;
    q.Y_p = fixed->Y_p;
    q.N_nu = fixed->N_nu;
    return dual_build(q, x_start, x_step, x_stop, nq, recfast_tol, recfast_atol);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_dual_cosmo_theta: %s\n", e.what());
    return nullptr;
  }
}

// As above with the parameters of p and partial 0 along Omega_b alone (the
// reference's bg_fwddiff / ih_fwddiff tests, runtests.jl:54-80).
void* oracle_dual_cosmo_omega_b(const oracle_params* p, double x_start, double x_step, double x_stop, int nq,
                                double recfast_tol) {
  try {
    ParamsT<G6> q;
    q.h = p->h; q.Omega_r = p->Omega_r; q.Omega_c = p->Omega_c; q.A = p->A; q.n = p->n;
    q.Y_p = p->Y_p; q.N_nu = p->N_nu; q.Sigma_m_nu = p->Sigma_m_nu;
    q.Omega_b = G6::seed(p->Omega_b, 0);
    return dual_build(q, x_start, x_step, x_stop, nq, recfast_tol, -1.0);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_dual_cosmo_omega_b: %s\n", e.what());
    return nullptr;
  }
}

void oracle_dual_free(void* h) { delete static_cast<ODual*>(h); }

static void put7(const G6& v, double* out) {
  out[0] = v.v;
  for (int j = 0; j < kThetaN; ++j) out[1 + j] = v.d[j];
}

// Table `which` (as oracle_table_eval) at x: out[i * 7 + 0] the value,
// out[i * 7 + 1 + j] its partial j.
int oracle_dual_table(void* h, int which, const double* x, int n, double* out) {
  ODual* o = static_cast<ODual*>(h);
  const SplineT<G6>* s = nullptr;
  switch (which) {
    case 0: s = &o->bg->H; break;
    case 3: s = &o->bg->eta; break;
    case 6: s = &o->bg->rho0M; break;
    case 7: s = &o->ih->Xe; break;
    case 8: s = &o->ih->tau; break;
    case 9: s = &o->ih->taup; break;
    case 11: s = &o->ih->g; break;
    case 14: s = &o->ih->Tmat; break;
    case 15: s = &o->ih->csb2; break;
    default: return -1;
  }
  for (int i = 0; i < n; ++i) put7((*s)(x[i]), out + 7 * size_t(i));
  return 0;
}

// eta0 and its partials (out[7]).
void oracle_dual_eta0(void* h, double* out) { put7(static_cast<ODual*>(h)->bg->eta0, out); }

// plin(k) at x with its partials (out[7]); returns the solver status.
int oracle_dual_plin(void* h, double k, int nq, int lg, int lnu, int lmnu, double x, double reltol, double abstol,
                     double* out) {
  ODual* o = static_cast<ODual*>(h);
  int st = 0;
  put7(plin_of(o->C, k, nq, lg, lnu, lmnu, x, reltol, abstol, &st), out);
  return st;
}

// cltt (spectra.jl:84-100) with its partials from the source grid on kg
// (frozen), the dense k grid quadratic_k(kd_min, kd_max, nkd) and the Bessel
// grid's upper end argmax (both frozen): out[il * 7 + ...].
int oracle_dual_cltt(void* h, const double* kg, int nk, int lg, int lnu, int lmnu, int nq, double reltol,
                     double abstol, const int* ells, int nell, double kd_min, double kd_max, int nkd, double argmax,
                     double* out, int nthreads) {
  ODual* o = static_cast<ODual*>(h);
  const int nx = o->bg->xg.n;
  std::vector<G6> ST(size_t(nk) * nx), SE(size_t(nk) * nx), tt(nell);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int st = source_grid_of(o->C, kg, nk, lg, lnu, lmnu, nq, reltol, abstol, ST.data(), SE.data(), nullptr);
  std::vector<double> kd(nkd);
  oracle_quadratic_k(kd_min, kd_max, nkd, kd.data());
  cl_of<G6>(o->C, ST.data(), nullptr, kg, nk, ells, nell, kd, argmax, tt.data(), nullptr, nullptr);
  for (int i = 0; i < nell; ++i) put7(tt[i], out + 7 * size_t(i));
  return st;
}

// ------------------------------------------- Bessel moments and Filon ---
// src/bessel/moments.jl, interpolator.jl, integrator.jl.
double oracle_sphj(int n, double t) { return sphj1(n, t); }

// int_0^x t^m j_n(t) dt; method 0 by range, 1 series, 2 large-argument form, 3 quadrature.
double oracle_sphj_moment(int n, double m, double x, int method) { return sphj_moment(n, m, x, method); }

void* oracle_moment_table_new(int n, int order, double kmin, double kmax, int N) {
  if (order < 1 || order > 4 || N < 2 || !(kmax > kmin) || n < 0) return nullptr;
  return new MomentTableO(n, order, kmin, kmax, N);
}
void oracle_moment_table_free(void* h) { delete static_cast<MomentTableO*>(h); }

// out[i * order + m] = I_m(x_i)
void oracle_moment_table_eval(void* h, const double* x, int nx, double* out) {
  const MomentTableO* T = static_cast<MomentTableO*>(h);
  for (int i = 0; i < nx; ++i) T->eval(x[i], out + size_t(i) * T->order);
}

void oracle_filon(void* h, int n, const double* f, const double* fp, const double* fpp, const double* k,
                  const double* a, const double* b, double* out) {
  const MomentTableO* T = static_cast<MomentTableO*>(h);
  for (int i = 0; i < n; ++i) out[i] = filon_segment(*T, f[i], fp[i], fpp[i], k[i], a[i], b[i]);
}

void oracle_filon_piecewise(void* h, int nt, const double* t, const double* f, const double* fp, const double* fpp,
                            int nk, const double* k, double* out, int nthreads) {
  const MomentTableO* T = static_cast<MomentTableO*>(h);
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = 0; i < nk; ++i) out[i] = filon_piecewise(*T, nt, t, f, fp, fpp, k[i]);
}

}  // extern "C"
