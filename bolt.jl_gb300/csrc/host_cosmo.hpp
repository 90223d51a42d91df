// Host-side construction of the per-cosmology background and ionization
// tables that the device kernels read.  This is the GB300 library's own
// implementation of Bolt.jl's Background (src/background.jl:104-128) and
// IonizationHistory(RECFAST) (src/ionization/recfast.jl:446-536, 674-726;
// src/ionization/ionization.jl:105-137); the Julia drop-in can instead hand
// the node values of its own splines to bolt_cosmo_upload().
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace bolt {

// Table slots, all sampled on the uniform x grid and stored as cubic
// B-spline coefficients with Interpolations.jl's Cubic(Line(OnGrid()))
// boundary rows (vanishing second derivative at both ends).
enum TableId {
  T_H = 0,    // conformal Hubble rate (bg.ℋ)
  T_HP,       // bg.ℋ′  (re-splined gradient)
  T_HPP,      // bg.ℋ′′ (re-splined Hessian)
  T_ETA,      // conformal time bg.η
  T_ETAP,     // bg.η′
  T_ETAPP,    // bg.η′′
  T_RHO0M,    // massive-neutrino background density bg.ρ₀ℳ
  T_XE,       // ih.Xₑ
  T_TAU,      // ih.τ
  T_TAUP,     // ih.τ′
  T_TAUPP,    // ih.τ′′
  T_G,        // visibility ih.g̃
  T_GP,       // ih.g̃′
  T_GPP,      // ih.g̃′′
  T_TMAT,     // ih.Tmat
  T_CSB2,     // baryon sound speed squared ih.csb²
  T_COUNT
};

struct CosmoParamsH {
  double h, Omega_r, Omega_b, Omega_c, A, n, Y_p, N_nu, Sigma_m_nu;  // Sigma_m_nu in Mpc^-1
};

struct RecfastOpts {
  double Yp, OmegaB, OmegaG;
  double Tnow;  // <= 0: derived from OmegaG and the background
  double tol;
  // 0: RECFAST (recfast.jl:446-536, 674-726); 1: Saha until z = 1587.4, then
  // the Peebles equation (ionization.jl:1-93, saha_peebles_recombination),
  // with T_mat = 2.725 K (1 + z) and the RECFAST path's sound speed formula
  // on it (customion, ionization.jl:141-164, takes both from its caller)
  int ionization = 0;
};

struct GridSpec {
  int n;
  double x0, h;
  long i0, M;  // x_j = (i0 + j) / M when M > 0 (Julia's correctly rounded range)
  double at(int j) const { return M > 0 ? double(i0 + j) / double(M) : x0 + j * h; }
};

GridSpec make_grid(double start, double step, double stop);

struct CosmoTables {
  CosmoParamsH par;
  GridSpec grid;
  int nq;
  double H0, eta0, rho_crit, Omega_Lambda, Tnu, logqmin, logqmax;
  double z_He_evo_start, z_H_He_evo_start, Tnow;
  std::vector<double> quad_pts, quad_wts;
  std::vector<double> nodes[T_COUNT];  // values at grid nodes
  std::vector<double> coef[T_COUNT];   // n + 2 B-spline coefficients
};

// Natural cubic B-spline prefilter (c has n + 2 entries).
void spline_coefs(const double* y, int n, double* c);
double spline_eval(const double* c, int n, double x0, double h, double x);
double spline_deriv(const double* c, int n, double x0, double h, double x);
double spline_deriv2(const double* c, int n, double x0, double h, double x);

// Unit conversions (Bolt.jl:43-51).
double units_km_s_Mpc_100();
double units_mass_eV();

// The discretisation choices of one RECFAST run: the two Saha switch
// redshifts (root finds), the accepted abscissae and step sizes of its three
// Tsit5 integrations, and the sides of the right-hand side's state-dependent
// switches at every stage of the accepted steps.  Replaying them makes the tables a smooth function of the
// parameters, for derivatives by central differences; the switch redshifts
// are held fixed as the reference's ForwardDiff gradient does
// (recfast.jl:451-456, assume_nondual).
struct RecfastFreeze {
  bool have = false;
  double zHe = 0.0, zHH = 0.0;
  std::vector<double> tHe, tHHe, tRe;  // accepted abscissae
  std::vector<double> hHe, hHHe, hRe;  // accepted step sizes
  std::vector<uint8_t> bHe, bHHe;      // sides of the right-hand side's switches taken
};

// Builds Background + RECFAST + IonizationHistory.  Throws std::runtime_error.
// freeze: null, or recorded into when empty, or replayed when filled.
void build_cosmo_tables(const CosmoParamsH& p, const GridSpec& g, int nq, const RecfastOpts& r, CosmoTables& out,
                        RecfastFreeze* freeze = nullptr);

// Gauss-Legendre nodes and weights on [-1, 1].
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w);

// Builds the remaining slots (re-splined derivatives) from caller-provided
// node values of the primary tables: H, eta, rho0M, Xe, tau, g, Tmat, csb2.
void finish_uploaded_tables(CosmoTables& t);

}  // namespace bolt
