// Oracle (test infrastructure only): Background (background.jl) and the
// RECFAST ionization history (recfast.jl, ionization.jl) restated in C++.
#pragma once
#include "oracle_common.hpp"

namespace orc {

constexpr double ZETA3 = 1.2020569;  // background.jl:3

// ---------------------------------------------------------- background -----
// T = double, or a dual number carrying derivatives with respect to theta.
template <class T>
struct BackgroundT {
  ParamsT<T> par;
  Grid xg;
  int nq = 15;
  std::vector<double> quad_pts, quad_wts;
  T H0 = 0.0, eta0 = 0.0, rho_crit = 0.0, Omega_Lambda = 0.0;
  T Tnu = 0.0, logqmin = 0.0, logqmax = 0.0;
  SplineT<T> H, Hp, Hpp, eta, etap, etapp, rho0M;

  // background.jl:5-6
  static T H0_of(const ParamsT<T>& p) { return p.h * units().km_s_Mpc_100; }
  static T rho_crit_of(const ParamsT<T>& p) {
    T H = H0_of(p);
    return (3.0 / (8.0 * M_PI)) * H * H / units().G_natural;
  }
  // background.jl:7-18
  static T Omega_Lambda_of(const ParamsT<T>& p) {
    T Tg = pow(15.0 / (M_PI * M_PI) * rho_crit_of(p) * p.Omega_r, 0.25);
    T nufac = (90.0 * ZETA3 / (11.0 * pow(M_PI, 4))) * (p.Omega_r * p.h * p.h / Tg) *
                   pow(p.N_nu / 3.0, 0.75);
    T Omega_nu = p.Sigma_m_nu * nufac / (p.h * p.h);
    return 1.0 - (p.Omega_r * (1.0 + (2.0 / 3.0) * (7.0 * p.N_nu / 8.0) * pow(4.0 / 11.0, 4.0 / 3.0)) +
                  p.Omega_b + p.Omega_c + Omega_nu);
  }
  static T Tnu_of(const ParamsT<T>& p) {
    return pow(p.N_nu / 3.0, 0.25) * pow(4.0 / 11.0, 1.0 / 3.0) *
           pow(15.0 / (M_PI * M_PI) * rho_crit_of(p) * p.Omega_r, 0.25);
  }
  // util.jl:24-27 (q <-> unit interval)
  template <class U, class V, class W>
  static auto to_ui(U lq, V lqmi, W lqma) { return -1.0 + (1.0 - (-1.0)) / (lqma - lqmi) * (lq - lqmi); }
  template <class U, class V, class W>
  static auto from_ui(U x, V lqmi, W lqma) { return lqmi + (lqma - lqmi) / (1.0 - (-1.0)) * (x - (-1.0)); }
  template <class U, class V, class W>
  static auto dxdq(U q, V lqmi, W lqma) { return (1.0 + to_ui(1.0 + lqmi, lqmi, lqma)) / (q * log(10.0)); }
  template <class U, class V, class W>
  static auto xq2q(U x, V lqmi, W lqma) { return pow(10.0, from_ui(x, lqmi, lqma)); }
  // background.jl:21-30
  T f0(const T& q) const { return 2.0 / pow(2.0 * M_PI, 3) / (exp(q / Tnu) + 1.0); }
  T dlnf0dlnq(const T& q) const { return -q / Tnu / (1.0 + exp(-q / Tnu)); }
  // background.jl:33-48 (energy density of the massive neutrinos)
  T rhoP0(double a, T* P = nullptr) const {
    T m = par.Sigma_m_nu, rho = 0.0, pr = 0.0;
    for (int i = 0; i < nq; ++i) {
      T q = xq2q(quad_pts[i], logqmin, logqmax);
      T eps = sqrt(q * q + (a * m) * (a * m));
      T dx = dxdq(q, logqmin, logqmax);
      rho += q * q * eps * f0(q) / dx * quad_wts[i];
      pr += q * q * (q * q / eps) * f0(q) / dx * quad_wts[i];
    }
    if (P) *P = 4.0 * M_PI / 3.0 * pow(a, -4) * pr;
    return 4.0 * M_PI * pow(a, -4) * rho;
  }
  // background.jl:58-70
  T H_a(double a) const {
    T rho_nu = rhoP0(a);
    const ParamsT<T>& p = par;
    return H0 * sqrt((p.Omega_c + p.Omega_b) * pow(a, -3) + rho_nu / rho_crit +
                          p.Omega_r * pow(a, -4) * (1.0 + (2.0 / 3.0) * (7.0 * p.N_nu / 8.0) * pow(4.0 / 11.0, 4.0 / 3.0)) +
                          Omega_Lambda);
  }
  T Hc_a(double a) const { return a * H_a(a); }
  // background.jl:73-77
  T eta_of(double x) const {
    double lamin = -13.75, lamax = log10(exp(x));
    T s = 0.0;
    for (int i = 0; i < nq; ++i) {
      double aa = xq2q(quad_pts[i], lamin, lamax);
      s += 1.0 / (aa * Hc_a(aa)) / dxdq(aa, lamin, lamax) * quad_wts[i];
    }
    return s;
  }

  // background.jl:104-128
  BackgroundT(const ParamsT<T>& p, const Grid& g, int nq_) : par(p), xg(g), nq(nq_) {
    gauss_legendre(nq, quad_pts, quad_wts);
    H0 = H0_of(p);
    rho_crit = rho_crit_of(p);
    Omega_Lambda = Omega_Lambda_of(p);
    Tnu = Tnu_of(p);
    logqmin = log10(Tnu / 30.0);
    logqmax = log10(Tnu * 30.0);
    std::vector<T> yr(g.n), yh(g.n), ye(g.n);
    for (int j = 0; j < g.n; ++j) {
      double x = g.at(j), a = exp(x);
      yr[j] = rhoP0(a);
      yh[j] = Hc_a(a);
      ye[j] = eta_of(x);
    }
    double x0 = g.at(0);
    rho0M.build(yr, x0, g.h);
    H.build(yh, x0, g.h);
    eta.build(ye, x0, g.h);
    Hp = spline_dx(H, g);
    Hpp = spline_dx2(H, g);
    etap = spline_dx(eta, g);
    etapp = spline_dx2(eta, g);
    eta0 = eta_of(0.0);
  }
};
using Background = BackgroundT<double>;

// --------------------------------------------------------------- RECFAST ---
// recfast.jl:22-121 (SI constants and derived coefficients, same defaults).
template <class T>
struct RecfastT {
  const BackgroundT<T>* bg;
  double C = 2.99792458e8, k_B = 1.380658e-23, h_P = 6.6260755e-34, m_e = 9.1093897e-31,
         m_H = 1.673575e-27, not4 = 3.9715e0, sigma = 6.6524616e-29, a = 7.565914e-16,
         G = 6.6742e-11;
  double Lambda = 8.2245809e0, Lambda_He = 51.3e0, L_H_ion = 1.096787737e7, L_H_alpha = 8.225916453e6,
         L_He1_ion = 1.98310772e7, L_He2_ion = 4.389088863e7, L_He_2s = 1.66277434e7,
         L_He_2p = 1.71134891e7;
  double A2P_s = 1.798287e9, A2P_t = 177.58e0, L_He_2Pt = 1.690871466e7, L_He_2St = 1.5985597526e7,
         L_He2St_ion = 3.8454693845e6, sigma_He_2Ps = 1.436289e-22, sigma_He_2Pt = 1.484872e-22;
  double AGauss1 = -0.14, AGauss2 = 0.079, zGauss1 = 7.28, zGauss2 = 6.73, wGauss1 = 0.18,
         wGauss2 = 0.33;
  double a_PPB = 4.309, b_PPB = -0.6166, c_PPB = 0.6703, d_PPB = 0.5300;
  double a_VF, b_VF = 0.711, T_0, T_1, a_trip, b_trip = 0.761;
  double Lalpha, Lalpha_He, DeltaB, CDB, DeltaB_He, CDB_He, CB1, CB1_He1, CB1_He2, CR, CK, CK_He, CL,
      CL_He, CT, Bfact;
  double H_frac = 1e-3;
  int Hswitch = 1, Heswitch = 6;
  T Yp, OmegaB, HO, OmegaG, Tnow, mu_H, mu_T, fHe, Nnow;
  double fu, b_He = 0.86, tol = 1e-8;
  double atol = 1e-6;  // OrdinaryDiffEq's default abstol in recfast.jl's solves

  // Tnow < 0 means "derive from OmegaG and the background" (recfast.jl:108)
  RecfastT(const BackgroundT<T>* b, T Yp_, T OmegaB_, T OmegaG_, double Tnow_ = -1.0, double tol_ = 1e-8)
      : bg(b), Yp(Yp_), OmegaB(OmegaB_), OmegaG(OmegaG_), tol(tol_) {
    a_VF = pow(10.0, -16.744);
    T_0 = pow(10.0, 0.477121);
    T_1 = pow(10.0, 5.114);
    a_trip = pow(10.0, -16.306);
    Lalpha = 1.0 / L_H_alpha;
    Lalpha_He = 1.0 / L_He_2p;
    DeltaB = h_P * C * (L_H_ion - L_H_alpha);
    CDB = DeltaB / k_B;
    DeltaB_He = h_P * C * (L_He1_ion - L_He_2s);
    CDB_He = DeltaB_He / k_B;
    CB1 = h_P * C * L_H_ion / k_B;
    CB1_He1 = h_P * C * L_He1_ion / k_B;
    CB1_He2 = h_P * C * L_He2_ion / k_B;
    CR = 2.0 * M_PI * (m_e / h_P) * (k_B / h_P);
    CK = Lalpha * Lalpha * Lalpha / (8.0 * M_PI);
    CK_He = Lalpha_He * Lalpha_He * Lalpha_He / (8.0 * M_PI);
    CL = C * h_P / (k_B * Lalpha);
    CL_He = C * h_P / (k_B / L_He_2s);
    CT = (8.0 / 3.0) * (sigma / (m_e * C)) * a;
    Bfact = h_P * C * (L_He_2p - L_He_2s) / k_B;
    HO = bg->H0 / units().H0_conv;
    Tnow = Tnow_ > 0 ? T(Tnow_) : pow(15.0 / (M_PI * M_PI) * bg->rho_crit * OmegaG, 0.25) * units().K_conv;
    mu_H = 1.0 / (1.0 - Yp);
    mu_T = not4 / (not4 - (not4 - 1.0) * Yp);
    fHe = Yp / (not4 * (1.0 - Yp));
    Nnow = 3.0 * HO * HO * OmegaB / (8.0 * M_PI * G * mu_H * m_H);
    fu = (Hswitch == 0) ? 1.14 : 1.125;
  }

  // recfast.jl:156-310
  void ion(const T* y, double z, T* f) const {
    T f1 = 0.0, f2 = 0.0, f3 = 0.0;
    T x_H = y[0], x_He = y[1], x = x_H + fHe * x_He, Tmat = y[2];
    T n = Nnow * pow(1 + z, 3), n_He = fHe * Nnow * pow(1 + z, 3), Trad = Tnow * (1 + z);
    double aa = 1.0 / (1 + z), x_a = log(aa);
    T Hz = bg->H(x_a) / aa / units().H0_conv;
    T dHdz = (-bg->Hp(x_a) + bg->H(x_a)) / units().H0_conv;
    T Rdown = 1e-19 * a_PPB * pow(Tmat / 1e4, b_PPB) / (1.0 + c_PPB * pow(Tmat / 1e4, d_PPB));
    T Rup = Rdown * pow(CR * Tmat, 1.5) * exp(-CDB / Tmat);
    T sq_0 = sqrt(Tmat / T_0), sq_1 = sqrt(Tmat / T_1);
    T Rdown_He = a_VF / (sq_0 * pow(1 + sq_0, 1 - b_VF));
    Rdown_He = Rdown_He / pow(1 + sq_1, 1 + b_VF);
    T Rup_He = Rdown_He * pow(CR * Tmat, 1.5) * exp(-CDB_He / Tmat);
    Rup_He = 4.0 * Rup_He;
    T He_Boltz = (Bfact / Tmat > 680.0) ? T(exp(680.0)) : exp(Bfact / Tmat);
    T K;
    if (Hswitch == 0)
      K = CK / Hz;
    else
      K = CK / Hz *
          (1.0 + AGauss1 * exp(-pow((log(1 + z) - zGauss1) / wGauss1, 2)) +
           AGauss2 * exp(-pow((log(1 + z) - zGauss2) / wGauss2, 2)));
    T Rdown_trip = a_trip / (sq_0 * pow(1 + sq_0, 1 - b_trip));
    Rdown_trip = Rdown_trip / pow(1 + sq_1, 1 + b_trip);
    T Rup_trip = Rdown_trip * exp(-h_P * C * L_He2St_ion / (k_B * Tmat));
    Rup_trip = Rup_trip * pow(CR * Tmat, 1.5) * (4.0 / 3.0);
    int Heflag = ((x_He < 5.e-9) || (x_He > 0.980)) ? 0 : Heswitch;
    T K_He = 0.0, CfHe_t = 0.0;
    if (Heflag == 0) {
      K_He = CK_He / Hz;
    } else {
      T tauHe_s = A2P_s * CK_He * 3 * n_He * (1 - x_He) / Hz;
      T pHe_s = (1 - exp(-tauHe_s)) / tauHe_s;
      K_He = 1.0 / (A2P_s * pHe_s * 3 * n_He * (1 - x_He));
      if (((Heflag == 2) || (Heflag >= 5)) && (x_H < 0.9999999)) {
        T Doppler = 2 * k_B * Tmat / (m_H * not4 * C * C);
        Doppler = C * L_He_2p * sqrt(Doppler);
        T gamma_2Ps = 3 * A2P_s * fHe * (1 - x_He) * C * C /
                           (sqrt(M_PI) * sigma_He_2Ps * 8 * M_PI * Doppler * (1 - x_H)) /
                           pow(C * L_He_2p, 2);
        double pb = 0.36, qb = b_He;
        T AHcon = A2P_s / (1 + pb * pow(gamma_2Ps, qb));
        K_He = 1.0 / ((A2P_s * pHe_s + AHcon) * 3 * n_He * (1 - x_He));
      }
      if (Heflag >= 3) {
        T tauHe_t = A2P_t * n_He * (1. - x_He) * 3;
        tauHe_t = tauHe_t / (8 * M_PI * Hz * pow(L_He_2Pt, 3));
        T pHe_t = (1 - exp(-tauHe_t)) / tauHe_t;
        double CL_PSt = h_P * C * (L_He_2Pt - L_He_2St) / k_B;
        if ((Heflag == 3) || (Heflag == 5) || (x_H > 0.99999)) {
          CfHe_t = A2P_t * pHe_t * exp(-CL_PSt / Tmat);
          CfHe_t = CfHe_t / (Rup_trip + CfHe_t);
        } else {
          T Doppler = 2 * k_B * Tmat / (m_H * not4 * C * C);
          Doppler = C * L_He_2Pt * sqrt(Doppler);
          T gamma_2Pt = 3 * A2P_t * fHe * (1 - x_He) * C * C /
                             (sqrt(M_PI) * sigma_He_2Pt * 8 * M_PI * Doppler * (1 - x_H)) /
                             pow(C * L_He_2Pt, 2);
          double pb = 0.66, qb = 0.9;
          T AHcon = A2P_t / (1 + pb * pow(gamma_2Pt, qb)) / 3;
          CfHe_t = (A2P_t * pHe_t + AHcon) * exp(-CL_PSt / Tmat);
          CfHe_t = CfHe_t / (Rup_trip + CfHe_t);
        }
      }
    }
    T timeTh = (1.0 / (CT * pow(Trad, 4))) * (1 + x + fHe) / x;
    T timeH = 2.0 / (3.0 * HO * pow(1 + z, 1.5));
    if (x_H > 0.99) {
      f1 = T(0.0);
    } else if (x_H > 0.985) {
      f1 = (x * x_H * n * Rdown - Rup * (1 - x_H) * exp(-CL / Tmat)) / (Hz * (1 + z));
    } else {
      f1 = ((x * x_H * n * Rdown - Rup * (1.0 - x_H) * exp(-CL / Tmat)) *
            (1.0 + K * Lambda * n * (1.0 - x_H))) /
           (Hz * (1.0 + z) * (1.0 / fu + K * Lambda * n * (1.0 - x_H) / fu + K * Rup * n * (1.0 - x_H)));
    }
    if (x_He < 1e-15) {
      f2 = T(0.0);
    } else {
      f2 = ((x * x_He * n * Rdown_He - Rup_He * (1 - x_He) * exp(-CL_He / Tmat)) *
            (1 + K_He * Lambda_He * n_He * (1 - x_He) * He_Boltz)) /
           (Hz * (1 + z) * (1 + K_He * (Lambda_He + Rup_He) * n_He * (1 - x_He) * He_Boltz));
      if (Heflag >= 3)
        f2 = f2 + (x * x_He * n * Rdown_trip -
                   (1 - x_He) * 3 * Rup_trip * exp(-h_P * C * L_He_2St / (k_B * Tmat))) *
                      CfHe_t / (Hz * (1 + z));
    }
    if (timeTh < H_frac * timeH) {
      T epsilon = Hz * (1 + x + fHe) / (CT * pow(Trad, 3) * x);
      f3 = Tnow + epsilon * ((1 + fHe) / (1 + fHe + x)) * ((f1 + fHe * f2) / x) - epsilon * dHdz / Hz +
           3 * epsilon / (1 + z);
    } else {
      f3 = CT * pow(Trad, 4) * x / (1 + x + fHe) * (Tmat - Trad) / (Hz * (1 + z)) + 2 * Tmat / (1 + z);
    }
    f[0] = f1; f[1] = f2; f[2] = f3;
  }

  // Root 0.5 (sqrt(b^2 + 4c) - b) of the Saha equations (recfast.jl:373-411),
  // written as 2c / (sqrt(b^2 + 4c) + b) when b > 0: the same number without
  // the cancellation that leaves ~1e-6 of rounding noise at early times.
  static T quad_root(const T& b, const T& c) {
    T s = sqrt(b * b + 4.0 * c);
    return b > 0.0 ? 2.0 * c / (s + b) : 0.5 * (s - b);
  }
  T saha_rhs(double z, double CB) const {
    return exp(1.5 * log(CR * Tnow / (1 + z)) - CB / (Tnow * (1 + z))) / Nnow;
  }
  // recfast.jl:373-380
  T end_of_saha_condition(double z) const {
    T rhs = saha_rhs(z, CB1_He1) * 4;
    T x0 = quad_root(rhs - 1, (1 + fHe) * rhs);
    return (x0 - 1) / fHe - 0.99;
  }
  // recfast.jl:402-408
  T x_H0_H_Saha(double z) const {
    T rhs = saha_rhs(z, CB1);
    return quad_root(rhs, rhs);
  }
  T end_He_evo_condition(double z) const { return x_H0_H_Saha(z) - 0.985; }
};
using Recfast = RecfastT<double>;

// NonlinearSolve 0.3 Falsi on an interval: regula-falsi steps, then
// bisection once those stall, to floating-point resolution; returns the end
// of the final bracket on the side of the initial left point.
inline double falsi(const std::function<double(double)>& f, double left, double right) {
  double fl = f(left), fr = f(right);
  if (fl == 0) return left;
  if (fr == 0) return right;
  bool use_falsi = true;
  int i = 1;
  const int maxiters = 1000;
  auto prevtowards = [&](double v) { return std::nextafter(v, left); };
  while (use_falsi && i < maxiters) {
    if (std::nextafter(left, right) == right) return left;
    double mid = (fr * left - fl * right) / (fr - fl);
    for (int k = 0; k < 10; ++k) {
      double pm = prevtowards(mid);
      mid = (right > left) ? std::max(left, pm) : std::min(left, pm);
    }
    if (mid == right || mid == left) { use_falsi = false; break; }
    double fm = f(mid);
    if (fm == 0) { right = mid; use_falsi = false; break; }
    if ((fl > 0) == (fm > 0)) { fl = fm; left = mid; }
    else { fr = fm; right = mid; }
    ++i;
  }
  while (i < maxiters) {
    double mid = 0.5 * (left + right);
    if (mid == left || mid == right) return left;
    double fm = f(mid);
    if (fm == 0) { right = mid; }
    else if ((fm > 0) == (fl > 0)) { left = mid; fl = fm; }
    else { right = mid; fr = fm; }
    ++i;
  }
  return left;
}

// recfastsolve + tanh_reio_solve (recfast.jl:446-536)
// The two switch redshifts come from root finds on the values alone: the
// reference wraps them in assume_nondual (recfast.jl:451,456), so under
// ForwardDiff they carry no derivative.
template <class T>
struct RecfastHistoryT {
  const RecfastT<T>* r;
  double zinitial = 10000.0, zfinal = 0.0, z_He_evo_start = 0, z_H_He_evo_start = 0;
  double zre_ini = 50.0;
  Tsit5SolT<T> sol_He, sol_H_He, sol_reio;

  RecfastHistoryT(const RecfastT<T>* rr, const std::vector<double>& zout) : r(rr) {
    double zb = std::min(zinitial, 3500.0);
    z_He_evo_start = falsi([&](double z) { return val(r->end_of_saha_condition(z)); }, zb, zfinal);
    z_H_He_evo_start = falsi([&](double z) { return val(r->end_He_evo_condition(z)); }, z_He_evo_start, zfinal);
    // He + Tmat with H in Saha (recfast.jl:383-389, 462-465)
    T y2[2];
    {
      T rhs = r->saha_rhs(z_He_evo_start, r->CB1_He1) * 4.0;
      T x0 = RecfastT<T>::quad_root(rhs - 1, (1 + r->fHe) * rhs);
      y2[0] = (x0 - 1) / r->fHe;
      y2[1] = r->Tnow * (1 + z_He_evo_start);
    }
    RhsT<T> fHe = [this](double z, const T* u, T* du) {
      T yy[3] = {r->x_H0_H_Saha(z), u[0], u[1]}, d[3];
      r->ion(yy, z, d);
      du[0] = d[1];
      du[1] = d[2];
    };
    sol_He = tsit5(fHe, 2, y2, z_He_evo_start, z_H_He_evo_start, r->tol, r->atol, zout);
    double z3 = z_H_He_evo_start;
    T y3[3] = {r->x_H0_H_Saha(z3), sol_He.y[sol_He.y.size() - 2], sol_He.y[sol_He.y.size() - 1]};
    RhsT<T> fH = [this](double z, const T* u, T* du) { r->ion(u, z, du); };
    std::vector<double> stops3 = zout;
    stops3.push_back(zre_ini);
    sol_H_He = tsit5(fH, 3, y3, z3, zfinal, r->tol, r->atol, stops3);
    T T50 = Tmat_RECFAST(zre_ini);
    RhsT<T> fR = [this](double z, const T* u, T* du) {
      T x_reio = reionization_Xe(z);
      double aa = 1.0 / (1 + z), x_a = log(aa);
      T Hz = r->bg->H(x_a) / aa / units().H0_conv;
      T Trad = r->Tnow * (1 + z);
      du[0] = r->CT * pow(Trad, 4) * x_reio / (1 + x_reio + r->fHe) * (u[0] - Trad) / (Hz * (1 + z)) +
              2 * u[0] / (1 + z);
    };
    sol_reio = tsit5(fR, 1, &T50, zre_ini, zfinal, r->tol, r->atol, zout);
  }
  // recfast.jl:413-433
  T Xe_RECFAST(double z) const {
    if (z > 8000.) return 1 + 2 * r->fHe;
    if (z > 5000.) {
      T rhs = r->saha_rhs(z, r->CB1_He2);
      return RecfastT<T>::quad_root(rhs - 1 - r->fHe, (1 + 2 * r->fHe) * rhs);
    }
    if (z > 3500.) return 1 + r->fHe;
    if (z > z_He_evo_start) {
      T rhs = r->saha_rhs(z, r->CB1_He1) * 4;
      return RecfastT<T>::quad_root(rhs - 1, (1 + r->fHe) * rhs);
    }
    if (z > z_H_He_evo_start) return r->x_H0_H_Saha(z) + r->fHe * sol_He.at(z, 0);
    T u[3];
    sol_H_He.at(z, u);
    return u[0] + r->fHe * u[1];
  }
  // recfast.jl:435-444
  T Tmat_RECFAST(double z) const {
    if (z > z_He_evo_start) return r->Tnow * (1 + z);
    if (z > z_H_He_evo_start) return sol_He.at(z, 1);
    return sol_H_He.at(z, 2);
  }
  // recfast.jl:478-488
  T reionization_Xe(double z) const {
    T X_fin = 1 + r->Yp / (r->not4 * (1 - r->Yp));
    double zre = 7.6711, al = 1.5, dH = 0.5, zHe = 3.5, dHe = 0.5;
    T fHe = X_fin - 1;
    T x_orig = Xe_RECFAST(z);
    T x_reio_H = (X_fin - x_orig) / 2 *
                          (1 + tanh((pow(1 + zre, al) - pow(1 + z, al)) / (al * pow(1 + zre, al - 1)) / dH)) +
                      x_orig;
    T x_reio_He = fHe / 2 * (1 + tanh((zHe - z) / dHe));
    return x_reio_H + x_reio_He;
  }
  // recfast.jl:512-526
  T Xe_TanhReio(double z) const { return z > zre_ini ? Xe_RECFAST(z) : reionization_Xe(z); }
  T Tmat_TanhReio(double z) const { return z > zre_ini ? Tmat_RECFAST(z) : sol_reio.at(z, 0); }
};
using RecfastHistory = RecfastHistoryT<double>;

// saha_peebles_recombination (ionization.jl:1-93): X_e from the Saha
// equation for hydrogen until z = 1587.4, then the Peebles equation by Tsit5
// at reltol = abstol = 1e-11, in Bolt's natural units (Mpc^-1), with
// T_b = 2.725 K / a.  (The Saha root as (sqrt(r^2 + 4r) - r) / 2 rounded
// without cancellation; beta2 = beta exp(3 eps0 / 4T) as exp(-eps0 / 4T),
// which the reference evaluates in BigFloat.)
struct SahaPeebles {
  const BackgroundT<double>* bg;
  double T0, eps0, me, mH, L2s, xtr;
  Tsit5Sol late;
  SahaPeebles(const BackgroundT<double>* b, const std::vector<double>& xout) : bg(b) {
    const Units& U = units();
    T0 = 2.725 / U.K_conv;                                      // ionization.jl:5 (PeeblesT0)
    eps0 = 13.605698 * U.mass_natural;                          // ionization.jl:26
    me = si::m_e * si::c / si::hbar * si::Mpc;                  // ionization.jl:27
    mH = U.m_H;                                                 // ionization.jl:28
    L2s = 8.227 * U.H0_conv;                                    // ionization.jl:25
    xtr = log(1.0 / (1.0 + 1587.4));                            // ionization.jl:83-84
    double x0 = saha(xtr);
    Rhs f = [&](double x, const double* y, double* dy) { dy[0] = peebles(x, y[0]); };
    std::vector<double> stops;
    for (double x : xout)
      if (x > xtr) stops.push_back(x);
    late = tsit5(f, 1, &x0, xtr, 0.0, 1e-11, 1e-11, stops);   // ionization.jl:70-74
  }
  double nH(double a) const {                                   // ionization.jl:6-7
    const ParamsT<double>& p = bg->par;
    return p.Omega_b * bg->rho_crit / (mH * a * a * a) * (1 - p.Y_p);
  }
  double saha(double x) const {                                 // ionization.jl:9-16
    double a = exp(x), Tb = T0 / a;
    double r = pow(me * Tb / (2 * M_PI), 1.5) / nH(a) * exp(-eps0 / Tb);
    return 2 * r / (sqrt(r * r + 4 * r) + r);
  }
  double oldH(double a) const {                                 // background.jl:51-55
    const ParamsT<double>& p = bg->par;
    return bg->H0 * sqrt((p.Omega_c + p.Omega_b) * pow(a, -3) +
                         p.Omega_r * (1 + (2.0 / 3.0) * (7 * p.N_nu / 8) * pow(4.0 / 11.0, 4.0 / 3.0)) * pow(a, -4) +
                         bg->Omega_Lambda);
  }
  double peebles(double x, double Xe) const {                   // ionization.jl:32-66
    double a = exp(x), Tb = T0 / a, H = oldH(a), n = nH(a);
    double phi2 = 0.448 * log(eps0 / Tb);
    double alpha2 = (64 * M_PI / sqrt(27 * M_PI)) * (si::alpha * si::alpha / (me * me)) * sqrt(eps0 / Tb) * phi2;
    double beta = alpha2 * pow(me * Tb / (2 * M_PI), 1.5) * exp(-eps0 / Tb);
    double beta2 = alpha2 * pow(me * Tb / (2 * M_PI), 1.5) * exp(-eps0 / (4 * Tb));
    double Lalpha = H * pow(3 * eps0, 3) / (pow(8 * M_PI, 2) * ((1 - Xe) * n));
    double Cr = (L2s + Lalpha) / (L2s + Lalpha + beta2);
    return Cr / H * (beta * (1 - Xe) - n * alpha2 * Xe * Xe);
  }
  double Xe(double x) const { return x < xtr ? saha(x) : late.at(x, 0); }  // ionization.jl:90-92
};

// IonizationHistory(RECFAST, par, bg) (recfast.jl:674-726, ionization.jl:107-137),
// or, with a SahaPeebles X_e, customion (ionization.jl:141-164) with
// T_mat = 2.725 K (1 + z) and RECFAST's sound-speed formula on it.
template <class T>
struct IonizationT {
  T tau0 = 0.0;
  SplineT<T> Xe, tau, taup, taupp, g, gp, gpp, Tmat, csb2;
  std::vector<T> Xe_nodes, Tmat_nodes;
  double z_He_evo_start = 0, z_H_He_evo_start = 0;

  IonizationT(const SahaPeebles& sp, const RecfastT<T>& r, const ParamsT<T>& par, const BackgroundT<T>& bg) {
    const Grid& g_ = bg.xg;
    int n = g_.n;
    Xe_nodes.resize(n);
    Tmat_nodes.resize(n);
    for (int j = 0; j < n; ++j) {
      double x = g_.at(j);
      Xe_nodes[j] = sp.Xe(x);
      Tmat_nodes[j] = 2.725 * (1 + (1.0 / exp(x) - 1.0));
    }
    finish(r, par, bg);
  }

  IonizationT(const RecfastT<T>& r, const ParamsT<T>& par, const BackgroundT<T>& bg) {
    const Grid& g_ = bg.xg;
    int n = g_.n;
    std::vector<double> zout;
    for (int j = 0; j < n; ++j) {
      double x = g_.at(j);
      double z = 1.0 / exp(x) - 1.0;
      if (z < 10000.0) zout.push_back(z);
    }
    RecfastHistoryT<T> rh(&r, zout);
    z_He_evo_start = rh.z_He_evo_start;
    z_H_He_evo_start = rh.z_H_He_evo_start;
    double xinit = log(1.0 / (rh.zinitial + 1.0));
    T Xe_initial = rh.Xe_RECFAST(rh.zinitial);
    Xe_nodes.resize(n);
    Tmat_nodes.resize(n);
    for (int j = 0; j < n; ++j) {
      double x = g_.at(j);
      double z = 1.0 / exp(x) - 1.0;
      Xe_nodes[j] = (x < xinit) ? Xe_initial : rh.Xe_TanhReio(z);
      Tmat_nodes[j] = (x < xinit) ? r.Tnow * (1 + z) : rh.Tmat_TanhReio(z);
    }
    finish(r, par, bg);
  }

  // tau, g, their splines and the sound speed from the X_e and T_mat nodes
  void finish(const RecfastT<T>& r, const ParamsT<T>& par, const BackgroundT<T>& bg) {
    const Grid& g_ = bg.xg;
    int n = g_.n;
    // tau' (ionization.jl:122-127) and reverse cumulative trapezoid (ionization.jl:105-115)
    const Units& U = units();
    T rc = BackgroundT<T>::rho_crit_of(par);
    std::vector<T> tp(n), ti(n);
    for (int j = 0; j < n; ++j) {
      double x = g_.at(j), a = exp(x);
      T nH = par.Omega_b * rc / (U.m_H * a * a * a) * (1 - par.Y_p);
      tp[j] = -Xe_nodes[j] * nH * a * U.sigma_T / bg.H(x);
    }
    {
      // cumul_integrate(reverse(x), reverse(tau')) then reverse
      std::vector<T> acc(n);
      acc[0] = T(0.0);
      for (int i = 1; i < n; ++i) {
        int jr = n - 1 - i, jp = n - i;
        double dx = g_.at(jr) - g_.at(jp);
        acc[i] = acc[i - 1] + dx * (tp[jr] + tp[jp]);
      }
      for (int i = 0; i < n; ++i) ti[n - 1 - i] = 0.5 * acc[i];
    }
    std::vector<T> gt(n);
    for (int j = 0; j < n; ++j) gt[j] = -tp[j] * exp(-ti[j]);
    double x0 = g_.at(0);
    Xe.build(Xe_nodes, x0, g_.h);
    tau.build(ti, x0, g_.h);
    g.build(gt, x0, g_.h);
    Tmat.build(Tmat_nodes, x0, g_.h);
    SplineT<T> Tp = spline_dx(Tmat, g_);
    std::vector<T> cs(n);
    for (int j = 0; j < n; ++j) {
      double x = g_.at(j);
      T pre = pow(r.C, -2) * r.k_B / r.m_H * (1.0 / r.mu_T + (1 - r.Yp) * Xe(x));
      cs[j] = pre * (Tmat(x) - 1.0 / 3.0 * Tp(x));
    }
    csb2.build(cs, x0, g_.h);
    taup = spline_dx(tau, g_);
    taupp = spline_dx2(tau, g_);
    gp = spline_dx(g, g_);
    gpp = spline_dx2(g, g_);
    tau0 = ti[n - 1];
  }
};
using Ionization = IonizationT<double>;

}  // namespace orc
