// Oracle (test infrastructure only): the Newtonian-gauge Boltzmann hierarchy
// (perturbations.jl), its solve, the source functions and the
// line-of-sight spectra (spectra.jl), restated in C++.
//
// Integrator: the reference calls OrdinaryDiffEq's KenCarp4
// (perturbations.jl:25-33).  The oracle integrates the same ODE with a
// Rodas4 Rosenbrock method (Hairer & Wanner, "Solving ODEs II", RODAS
// coefficient set 1) at a caller-chosen tolerance, landing exactly on every
// output node.  Parity is defined on tolerance-converged results.
#pragma once
#include "oracle_cosmo.hpp"

namespace orc {

// T = double, or G6 (a dual number carrying derivatives with respect to
// theta) for the gradient oracle.
template <class T>
struct CosmoT {
  ParamsT<T> par;
  BackgroundT<T>* bg = nullptr;
  IonizationT<T>* ih = nullptr;
};
using Cosmo = CosmoT<double>;

// Hierarchy (perturbations.jl:7-21) plus per-mode constants.
template <class T>
struct ModeT {
  const CosmoT<T>* C;
  double k;
  int lg, lnu, lmnu, nq, N;
  int iTp, iN, iM, iPhi;  // offsets (unpack, perturbations.jl:114-125)
  std::vector<T> q, df0, Aq;  // q nodes, dlnf0/dlnq, 4*pi*q^2 f0 / dxdq * w
  std::vector<T> Bq;          // 4*pi*q^3 f0 / dxdq * w  (theta integral)
  ModeT(const CosmoT<T>* c, double k_, int lg_, int lnu_, int lmnu_, int nq_)
      : C(c), k(k_), lg(lg_), lnu(lnu_), lmnu(lmnu_), nq(nq_) {
    N = 2 * (lg + 1) + (lnu + 1) + (lmnu + 1) * nq + 5;
    iTp = lg + 1;
    iN = 2 * (lg + 1);
    iM = iN + lnu + 1;
    iPhi = iM + (lmnu + 1) * nq;
    const BackgroundT<T>& bg = *C->bg;
    q.resize(nq); df0.resize(nq); Aq.resize(nq); Bq.resize(nq);
    for (int i = 0; i < nq; ++i) {
      T qq = BackgroundT<T>::xq2q(bg.quad_pts[i], bg.logqmin, bg.logqmax);
      q[i] = qq;
      df0[i] = bg.dlnf0dlnq(qq);
      T dx = BackgroundT<T>::dxdq(qq, bg.logqmin, bg.logqmax);
      Aq[i] = 4.0 * M_PI * qq * qq * bg.f0(qq) / dx * bg.quad_wts[i];
      Bq[i] = 4.0 * M_PI * qq * qq * qq * bg.f0(qq) / dx * bg.quad_wts[i];
    }
  }
  int M(int l, int iq) const { return iM + l * nq + iq; }
};
using Mode = ModeT<double>;

// rho_sigma (perturbations.jl:127-145): massive-neutrino density and shear
// q-integrals of the l = 0 and l = 2 moments.
template <class S, class T, class A>
inline void rho_sigma(const ModeT<T>& md, A a, const T* M0, const T* M2, S& rho, S& sig) {
  T m = md.C->par.Sigma_m_nu;
  rho = S(0.0);
  sig = S(0.0);
  for (int i = 0; i < md.nq; ++i) {
    S eps = sqrt(md.q[i] * md.q[i] + (a * m) * (a * m));
    rho = rho + md.Aq[i] * eps * M0[i * 1];
    sig = sig + md.Aq[i] * (md.q[i] * md.q[i] / eps) * M2[i * 1];
  }
}

struct RhsInfo { bool rsa = false; };

// The radiation-streaming switch of hierarchy! (perturbations.jl:216):
// k eta > 240 and -tau' H / eta > 100.
template <class T>
inline bool rsa_switch(const ModeT<T>& md, double x) {
  const BackgroundT<T>& bg = *md.C->bg;
  const IonizationT<T>& ih = *md.C->ih;
  double eta = val(bg.eta.eval(x)), tp = val(ih.taup.eval(x)), Hc = val(bg.H.eval(x));
  return (md.k * eta > 240.0) && (-tp * Hc / eta > 100.0);
}

// hierarchy! (perturbations.jl:161-271).  S = T for the plain RHS (x a
// double), S = D1T<T> (value, d/dx; x a D1) to obtain the explicit
// x-derivative of the RHS that a Rosenbrock method needs for a
// non-autonomous system.
template <class S> struct AbscissaOf { using type = double; };
template <class V> struct AbscissaOf<D1T<V>> { using type = D1; };
template <class S, class T>
inline void hierarchy_rhs(const ModeT<T>& md, typename AbscissaOf<S>::type x, const T* u, S* du,
                          RhsInfo* info = nullptr) {
  const CosmoT<T>& C = *md.C;
  const ParamsT<T>& p = C.par;
  const BackgroundT<T>& bg = *C.bg;
  const IonizationT<T>& ih = *C.ih;
  const double k = md.k;
  const int lg = md.lg, lnu = md.lnu, lmnu = md.lmnu, nq = md.nq;
  const T H0sq = bg.H0 * bg.H0;
  S Hc = bg.H.eval(x), eta = bg.eta.eval(x), tp = ih.taup.eval(x), cs2 = ih.csb2.eval(x);
  S a = S(exp(x));
  S R = 4.0 * p.Omega_r / (3.0 * p.Omega_b * a);
  T Omega_nu = 7.0 * (2.0 / 3.0) * p.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * p.Omega_r;
  const T* Th = u;
  const T* Tp = u + md.iTp;
  const T* Nn = u + md.iN;
  const T* Mm = u + md.iM;
  const T Phi = u[md.iPhi], del = u[md.iPhi + 1], v = u[md.iPhi + 2], delb = u[md.iPhi + 3], vb = u[md.iPhi + 4];
  S* dTh = du;
  S* dTp = du + md.iTp;
  S* dNn = du + md.iN;
  S* dMm = du + md.iM;
  std::vector<T> M0(nq), M2(nq);
  for (int i = 0; i < nq; ++i) { M0[i] = Mm[0 * nq + i]; M2[i] = Mm[2 * nq + i]; }
  S rhoM, sigM;
  rho_sigma(md, a, M0.data(), M2.data(), rhoM, sigM);
  S Psi = -Phi - 12.0 * H0sq / (k * k) / (a * a) * (p.Omega_r * Th[2] + Omega_nu * Nn[2] + sigM / bg.rho_crit / 4.0);
  S Phip = Psi - k * k / (3.0 * Hc * Hc) * Phi +
           H0sq / (2.0 * Hc * Hc) *
               (p.Omega_c / a * del + p.Omega_b / a * delb + 4.0 * p.Omega_r / (a * a) * Th[0] +
                4.0 * Omega_nu / (a * a) * Nn[0] + rhoM / (a * a) / bg.rho_crit);
  S ddel = k / Hc * v - 3.0 * Phip;
  S dv = -S(v) - k / Hc * Psi;
  S ddelb = k / Hc * vb - 3.0 * Phip;
  S dvb = -S(vb) - k / Hc * (Psi + cs2 * delb) + tp * R * (3.0 * Th[1] + vb);
  T m = p.Sigma_m_nu;
  for (int iq = 0; iq < nq; ++iq) {
    T q = md.q[iq];
    S eps = sqrt(q * q + (a * m) * (a * m));
    T df0 = md.df0[iq];
    dMm[0 * nq + iq] = -k / Hc * (q / eps) * Mm[1 * nq + iq] + Phip * df0;
    dMm[1 * nq + iq] = k / (3.0 * Hc) * ((q / eps) * (Mm[0 * nq + iq] - 2.0 * Mm[2 * nq + iq]) - eps / q * Psi * df0);
    for (int l = 2; l <= lmnu - 1; ++l)
      dMm[l * nq + iq] = k / Hc * q / ((2.0 * l + 1.0) * eps) * (l * Mm[(l - 1) * nq + iq] - (l + 1) * Mm[(l + 1) * nq + iq]);
    dMm[lmnu * nq + iq] = q / eps * k / Hc * Mm[(lmnu - 1) * nq + iq] - (lmnu + 1.0) / (Hc * eta) * Mm[lmnu * nq + iq];
  }
  bool rsa_on = rsa_switch(md, val(x));
  if (info) info->rsa = rsa_on;
  if (rsa_on) {
    // The reference also overwrites Theta_0..2 and N_0..2 of u here
    // (perturbations.jl:217-227); the solver applies that to the accepted
    // state after each step (rsa_overwrite).  Nothing below reads them.
    for (int l = 0; l <= lnu; ++l) dNn[l] = S(0.0);
    for (int l = 0; l <= lg; ++l) { dTh[l] = S(0.0); dTp[l] = S(0.0); }
  } else {
    dNn[0] = -k / Hc * Nn[1] - Phip;
    dNn[1] = k / (3.0 * Hc) * Nn[0] - 2.0 * k / (3.0 * Hc) * Nn[2] + k / (3.0 * Hc) * Psi;
    for (int l = 2; l <= lnu - 1; ++l)
      dNn[l] = k / ((2.0 * l + 1.0) * Hc) * (l * Nn[l - 1] - (l + 1) * Nn[l + 1]);
    dNn[lnu] = k / Hc * Nn[lnu - 1] - (lnu + 1.0) / (Hc * eta) * Nn[lnu];
    T Pi = Th[2] + Tp[2] + Tp[0];
    dTh[0] = -k / Hc * Th[1] - Phip;
    dTh[1] = k / (3.0 * Hc) * Th[0] - 2.0 * k / (3.0 * Hc) * Th[2] + k / (3.0 * Hc) * Psi + tp * (Th[1] + vb / 3.0);
    for (int l = 2; l <= lg - 1; ++l)
      dTh[l] = l * k / ((2.0 * l + 1.0) * Hc) * Th[l - 1] - (l + 1) * k / ((2.0 * l + 1.0) * Hc) * Th[l + 1] +
               tp * (Th[l] - Pi * (l == 2 ? 1.0 : 0.0) / 10.0);
    dTp[0] = -k / Hc * Tp[1] + tp * (Tp[0] - Pi / 2.0);
    for (int l = 1; l <= lg - 1; ++l)
      dTp[l] = l * k / ((2.0 * l + 1.0) * Hc) * Tp[l - 1] - (l + 1) * k / ((2.0 * l + 1.0) * Hc) * Tp[l + 1] +
               tp * (Tp[l] - Pi * (l == 2 ? 1.0 : 0.0) / 10.0);
    dTh[lg] = k / Hc * Th[lg - 1] - ((lg + 1.0) / (Hc * eta) - tp) * Th[lg];
    dTp[lg] = k / Hc * Tp[lg - 1] - ((lg + 1.0) / (Hc * eta) - tp) * Tp[lg];
  }
  du[md.iPhi] = Phip;
  du[md.iPhi + 1] = ddel;
  du[md.iPhi + 2] = dv;
  du[md.iPhi + 3] = ddelb;
  du[md.iPhi + 4] = dvb;
}

// The state overwrite of hierarchy!'s radiation-streaming branch
// (perturbations.jl:217-227) at x: Theta_0, Theta_1 from the metric and the
// baryons, Theta_2 = 0, N_0 = Phi, N_1 = -2 H Phi' / k, N_2 = 0, with Phi'
// formed from u before the overwrite (as the reference forms it).  OrdinaryDiffEq
// passes the integrator's own state to the right-hand side at the end of a
// step, so the accepted state carries these values into the next step; the
// solver applies them there.
template <class T>
inline void rsa_overwrite(const ModeT<T>& md, double x, T* u) {
  const CosmoT<T>& C = *md.C;
  const ParamsT<T>& p = C.par;
  const BackgroundT<T>& bg = *C.bg;
  const IonizationT<T>& ih = *C.ih;
  const double k = md.k, a = std::exp(x);
  const T H0sq = bg.H0 * bg.H0;
  const T Hc = bg.H(x), tp = ih.taup(x), tpp = ih.taupp(x), cs2 = ih.csb2(x);
  T Omega_nu = 7.0 * (2.0 / 3.0) * p.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * p.Omega_r;
  const int nq = md.nq;
  std::vector<T> M0(nq), M2(nq);
  for (int i = 0; i < nq; ++i) { M0[i] = u[md.iM + i]; M2[i] = u[md.iM + 2 * nq + i]; }
  T rhoM, sigM;
  rho_sigma(md, a, M0.data(), M2.data(), rhoM, sigM);
  const T Phi = u[md.iPhi], del = u[md.iPhi + 1], delb = u[md.iPhi + 3], vb = u[md.iPhi + 4];
  T Psi = -Phi - 12.0 * H0sq / (k * k) / (a * a) * (p.Omega_r * u[2] + Omega_nu * u[md.iN + 2] + sigM / bg.rho_crit / 4.0);
  T Phip = Psi - k * k / (3.0 * Hc * Hc) * Phi +
                H0sq / (2.0 * Hc * Hc) *
                    (p.Omega_c / a * del + p.Omega_b / a * delb + 4.0 * p.Omega_r / (a * a) * u[0] +
                     4.0 * Omega_nu / (a * a) * u[md.iN] + rhoM / (a * a) / bg.rho_crit);
  u[0] = Phi - Hc / k * tp * vb;
  u[1] = Hc / k * (-2.0 * Phip + tp * (Phi - cs2 * delb) + Hc / k * (tpp - tp) * vb);
  u[2] = 0.0;
  u[md.iN] = Phi;
  u[md.iN + 1] = -2.0 * Hc / k * Phip;
  u[md.iN + 2] = 0.0;
}

// initial_conditions (perturbations.jl:274-338)
template <class T>
inline void initial_conditions(const ModeT<T>& md, double xi, T* u) {
  const CosmoT<T>& C = *md.C;
  const ParamsT<T>& p = C.par;
  const BackgroundT<T>& bg = *C.bg;
  const IonizationT<T>& ih = *C.ih;
  double k = md.k;
  int lg = md.lg, lnu = md.lnu, lmnu = md.lmnu, nq = md.nq;
  std::fill(u, u + md.N, T(0.0));
  T Hc = bg.H(xi), eta = bg.eta(xi), tp = ih.taup(xi);
  double ai = std::exp(xi);
  T fnu = 1.0 / (1.0 + 1.0 / (7.0 * (3.0 / 3.0) * p.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0)));
  double Rc = 1.0;
  T Phi = (4.0 * fnu + 10.0) / (4.0 * fnu + 15.0) * Rc;
  T Cc = -((15.0 + 4.0 * fnu) / (20.0 + 8.0 * fnu)) * Phi;
  T* Th = u;
  T* Tp = u + md.iTp;
  T* Nn = u + md.iN;
  T* Mm = u + md.iM;
  Th[0] = -40.0 * Cc / (15.0 + 4.0 * fnu) / 4.0;
  Th[1] = 10.0 * Cc / (15.0 + 4.0 * fnu) * (k * k * eta) / (3.0 * k);
  Th[2] = -8.0 * k / (15.0 * Hc * tp) * Th[1];
  Tp[0] = (5.0 / 4.0) * Th[2];
  Tp[1] = -k / (4.0 * Hc * tp) * Th[2];
  Tp[2] = (1.0 / 4.0) * Th[2];
  for (int l = 3; l <= lg; ++l) {
    Th[l] = -l / (2.0 * l + 1.0) * k / (Hc * tp) * Th[l - 1];
    Tp[l] = -l / (2.0 * l + 1.0) * k / (Hc * tp) * Tp[l - 1];
  }
  T del = 3.0 / 4.0 * (4.0 * Th[0]);
  T delb = del;
  T v = -3.0 * k * Th[1];
  T vb = v;
  Nn[0] = Th[0];
  Nn[1] = Th[1];
  Nn[2] = -(k * k * eta * eta) / 15.0 * 1.0 / (1.0 + 2.0 / 5.0 * fnu) * Phi / 2.0;
  for (int l = 3; l <= lnu; ++l) Nn[l] = k / ((2.0 * l + 1.0) * Hc) * Nn[l - 1];
  for (int iq = 0; iq < nq; ++iq) {
    T q = md.q[iq];
    T eps = sqrt(q * q + (ai * p.Sigma_m_nu) * (ai * p.Sigma_m_nu));
    T df0 = md.df0[iq];
    Mm[0 * nq + iq] = -Nn[0] * df0;
    Mm[1 * nq + iq] = -eps / q * Nn[1] * df0;
    Mm[2 * nq + iq] = -Nn[2] * df0;
    for (int l = 3; l <= lmnu; ++l)
      Mm[l * nq + iq] = q / eps * k / ((2.0 * l + 1.0) * Hc) * Mm[(l - 1) * nq + iq];
  }
  u[md.iPhi] = Phi;
  u[md.iPhi + 1] = del;
  u[md.iPhi + 2] = v;
  u[md.iPhi + 3] = delb;
  u[md.iPhi + 4] = vb;
}

// source_function (perturbations.jl:343-383) and source_function_P (386-404)
template <class T>
inline void source_functions(const ModeT<T>& md, double x, const T* u, const T* du, T& ST, T& SE) {
  const CosmoT<T>& C = *md.C;
  const ParamsT<T>& p = C.par;
  const BackgroundT<T>& bg = *C.bg;
  const IonizationT<T>& ih = *C.ih;
  double k = md.k;
  int nq = md.nq;
  T H0sq = bg.H0 * bg.H0;
  T Hc = bg.H(x), Hcp = bg.Hp(x), Hcpp = bg.Hpp(x);
  T tau = ih.tau(x), tp = ih.taup(x), tpp = ih.taupp(x);
  T g = ih.g(x), gp = ih.gp(x), gpp = ih.gpp(x);
  double a = std::exp(x);
  T Omega_nu = 7.0 * (2.0 / 3.0) * p.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * p.Omega_r;
  const T* Th = u;
  const T* Tp = u + md.iTp;
  const T* Nn = u + md.iN;
  const T* Mm = u + md.iM;
  const T* dTh = du;
  const T* dTp = du + md.iTp;
  const T* dNn = du + md.iN;
  const T* dMm = du + md.iM;
  T Phip = du[md.iPhi], vbp = du[md.iPhi + 4], Phi = u[md.iPhi], vb = u[md.iPhi + 4];
  std::vector<T> M0(nq), M2(nq), dM0(nq), dM2(nq);
  for (int i = 0; i < nq; ++i) {
    M0[i] = Mm[i]; M2[i] = Mm[2 * nq + i];
    dM0[i] = dMm[i]; dM2[i] = dMm[2 * nq + i];
  }
  T r_, sigM, sigMp;
  rho_sigma(md, a, M0.data(), M2.data(), r_, sigM);
  rho_sigma(md, a, dM0.data(), dM2.data(), r_, sigMp);
  T Psi = -Phi - 12.0 * H0sq / (k * k) / (a * a) * (p.Omega_r * Th[2] + Omega_nu * Nn[2] + sigM / bg.rho_crit / 4.0);
  T Psip = -Phip - 12.0 * H0sq / (k * k) / (a * a) *
                            (p.Omega_r * (dTh[2] - 2.0 * Th[2]) + Omega_nu * (dNn[2] - 2.0 * Nn[2]) +
                             (sigMp - 2.0 * sigM) / bg.rho_crit / 4.0);
  T Pi = Th[2] + Tp[2] + Tp[0];
  T Pip = dTh[2] + dTp[2] + dTp[0];
  T term1 = g * (Th[0] + Psi + Pi / 4.0) + exp(-tau) * (Psip - Phip);
  T term2 = (-1.0 / k) * (Hcp * g * vb + Hc * gp * vb + Hc * g * vbp);
  T Pipp = 2.0 * k / (5.0 * Hc) * (-Hcp / Hc * Th[1] + dTh[1]) + (3.0 / 10.0) * (tpp * Pi + tp * Pip) -
                3.0 * k / (5.0 * Hc) * (-Hcp / Hc * (Th[3] + Tp[1] + Tp[3]) + (dTh[3] + dTp[1] + dTp[3]));
  T term3 = (3.0 / (4.0 * k * k)) *
                 ((Hcp * Hcp + Hc * Hcpp) * g * Pi + 3.0 * Hc * Hcp * (gp * Pi + g * Pip) +
                  Hc * Hc * (gpp * Pi + 2.0 * gp * Pip + g * Pipp));
  ST = term1 + term2 + term3;
  T y = k * (bg.eta(bg.xg.at(bg.xg.n - 1)) - bg.eta(x));
  SE = (3.0 / (4.0 * y * y)) * g * Pi;
}

// ------------------------------------------------------- linear algebra ----
// Banded LU with partial pivoting (LAPACK dgbtf2/dgbtrs layout) for the
// local part of the Rosenbrock matrix, plus a rank-3 Woodbury correction for
// the three global couplings (Phi', Psi, Pi) of the hierarchy.
template <class T>
struct BandLUT {
  int n = 0, kl = 2, ku = 2, ld = 0, kv = 0;
  std::vector<T> ab;
  std::vector<int> ipiv;
  void init(int n_) {
    n = n_;
    kv = kl + ku;
    ld = 2 * kl + ku + 1;
    ab.assign(size_t(ld) * n, T(0.0));
    ipiv.assign(n, 0);
  }
  T& at(int i, int j) { return ab[size_t(kv + i - j) + size_t(j) * ld]; }
  void zero() { std::fill(ab.begin(), ab.end(), T(0.0)); }
  bool factor() {
    int ju = 0;
    for (int j = 0; j < n; ++j) {
      int km = std::min(kl, n - 1 - j);
      int jp = 0;
      double best = std::fabs(val(at(j, j)));
      for (int r = 1; r <= km; ++r)
        if (std::fabs(val(at(j + r, j))) > best) { best = std::fabs(val(at(j + r, j))); jp = r; }
      ipiv[j] = j + jp;
      if (best == 0.0) return false;
      ju = std::max(ju, std::min(j + ku + jp, n - 1));
      if (jp != 0)
        for (int c = j; c <= ju; ++c) std::swap(at(j, c), at(j + jp, c));
      T piv = at(j, j);
      for (int r = 1; r <= km; ++r) at(j + r, j) /= piv;
      for (int c = j + 1; c <= ju; ++c) {
        T ujc = at(j, c);
        if (nonzero(ujc))
          for (int r = 1; r <= km; ++r) at(j + r, c) -= at(j + r, j) * ujc;
      }
    }
    return true;
  }
  void solve(T* b) {
    for (int j = 0; j < n - 1; ++j) {
      int lm = std::min(kl, n - 1 - j);
      int l = ipiv[j];
      if (l != j) std::swap(b[l], b[j]);
      for (int r = 1; r <= lm; ++r) b[j + r] -= at(j + r, j) * b[j];
    }
    for (int j = n - 1; j >= 0; --j) {
      b[j] /= at(j, j);
      T bj = b[j];
      for (int i = std::max(0, j - kl - ku); i < j; ++i) b[i] -= at(i, j) * bj;
    }
  }
};

// Jacobian split J = L + U W^T of the (linear) hierarchy at x.  L is stored
// in a permuted order in which every species is a contiguous chain and the
// baryon pair (delta_b, v_b) precedes the photon temperature chain, giving
// bandwidth 2; U and W are the three global couplings (Phi', Psi, Pi).
template <class T>
struct JacSplitT {
  int N = 0;
  std::vector<int> pos;   // state index -> banded position
  std::vector<int> st;    // banded position -> state index
  struct E { int r, c; T v; };
  std::vector<E> L;       // local entries (state indices)
  std::vector<T> U[3], W[3];
};
using JacSplit = JacSplitT<double>;
using BandLU = BandLUT<double>;

template <class T>
inline void build_perm(const ModeT<T>& md, std::vector<int>& pos, std::vector<int>& st) {
  int N = md.N;
  st.clear();
  st.push_back(md.iPhi + 3);  // delta_b
  st.push_back(md.iPhi + 4);  // v_b
  for (int l = 0; l <= md.lg; ++l) st.push_back(l);
  for (int l = 0; l <= md.lg; ++l) st.push_back(md.iTp + l);
  for (int l = 0; l <= md.lnu; ++l) st.push_back(md.iN + l);
  for (int iq = 0; iq < md.nq; ++iq)
    for (int l = 0; l <= md.lmnu; ++l) st.push_back(md.M(l, iq));
  st.push_back(md.iPhi + 1);  // delta
  st.push_back(md.iPhi + 2);  // v
  st.push_back(md.iPhi);      // Phi
  pos.assign(N, -1);
  for (int p = 0; p < N; ++p) pos[st[p]] = p;
}

template <class T>
inline void jacobian_split(const ModeT<T>& md, double x, JacSplitT<T>& J) {
  const CosmoT<T>& C = *md.C;
  const ParamsT<T>& p = C.par;
  const BackgroundT<T>& bg = *C.bg;
  const IonizationT<T>& ih = *C.ih;
  const double k = md.k;
  const int lg = md.lg, lnu = md.lnu, lmnu = md.lmnu, nq = md.nq, N = md.N;
  const T H0sq = bg.H0 * bg.H0;
  T Hc = bg.H(x), eta = bg.eta(x), tp = ih.taup(x), cs2 = ih.csb2(x);
  double a = std::exp(x);
  T R = 4.0 * p.Omega_r / (3.0 * p.Omega_b * a);
  T Omega_nu = 7.0 * (2.0 / 3.0) * p.N_nu / 8.0 * std::pow(4.0 / 11.0, 4.0 / 3.0) * p.Omega_r;
  T m = p.Sigma_m_nu;
  J.N = N;
  J.L.clear();
  for (int r = 0; r < 3; ++r) { J.U[r].assign(N, 0.0); J.W[r].assign(N, 0.0); }
  // with the radiation-streaming switch on, the photon and massless-neutrino
  // rows of the right-hand side are zero, and so are their Jacobian rows
  const bool rsa = rsa_switch(md, x);
  const int rad_end = md.iM;  // rows 0 .. iM-1: photon T, photon P, massless nu
  auto add = [&](int r, int c, T v) {
    if (!(rsa && r < rad_end)) J.L.push_back({r, c, v});
  };
  const int iPhi = md.iPhi, idel = iPhi + 1, iv = iPhi + 2, idelb = iPhi + 3, ivb = iPhi + 4;
  // gradients of Psi and Phi'
  T cpsi = 12.0 * H0sq / (k * k) / (a * a);
  std::vector<T>& Wpsi = J.W[1];
  std::vector<T>& Wphp = J.W[0];
  Wpsi[iPhi] += -1.0;
  Wpsi[2] += -cpsi * p.Omega_r;
  Wpsi[md.iN + 2] += -cpsi * Omega_nu;
  std::vector<T> eps(nq);
  for (int iq = 0; iq < nq; ++iq) {
    eps[iq] = sqrt(md.q[iq] * md.q[iq] + (a * m) * (a * m));
    Wpsi[md.M(2, iq)] += -cpsi * md.Aq[iq] * (md.q[iq] * md.q[iq] / eps[iq]) / bg.rho_crit / 4.0;
  }
  Wphp = Wpsi;
  T d = H0sq / (2.0 * Hc * Hc);
  Wphp[iPhi] += -k * k / (3.0 * Hc * Hc);
  Wphp[idel] += d * p.Omega_c / a;
  Wphp[idelb] += d * p.Omega_b / a;
  Wphp[0] += d * 4.0 * p.Omega_r / (a * a);
  Wphp[md.iN] += d * 4.0 * Omega_nu / (a * a);
  for (int iq = 0; iq < nq; ++iq) Wphp[md.M(0, iq)] += d * md.Aq[iq] * eps[iq] / (a * a) / bg.rho_crit;
  J.W[2][2] = 1.0;
  J.W[2][md.iTp + 2] = 1.0;
  J.W[2][md.iTp + 0] = 1.0;
  // U columns: coefficient of Phi', Psi, Pi in each row
  std::vector<T>& Uph = J.U[0];
  std::vector<T>& Ups = J.U[1];
  std::vector<T>& Upi = J.U[2];
  T kH = k / Hc;
  Uph[iPhi] = 1.0;
  Uph[idel] = -3.0;
  Uph[idelb] = -3.0;
  Ups[iv] = -kH;
  Ups[ivb] = -kH;
  // matter (local parts)
  add(idel, iv, kH);
  add(iv, iv, -1.0);
  add(idelb, ivb, kH);
  add(ivb, ivb, -1.0 + tp * R);
  add(ivb, idelb, -kH * cs2);
  add(ivb, 1, 3.0 * tp * R);
  // massive neutrinos
  for (int iq = 0; iq < nq; ++iq) {
    T q = md.q[iq], e = eps[iq], df0 = md.df0[iq];
    Uph[md.M(0, iq)] = df0;
    add(md.M(0, iq), md.M(1, iq), -kH * (q / e));
    add(md.M(1, iq), md.M(0, iq), k / (3.0 * Hc) * (q / e));
    add(md.M(1, iq), md.M(2, iq), -2.0 * k / (3.0 * Hc) * (q / e));
    Ups[md.M(1, iq)] = -k / (3.0 * Hc) * (e / q) * df0;
    for (int l = 2; l <= lmnu - 1; ++l) {
      T f = kH * q / ((2.0 * l + 1.0) * e);
      add(md.M(l, iq), md.M(l - 1, iq), f * l);
      add(md.M(l, iq), md.M(l + 1, iq), -f * (l + 1));
    }
    add(md.M(lmnu, iq), md.M(lmnu - 1, iq), q / e * kH);
    add(md.M(lmnu, iq), md.M(lmnu, iq), -(lmnu + 1.0) / (Hc * eta));
  }
  // massless neutrinos
  Uph[md.iN] = -1.0;
  add(md.iN, md.iN + 1, -kH);
  add(md.iN + 1, md.iN, k / (3.0 * Hc));
  add(md.iN + 1, md.iN + 2, -2.0 * k / (3.0 * Hc));
  Ups[md.iN + 1] = k / (3.0 * Hc);
  for (int l = 2; l <= lnu - 1; ++l) {
    T f = k / ((2.0 * l + 1.0) * Hc);
    add(md.iN + l, md.iN + l - 1, f * l);
    add(md.iN + l, md.iN + l + 1, -f * (l + 1));
  }
  add(md.iN + lnu, md.iN + lnu - 1, kH);
  add(md.iN + lnu, md.iN + lnu, -(lnu + 1.0) / (Hc * eta));
  // photons
  Uph[0] = -1.0;
  add(0, 1, -kH);
  add(1, 0, k / (3.0 * Hc));
  add(1, 2, -2.0 * k / (3.0 * Hc));
  add(1, 1, tp);
  add(1, ivb, tp / 3.0);
  Ups[1] = k / (3.0 * Hc);
  for (int l = 2; l <= lg - 1; ++l) {
    T f = k / ((2.0 * l + 1.0) * Hc);
    add(l, l - 1, f * l);
    add(l, l + 1, -f * (l + 1));
    add(l, l, tp);
  }
  Upi[2] = -tp / 10.0;
  add(md.iTp + 0, md.iTp + 1, -kH);
  add(md.iTp + 0, md.iTp + 0, tp);
  Upi[md.iTp + 0] = -tp / 2.0;
  for (int l = 1; l <= lg - 1; ++l) {
    T f = k / ((2.0 * l + 1.0) * Hc);
    add(md.iTp + l, md.iTp + l - 1, f * l);
    add(md.iTp + l, md.iTp + l + 1, -f * (l + 1));
    add(md.iTp + l, md.iTp + l, tp);
  }
  Upi[md.iTp + 2] = -tp / 10.0;
  add(lg, lg - 1, kH);
  add(lg, lg, -((lg + 1.0) / (Hc * eta) - tp));
  add(md.iTp + lg, md.iTp + lg - 1, kH);
  add(md.iTp + lg, md.iTp + lg, -((lg + 1.0) / (Hc * eta) - tp));
  if (rsa)
    for (int r = 0; r < 3; ++r)
      for (int i = 0; i < rad_end; ++i) J.U[r][i] = 0.0;
}

// ---------------------------------------------------------- Rodas4 ---------
struct SolveStats { long steps = 0, rejects = 0, rsa = 0; int status = 0; };

struct Rodas4 {
  static constexpr double gam = 0.25;
  static constexpr double c2 = 0.386, c3 = 0.21, c4 = 0.63;
  static constexpr double d1 = 0.25, d2 = -0.1043, d3 = 0.1035, d4 = -0.0362;
  static constexpr double a21 = 1.544, a31 = 0.9466785280815826, a32 = 0.2557011698983284,
                          a41 = 3.314825187068521, a42 = 2.896124015972201, a43 = 0.9986419139977817,
                          a51 = 1.221224509226641, a52 = 6.019134481288629, a53 = 12.53708332932087,
                          a54 = -0.687886036105895;
  static constexpr double C21 = -5.6688, C31 = -2.430093356833875, C32 = -0.2063599157091915,
                          C41 = -0.1073529058151375, C42 = -9.594562251023355, C43 = -20.47028614809616,
                          C51 = 7.496443313967647, C52 = -10.24680431464352, C53 = -33.99990352819905,
                          C54 = 11.7089089320616, C61 = 8.083246795921522, C62 = -7.981132988064893,
                          C63 = -31.52159432874371, C64 = 16.31930543123136, C65 = -6.058818238834054;
};

// Integrate one mode from x = -20 (first grid node) to 0, landing on every
// xout node (ascending), and call emit(j, x, u) there.
template <class T, class Emit>
inline SolveStats solve_mode(const ModeT<T>& md, double reltol, double abstol, const std::vector<double>& xout,
                             Emit emit, long maxsteps = 20000000) {
  typedef Rodas4 R;
  const int N = md.N;
  const BackgroundT<T>& bg = *md.C->bg;
  double x = bg.xg.at(0), xend = bg.xg.at(bg.xg.n - 1);
  std::vector<T> y(N), ynew(N), tmp(N), f(N), fx(N);
  std::vector<T> k1(N), k2(N), k3(N), k4(N), k5(N), k6(N);
  std::vector<D1T<T>> fd(N);
  std::vector<int> pos, st;
  build_perm(md, pos, st);
  JacSplitT<T> J;
  BandLUT<T> B;
  B.init(N);
  std::vector<T> Z[3];
  for (int r = 0; r < 3; ++r) Z[r].assign(N, T(0.0));
  T Cinv[3][3];
  initial_conditions(md, x, y.data());
  SolveStats stats;
  size_t jo = 0;
  while (jo < xout.size() && xout[jo] <= x) { emit(int(jo), x, y.data()); ++jo; }
  double h = 1e-3;
  std::vector<T> pb(N);
  auto wsolve = [&](T* b) {  // b <- A^{-1} b (state order)
    for (int p = 0; p < N; ++p) pb[p] = b[st[p]];
    B.solve(pb.data());
    for (int p = 0; p < N; ++p) b[st[p]] = pb[p];
    T t[3] = {0, 0, 0};
    for (int r = 0; r < 3; ++r)
      for (int i = 0; i < N; ++i) t[r] += J.W[r][i] * b[i];
    T s[3];
    for (int r = 0; r < 3; ++r) s[r] = Cinv[r][0] * t[0] + Cinv[r][1] * t[1] + Cinv[r][2] * t[2];
    for (int i = 0; i < N; ++i) b[i] += Z[0][i] * s[0] + Z[1][i] * s[1] + Z[2][i] * s[2];
  };
  while (x < xend) {
    double target = jo < xout.size() ? std::min(xout[jo], xend) : xend;
    bool landing = false;
    double hs = h;
    if (x + hs >= target - 1e-14 * std::fabs(target)) { hs = target - x; landing = true; }
    // Jacobian split, explicit x-derivative, factorisation
    jacobian_split(md, x, J);
    hierarchy_rhs<D1T<T>>(md, D1(x, 1.0), y.data(), fd.data());
    for (int i = 0; i < N; ++i) { f[i] = fd[i].v; fx[i] = fd[i].d; }
    B.zero();
    double inv = 1.0 / (hs * R::gam);
    for (int p = 0; p < N; ++p) B.at(p, p) = inv;
    for (auto& e : J.L) {
      int pr = pos[e.r], pc = pos[e.c];
      if (std::abs(pr - pc) > 2) throw std::runtime_error("band violation");
      B.at(pr, pc) -= e.v;
    }
    if (!B.factor()) { stats.status = 4; return stats; }
    for (int r = 0; r < 3; ++r) {
      for (int i = 0; i < N; ++i) Z[r][i] = J.U[r][i];
      for (int p = 0; p < N; ++p) pb[p] = Z[r][st[p]];
      B.solve(pb.data());
      for (int p = 0; p < N; ++p) Z[r][st[p]] = pb[p];
    }
    T Cm[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        T s = 0.0;
        for (int i = 0; i < N; ++i) s += J.W[r][i] * Z[c][i];
        Cm[r][c] = (r == c ? 1.0 : 0.0) - s;
      }
    {
      T det = Cm[0][0] * (Cm[1][1] * Cm[2][2] - Cm[1][2] * Cm[2][1]) -
                   Cm[0][1] * (Cm[1][0] * Cm[2][2] - Cm[1][2] * Cm[2][0]) +
                   Cm[0][2] * (Cm[1][0] * Cm[2][1] - Cm[1][1] * Cm[2][0]);
      if (val(det) == 0.0 || !(val(det) == val(det))) { stats.status = 4; return stats; }
      Cinv[0][0] = (Cm[1][1] * Cm[2][2] - Cm[1][2] * Cm[2][1]) / det;
      Cinv[0][1] = (Cm[0][2] * Cm[2][1] - Cm[0][1] * Cm[2][2]) / det;
      Cinv[0][2] = (Cm[0][1] * Cm[1][2] - Cm[0][2] * Cm[1][1]) / det;
      Cinv[1][0] = (Cm[1][2] * Cm[2][0] - Cm[1][0] * Cm[2][2]) / det;
      Cinv[1][1] = (Cm[0][0] * Cm[2][2] - Cm[0][2] * Cm[2][0]) / det;
      Cinv[1][2] = (Cm[0][2] * Cm[1][0] - Cm[0][0] * Cm[1][2]) / det;
      Cinv[2][0] = (Cm[1][0] * Cm[2][1] - Cm[1][1] * Cm[2][0]) / det;
      Cinv[2][1] = (Cm[0][1] * Cm[2][0] - Cm[0][0] * Cm[2][1]) / det;
      Cinv[2][2] = (Cm[0][0] * Cm[1][1] - Cm[0][1] * Cm[1][0]) / det;
    }
    double hd1 = hs * R::d1, hd2 = hs * R::d2, hd3 = hs * R::d3, hd4 = hs * R::d4;
    double ih = 1.0 / hs;
    RhsInfo info;
    for (int i = 0; i < N; ++i) k1[i] = f[i] + hd1 * fx[i];
    wsolve(k1.data());
    for (int i = 0; i < N; ++i) tmp[i] = y[i] + R::a21 * k1[i];
    hierarchy_rhs<T>(md, x + R::c2 * hs, tmp.data(), f.data(), &info);
    stats.rsa += info.rsa;
    for (int i = 0; i < N; ++i) k2[i] = f[i] + hd2 * fx[i] + R::C21 * ih * k1[i];
    wsolve(k2.data());
    for (int i = 0; i < N; ++i) tmp[i] = y[i] + R::a31 * k1[i] + R::a32 * k2[i];
    hierarchy_rhs<T>(md, x + R::c3 * hs, tmp.data(), f.data(), &info);
    stats.rsa += info.rsa;
    for (int i = 0; i < N; ++i) k3[i] = f[i] + hd3 * fx[i] + ih * (R::C31 * k1[i] + R::C32 * k2[i]);
    wsolve(k3.data());
    for (int i = 0; i < N; ++i) tmp[i] = y[i] + R::a41 * k1[i] + R::a42 * k2[i] + R::a43 * k3[i];
    hierarchy_rhs<T>(md, x + R::c4 * hs, tmp.data(), f.data(), &info);
    stats.rsa += info.rsa;
    for (int i = 0; i < N; ++i)
      k4[i] = f[i] + hd4 * fx[i] + ih * (R::C41 * k1[i] + R::C42 * k2[i] + R::C43 * k3[i]);
    wsolve(k4.data());
    for (int i = 0; i < N; ++i) tmp[i] = y[i] + R::a51 * k1[i] + R::a52 * k2[i] + R::a53 * k3[i] + R::a54 * k4[i];
    double xn = landing ? target : x + hs;
    hierarchy_rhs<T>(md, xn, tmp.data(), f.data(), &info);
    stats.rsa += info.rsa;
    for (int i = 0; i < N; ++i)
      k5[i] = f[i] + ih * (R::C51 * k1[i] + R::C52 * k2[i] + R::C53 * k3[i] + R::C54 * k4[i]);
    wsolve(k5.data());
    for (int i = 0; i < N; ++i) tmp[i] += k5[i];
    hierarchy_rhs<T>(md, xn, tmp.data(), f.data(), &info);
    stats.rsa += info.rsa;
    for (int i = 0; i < N; ++i)
      k6[i] = f[i] + ih * (R::C61 * k1[i] + R::C62 * k2[i] + R::C63 * k3[i] + R::C64 * k4[i] + R::C65 * k5[i]);
    wsolve(k6.data());
    double en = 0.0;
    bool finite = true;
    for (int i = 0; i < N; ++i) {
      ynew[i] = tmp[i] + k6[i];
      double sc = abstol + reltol * std::max(std::fabs(val(y[i])), std::fabs(val(ynew[i])));
      double e = val(k6[i]) / sc;
      en += e * e;
      if (!std::isfinite(val(ynew[i]))) finite = false;
    }
    en = std::sqrt(en / N);
    if (!finite || !(en == en)) en = 1e10;
    double fac = 0.9 * std::pow(std::max(en, 1e-12), -0.25);
    fac = std::min(6.0, std::max(0.2, fac));
    if (en <= 1.0) {
      x = xn;
      std::swap(y, ynew);
      if (rsa_switch(md, x)) rsa_overwrite(md, x, y.data());
      ++stats.steps;
      while (jo < xout.size() && xout[jo] <= x + 1e-14 * std::fabs(x)) { emit(int(jo), xout[jo], y.data()); ++jo; }
      double hp = hs * fac;
      h = landing ? std::max(h, hp) : hp;
    } else {
      ++stats.rejects;
      h = hs * std::min(1.0, fac);
      if (h < 1e-14) { stats.status = 2; return stats; }
    }
    if (stats.steps + stats.rejects > maxsteps) { stats.status = 1; return stats; }
  }
  return stats;
}

// --------------------------------------------------------- spherical j_l ---
// j_l(x) for l = 0..L at one x: upward recurrence from the closed forms of
// j_0 and j_1 while l <= x (the oscillatory region, where it is stable), and
// above the turning point the ratios j_l / j_{l+1} from a downward
// recurrence started well past max(L, x).
inline void sph_bessel_all(int L, double x, double* out) {
  if (x <= 1.4901161193847656e-8) {  // sqrt(eps): SpecialFunctions' small-x branch
    out[0] = 1.0;
    for (int l = 1; l <= L; ++l) out[l] = 0.0;
    return;
  }
  double s = std::sin(x), c = std::cos(x);
  double j0 = s / x, j1 = s / (x * x) - c / x;
  out[0] = j0;
  if (L >= 1) out[1] = j1;
  int lt = std::min(L, int(std::floor(x)));
  for (int l = 1; l < lt; ++l) out[l + 1] = (2.0 * l + 1.0) / x * out[l] - out[l - 1];
  if (lt >= L) return;
  int ls = std::max(L, int(std::ceil(x))) + 20 + int(std::ceil(10.0 * std::cbrt(x)));
  std::vector<double> r(ls + 2, 0.0);
  // r_l = j_l / j_{l+1};  r_{l} = (2l+3)/x - 1/r_{l+1}
  double rl = (2.0 * ls + 3.0) / x;
  for (int l = ls - 1; l >= lt; --l) {
    rl = (2.0 * l + 3.0) / x - 1.0 / rl;
    if (l <= L) r[l] = rl;
  }
  if (ls - 1 < lt) r[lt] = rl;
  for (int l = lt; l < L; ++l) {
    out[l + 1] = out[l] / r[l];
  }
}

}  // namespace orc
