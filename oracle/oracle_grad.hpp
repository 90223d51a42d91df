// Oracle (test infrastructure only): the number-type-generic tail of the
// pipeline -- plin (spectra.jl:163-198) and the line-of-sight C_l
// (spectra.jl:49-160) -- used with T = double by the plain oracle and with
// T = G6 by the gradient oracle, which restates the reference's ForwardDiff
// gradient (examples/plot_deriv_cl.jl): every quantity carries its partial
// derivatives with respect to theta = (h, omega_b, omega_c, n_s, A_s,
// Sigma m_nu), while the quantities the reference wraps in assume_nondual
// keep none -- the k grids (spectra.jl:60-68), the Bessel grid's upper end
// (spectra.jl:49-52) and RECFAST's two switch redshifts (recfast.jl:451,456).
// Step sizes of the ODE solvers are plain numbers chosen from the values, so
// the derivatives are those of the discrete solution on the value's steps.
#pragma once
#include <omp.h>

#include "oracle_perturb.hpp"

namespace orc {

inline double spline_at(const Spline& s, double u) { return s(u); }
template <int P> inline Dual<P> spline_at(const Spline& s, const Dual<P>& u) { return s.at(u); }

// plin (spectra.jl:163-198) for one k at x.
template <class T>
T plin_of(const CosmoT<T>& C, double k, int nq, int lg, int lnu, int lmnu, double x, double reltol, double abstol,
          int* status) {
  const BackgroundT<T>& bg = *C.bg;
  const ParamsT<T>& p = C.par;
  ModeT<T> md(&C, k, lg, lnu, lmnu, nq);
  std::vector<T> u(md.N);
  std::vector<double> xo(1, x);
  SolveStats s = solve_mode(md, reltol, abstol, xo, [&](int, double, const T* y) {
    std::copy(y, y + md.N, u.begin());
  });
  if (status) *status = s.status;
  double a = std::exp(x);
  std::vector<T> M0(nq), M1(nq), M2(nq);
  for (int i = 0; i < nq; ++i) { M0[i] = u[md.M(0, i)]; M1[i] = u[md.M(1, i)]; M2[i] = u[md.M(2, i)]; }
  T rho, sig;
  rho_sigma(md, a, M0.data(), M2.data(), rho, sig);
  T r0 = bg.rho0M(x);
  T Mrho = rho / r0;
  T th = 0.0;
  for (int i = 0; i < nq; ++i) th += md.Bq[i] * M1[i];
  T Mth = k * th / r0;
  T dcN = u[md.iPhi + 1], dbN = u[md.iPhi + 3], vcN = u[md.iPhi + 2], vbN = u[md.iPhi + 4];
  T vmnuN = -Mth / k;
  T Tg = pow(15.0 / (M_PI * M_PI) * bg.rho_crit * p.Omega_r, 0.25);
  T nufac = (90.0 * ZETA3 / (11.0 * std::pow(M_PI, 4))) * (p.Omega_r * p.h * p.h / Tg) * pow(p.N_nu / 3.0, 0.75);
  T Omega_nu = p.Sigma_m_nu * nufac / (p.h * p.h);
  T Om = p.Omega_c + p.Omega_b + Omega_nu;
  T Hc = bg.H(x);
  T dc = dcN - 3.0 * Hc * vcN / k;
  T db = dbN - 3.0 * Hc * vbN / k;
  T dmnu = Mrho - 3.0 * Hc * vmnuN / k;
  T dm = (p.Omega_c * dc + p.Omega_b * db + Omega_nu * dmnu) / Om;
  T Pprim = p.A * pow(k / 0.05, p.n - 1.0);
  return (2.0 * M_PI * M_PI / (k * k * k)) * dm * dm * Pprim;
}

// j_l on the Bessel grid [0, argmax] (5001 points, spectra.jl:49-58) for the
// requested multipoles: jtab[il][ib].
inline void bessel_table(const int* ells, int nell, double argmax, std::vector<double>& jtab) {
  const int nb = 5001;
  const double dg = argmax / 5000.0;
  int Lmax = 0;
  for (int i = 0; i < nell; ++i) Lmax = std::max(Lmax, ells[i]);
  jtab.assign(size_t(nell) * nb, 0.0);
#pragma omp parallel
  {
    std::vector<double> all(Lmax + 1);
#pragma omp for schedule(dynamic, 16)
    for (int ib = 0; ib < nb; ++ib) {
      double xb = ib * dg;
      sph_bessel_all(Lmax, xb, all.data());
      for (int i = 0; i < nell; ++i) jtab[size_t(i) * nb + ib] = all[ells[i]];
    }
  }
}

// cltt / clte / clee (spectra.jl:84-160) on a source grid S[ik * nx + ix]
// (bilinear in (x, k), spectra.jl:21), the dense k grid kd (5000 quadratic
// k, frozen) and the Bessel grid's upper end argmax (frozen).  Any of
// tt / te / ee may be null; SE may be null when te and ee are.
template <class T>
void cl_of(const CosmoT<T>& C, const T* ST, const T* SE, const double* kg, int nk, const int* ells, int nell,
           const std::vector<double>& kd, double argmax, T* tt, T* te, T* ee) {
  const BackgroundT<T>& bg = *C.bg;
  const ParamsT<T>& par = C.par;
  const Grid& g = bg.xg;
  const int nx = g.n, nkd = int(kd.size()), nb = 5001;
  const double dg = argmax / 5000.0;
  std::vector<double> jtab;
  bessel_table(ells, nell, argmax, jtab);
  int xi = 0;
  while (xi < nx && !(g.at(xi) > -8.0)) ++xi;
  std::vector<T> yv(nx);
  std::vector<double> dx(nx);
  for (int i = xi; i < nx - 1; ++i) {
    yv[i] = bg.eta0 - bg.eta(g.at(i));
    dx[i] = g.at(i + 1) - g.at(i);
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int il = 0; il < nell; ++il) {
    int l = ells[il];
    std::vector<double> col(jtab.begin() + size_t(il) * nb, jtab.begin() + size_t(il + 1) * nb);
    Spline bes(col, 0.0, dg);
    double lfac = std::sqrt(double(int64_t(l + 2) * int64_t(l + 1) * int64_t(l) * int64_t(l - 1)));
    T stt = 0.0, ste = 0.0, see = 0.0;
    for (int m = 0; m < nkd - 1; ++m) {
      double k = (kd[m] + kd[m + 1]) / 2.0;
      double dk = kd[m + 1] - kd[m];
      int j = 0;
      if (k >= kg[nk - 1]) j = nk - 2;
      else { while (j < nk - 2 && kg[j + 1] <= k) ++j; }
      double w = (k - kg[j]) / (kg[j + 1] - kg[j]);
      const T* sT0 = ST + size_t(j) * nx;
      const T* sT1 = ST + size_t(j + 1) * nx;
      const T* sE0 = SE ? SE + size_t(j) * nx : nullptr;
      const T* sE1 = SE ? SE + size_t(j + 1) * nx : nullptr;
      T th = 0.0, ep = 0.0;
      for (int i = xi; i < nx - 1; ++i) {
        T b = spline_at(bes, k * yv[i]);
        th += b * ((1.0 - w) * sT0[i] + w * sT1[i]) * dx[i];
        if (sE0) ep += b * ((1.0 - w) * sE0[i] + w * sE1[i]) * dx[i];
      }
      ep *= lfac;
      T Pp = par.A * pow(k / 0.05, par.n - 1.0);
      stt += th * th * Pp * dk / k;
      ste += th * ep * Pp * dk / k;
      see += ep * ep * Pp * dk / k;
    }
    if (tt) tt[il] = 4.0 * M_PI * stt;
    if (te) te[il] = 4.0 * M_PI * ste;
    if (ee) ee[il] = 4.0 * M_PI * see;
  }
}

// The source grid (spectra.jl:6-42) on every x node: S[ik * nx + ix].
template <class T>
int source_grid_of(const CosmoT<T>& C, const double* kg, int nk, int lg, int lnu, int lmnu, int nq, double reltol,
                   double abstol, T* ST, T* SE, long* steps) {
  const Grid& g = C.bg->xg;
  const int nx = g.n;
  std::vector<double> xo(nx);
  for (int j = 0; j < nx; ++j) xo[j] = g.at(j);
  int worst = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : worst)
  for (int ik = 0; ik < nk; ++ik) {
    ModeT<T> md(&C, kg[ik], lg, lnu, lmnu, nq);
    std::vector<T> du(md.N);
    SolveStats s = solve_mode(md, reltol, abstol, xo, [&](int j, double x, const T* y) {
      hierarchy_rhs<T>(md, x, y, du.data());
      T st, se;
      source_functions(md, x, y, du.data(), st, se);
      ST[size_t(ik) * nx + j] = st;
      SE[size_t(ik) * nx + j] = se;
    });
    if (steps) steps[ik] = s.steps;
    worst = std::max(worst, s.status);
  }
  return worst;
}

}  // namespace orc
