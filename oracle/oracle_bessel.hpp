// Oracle (test infrastructure only): moments of the spherical Bessel
// functions, I_m(x) = int_0^x t^m j_n(t) dt, their cubic B-spline table and
// the Filon-type integral of a local quadratic times j_n(k t), restated from
// Bolt.jl src/bessel/moments.jl, interpolator.jl and integrator.jl.
//
// The reference evaluates the table nodes below x = 50 with a Weniger
// transformation of 1F2 in Double64 (weniger.jl, adapted from
// HypergeometricFunctions.jl).  The oracle restates the value, not that
// algorithm: those nodes come from composite Gauss-Legendre quadrature of
// t^m j_n(t) (the first unit of t in u = sqrt(t), where t^m for half-integer
// m is not smooth), which converges to the same number.  The Maclaurin
// series (moments.jl:87-92, weniger.jl:238-248) and the Lommel-function
// asymptotic (moments.jl:4-20,56-73) are restated as published: the closed
// form of int_0^x t^mu J_nu(t) dt through the Lommel function S_{mu,nu}
// (Watson, Treatise on the Theory of Bessel Functions, sec. 5.13) with the
// large-argument expansion of S_{mu,nu} (DLMF sec. 11.9), for
// mu = m - 1/2, nu = n + 1/2.
#pragma once

#include <cmath>
#include <vector>

#include "oracle_common.hpp"

namespace orc {

// j_n(t) of one order; n = -1 gives cos(t) / t (= J_{-1/2} sqrt(pi / 2t)).
// Power series below t = 1, upward recurrence from j_0, j_1 where t >= n,
// otherwise the ratios r_l = j_l / j_{l+1} by the backward recurrence
// r_l = (2l + 3) / t - 1 / r_{l+1} anchored on j_floor(t).
inline double sphj1(int n, double t) {
  if (n < 0) return std::cos(t) / t;
  if (t == 0.0) return n == 0 ? 1.0 : 0.0;
  if (t < 1.0) {
    double pre = 1.0;
    for (int i = 1; i <= n; ++i) pre *= t / (2.0 * i + 1.0);
    double term = 1.0, s = 1.0;
    for (int k = 1; k < 80; ++k) {
      term *= -t * t / (2.0 * k * (2.0 * n + 2.0 * k + 1.0));
      s += term;
      if (std::fabs(term) < 1e-18 * std::fabs(s)) break;
    }
    return pre * s;
  }
  const double sn = std::sin(t), cs = std::cos(t);
  const double j0 = sn / t, j1 = sn / (t * t) - cs / t;
  if (n == 0) return j0;
  if (n == 1) return j1;
  if (t >= n) {
    double a = j0, b = j1;
    for (int l = 1; l < n; ++l) {
      double c = (2.0 * l + 1.0) / t * b - a;
      a = b;
      b = c;
    }
    return b;
  }
  const int lt = int(std::floor(t));
  double a = j0, b = j1;
  for (int l = 1; l < lt; ++l) {
    double c = (2.0 * l + 1.0) / t * b - a;
    a = b;
    b = c;
  }
  const int ls = n + 20 + int(std::ceil(10.0 * std::cbrt(t)));
  double r = (2.0 * ls + 3.0) / t, prod = 1.0;
  for (int l = ls - 1; l >= lt; --l) {
    r = (2.0 * l + 3.0) / t - 1.0 / r;
    if (l < n) prod /= r;
  }
  return b * prod;
}

// log((2n + 1)!!)
inline double log_dfact(int n) { return std::lgamma(2.0 * n + 2.0) - n * std::log(2.0) - std::lgamma(n + 1.0); }

// Maclaurin series (the 1F2 of moments.jl:87-92 written term by term):
// I_m(x) = x^{n+m+1} / ((n+m+1)(2n+1)!!) sum_k a_k, a_0 = 1,
// a_k = -a_{k-1} x^2 (n+m+2k-1) / (2k (n+m+2k+1) (2n+2k+1)).
inline double sphj_moment_maclaurin(int n, double m, double x) {
  const double a = n + m;
  double pre;
  if (n <= 100) {
    double df = 1.0;
    for (int i = 1; i <= n; ++i) df *= 2.0 * i + 1.0;
    pre = std::pow(x, a + 1.0) / ((a + 1.0) * df);
  } else {
    pre = std::exp((a + 1.0) * std::log(x) - std::log(a + 1.0) - log_dfact(n));
  }
  double term = 1.0, s = 1.0;
  for (int k = 1; k < 2000; ++k) {
    term *= -x * x * (a + 2.0 * k - 1.0) / (2.0 * k * (a + 2.0 * k + 1.0) * (2.0 * n + 2.0 * k + 1.0));
    s += term;
    if (std::fabs(term) < 1e-17 * std::fabs(s)) break;
  }
  return pre * s;
}

// S_{p,q}(x) / x^{p-1} by its large-argument expansion: sum_j c_j, c_0 = 1,
// c_{j+1} = c_j (q^2 - (p - 1 - 2j)^2) / x^2, cut at the smallest term.
inline double lommel_series(double p, double q, double x) {
  const double ix2 = 1.0 / (x * x);
  double s = 1.0, c = 1.0;
  for (int j = 0; j < 80; ++j) {
    double f = p - 1.0 - 2.0 * j;
    double cn = c * (q * q - f * f) * ix2;
    if (cn == 0.0) break;
    if (std::fabs(cn) >= std::fabs(c)) break;
    c = cn;
    s += c;
    if (std::fabs(c) < 1e-18 * std::fabs(s)) break;
  }
  return s;
}

// Gamma(a) / Gamma(b) for a > 0 (0 where b is a pole).
inline double gamma_ratio(double a, double b) {
  if (b <= 0.0 && b == std::floor(b)) return 0.0;
  if (a < 150.0 && std::fabs(b) < 150.0) return std::tgamma(a) / std::tgamma(b);
  double sg = 1.0;
  if (b < 0.0) sg = (long(std::ceil(-b)) % 2 == 1) ? -1.0 : 1.0;
  return sg * std::exp(std::lgamma(a) - std::lgamma(b));
}

// The limit of I_m(x) as x -> infinity where it exists (the constant of the
// Lommel form): sqrt(pi) 2^{m-1} Gamma((n+m+1)/2) / Gamma((n-m)/2 + 1).
inline double sphj_moment_const(int n, double m) {
  return std::sqrt(M_PI) * std::pow(2.0, m - 1.0) * gamma_ratio(0.5 * (n + m + 1.0), 0.5 * (n - m) + 1.0);
}

// Large-argument form: I_m(x) = P + (m+n-1) x^{m-1} j_n(x) S_{m-3/2,n-1/2}/x^{m-5/2}
//                                 - x^m j_{n-1}(x) S_{m-1/2,n+1/2}/x^{m-3/2}.
inline double sphj_moment_asymp(int n, double m, double x) {
  const double s1 = lommel_series(m - 1.5, n - 0.5, x);
  const double s2 = lommel_series(m - 0.5, n + 0.5, x);
  const double xm = std::pow(x, m);
  return sphj_moment_const(n, m) + (m + n - 1.0) * (xm / x) * sphj1(n, x) * s1 - xm * sphj1(n - 1, x) * s2;
}

struct GL20 {
  std::vector<double> x, w;
  GL20() { gauss_legendre(20, x, w); }
};
inline const std::vector<double>& gl20(int which) {
  static const GL20 g;  // initialised once, thread-safe
  return which == 0 ? g.x : g.w;
}

// int_a^b t^m j_n(t) dt, 20-point Gauss-Legendre on panels of width
// <= 0.5, narrowed below the turning point where the integrand grows like
// t^(n+m) (for a >= 1, or integer m: the integrand is smooth on [a, b]).
inline double sphj_moment_panels(int n, double m, double a, double b) {
  if (!(b > a)) return 0.0;
  const std::vector<double>& gx = gl20(0);
  const std::vector<double>& gw = gl20(1);
  const double tfl = (n + 1.0) / 100.0, rate = 3.0 / (n + std::fabs(m) + 1.0);
  double s = 0.0, t0 = a;
  while (t0 < b) {
    double w = std::min(0.5, rate * std::max(t0, tfl));
    double t1 = (b - t0 <= 1.5 * w) ? b : t0 + w;
    double h = t1 - t0, mid = t0 + 0.5 * h, ps = 0.0;
    t0 = t1;
    for (int g = 0; g < 20; ++g) {
      double t = mid + 0.5 * h * gx[g];
      ps += gw[g] * std::pow(t, m) * sphj1(n, t);
    }
    s += 0.5 * h * ps;
  }
  return s;
}

// int_0^x t^m j_n(t) dt by quadrature: [0, min(x, 1)] as int 2 u^{2m+1} j_n(u^2) du,
// the rest in t.
inline double sphj_moment_quad(int n, double m, double x) {
  const std::vector<double>& gx = gl20(0);
  const std::vector<double>& gw = gl20(1);
  const double x1 = std::min(x, 1.0), u1 = std::sqrt(x1);
  double s = 0.0;
  const int npu = 4;
  const double hu = u1 / npu;
  for (int p = 0; p < npu; ++p) {
    double mid = (p + 0.5) * hu, ps = 0.0;
    for (int g = 0; g < 20; ++g) {
      double u = mid + 0.5 * hu * gx[g];
      ps += gw[g] * 2.0 * std::pow(u, 2.0 * m + 1.0) * sphj1(n, u * u);
    }
    s += 0.5 * hu * ps;
  }
  return s + sphj_moment_panels(n, m, x1, x);
}

// Argument above which the table nodes take the large-argument form (the
// reference's weniger_cut = 50, interpolator.jl:81, raised with the order
// for high orders, where the expansion needs x well above n).
inline double moment_asymp_cut(int n) { return std::max(50.0, 4.0 * n); }

// The moment by range: series below x = 2, quadrature up to the cut, the
// large-argument form above.  method 1/2/3 forces series/asymptotic/quadrature.
inline double sphj_moment(int n, double m, double x, int method = 0) {
  if (method == 1) return sphj_moment_maclaurin(n, m, x);
  if (method == 2) return sphj_moment_asymp(n, m, x);
  if (method == 3) return sphj_moment_quad(n, m, x);
  if (x <= 2.0) return sphj_moment_maclaurin(n, m, x);
  if (x < moment_asymp_cut(n)) return sphj_moment_quad(n, m, x);
  return sphj_moment_asymp(n, m, x);
}

// sph_bessel_interpolator(nu, order, kmin, kmax, N) (interpolator.jl:81-94)
// and its call (interpolator.jl:67-75): moments m = 0..order-1 on N uniform
// nodes of [kmin, kmax], one cubic B-spline per order; the Maclaurin series
// below kmin, the large-argument form above kmax.
struct MomentTableO {
  int n = 0, order = 3;
  double kmin = 0.0, kmax = 1.0;
  std::vector<SplineT<double>> sp;

  // Node values: at and above the cut the large-argument form; below it
  // I_m(x_0) (series for x_0 <= 2, else quadrature from 0) plus the
  // integrals over the node intervals, accumulated in long double.
  MomentTableO(int n_, int order_, double kmin_, double kmax_, int N) : n(n_), order(order_), kmin(kmin_), kmax(kmax_) {
    const double h = (kmax - kmin) / (N - 1);
    const double cut = moment_asymp_cut(n);
    auto node = [&](int i) { return (i == N - 1) ? kmax : kmin + i * h; };
    std::vector<std::vector<double>> y(order, std::vector<double>(N));
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < N; ++i) {
      const double x = node(i);
      for (int m = 0; m < order; ++m) {
        if (x >= cut) y[m][i] = sphj_moment_asymp(n, m, x);
        else if (i == 0) y[m][i] = x <= 2.0 ? sphj_moment_maclaurin(n, m, x) : sphj_moment_quad(n, m, x);
        else y[m][i] = sphj_moment_panels(n, m, node(i - 1), x);  // the interval, summed below
      }
    }
    for (int m = 0; m < order; ++m) {
      long double acc = 0.0L;
      for (int i = 0; i < N && node(i) < cut; ++i) {
        acc += y[m][i];
        y[m][i] = double(acc);
      }
    }
    for (int m = 0; m < order; ++m) sp.emplace_back(y[m], kmin, h);
  }
  void eval(double x, double* out) const {
    for (int m = 0; m < order; ++m) {
      if (x >= kmin && x <= kmax) out[m] = sp[m](x);
      else if (x > kmax) out[m] = sphj_moment_asymp(n, m, x);
      else out[m] = sphj_moment_maclaurin(n, m, x);
    }
  }
};

// integrate_sph_bessel_filon(f, f', f'', k, a, b, itp) (integrator.jl:7-19):
// int_a^b p(t) j_n(k t) dt for the quadratic p with p(a) = f, p'(a) = f',
// p'' = f'', written p = c0 + c1 t + c2 t^2, with
// int_a^b t^j j_n(k t) dt = k^{-j-1} (I_j(k b) - I_j(k a)).
inline double filon_segment(const MomentTableO& T, double f, double fp, double fpp, double k, double a, double b) {
  const double c2 = 0.5 * fpp, c1 = fp - a * fpp, c0 = f - a * fp + 0.5 * a * a * fpp;
  double Ia[4], Ib[4];
  T.eval(k * a, Ia);
  T.eval(k * b, Ib);
  const double ik = 1.0 / k;
  return c0 * ik * (Ib[0] - Ia[0]) + c1 * ik * ik * (Ib[1] - Ia[1]) + c2 * ik * ik * ik * (Ib[2] - Ia[2]);
}

// The piecewise form (_loop_integrate_sph_bessel_filon, integrator.jl:25-38,
// summed over consecutive segments [t_i, t_{i+1}] with the local quadratic
// at t_i).
inline double filon_piecewise(const MomentTableO& T, int nt, const double* t, const double* f, const double* fp,
                              const double* fpp, double k) {
  double s = 0.0;
  for (int i = 0; i + 1 < nt; ++i) s += filon_segment(T, f[i], fp[i], fpp[i], k, t[i], t[i + 1]);
  return s;
}

}  // namespace orc
