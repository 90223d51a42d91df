// Oracle (test infrastructure only): a CPU FP64 restatement of Bolt.jl's
// algorithm for the Boltzmann hot path.  Nothing in the product links this
// code; tests, smoke() and the CPU-baseline leg of bench.py call it as the
// checker.  Parity is pinned against the reference's own fixtures
// (test/data/*.dat) -- see tests/test_oracle_fixtures.py.
//
// This header holds the shared pieces: unit constants, cosmological
// parameters, the cubic B-spline with Interpolations.jl's
// BSpline(Cubic(Line(OnGrid()))) semantics, Gauss-Legendre nodes, a
// first-derivative dual number and the Tsit5 integrator used by RECFAST.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- units ---
// Bolt.jl:43-51 (natural units, hbar = c = k_B = 1, lengths in Mpc).  The SI
// values are the exact 2019 SI constants and CODATA 2018 values that
// PhysicalConstants.CODATA2018 / Unitful carry; the parsec is UnitfulAstro's.
namespace si {
constexpr double c = 299792458.0;
constexpr double h_planck = 6.62607015e-34;
constexpr double hbar = h_planck / (2.0 * M_PI);
constexpr double k_B = 1.380649e-23;
constexpr double eV = 1.602176634e-19;
constexpr double Mpc = 3.0856775814913673e22;
constexpr double G = 6.67430e-11;             // CODATA 2018
constexpr double m_e = 9.1093837015e-31;      // CODATA 2018
constexpr double m_p = 1.67262192369e-27;     // CODATA 2018 (ProtonMass)
constexpr double sigma_T = 6.6524587321e-29;  // CODATA 2018
constexpr double alpha = 7.2973525693e-3;      // CODATA 2018 fine-structure constant
}  // namespace si

struct Units {
  double km_s_Mpc_100;    // 100 km/s/Mpc in Mpc^-1          (Bolt.jl:49)
  double G_natural;       // G in Mpc^2                        (Bolt.jl:50)
  double mass_natural;    // 1 eV in Mpc^-1                    (Bolt.jl:51)
  double m_H;             // proton mass in Mpc^-1             (ionization.jl:224)
  double sigma_T;         // Thomson cross-section in Mpc^2    (ionization.jl:226)
  double H0_conv;         // seconds per natural time unit     (recfast.jl:4)
  double K_conv;          // Kelvin per Mpc^-1                 (recfast.jl:5)
  Units() {
    km_s_Mpc_100 = 1e5 / si::c;
    G_natural = si::G * si::hbar / (si::c * si::c * si::c) / (si::Mpc * si::Mpc);
    mass_natural = si::eV / (si::hbar * si::c) * si::Mpc;
    m_H = si::m_p * si::c / si::hbar * si::Mpc;
    sigma_T = si::sigma_T / (si::Mpc * si::Mpc);
    H0_conv = si::Mpc / si::c;
    K_conv = si::hbar * si::c / (si::k_B * si::Mpc);
  }
};
inline const Units& units() {
  static Units u;
  return u;
}


// ------------------------------------------------------- dual numbers -----
// Dual<P>: a value and its partial derivatives along P directions, the
// arithmetic of ForwardDiff.Dual (the reference's gradient path).  Math
// functions propagate the chain rule; comparisons compare values.
template <int P>
struct Dual {
  double v = 0.0;
  double d[P] = {};
  Dual() {}
  Dual(double a) : v(a) {}  // a constant: zero partials
  static Dual seed(double a, int j) { Dual r(a); r.d[j] = 1.0; return r; }
  Dual& operator+=(const Dual& b) { v += b.v; for (int i = 0; i < P; ++i) d[i] += b.d[i]; return *this; }
  Dual& operator-=(const Dual& b) { v -= b.v; for (int i = 0; i < P; ++i) d[i] -= b.d[i]; return *this; }
  Dual& operator*=(const Dual& b) { *this = *this * b; return *this; }
  Dual& operator/=(const Dual& b) { *this = *this / b; return *this; }
  friend Dual operator+(Dual a, const Dual& b) { a += b; return a; }
  friend Dual operator-(Dual a, const Dual& b) { a -= b; return a; }
  friend Dual operator-(Dual a) { a.v = -a.v; for (int i = 0; i < P; ++i) a.d[i] = -a.d[i]; return a; }
  friend Dual operator*(const Dual& a, const Dual& b) {
    Dual r(a.v * b.v);
    for (int i = 0; i < P; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
  }
  friend Dual operator/(const Dual& a, const Dual& b) {
    Dual r(a.v / b.v);
    const double ib = 1.0 / b.v;
    for (int i = 0; i < P; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
  }
  friend Dual operator+(Dual a, double b) { a.v += b; return a; }
  friend Dual operator+(double b, Dual a) { a.v += b; return a; }
  friend Dual operator-(Dual a, double b) { a.v -= b; return a; }
  friend Dual operator-(double b, const Dual& a) { return Dual(b) - a; }
  friend Dual operator*(Dual a, double b) { a.v *= b; for (int i = 0; i < P; ++i) a.d[i] *= b; return a; }
  friend Dual operator*(double b, Dual a) { return a * b; }
  friend Dual operator/(Dual a, double b) { a.v /= b; for (int i = 0; i < P; ++i) a.d[i] /= b; return a; }
  friend Dual operator/(double b, const Dual& a) { return Dual(b) / a; }
  friend bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
  friend bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
  friend bool operator<(const Dual& a, double b) { return a.v < b; }
  friend bool operator>(const Dual& a, double b) { return a.v > b; }
  friend bool operator<=(const Dual& a, double b) { return a.v <= b; }
  friend bool operator>=(const Dual& a, double b) { return a.v >= b; }
  friend bool operator<(double a, const Dual& b) { return a < b.v; }
  friend bool operator>(double a, const Dual& b) { return a > b.v; }
  friend bool operator==(const Dual& a, double b) { return a.v == b; }
  friend bool operator!=(const Dual& a, double b) { return a.v != b; }
};
template <int P> Dual<P> chain(const Dual<P>& a, double f, double df) {
  Dual<P> r(f);
  for (int i = 0; i < P; ++i) r.d[i] = df * a.d[i];
  return r;
}
template <int P> Dual<P> exp(const Dual<P>& a) { double e = std::exp(a.v); return chain(a, e, e); }
template <int P> Dual<P> log(const Dual<P>& a) { return chain(a, std::log(a.v), 1.0 / a.v); }
template <int P> Dual<P> log10(const Dual<P>& a) { return chain(a, std::log10(a.v), 1.0 / (a.v * std::log(10.0))); }
template <int P> Dual<P> sqrt(const Dual<P>& a) { double s = std::sqrt(a.v); return chain(a, s, 0.5 / s); }
template <int P> Dual<P> tanh(const Dual<P>& a) { double t = std::tanh(a.v); return chain(a, t, 1.0 - t * t); }
template <int P> Dual<P> fabs(const Dual<P>& a) { return a.v < 0 ? -a : a; }
template <int P> Dual<P> pow(const Dual<P>& a, double b) {
  double p = std::pow(a.v, b);
  return chain(a, p, b * std::pow(a.v, b - 1.0));
}
template <int P> Dual<P> pow(double a, const Dual<P>& b) { double p = std::pow(a, b.v); return chain(b, p, p * std::log(a)); }
template <int P> Dual<P> pow(const Dual<P>& a, const Dual<P>& b) { return exp(b * log(a)); }

// The value of a number (a double is its own value).
inline double val(double a) { return a; }
template <int P> inline double val(const Dual<P>& a) { return a.v; }
// Whether a number or any of its partials is nonzero (elimination skips).
inline bool nonzero(double a) { return a != 0.0; }
template <int P> inline bool nonzero(const Dual<P>& a) {
  if (a.v != 0.0) return true;
  for (int i = 0; i < P; ++i)
    if (a.d[i] != 0.0) return true;
  return false;
}
// Sum of squares of the value and partials, and their count (error norms).
inline double sse(double a) { return a * a; }
template <int P> inline double sse(const Dual<P>& a) {
  double s = a.v * a.v;
  for (int i = 0; i < P; ++i) s += a.d[i] * a.d[i];
  return s;
}

// The parameter-gradient type of the gradient oracle: partials along
// theta = (h, omega_b, omega_c, n_s, A_s, Sigma m_nu).
constexpr int kThetaN = 6;
using G6 = Dual<kThetaN>;

inline double exp(double a) { return std::exp(a); }
inline double sqrt(double a) { return std::sqrt(a); }
inline double log(double a) { return std::log(a); }
inline double log10(double a) { return std::log10(a); }
inline double pow(double a, double b) { return std::pow(a, b); }
inline double tanh(double a) { return std::tanh(a); }
inline double fabs(double a) { return std::fabs(a); }

// ------------------------------------------------------------ dual (d/dx) --
// D1T<V>: a value of type V and its derivative in x (one direction), for the
// explicit x-derivative of the right-hand side a Rosenbrock step needs.
template <class V>
struct D1T {
  V v, d;
  D1T() : v(0.0), d(0.0) {}
  D1T(V a) : v(a), d(0.0) {}
  D1T(V a, V b) : v(a), d(b) {}
  template <class W, class = typename std::enable_if<!std::is_same<V, W>::value>::type>
  D1T(const D1T<W>& o) : v(o.v), d(o.d) {}
};
template <class V> inline D1T<V> operator+(const D1T<V>& a, const D1T<V>& b) { return {a.v + b.v, a.d + b.d}; }
template <class V> inline D1T<V> operator-(const D1T<V>& a, const D1T<V>& b) { return {a.v - b.v, a.d - b.d}; }
template <class V> inline D1T<V> operator-(const D1T<V>& a) { return {-a.v, -a.d}; }
template <class V> inline D1T<V> operator*(const D1T<V>& a, const D1T<V>& b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
template <class V> inline D1T<V> operator/(const D1T<V>& a, const D1T<V>& b) {
  return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)};
}
template <class V> inline D1T<V> operator+(const D1T<V>& a, const V& b) { return {a.v + b, a.d}; }
template <class V> inline D1T<V> operator+(const V& b, const D1T<V>& a) { return {a.v + b, a.d}; }
template <class V> inline D1T<V> operator-(const D1T<V>& a, const V& b) { return {a.v - b, a.d}; }
template <class V> inline D1T<V> operator-(const V& b, const D1T<V>& a) { return {b - a.v, -a.d}; }
template <class V> inline D1T<V> operator*(const D1T<V>& a, const V& b) { return {a.v * b, a.d * b}; }
template <class V> inline D1T<V> operator*(const V& b, const D1T<V>& a) { return {a.v * b, a.d * b}; }
template <class V> inline D1T<V> operator/(const D1T<V>& a, const V& b) { return {a.v / b, a.d / b}; }
template <class V> inline D1T<V> operator/(const V& b, const D1T<V>& a) { return {b / a.v, -b * a.d / (a.v * a.v)}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator+(const D1T<V>& a, double b) { return {a.v + b, a.d}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator+(double b, const D1T<V>& a) { return {a.v + b, a.d}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator-(const D1T<V>& a, double b) { return {a.v - b, a.d}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator-(double b, const D1T<V>& a) { return {b - a.v, -a.d}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator*(const D1T<V>& a, double b) { return {a.v * b, a.d * b}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator*(double b, const D1T<V>& a) { return {a.v * b, a.d * b}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator/(const D1T<V>& a, double b) { return {a.v / b, a.d / b}; }
template <class V, class = typename std::enable_if<!std::is_same<V, double>::value>::type>
inline D1T<V> operator/(double b, const D1T<V>& a) { return {b / a.v, -b * a.d / (a.v * a.v)}; }
template <class V> inline D1T<V> exp(const D1T<V>& a) { V e = exp(a.v); return {e, e * a.d}; }
template <class V> inline D1T<V> sqrt(const D1T<V>& a) { V s = sqrt(a.v); return {s, 0.5 * a.d / s}; }
using D1 = D1T<double>;
template <class V> inline double val(const D1T<V>& a) { return val(a.v); }
// The value part of a number of the gradient type, kept in that type.
template <class V> inline V base_of(const D1T<V>& a) { return a.v; }
inline double base_of(double a) { return a; }
template <int P> inline Dual<P> base_of(const Dual<P>& a) { return a; }

// CosmoParams (Bolt.jl:56-66).  Sigma_m_nu is in Mpc^-1 like the reference.
// T = double, or a dual number carrying derivatives with respect to theta.
template <class T>
struct ParamsT {
  T h = 0.7, Omega_r = 5.0469e-5, Omega_b = 0.046, Omega_c = 0.224;
  T A = 2.097e-9, n = 1.0, Y_p = 0.24, N_nu = 3.046, Sigma_m_nu = 0.0;
};
using Params = ParamsT<double>;

// ---------------------------------------------------------------- spline ---
// Uniform grid x_j = (i0 + j) / M  (j = 0..n-1) reproducing Julia's
// correctly-rounded range values for start:1/M:stop.
struct Grid {
  int n = 0;
  double x0 = 0.0, h = 0.0;
  long i0 = 0;
  long M = 0;  // 0 => x_j = x0 + j*h
  double at(int j) const {
    if (M > 0) return double(i0 + j) / double(M);
    return x0 + j * h;
  }
  static Grid range(double start, double step, double stop) {
    Grid g;
    double inv = 1.0 / step;
    double Mr = std::round(inv);
    g.n = int(std::floor((stop - start) / step + 1e-9)) + 1;
    g.h = step;
    g.x0 = start;
    if (std::fabs(inv - Mr) < 1e-9 * Mr && std::fabs(start * Mr - std::round(start * Mr)) < 1e-6) {
      g.M = long(Mr);
      g.i0 = long(std::round(start * Mr));
    }
    return g;
  }
};

// Interpolations.jl 0.13 scale(interpolate(y, BSpline(Cubic(Line(OnGrid())))), r)
// (util.jl:11).  Coefficients are padded by one on each side; the boundary
// rows impose a vanishing second derivative at the first and last data point
// (c[0] - 2c[1] + c[2] = 0), which fixes c[1] = y[0] and c[n] = y[n-1].
// T is the number type of the data (double, or a dual number when the
// tables carry parameter derivatives); the abscissa is always a double.
template <class T>
struct SplineT {
  double x0 = 0.0, h = 1.0;
  int n = 0;
  std::vector<T> c;  // n + 2

  SplineT() {}
  SplineT(const std::vector<T>& y, double x0_, double h_) { build(y, x0_, h_); }
  void build(const std::vector<T>& y, double x0_, double h_) {
    x0 = x0_;
    h = h_;
    n = int(y.size());
    c.assign(n + 2, T(0.0));
    if (n == 1) { c[0] = c[1] = c[2] = y[0]; return; }
    c[1] = y[0];
    c[n] = y[n - 1];
    // interior: c[i-1]/6 + 2/3 c[i] + c[i+1]/6 = y[i-1], i = 2..n-1
    int m = n - 2;
    if (m > 0) {
      std::vector<double> cp(m);
      std::vector<T> dp(m);
      for (int r = 0; r < m; ++r) {
        int i = r + 2;
        T rhs = y[i - 1];
        if (r == 0) rhs -= c[1] / 6.0;
        if (r == m - 1) rhs -= c[n] / 6.0;
        double b = 2.0 / 3.0, a = 1.0 / 6.0, cc = 1.0 / 6.0;
        if (r == 0) {
          cp[r] = cc / b;
          dp[r] = rhs / b;
        } else {
          double den = b - a * cp[r - 1];
          cp[r] = cc / den;
          dp[r] = (rhs - a * dp[r - 1]) / den;
        }
      }
      c[m + 1] = dp[m - 1];
      for (int r = m - 2; r >= 0; --r) c[r + 2] = dp[r] - cp[r] * c[r + 3];
    }
    c[0] = 2.0 * c[1] - c[2];
    c[n + 1] = 2.0 * c[n] - c[n - 1];
  }
  inline void locate(double x, int& i, double& t) const {
    double u = (x - x0) / h;
    double fl = std::floor(u);
    if (fl < 0) fl = 0;
    if (fl > n - 2) fl = n - 2;
    i = int(fl);
    t = u - fl;
  }
  T operator()(double x) const {
    int i; double t; locate(x, i, t);
    double s = 1.0 - t;
    double w0 = s * s * s / 6.0;
    double w1 = 2.0 / 3.0 - t * t + t * t * t / 2.0;
    double w2 = 2.0 / 3.0 - s * s + s * s * s / 2.0;
    double w3 = t * t * t / 6.0;
    return c[i] * w0 + c[i + 1] * w1 + c[i + 2] * w2 + c[i + 3] * w3;
  }
  T d1(double x) const {
    int i; double t; locate(x, i, t);
    double s = 1.0 - t;
    double w0 = -s * s / 2.0;
    double w1 = -2.0 * t + 1.5 * t * t;
    double w2 = 2.0 * s - 1.5 * s * s;
    double w3 = t * t / 2.0;
    return (c[i] * w0 + c[i + 1] * w1 + c[i + 2] * w2 + c[i + 3] * w3) / h;
  }
  T d2(double x) const {
    int i; double t; locate(x, i, t);
    double w0 = 1.0 - t;
    double w1 = -2.0 + 3.0 * t;
    double w2 = 1.0 - 3.0 * t;
    double w3 = t;
    return (c[i] * w0 + c[i + 1] * w1 + c[i + 2] * w2 + c[i + 3] * w3) / (h * h);
  }
  D1T<T> eval(D1 x) const { return D1T<T>((*this)(x.v), d1(x.v) * x.d); }
  T eval(double x) const { return (*this)(x); }
  // a spline of plain numbers at an abscissa that carries parameter
  // derivatives (the Bessel argument k (eta0 - eta(x)) under ForwardDiff)
  template <int P> Dual<P> at(const Dual<P>& x) const { return chain(x, val((*this)(x.v)), val(d1(x.v))); }
};
using Spline = SplineT<double>;

// spline_d_x / spline_d_x2 (util.jl:12-13): re-spline the gradient / Hessian
// of a spline sampled at the grid nodes.
template <class T>
inline SplineT<T> spline_dx(const SplineT<T>& s, const Grid& g) {
  std::vector<T> y(g.n);
  for (int j = 0; j < g.n; ++j) y[j] = s.d1(g.at(j));
  return SplineT<T>(y, s.x0, s.h);
}
template <class T>
inline SplineT<T> spline_dx2(const SplineT<T>& s, const Grid& g) {
  std::vector<T> y(g.n);
  for (int j = 0; j < g.n; ++j) y[j] = s.d2(g.at(j));
  return SplineT<T>(y, s.x0, s.h);
}

// ------------------------------------------------------- Gauss-Legendre ----
// FastGaussQuadrature.gausslegendre(n): nodes ascending on [-1, 1].
inline void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      double dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) {
        // one more polish step
        p0 = 1.0; p1 = z;
        for (int k = 2; k <= n; ++k) {
          double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1; p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
        break;
      }
    }
  }
}

// ------------------------------------------------------------ Tsit5 --------
// Tsitouras (2011) 5(4) pair with a standard step-size controller, the error
// norm of OrdinaryDiffEq (RMS of err / (abstol + reltol*max|u|)), and
// landing on every requested output time.  Dense output between stored steps
// is cubic Hermite (used only where a solution is queried off the landing
// points).  Integrates forward or backward in t.  The state may carry
// parameter derivatives (T a dual number): the step sizes are plain numbers
// chosen from the values, so the derivatives are those of the discrete
// solution on the value's steps.
template <class T>
struct Tsit5SolT {
  int dim = 0;
  std::vector<double> t;   // accepted step end points (incl. start)
  std::vector<T> y;        // dim per point
  std::vector<T> f;        // dim per point
  double t0() const { return t.front(); }
  double t1() const { return t.back(); }
  void at(double tq, T* out) const {
    int n = int(t.size());
    bool fwd = t.back() > t.front();
    // binary search for interval
    int lo = 0, hi = n - 1;
    if (n == 1) { for (int d = 0; d < dim; ++d) out[d] = y[d]; return; }
    while (hi - lo > 1) {
      int mid = (lo + hi) / 2;
      bool right = fwd ? (t[mid] <= tq) : (t[mid] >= tq);
      if (right) lo = mid; else hi = mid;
    }
    double ta = t[lo], tb = t[lo + 1], hh = tb - ta;
    if (tq == ta) { for (int d = 0; d < dim; ++d) out[d] = y[lo * dim + d]; return; }
    if (tq == tb) { for (int d = 0; d < dim; ++d) out[d] = y[(lo + 1) * dim + d]; return; }
    double s = (tq - ta) / hh;
    double h00 = (1 + 2 * s) * (1 - s) * (1 - s), h10 = s * (1 - s) * (1 - s);
    double h01 = s * s * (3 - 2 * s), h11 = s * s * (s - 1);
    for (int d = 0; d < dim; ++d)
      out[d] = h00 * y[lo * dim + d] + h10 * hh * f[lo * dim + d] + h01 * y[(lo + 1) * dim + d] +
               h11 * hh * f[(lo + 1) * dim + d];
  }
  T at(double tq, int idx) const {
    std::vector<T> o(dim);
    at(tq, o.data());
    return o[idx];
  }
};
using Tsit5Sol = Tsit5SolT<double>;

template <class T>
using RhsT = std::function<void(double t, const T* y, T* dy)>;
using Rhs = RhsT<double>;

template <class T>
inline Tsit5SolT<T> tsit5(const RhsT<T>& f, int dim, const T* y0, double ta, double tb, double reltol,
                          double abstol, const std::vector<double>& stops) {
  static const double c2 = 0.161, c3 = 0.327, c4 = 0.9, c5 = 0.9800255409045097;
  static const double a21 = 0.161;
  static const double a31 = -0.008480655492356989, a32 = 0.335480655492357;
  static const double a41 = 2.897153057105493, a42 = -6.359448489975075, a43 = 4.3622954328695815;
  static const double a51 = 5.325864828439257, a52 = -11.748883564062828, a53 = 7.4955393428898365,
                      a54 = -0.09249506636175525;
  static const double a61 = 5.86145544294642, a62 = -12.92096931784711, a63 = 8.159367898576159,
                      a64 = -0.071584973281401, a65 = -0.028269050394068383;
  static const double a71 = 0.09646076681806523, a72 = 0.01, a73 = 0.4798896504144996,
                      a74 = 1.379008574103742, a75 = -3.290069515436081, a76 = 2.324710524099774;
  static const double e1 = -0.00178001105222577714, e2 = -0.0008164344596567469,
                      e3 = 0.007880878010261995, e4 = -0.1447110071732629, e5 = 0.5823571654525552,
                      e6 = -0.45808210592918697, e7 = 1.0 / 66.0;
  Tsit5SolT<T> sol;
  sol.dim = dim;
  double dir = tb > ta ? 1.0 : -1.0;
  std::vector<T> y(y0, y0 + dim), k1(dim), k2(dim), k3(dim), k4(dim), k5(dim), k6(dim), k7(dim),
      tmp(dim), ynew(dim);
  // landing points strictly inside (ta, tb], sorted in the direction of travel
  std::vector<double> land;
  for (double s : stops)
    if ((s - ta) * dir > 0 && (tb - s) * dir > 0) land.push_back(s);
  land.push_back(tb);
  std::sort(land.begin(), land.end(), [dir](double a, double b) { return a * dir < b * dir; });
  f(ta, y.data(), k1.data());
  sol.t.push_back(ta);
  sol.y.insert(sol.y.end(), y.begin(), y.end());
  sol.f.insert(sol.f.end(), k1.begin(), k1.end());
  double t = ta;
  double hmag = std::fabs(tb - ta) * 1e-6;
  size_t li = 0;
  int steps = 0;
  while (li < land.size()) {
    double target = land[li];
    double remain = (target - t) * dir;
    bool landing = false;
    double hs = hmag;
    if (hs >= remain * (1 - 1e-12)) { hs = remain; landing = true; }
    double hh = hs * dir;
    for (int d = 0; d < dim; ++d) tmp[d] = y[d] + hh * a21 * k1[d];
    f(t + c2 * hh, tmp.data(), k2.data());
    for (int d = 0; d < dim; ++d) tmp[d] = y[d] + hh * (a31 * k1[d] + a32 * k2[d]);
    f(t + c3 * hh, tmp.data(), k3.data());
    for (int d = 0; d < dim; ++d) tmp[d] = y[d] + hh * (a41 * k1[d] + a42 * k2[d] + a43 * k3[d]);
    f(t + c4 * hh, tmp.data(), k4.data());
    for (int d = 0; d < dim; ++d)
      tmp[d] = y[d] + hh * (a51 * k1[d] + a52 * k2[d] + a53 * k3[d] + a54 * k4[d]);
    f(t + c5 * hh, tmp.data(), k5.data());
    for (int d = 0; d < dim; ++d)
      tmp[d] = y[d] + hh * (a61 * k1[d] + a62 * k2[d] + a63 * k3[d] + a64 * k4[d] + a65 * k5[d]);
    double tn = landing ? target : t + hh;
    f(tn, tmp.data(), k6.data());
    for (int d = 0; d < dim; ++d)
      ynew[d] = y[d] + hh * (a71 * k1[d] + a72 * k2[d] + a73 * k3[d] + a74 * k4[d] + a75 * k5[d] +
                             a76 * k6[d]);
    f(tn, ynew.data(), k7.data());
    double en = 0.0;
    for (int d = 0; d < dim; ++d) {
      double e = hh * (e1 * val(k1[d]) + e2 * val(k2[d]) + e3 * val(k3[d]) + e4 * val(k4[d]) + e5 * val(k5[d]) +
                       e6 * val(k6[d]) + e7 * val(k7[d]));
      double sc = abstol + reltol * std::max(std::fabs(val(y[d])), std::fabs(val(ynew[d])));
      en += (e / sc) * (e / sc);
    }
    en = std::sqrt(en / dim);
    if (!(en == en)) en = 1e10;
    double fac = 0.9 * std::pow(std::max(en, 1e-10), -0.2);
    fac = std::min(10.0, std::max(0.2, fac));
    if (en <= 1.0) {
      t = tn;
      y = ynew;
      k1 = k7;
      sol.t.push_back(t);
      sol.y.insert(sol.y.end(), y.begin(), y.end());
      sol.f.insert(sol.f.end(), k1.begin(), k1.end());
      if (landing) ++li;
      double hprop = hs * fac;
      if (!landing || hprop > hmag) hmag = std::max(hprop, landing ? hmag : 0.0);
      if (landing) hmag = std::max(hmag, hs * fac);
    } else {
      hmag = hs * std::min(1.0, fac);
    }
    if (++steps > 10000000) throw std::runtime_error("tsit5: too many steps");
  }
  return sol;
}

}  // namespace orc
