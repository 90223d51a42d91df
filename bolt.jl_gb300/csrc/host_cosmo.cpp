// Host construction of the background and ionization tables (see
// host_cosmo.hpp).  Every formula cites the Bolt.jl line it restates.
#include "host_cosmo.hpp"

#include <algorithm>
#include <cmath>
#include <functional>
#include <stdexcept>

namespace bolt {
namespace {

// Exact SI constants and CODATA 2018 values (PhysicalConstants.CODATA2018 as
// used by Bolt.jl:38-39); parsec from UnitfulAstro.
const double kC = 299792458.0;
const double kHbar = 6.62607015e-34 / (2.0 * M_PI);
const double kKB = 1.380649e-23;
const double kEV = 1.602176634e-19;
const double kMpc = 3.0856775814913673e22;
const double kG = 6.67430e-11;
const double kMp = 1.67262192369e-27;
const double kSigmaT = 6.6524587321e-29;
const double kMe = 9.1093837015e-31;
const double kAlphaFS = 7.2973525693e-3;
const double kZeta3 = 1.2020569;  // background.jl:3

double nat_G() { return kG * kHbar / (kC * kC * kC) / (kMpc * kMpc); }
double nat_mH() { return kMp * kC / kHbar * kMpc; }
double nat_sigmaT() { return kSigmaT / (kMpc * kMpc); }
double sec_per_nat() { return kMpc / kC; }        // recfast.jl:4
double kelvin_per_nat() { return kHbar * kC / (kKB * kMpc); }  // recfast.jl:5

}  // namespace

double units_km_s_Mpc_100() { return 1e5 / kC; }
double units_mass_eV() { return kEV / (kHbar * kC) * kMpc; }

GridSpec make_grid(double start, double step, double stop) {
  GridSpec g;
  g.n = int(std::floor((stop - start) / step + 1e-9)) + 1;
  g.x0 = start;
  g.h = step;
  g.i0 = 0;
  g.M = 0;
  double inv = 1.0 / step, Mr = std::round(inv);
  if (std::fabs(inv - Mr) < 1e-9 * Mr && std::fabs(start * Mr - std::round(start * Mr)) < 1e-6) {
    g.M = long(Mr);
    g.i0 = long(std::round(start * Mr));
  }
  return g;
}

// ------------------------------------------------------------------ splines
// Interior rows (c[i-1] + 4 c[i] + c[i+1]) / 6 = y[i-1]; the natural
// boundary rows reduce to c[1] = y[0], c[n] = y[n-1] (util.jl:11).
void spline_coefs(const double* y, int n, double* c) {
  if (n == 1) { c[0] = c[1] = c[2] = y[0]; return; }
  c[1] = y[0];
  c[n] = y[n - 1];
  int m = n - 2;  // unknowns c[2..n-1]
  if (m > 0) {
    std::vector<double> w(m);
    // forward elimination of the constant (1, 4, 1) system scaled by 6
    double denom = 4.0;
    c[2] = 6.0 * y[1] - c[1];
    w[0] = 1.0 / denom;
    for (int r = 1; r < m; ++r) {
      double rhs = 6.0 * y[r + 1];
      denom = 4.0 - w[r - 1];
      c[r + 2] = rhs - c[r + 1] * w[r - 1];
      w[r] = 1.0 / denom;
    }
    // c[2..n-1] currently hold the forward-swept right-hand sides
    c[n - 1] -= (m >= 1 ? c[n] : 0.0);
    c[n - 1] *= w[m - 1];
    for (int r = m - 2; r >= 0; --r) c[r + 2] = (c[r + 2] - c[r + 3]) * w[r];
  }
  c[0] = 2.0 * c[1] - c[2];
  c[n + 1] = 2.0 * c[n] - c[n - 1];
}

static inline void spl_locate(int n, double x0, double h, double x, int& i, double& t) {
  double u = (x - x0) / h;
  double f = std::floor(u);
  f = std::min(std::max(f, 0.0), double(n - 2));
  i = int(f);
  t = u - f;
}

double spline_eval(const double* c, int n, double x0, double h, double x) {
  int i; double t; spl_locate(n, x0, h, x, i, t);
  double s = 1.0 - t, t2 = t * t, s2 = s * s;
  return (c[i] * s2 * s + c[i + 1] * (4.0 - 6.0 * t2 + 3.0 * t2 * t) + c[i + 2] * (4.0 - 6.0 * s2 + 3.0 * s2 * s) +
          c[i + 3] * t2 * t) / 6.0;
}

double spline_deriv(const double* c, int n, double x0, double h, double x) {
  int i; double t; spl_locate(n, x0, h, x, i, t);
  double s = 1.0 - t;
  return (-0.5 * s * s * c[i] + (-2.0 * t + 1.5 * t * t) * c[i + 1] + (2.0 * s - 1.5 * s * s) * c[i + 2] +
          0.5 * t * t * c[i + 3]) / h;
}

double spline_deriv2(const double* c, int n, double x0, double h, double x) {
  int i; double t; spl_locate(n, x0, h, x, i, t);
  return ((1.0 - t) * c[i] + (3.0 * t - 2.0) * c[i + 1] + (1.0 - 3.0 * t) * c[i + 2] + t * c[i + 3]) / (h * h);
}

namespace {

struct Spl {
  const GridSpec* g;
  std::vector<double> c;
  void fit(const GridSpec& gg, const std::vector<double>& y) {
    g = &gg;
    c.assign(gg.n + 2, 0.0);
    spline_coefs(y.data(), gg.n, c.data());
  }
  double operator()(double x) const { return spline_eval(c.data(), g->n, g->x0, g->h, x); }
  double d1(double x) const { return spline_deriv(c.data(), g->n, g->x0, g->h, x); }
  double d2(double x) const { return spline_deriv2(c.data(), g->n, g->x0, g->h, x); }
};

// ------------------------------------------------------------ quadrature
void gauss_legendre_nodes(int n, std::vector<double>& x, std::vector<double>& w) {
  x.resize(n);
  w.resize(n);
  int half = (n + 1) / 2;
  for (int i = 0; i < half; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 64; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    double wt = 2.0 / ((1.0 - z * z) * dp * dp);
    x[n - 1 - i] = z;
    w[n - 1 - i] = wt;
    x[i] = -z;
    w[i] = wt;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

// ------------------------------------------------------------ background
struct Bg {
  CosmoParamsH p;
  int nq;
  std::vector<double> xq, wq;
  double H0, rc, OL, Tnu, lqmin, lqmax;

  static double ui_scale(double lqmi, double lqma) { return (lqma - lqmi) / 2.0; }
  double q_of(double xx, double lqmi, double lqma) const { return std::pow(10.0, lqmi + ui_scale(lqmi, lqma) * (xx + 1.0)); }
  double dxdq(double q, double lqmi, double lqma) const {  // util.jl:26
    return (1.0 + (-1.0 + 2.0 / (lqma - lqmi) * ((1.0 + lqmi) - lqmi))) / (q * std::log(10.0));
  }
  double f0(double q) const { return 2.0 / std::pow(2.0 * M_PI, 3) / (std::exp(q / Tnu) + 1.0); }

  void init(const CosmoParamsH& pp, int n) {
    p = pp;
    nq = n;
    gauss_legendre_nodes(n, xq, wq);
    H0 = p.h * units_km_s_Mpc_100();                       // background.jl:5
    rc = (3.0 / (8.0 * M_PI)) * H0 * H0 / nat_G();           // background.jl:6
    double Tg = std::pow(15.0 / (M_PI * M_PI) * rc * p.Omega_r, 0.25);
    double nufac = (90.0 * kZeta3 / (11.0 * std::pow(M_PI, 4))) * (p.Omega_r * p.h * p.h / Tg) * std::pow(p.N_nu / 3.0, 0.75);
    double Omega_nu = p.Sigma_m_nu * nufac / (p.h * p.h);
    OL = 1.0 - (p.Omega_r * (1.0 + (2.0 / 3.0) * (7.0 * p.N_nu / 8.0) * std::pow(4.0 / 11.0, 4.0 / 3.0)) + p.Omega_b +
                p.Omega_c + Omega_nu);                           // background.jl:7-18
    Tnu = std::pow(p.N_nu / 3.0, 0.25) * std::pow(4.0 / 11.0, 1.0 / 3.0) * Tg;
    lqmin = std::log10(Tnu / 30.0);
    lqmax = std::log10(Tnu * 30.0);
  }
  // background.jl:33-48
  double rho_nu(double a) const {
    double s = 0.0, am = a * p.Sigma_m_nu;
    for (int i = 0; i < nq; ++i) {
      double q = q_of(xq[i], lqmin, lqmax);
      s += q * q * std::sqrt(q * q + am * am) * f0(q) / dxdq(q, lqmin, lqmax) * wq[i];
    }
    return 4.0 * M_PI * std::pow(a, -4) * s;
  }
  // background.jl:58-64, conformal rate a*H
  double Hconf(double a) const {
    double rad = p.Omega_r * std::pow(a, -4) * (1.0 + (2.0 / 3.0) * (7.0 * p.N_nu / 8.0) * std::pow(4.0 / 11.0, 4.0 / 3.0));
    return a * H0 * std::sqrt((p.Omega_c + p.Omega_b) * std::pow(a, -3) + rho_nu(a) / rc + rad + OL);
  }
  // background.jl:73-77: GL quadrature in log10(a) from -13.75
  double eta(double x) const {
    double lo = -13.75, hi = std::log10(std::exp(x)), s = 0.0;
    for (int i = 0; i < nq; ++i) {
      double a = q_of(xq[i], lo, hi);
      s += 1.0 / (a * Hconf(a)) / dxdq(a, lo, hi) * wq[i];
    }
    return s;
  }
};

// ---------------------------------------------------------------- Tsit5
// Tsitouras 5(4) with landing on requested points; Hermite dense output.
// Which side of each state-dependent switch of the RECFAST right-hand side
// every stage evaluation of the accepted steps took (one byte per
// evaluation); replayed, perturbed runs take the same sides, as a
// ForwardDiff derivative follows the branch of the unperturbed run.
struct BranchLog {
  std::vector<uint8_t>* bits = nullptr;
  size_t pos = 0;
  bool replay = false;
};

struct Traj {
  int dim = 0;
  std::vector<double> t, y, f;
  std::vector<double> h;  // signed size of each accepted step
  void eval(double tq, double* out) const {
    size_t n = t.size();
    bool up = t.back() > t.front();
    size_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
      size_t mid = (lo + hi) / 2;
      if (up ? (t[mid] <= tq) : (t[mid] >= tq)) lo = mid; else hi = mid;
    }
    double ta = t[lo], tb = t[lo + 1], hh = tb - ta;
    if (tq == ta || n == 1) { for (int d = 0; d < dim; ++d) out[d] = y[lo * dim + d]; return; }
    if (tq == tb) { for (int d = 0; d < dim; ++d) out[d] = y[(lo + 1) * dim + d]; return; }
    double s = (tq - ta) / hh, s2 = s * s, s3 = s2 * s;
    double h00 = 2 * s3 - 3 * s2 + 1, h10 = s3 - 2 * s2 + s, h01 = -2 * s3 + 3 * s2, h11 = s3 - s2;
    for (int d = 0; d < dim; ++d)
      out[d] = h00 * y[lo * dim + d] + h10 * hh * f[lo * dim + d] + h01 * y[(lo + 1) * dim + d] + h11 * hh * f[(lo + 1) * dim + d];
  }
  double eval1(double tq, int i) const { double b[4]; eval(tq, b); return b[i]; }
  const double* last() const { return &y[y.size() - dim]; }
};

typedef std::function<void(double, const double*, double*)> OdeFn;

// replay / replay_h: if non-null, the accepted abscissae (replay[0] == t0)
// and step sizes of an earlier run; the same steps are taken without error
// control, so the result is a smooth function of the right-hand side's
// parameters, and bitwise the earlier run's for the same right-hand side.
Traj tsit5_integrate(const OdeFn& fn, int dim, const double* y0, double t0, double t1, double rtol, double atol,
                     std::vector<double> land, const std::vector<double>* replay = nullptr,
                     const std::vector<double>* replay_h = nullptr, BranchLog* blog = nullptr) {
  const double C[7] = {0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
  const double A[7][6] = {
      {0, 0, 0, 0, 0, 0},
      {0.161, 0, 0, 0, 0, 0},
      {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
      {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
      {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
      {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
      {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
  const double E[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995, -0.1447110071732629,
                       0.5823571654525552, -0.45808210592918697, 1.0 / 66.0};
  double dir = t1 > t0 ? 1.0 : -1.0;
  land.erase(std::remove_if(land.begin(), land.end(), [&](double s) { return !((s - t0) * dir > 0 && (t1 - s) * dir > 0); }),
             land.end());
  land.push_back(t1);
  std::sort(land.begin(), land.end(), [dir](double a, double b) { return a * dir < b * dir; });
  Traj tr;
  tr.dim = dim;
  std::vector<double> y(y0, y0 + dim), yn(dim), tmp(dim), K(7 * dim);
  fn(t0, y.data(), &K[0]);
  tr.t.push_back(t0);
  tr.y.insert(tr.y.end(), y.begin(), y.end());
  tr.f.insert(tr.f.end(), K.begin(), K.begin() + dim);
  double t = t0, hnext = std::fabs(t1 - t0) * 1e-6;
  if (replay) {
    if (replay->empty() || (*replay)[0] != t0 || !replay_h || replay_h->size() + 1 != replay->size())
      throw std::runtime_error("RECFAST replay does not match this integration");
    for (size_t i = 1; i < replay->size(); ++i) {
      const double tn = (*replay)[i], h = (*replay_h)[i - 1];
      for (int s = 1; s < 7; ++s) {
        for (int d = 0; d < dim; ++d) {
          double acc = 0.0;
          for (int j = 0; j < s; ++j) acc += A[s][j] * K[j * dim + d];
          tmp[d] = y[d] + h * acc;
        }
        double ts = s >= 5 ? tn : t + C[s] * h;
        if (s == 6) std::copy(tmp.begin(), tmp.end(), yn.begin());
        fn(ts, tmp.data(), &K[s * dim]);
      }
      t = tn;
      y = yn;
      std::copy(K.begin() + 6 * dim, K.begin() + 7 * dim, K.begin());
      tr.t.push_back(t);
      tr.y.insert(tr.y.end(), y.begin(), y.end());
      tr.f.insert(tr.f.end(), K.begin(), K.begin() + dim);
    }
    return tr;
  }
  size_t li = 0;
  long guard = 0;
  while (li < land.size()) {
    const size_t mark = (blog && blog->bits && !blog->replay) ? blog->bits->size() : 0;
    double rem = (land[li] - t) * dir;
    bool hit = hnext >= rem * (1.0 - 1e-12);
    double hs = hit ? rem : hnext, h = hs * dir;
    for (int s = 1; s < 7; ++s) {
      for (int d = 0; d < dim; ++d) {
        double acc = 0.0;
        for (int j = 0; j < s; ++j) acc += A[s][j] * K[j * dim + d];
        tmp[d] = y[d] + h * acc;
      }
      double ts = (s >= 5 && hit) ? land[li] : t + C[s] * h;
      if (s == 6) std::copy(tmp.begin(), tmp.end(), yn.begin());
      fn(ts, tmp.data(), &K[s * dim]);
    }
    // stage 7 (FSAL) was evaluated at yn: K[6]
    double err = 0.0;
    for (int d = 0; d < dim; ++d) {
      double e = 0.0;
      for (int j = 0; j < 7; ++j) e += E[j] * K[j * dim + d];
      e *= h;
      double sc = atol + rtol * std::max(std::fabs(y[d]), std::fabs(yn[d]));
      err += (e / sc) * (e / sc);
    }
    err = std::sqrt(err / dim);
    if (!(err == err)) err = 1e10;
    double fac = std::min(10.0, std::max(0.2, 0.9 * std::pow(std::max(err, 1e-10), -0.2)));
    if (err <= 1.0) {
      t = hit ? land[li] : t + h;
      tr.h.push_back(h);
      y = yn;
      std::copy(K.begin() + 6 * dim, K.begin() + 7 * dim, K.begin());
      tr.t.push_back(t);
      tr.y.insert(tr.y.end(), y.begin(), y.end());
      tr.f.insert(tr.f.end(), K.begin(), K.begin() + dim);
      if (hit) { ++li; hnext = std::max(hnext, hs * fac); }
      else hnext = hs * fac;
    } else {
      hnext = hs * std::min(1.0, fac);
      if (blog && blog->bits && !blog->replay) blog->bits->resize(mark);  // forget the rejected attempt
    }
    if (++guard > 20000000) throw std::runtime_error("RECFAST integration did not finish");
  }
  return tr;
}

// --------------------------------------------------------------- RECFAST
// Constants and derived coefficients: recfast.jl:22-121.
struct Rf {
  const Bg* bg;
  const Spl *H, *Hp;
  double C = 2.99792458e8, k_B = 1.380658e-23, h_P = 6.6260755e-34, m_e = 9.1093897e-31, m_H = 1.673575e-27,
         not4 = 3.9715, sigma = 6.6524616e-29, arad = 7.565914e-16, G = 6.6742e-11;
  double Lambda = 8.2245809, Lambda_He = 51.3, L_H_ion = 1.096787737e7, L_H_alpha = 8.225916453e6,
         L_He1_ion = 1.98310772e7, L_He2_ion = 4.389088863e7, L_He_2s = 1.66277434e7, L_He_2p = 1.71134891e7;
  double A2P_s = 1.798287e9, A2P_t = 177.58, L_He_2Pt = 1.690871466e7, L_He_2St = 1.5985597526e7,
         L_He2St_ion = 3.8454693845e6, sigma_He_2Ps = 1.436289e-22, sigma_He_2Pt = 1.484872e-22;
  double AG1 = -0.14, AG2 = 0.079, zG1 = 7.28, zG2 = 6.73, wG1 = 0.18, wG2 = 0.33;
  double aP = 4.309, bP = -0.6166, cP = 0.6703, dP = 0.53;
  double aVF, bVF = 0.711, T0, T1, atr, btr = 0.761;
  double CDB, CDB_He, CB1, CB1_He1, CB1_He2, CR, CK, CK_He, CL, CL_He, CT, Bfact;
  double Yp, OmegaB, HO, Tnow, mu_T, fHe, Nnow, fu = 1.125, b_He = 0.86, H_frac = 1e-3, tol;
  int Heswitch = 6;

  void init(const Bg* b, const Spl* h, const Spl* hp, const RecfastOpts& o) {
    bg = b; H = h; Hp = hp;
    aVF = std::pow(10.0, -16.744);
    T0 = std::pow(10.0, 0.477121);
    T1 = std::pow(10.0, 5.114);
    atr = std::pow(10.0, -16.306);
    double La = 1.0 / L_H_alpha, LaHe = 1.0 / L_He_2p;
    CDB = h_P * C * (L_H_ion - L_H_alpha) / k_B;
    CDB_He = h_P * C * (L_He1_ion - L_He_2s) / k_B;
    CB1 = h_P * C * L_H_ion / k_B;
    CB1_He1 = h_P * C * L_He1_ion / k_B;
    CB1_He2 = h_P * C * L_He2_ion / k_B;
    CR = 2.0 * M_PI * (m_e / h_P) * (k_B / h_P);
    CK = La * La * La / (8.0 * M_PI);
    CK_He = LaHe * LaHe * LaHe / (8.0 * M_PI);
    CL = C * h_P / (k_B * La);
    CL_He = C * h_P / (k_B / L_He_2s);
    CT = (8.0 / 3.0) * (sigma / (m_e * C)) * arad;
    Bfact = h_P * C * (L_He_2p - L_He_2s) / k_B;
    Yp = o.Yp;
    OmegaB = o.OmegaB;
    tol = o.tol;
    HO = bg->H0 / sec_per_nat();
    Tnow = o.Tnow > 0 ? o.Tnow : std::pow(15.0 / (M_PI * M_PI) * bg->rc * o.OmegaG, 0.25) * kelvin_per_nat();
    double mu_H = 1.0 / (1.0 - Yp);
    mu_T = not4 / (not4 - (not4 - 1.0) * Yp);
    fHe = Yp / (not4 * (1.0 - Yp));
    Nnow = 3.0 * HO * HO * OmegaB / (8.0 * M_PI * G * mu_H * m_H);
  }
  double saha(double z, double CBx) const {
    return std::exp(1.5 * std::log(CR * Tnow / (1 + z)) - CBx / (Tnow * (1 + z))) / Nnow;
  }
  // The Saha roots (recfast.jl:396-411) 0.5 (sqrt(b^2 + 4c) - b) are
  // evaluated as 2c / (sqrt(b^2 + 4c) + b) when b > 0: the same number
  // without the cancellation that leaves ~1e-6 of rounding noise when
  // r ~ 1e10 (early times), noise a central difference would amplify.
  static double quad_root(double b, double c) {
    double s = std::sqrt(b * b + 4.0 * c);
    return b > 0.0 ? 2.0 * c / (s + b) : 0.5 * (s - b);
  }
  double xH_saha(double z) const { double r = saha(z, CB1); return quad_root(r, r); }
  double xtot_He1_saha(double z) const {
    double r = 4.0 * saha(z, CB1_He1);
    return quad_root(r - 1, (1 + fHe) * r);
  }
  // recfast.jl:156-310
  mutable BranchLog* blog = nullptr;

  void rhs(double z, const double* y, double* f) const {
    double xH = y[0], xHe = y[1], Tm = y[2], x = xH + fHe * xHe;
    uint8_t br = uint8_t((xHe < 5e-9 || xHe > 0.98) ? 1 : 0) | uint8_t(xH < 0.9999999 ? 2 : 0) |
                 uint8_t(xH > 0.99999 ? 4 : 0) | uint8_t(xH > 0.99 ? 8 : 0) | uint8_t(xH > 0.985 ? 16 : 0) |
                 uint8_t(xHe < 1e-15 ? 32 : 0);
    {  // the temperature equation's switch (recfast.jl:293-307)
      double tTh0 = (1.0 / (CT * std::pow(Tnow * (1.0 + z), 4))) * (1 + x + fHe) / x;
      double tH0 = 2.0 / (3.0 * HO * std::pow(1.0 + z, 1.5));
      if (tTh0 < H_frac * tH0) br |= 64;
    }
    if (blog && blog->bits) {
      if (blog->replay) {
        if (blog->pos >= blog->bits->size()) throw std::runtime_error("RECFAST branch replay ran out");
        br = (*blog->bits)[blog->pos++];
      } else {
        blog->bits->push_back(br);
      }
    }
    double zp = 1.0 + z, n = Nnow * zp * zp * zp, nHe = fHe * n, Trad = Tnow * zp;
    double a = 1.0 / zp, xa = std::log(a);
    double Hz = (*H)(xa) / a / sec_per_nat();
    double dHdz = (-Hp->operator()(xa) + (*H)(xa)) / sec_per_nat();
    double Rdown = 1e-19 * aP * std::pow(Tm / 1e4, bP) / (1.0 + cP * std::pow(Tm / 1e4, dP));
    double Rup = Rdown * std::pow(CR * Tm, 1.5) * std::exp(-CDB / Tm);
    double s0 = std::sqrt(Tm / T0), s1 = std::sqrt(Tm / T1);
    double RdHe = aVF / (s0 * std::pow(1 + s0, 1 - bVF)) / std::pow(1 + s1, 1 + bVF);
    double RuHe = 4.0 * RdHe * std::pow(CR * Tm, 1.5) * std::exp(-CDB_He / Tm);
    double HeB = std::exp(std::min(Bfact / Tm, 680.0));
    double lz = std::log(zp);
    double K = CK / Hz * (1.0 + AG1 * std::exp(-std::pow((lz - zG1) / wG1, 2)) + AG2 * std::exp(-std::pow((lz - zG2) / wG2, 2)));
    double Rdtr = atr / (s0 * std::pow(1 + s0, 1 - btr)) / std::pow(1 + s1, 1 + btr);
    double Rutr = Rdtr * std::exp(-h_P * C * L_He2St_ion / (k_B * Tm)) * std::pow(CR * Tm, 1.5) * (4.0 / 3.0);
    int flag = (br & 1) ? 0 : Heswitch;
    double KHe, Cft = 0.0;
    if (flag == 0) {
      KHe = CK_He / Hz;
    } else {
      double tauS = A2P_s * CK_He * 3 * nHe * (1 - xHe) / Hz;
      double pS = (1 - std::exp(-tauS)) / tauS;
      KHe = 1.0 / (A2P_s * pS * 3 * nHe * (1 - xHe));
      if ((flag == 2 || flag >= 5) && (br & 2)) {
        double Dop = C * L_He_2p * std::sqrt(2 * k_B * Tm / (m_H * not4 * C * C));
        double g2 = 3 * A2P_s * fHe * (1 - xHe) * C * C / (std::sqrt(M_PI) * sigma_He_2Ps * 8 * M_PI * Dop * (1 - xH)) /
                    std::pow(C * L_He_2p, 2);
        double AH = A2P_s / (1 + 0.36 * std::pow(g2, b_He));
        KHe = 1.0 / ((A2P_s * pS + AH) * 3 * nHe * (1 - xHe));
      }
      if (flag >= 3) {
        double tauT = A2P_t * nHe * (1. - xHe) * 3 / (8 * M_PI * Hz * std::pow(L_He_2Pt, 3));
        double pT = (1 - std::exp(-tauT)) / tauT;
        double CLPSt = h_P * C * (L_He_2Pt - L_He_2St) / k_B;
        if (flag == 3 || flag == 5 || (br & 4)) {
          Cft = A2P_t * pT * std::exp(-CLPSt / Tm);
        } else {
          double Dop = C * L_He_2Pt * std::sqrt(2 * k_B * Tm / (m_H * not4 * C * C));
          double g2 = 3 * A2P_t * fHe * (1 - xHe) * C * C / (std::sqrt(M_PI) * sigma_He_2Pt * 8 * M_PI * Dop * (1 - xH)) /
                      std::pow(C * L_He_2Pt, 2);
          double AH = A2P_t / (1 + 0.66 * std::pow(g2, 0.9)) / 3;
          Cft = (A2P_t * pT + AH) * std::exp(-CLPSt / Tm);
        }
        Cft = Cft / (Rutr + Cft);
      }
    }
    double f1;
    if (br & 8) f1 = 0.0;
    else if (br & 16) f1 = (x * xH * n * Rdown - Rup * (1 - xH) * std::exp(-CL / Tm)) / (Hz * zp);
    else
      f1 = ((x * xH * n * Rdown - Rup * (1.0 - xH) * std::exp(-CL / Tm)) * (1.0 + K * Lambda * n * (1.0 - xH))) /
           (Hz * zp * (1.0 / fu + K * Lambda * n * (1.0 - xH) / fu + K * Rup * n * (1.0 - xH)));
    double f2 = 0.0;
    if (!(br & 32)) {
      f2 = ((x * xHe * n * RdHe - RuHe * (1 - xHe) * std::exp(-CL_He / Tm)) * (1 + KHe * Lambda_He * nHe * (1 - xHe) * HeB)) /
           (Hz * zp * (1 + KHe * (Lambda_He + RuHe) * nHe * (1 - xHe) * HeB));
      if (flag >= 3)
        f2 += (x * xHe * n * Rdtr - (1 - xHe) * 3 * Rutr * std::exp(-h_P * C * L_He_2St / (k_B * Tm))) * Cft / (Hz * zp);
    }
    double f3;
    if (br & 64) {
      double eps = Hz * (1 + x + fHe) / (CT * std::pow(Trad, 3) * x);
      f3 = Tnow + eps * ((1 + fHe) / (1 + fHe + x)) * ((f1 + fHe * f2) / x) - eps * dHdz / Hz + 3 * eps / zp;
    } else {
      f3 = CT * std::pow(Trad, 4) * x / (1 + x + fHe) * (Tm - Trad) / (Hz * zp) + 2 * Tm / zp;
    }
    f[0] = f1; f[1] = f2; f[2] = f3;
  }
};

// ----------------------------------------------------------- Saha-Peebles
// The Saha equation for hydrogen and the Peebles equation (ionization.jl:1-93)
// in Bolt's natural units (Mpc^-1), T_b = 2.725 K / a.  The Saha root is
// taken without cancellation, 2r / (sqrt(r^2 + 4r) + r), the same number as
// the reference's (sqrt(r^2 + 4r) - r) / 2; beta2 = beta exp(3 eps0 / 4T) is
// formed as one exponential, exp(-eps0 / 4T), which the reference reaches in
// BigFloat (its ODE right-hand side, ionization.jl:61-66).
struct SahaPeebles {
  const Bg* bg;
  double T0, eps0, me, mH, alpha, L2s;
  void init(const Bg* b) {
    bg = b;
    T0 = 2.725 / kelvin_per_nat();                  // ionization.jl:5
    eps0 = 13.605698 * units_mass_eV();             // ionization.jl:26
    me = kMe * kC / kHbar * kMpc;
    mH = nat_mH();
    alpha = kAlphaFS;
    L2s = 8.227 * sec_per_nat();                    // ionization.jl:25
  }
  double nH(double a) const { return bg->p.Omega_b * bg->rc / (mH * a * a * a) * (1 - bg->p.Y_p); }
  double xe_saha(double x) const {                 // ionization.jl:12-16
    double a = std::exp(x), Tb = T0 / a;
    double r = std::pow(me * Tb / (2 * M_PI), 1.5) / nH(a) * std::exp(-eps0 / Tb);
    return 2 * r / (std::sqrt(r * r + 4 * r) + r);
  }
  double Hold(double a) const {                    // background.jl:51-55
    const CosmoParamsH& p = bg->p;
    return bg->H0 * std::sqrt((p.Omega_c + p.Omega_b) * std::pow(a, -3) +
                              p.Omega_r * (1 + (2.0 / 3.0) * (7 * p.N_nu / 8) * std::pow(4.0 / 11.0, 4.0 / 3.0)) *
                                  std::pow(a, -4) +
                              bg->OL);
  }
  double dxe_dx(double x, double xe) const {       // ionization.jl:36-66
    double a = std::exp(x), Tb = T0 / a, H = Hold(a), n = nH(a);
    double a2 = (64 * M_PI / std::sqrt(27 * M_PI)) * (alpha * alpha / (me * me)) * std::sqrt(eps0 / Tb) *
                (0.448 * std::log(eps0 / Tb));
    double pre = a2 * std::pow(me * Tb / (2 * M_PI), 1.5);
    double beta = pre * std::exp(-eps0 / Tb), beta2 = pre * std::exp(-eps0 / (4 * Tb));
    double La = H * std::pow(3 * eps0, 3) / (std::pow(8 * M_PI, 2) * (1 - xe) * n);
    double Cr = (L2s + La) / (L2s + La + beta2);
    return Cr / H * (beta * (1 - xe) - n * a2 * xe * xe);
  }
};

// Bracketing root of f on [a, b]: regula falsi then bisection, to floating
// point resolution (the NonlinearSolve Falsi call at recfast.jl:451-459).
double bracket_root(const std::function<double(double)>& f, double a, double b) {
  double fa = f(a), fb = f(b);
  if (fa == 0.0) return a;
  if (fb == 0.0) return b;
  bool falsi = true;
  int it = 1;
  while (falsi && it < 1000) {
    if (std::nextafter(a, b) == b) return a;
    double m = (fb * a - fa * b) / (fb - fa);
    for (int r = 0; r < 10; ++r) {
      double pm = std::nextafter(m, a);
      m = (b > a) ? std::max(a, pm) : std::min(a, pm);
    }
    if (m == a || m == b) break;
    double fm = f(m);
    if (fm == 0.0) { b = m; break; }
    if ((fm > 0) == (fa > 0)) { a = m; fa = fm; } else { b = m; fb = fm; }
    ++it;
  }
  for (; it < 1000; ++it) {
    double m = 0.5 * (a + b);
    if (m == a || m == b) return a;
    double fm = f(m);
    if (fm == 0.0) b = m;
    else if ((fm > 0) == (fa > 0)) { a = m; fa = fm; }
    else { b = m; fb = fm; }
  }
  return a;
}

}  // namespace

void build_cosmo_tables(const CosmoParamsH& p, const GridSpec& g, int nq, const RecfastOpts& ro, CosmoTables& T,
                        RecfastFreeze* fz) {
  const bool replay = fz && fz->have;
  if (g.n < 4) throw std::runtime_error("x grid needs at least 4 nodes");
  if (nq < 1) throw std::runtime_error("nq must be positive");
  if (!(p.h > 0) || !(p.Omega_b > 0) || !(p.Omega_r > 0) || !(p.N_nu > 0) || p.Sigma_m_nu < 0 || !(p.A > 0))
    throw std::runtime_error("cosmological parameters out of range");
  Bg bg;
  bg.init(p, nq);
  T.par = p;
  T.grid = g;
  T.nq = nq;
  T.H0 = bg.H0;
  T.rho_crit = bg.rc;
  T.Omega_Lambda = bg.OL;
  T.Tnu = bg.Tnu;
  T.logqmin = bg.lqmin;
  T.logqmax = bg.lqmax;
  T.quad_pts = bg.xq;
  T.quad_wts = bg.wq;
  const int n = g.n;
  for (int s = 0; s < T_COUNT; ++s) T.nodes[s].assign(n, 0.0);
  for (int j = 0; j < n; ++j) {
    double x = g.at(j), a = std::exp(x);
    T.nodes[T_RHO0M][j] = bg.rho_nu(a);
    T.nodes[T_H][j] = bg.Hconf(a);
    T.nodes[T_ETA][j] = bg.eta(x);
  }
  T.eta0 = bg.eta(0.0);
  Spl sH, sHp;
  sH.fit(g, T.nodes[T_H]);
  for (int j = 0; j < n; ++j) T.nodes[T_HP][j] = sH.d1(g.at(j));
  sHp.fit(g, T.nodes[T_HP]);

  // --- RECFAST (recfast.jl:446-536)
  Rf rf;
  rf.init(&bg, &sH, &sHp, ro);
  T.Tnow = rf.Tnow;
  if (ro.ionization == 1) {
    // Saha-Peebles (ionization.jl:83-93) through customion (ionization.jl:141-164)
    if (fz) throw std::runtime_error("gradients of a Saha-Peebles ionization history are not available");
    SahaPeebles sp;
    sp.init(&bg);
    const double xtr = std::log(1.0 / (1.0 + 1587.4));  // z2x(1587.4)
    std::vector<double> land;
    for (int j = 0; j < n; ++j)
      if (g.at(j) > xtr) land.push_back(g.at(j));
    double x0 = sp.xe_saha(xtr);
    Traj Pe = tsit5_integrate([&](double x, const double* u, double* du) { du[0] = sp.dxe_dx(x, u[0]); }, 1, &x0, xtr,
                              0.0, 1e-11, 1e-11, land);
    T.z_He_evo_start = T.z_H_He_evo_start = 0.0;
    for (int j = 0; j < n; ++j) {
      double x = g.at(j), z = 1.0 / std::exp(x) - 1.0;
      T.nodes[T_XE][j] = x < xtr ? sp.xe_saha(x) : Pe.eval1(x, 0);
      T.nodes[T_TMAT][j] = 2.725 * (1 + z);  // saha_T_b (ionization.jl:8)
    }
  } else {
    const double zini = 10000.0, zfin = 0.0, zre_ini = 50.0;
    double zHe = replay ? fz->zHe
                        : bracket_root([&](double z) { return (rf.xtot_He1_saha(z) - 1.0) / rf.fHe - 0.99; },
                                       std::min(zini, 3500.0), zfin);
    double zHH = replay ? fz->zHH : bracket_root([&](double z) { return rf.xH_saha(z) - 0.985; }, zHe, zfin);
    T.z_He_evo_start = zHe;
    T.z_H_He_evo_start = zHH;
    std::vector<double> zland;
    for (int j = 0; j < n; ++j) {
      double z = 1.0 / std::exp(g.at(j)) - 1.0;
      if (z < zini) zland.push_back(z);
    }
    BranchLog logHe, logHHe;
    if (fz) {
      logHe.bits = &fz->bHe;
      logHHe.bits = &fz->bHHe;
      logHe.replay = logHHe.replay = replay;
      if (!replay) { fz->bHe.clear(); fz->bHHe.clear(); }
    }
    double y2[2] = {(rf.xtot_He1_saha(zHe) - 1.0) / rf.fHe, rf.Tnow * (1 + zHe)};
    rf.blog = fz ? &logHe : nullptr;
    Traj He = tsit5_integrate(
        [&](double z, const double* u, double* du) {
          double yy[3] = {rf.xH_saha(z), u[0], u[1]}, d[3];
          rf.rhs(z, yy, d);
          du[0] = d[1];
          du[1] = d[2];
        },
        2, y2, zHe, zHH, rf.tol, 1e-6, zland, replay ? &fz->tHe : nullptr, replay ? &fz->hHe : nullptr,
        fz ? &logHe : nullptr);
    rf.blog = fz ? &logHHe : nullptr;
    double y3[3] = {rf.xH_saha(zHH), He.last()[0], He.last()[1]};
    std::vector<double> land3 = zland;
    land3.push_back(zre_ini);
    Traj HHe = tsit5_integrate([&](double z, const double* u, double* du) { rf.rhs(z, u, du); }, 3, y3, zHH, zfin, rf.tol,
                               1e-6, land3, replay ? &fz->tHHe : nullptr, replay ? &fz->hHHe : nullptr,
                               fz ? &logHHe : nullptr);
    rf.blog = nullptr;
    auto xe_recfast = [&](double z) -> double {  // recfast.jl:413-433
      if (z > 8000.) return 1 + 2 * rf.fHe;
      if (z > 5000.) {
        double r = rf.saha(z, rf.CB1_He2);
        return Rf::quad_root(r - 1 - rf.fHe, (1 + 2 * rf.fHe) * r);
      }
      if (z > 3500.) return 1 + rf.fHe;
      if (z > zHe) return rf.xtot_He1_saha(z);
      if (z > zHH) return rf.xH_saha(z) + rf.fHe * He.eval1(z, 0);
      double b[3];
      HHe.eval(z, b);
      return b[0] + rf.fHe * b[1];
    };
    auto tmat_recfast = [&](double z) -> double {  // recfast.jl:435-444
      if (z > zHe) return rf.Tnow * (1 + z);
      if (z > zHH) return He.eval1(z, 1);
      return HHe.eval1(z, 2);
    };
    const double Xfin = 1 + rf.Yp / (rf.not4 * (1 - rf.Yp));
    auto xe_reio = [&](double z) -> double {  // recfast.jl:478-488
      const double zre = 7.6711, al = 1.5, dH = 0.5, zHe2 = 3.5, dHe = 0.5;
      double xo = xe_recfast(z);
      double xH = (Xfin - xo) / 2 * (1 + std::tanh((std::pow(1 + zre, al) - std::pow(1 + z, al)) / (al * std::pow(1 + zre, al - 1)) / dH)) + xo;
      return xH + (Xfin - 1) / 2 * (1 + std::tanh((zHe2 - z) / dHe));
    };
    double T50 = tmat_recfast(zre_ini);
    Traj Re = tsit5_integrate(
        [&](double z, const double* u, double* du) {  // recfast.jl:491-502
          double xr = xe_reio(z), a = 1.0 / (1 + z);
          double Hz = sH(std::log(a)) / a / sec_per_nat(), Trad = rf.Tnow * (1 + z);
          du[0] = rf.CT * std::pow(Trad, 4) * xr / (1 + xr + rf.fHe) * (u[0] - Trad) / (Hz * (1 + z)) + 2 * u[0] / (1 + z);
        },
        1, &T50, zre_ini, zfin, rf.tol, 1e-6, zland, replay ? &fz->tRe : nullptr, replay ? &fz->hRe : nullptr);
    if (fz && !replay) {
      fz->zHe = zHe;
      fz->zHH = zHH;
      fz->tHe = He.t;
      fz->tHHe = HHe.t;
      fz->tRe = Re.t;
      fz->hHe = He.h;
      fz->hHHe = HHe.h;
      fz->hRe = Re.h;
      fz->have = true;
    }

    // --- node values (recfast.jl:689-708)
    double xini = std::log(1.0 / (zini + 1.0));
    for (int j = 0; j < n; ++j) {
      double x = g.at(j), z = 1.0 / std::exp(x) - 1.0;
      if (x < xini) {
        T.nodes[T_XE][j] = 1 + 2 * rf.fHe;
        T.nodes[T_TMAT][j] = rf.Tnow * (1 + z);
      } else {
        T.nodes[T_XE][j] = z > zre_ini ? xe_recfast(z) : xe_reio(z);
        T.nodes[T_TMAT][j] = z > zre_ini ? tmat_recfast(z) : Re.eval1(z, 0);
      }
    }
  }
  // tau' and its reverse cumulative trapezoid (ionization.jl:105-127)
  double mH = nat_mH(), sT = nat_sigmaT();
  std::vector<double> tp(n), tau(n);
  for (int j = 0; j < n; ++j) {
    double x = g.at(j), a = std::exp(x);
    double nH = p.Omega_b * bg.rc / (mH * a * a * a) * (1 - p.Y_p);
    tp[j] = -T.nodes[T_XE][j] * nH * a * sT / sH(x);
  }
  {
    double acc = 0.0;
    tau[n - 1] = 0.0;
    for (int i = 1; i < n; ++i) {
      int jr = n - 1 - i;
      acc += (g.at(jr) - g.at(jr + 1)) * (tp[jr] + tp[jr + 1]);
      tau[jr] = 0.5 * acc;
    }
  }
  for (int j = 0; j < n; ++j) {
    T.nodes[T_TAU][j] = tau[j];
    T.nodes[T_G][j] = -tp[j] * std::exp(-tau[j]);
  }
  // baryon sound speed from Tmat and its re-splined gradient (recfast.jl:709-712)
  Spl sT_, sXe;
  sT_.fit(g, T.nodes[T_TMAT]);
  sXe.fit(g, T.nodes[T_XE]);
  std::vector<double> tgrad(n);
  for (int j = 0; j < n; ++j) tgrad[j] = sT_.d1(g.at(j));
  Spl sTg;
  sTg.fit(g, tgrad);
  for (int j = 0; j < n; ++j) {
    double x = g.at(j);
    double pre = std::pow(rf.C, -2) * rf.k_B / rf.m_H * (1.0 / rf.mu_T + (1 - rf.Yp) * sXe(x));
    T.nodes[T_CSB2][j] = pre * (sT_(x) - 1.0 / 3.0 * sTg(x));
  }
  finish_uploaded_tables(T);
}

void finish_uploaded_tables(CosmoTables& T) {
  const GridSpec& g = T.grid;
  const int n = g.n;
  auto fit = [&](int s) {
    T.coef[s].assign(n + 2, 0.0);
    spline_coefs(T.nodes[s].data(), n, T.coef[s].data());
  };
  auto grad_of = [&](int src, int dst, int order) {
    T.nodes[dst].assign(n, 0.0);
    for (int j = 0; j < n; ++j)
      T.nodes[dst][j] = order == 1 ? spline_deriv(T.coef[src].data(), n, g.x0, g.h, g.at(j))
                                   : spline_deriv2(T.coef[src].data(), n, g.x0, g.h, g.at(j));
    fit(dst);
  };
  const int prim[] = {T_H, T_ETA, T_RHO0M, T_XE, T_TAU, T_G, T_TMAT, T_CSB2};
  for (int s : prim) fit(s);
  grad_of(T_H, T_HP, 1);
  grad_of(T_H, T_HPP, 2);
  grad_of(T_ETA, T_ETAP, 1);
  grad_of(T_ETA, T_ETAPP, 2);
  grad_of(T_TAU, T_TAUP, 1);
  grad_of(T_TAU, T_TAUPP, 2);
  grad_of(T_G, T_GP, 1);
  grad_of(T_G, T_GPP, 2);
}

}  // namespace bolt

namespace bolt {
// Gauss-Legendre nodes and weights on [-1, 1] (FastGaussQuadrature.gausslegendre).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) { gauss_legendre_nodes(n, x, w); }
}  // namespace bolt
