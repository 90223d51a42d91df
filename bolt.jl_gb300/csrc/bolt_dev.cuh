// Device-side data layout shared by the GB300 kernels.
//
// Per cosmology, HBM holds one CosmoDev record plus its spline tables.  The
// four tables the Rosenbrock right-hand side reads at every stage
// (conformal Hubble rate, conformal time, opacity tau', baryon sound speed)
// are interleaved coefficient-by-coefficient (hot[j][4]) so one 32-byte
// sector delivers all four coefficients of node j; the remaining tables are
// stored one after another (cold[t][n+2]).
#pragma once
#include <cstdint>

namespace bolt {

enum ColdId {
  C_H = 0, C_HP, C_HPP, C_ETA, C_TAU, C_TAUP, C_TAUPP, C_G, C_GP, C_GPP, C_CSB2, C_RHO0M, C_COUNT
};

struct CosmoDev {
  // cosmological parameters (CosmoParams, Bolt.jl:56-66); Sigma_m_nu in Mpc^-1
  double h, Omega_r, Omega_b, Omega_c, A, n_s, Y_p, N_nu, Sigma_m_nu;
  // background scalars
  double H0, eta0, rho_crit, eta_last;  // eta_last = bg.η(x_grid[end]) (host evaluation)
  double x_last;                        // x_grid[end]
  double Tnu, logqmin, logqmax;
  double Omega_nu;  // massless-neutrino density 7(2/3)N_nu/8 (4/11)^(4/3) Omega_r (perturbations.jl:171)
  // uniform x grid: x_j = x0 + j * hx, n nodes; inv_hx = 1 / hx
  double x0, hx, inv_hx;
  int n, nq;
  const double* hot;   // [n + 2][4]: H, eta, tau', csb2
  const double* cold;  // [C_COUNT][n + 2]
  const double* qw;    // [nq] Gauss-Legendre weights (on [-1, 1])
  const double* qx;    // [nq] Gauss-Legendre nodes
};

// One k-mode of one cosmology.
struct ModeDev {
  double k;
  int cosmo;
  int lg, lnu, lmnu, nq;
  int flags;          // MODE_* bits
  int nout;           // landing nodes
  const double* xout; // ascending landing nodes (device)
  double* src_T;      // [nout] source S_T at the landing nodes (MODE_SOURCES)
  double* src_E;      // [nout] source S_E
  double* traj;       // [nout][N] state at the landing nodes (MODE_TRAJ)
  double* plin;       // [1] P_lin at the last node (MODE_PLIN)
  int32_t* status;    // [1]
  int64_t* counters;  // [2] accepted steps, rejected steps
  double* rec;        // [rec_cap] end abscissae of the accepted steps (MODE_RECORD / MODE_REPLAY)
  int rec_cap;
  // MODE_TANGENT: the cosmologies (indices) of the four perturbed parameter
  // sets with 1 / their steps, and where the tangents of the outputs go
  // (null: not wanted)
  int tcos[4];
  double tinv[4];
  double* tsrc_T[4];  // [nout]
  double* tsrc_E[4];  // [nout]
  double* tplin[4];   // [1]
  // MODE_CKPT (with MODE_RECORD): the state at the start of every
  // kCkptEvery-th accepted step, [rec_cap / kCkptEvery + 1][N].
  // MODE_ADJOINT: the reverse sweep of such a forward mode (same ckpt / rec,
  // tcos / tinv as a tangent mode): its accepted steps (nfwd, the forward
  // mode's counters), the cotangents of its outputs (sbar: of S_T at the
  // nodes [nout], or of P_lin [1]) and where the cotangent's partial
  // derivatives along the four tangent directions go (tbar [4]).
  double* ckpt;
  const int64_t* nfwd;
  const double* sbar;
  double* tbar;
};
constexpr int kCkptEvery = 32;

// MODE_RECORD stores the end abscissa of every accepted step; MODE_REPLAY
// takes exactly those steps (no error control), so a mode of perturbed
// parameters is integrated on the same discretisation as the recorded one.
// MODE_TANGENT integrates, with the state, its derivatives with respect to
// four parameters (the tangent-linear solver, tangent.cuh).  MODE_CKPT
// keeps checkpoints of a recorded forward solve; MODE_ADJOINT runs its
// discrete adjoint backwards (adjoint.cuh).
enum ModeFlags {
  MODE_SOURCES = 1,
  MODE_TRAJ = 2,
  MODE_PLIN = 4,
  MODE_RECORD = 8,
  MODE_REPLAY = 16,
  MODE_TANGENT = 32,
  MODE_CKPT = 64,
  MODE_ADJOINT = 128
};

enum StatusBits {
  ST_OK = 0,
  ST_MAXITERS = 1,
  ST_DT_UNDERFLOW = 2,
  ST_NONFINITE = 3,
  ST_LU_FAIL = 4,
  ST_BAD_INPUT = 5,
  ST_REPLAY_SHORT = 6,   // MODE_REPLAY ran past the recorded steps
  ST_TANGENT_RSA = 7,    // MODE_TANGENT / MODE_ADJOINT: the radiation-streaming overwrite fired (no derivative here)
  ST_RSA_FIRED = 256,    // informational, OR-ed into the code
  ST_REC_OVERFLOW = 512  // MODE_RECORD: more accepted steps than rec_cap (record unusable)
};

struct SolverCfg {
  double reltol, abstol, h0;
  double x_dense;  // source nodes below this x come from dense output
  long long max_steps;
  int land_stride;  // source nodes at or above x_dense: every land_stride-th (and the last) is landed on,
                    // the others come from dense output (1: every node is landed on)
};

// Argument block of one solver launch captured as a graph kernel node.
struct RodasNodeArgs {
  const ModeDev* modes;
  int nmodes;
  const CosmoDev* cosmos;
  SolverCfg cfg;
  int* queue;
  double* scratch;
  int spm;
  void* ptrs[7];
};

// Reciprocal: the hardware approximation (rcp.approx.ftz.f64) refined by two
// Newton-Raphson iterations r <- r + r (1 - x r) (quadratic convergence to
// about an ulp of 1/x).  For finite, nonzero, normal x; 0 and non-finite x
// give non-finite results, which the callers test for.
__device__ __forceinline__ double frcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// ---------------------------------------------------------------- duals ----
struct dd {
  double v, d;
};
__device__ __forceinline__ dd mk(double v, double d) { dd r; r.v = v; r.d = d; return r; }
__device__ __forceinline__ dd operator+(dd a, dd b) { return mk(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return mk(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ dd operator-(dd a) { return mk(-a.v, -a.d); }
__device__ __forceinline__ dd operator*(dd a, dd b) { return mk(a.v * b.v, fma(a.d, b.v, a.v * b.d)); }
__device__ __forceinline__ dd operator*(dd a, double b) { return mk(a.v * b, a.d * b); }
__device__ __forceinline__ dd operator*(double b, dd a) { return mk(a.v * b, a.d * b); }
__device__ __forceinline__ dd operator+(dd a, double b) { return mk(a.v + b, a.d); }
__device__ __forceinline__ dd operator+(double b, dd a) { return mk(a.v + b, a.d); }
__device__ __forceinline__ dd operator-(dd a, double b) { return mk(a.v - b, a.d); }
__device__ __forceinline__ dd operator-(double b, dd a) { return mk(b - a.v, -a.d); }
__device__ __forceinline__ dd operator/(dd a, dd b) {
  double q = a.v / b.v;
  return mk(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ dd operator/(dd a, double b) { return mk(a.v / b, a.d / b); }
__device__ __forceinline__ dd operator/(double a, dd b) {
  double q = a / b.v;
  return mk(q, -q * b.d / b.v);
}
__device__ __forceinline__ double vof(double a) { return a; }
__device__ __forceinline__ double vof(dd a) { return a.v; }
template <class T> __device__ __forceinline__ T cst(double v);
template <> __device__ __forceinline__ double cst<double>(double v) { return v; }
template <> __device__ __forceinline__ dd cst<dd>(double v) { return mk(v, 0.0); }
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ dd dsqrt(dd a) { double s = sqrt(a.v); return mk(s, 0.5 * a.d / s); }
__device__ __forceinline__ double dexp(double a) { return exp(a); }
__device__ __forceinline__ dd dexp(dd a) { double e = exp(a.v); return mk(e, e * a.d); }

// Tangent numbers of the tangent-linear solver: a value and its derivatives
// along kTD parameter directions (d4), and the x-dual of such a number (x4:
// value and d/dx, each a d4), for the explicit x-derivative of the
// right-hand side's tangent.
constexpr int kTD = 4;
struct d4 {
  double v, t[kTD];
};
__device__ __forceinline__ d4 c4(double v) { d4 r; r.v = v; for (int j = 0; j < kTD; ++j) r.t[j] = 0.0; return r; }
__device__ __forceinline__ d4 operator+(const d4& a, const d4& b) {
  d4 r; r.v = a.v + b.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = a.t[j] + b.t[j];
  return r;
}
__device__ __forceinline__ d4 operator-(const d4& a, const d4& b) {
  d4 r; r.v = a.v - b.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = a.t[j] - b.t[j];
  return r;
}
__device__ __forceinline__ d4 operator-(const d4& a) {
  d4 r; r.v = -a.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = -a.t[j];
  return r;
}
__device__ __forceinline__ d4 operator*(const d4& a, const d4& b) {
  d4 r; r.v = a.v * b.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = fma(a.t[j], b.v, a.v * b.t[j]);
  return r;
}
__device__ __forceinline__ d4 operator*(const d4& a, double b) {
  d4 r; r.v = a.v * b;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = a.t[j] * b;
  return r;
}
__device__ __forceinline__ d4 operator*(double b, const d4& a) { return a * b; }
__device__ __forceinline__ d4 operator+(const d4& a, double b) { d4 r = a; r.v += b; return r; }
__device__ __forceinline__ d4 operator+(double b, const d4& a) { d4 r = a; r.v += b; return r; }
__device__ __forceinline__ d4 operator-(const d4& a, double b) { d4 r = a; r.v -= b; return r; }
__device__ __forceinline__ d4 operator-(double b, const d4& a) { return c4(b) - a; }
__device__ __forceinline__ d4 operator/(const d4& a, const d4& b) {
  d4 r; r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = (a.t[j] - r.v * b.t[j]) * ib;
  return r;
}
__device__ __forceinline__ d4 operator/(const d4& a, double b) {
  d4 r; r.v = a.v / b;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = a.t[j] / b;
  return r;
}
__device__ __forceinline__ d4 operator/(double a, const d4& b) { return c4(a) / b; }
__device__ __forceinline__ double vof(const d4& a) { return a.v; }
template <> __device__ __forceinline__ d4 cst<d4>(double v) { return c4(v); }
__device__ __forceinline__ d4 dsqrt(const d4& a) {
  d4 r; r.v = sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = a.t[j] * h;
  return r;
}
__device__ __forceinline__ d4 dexp(const d4& a) {
  d4 r; r.v = exp(a.v);
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = a.t[j] * r.v;
  return r;
}
__device__ __forceinline__ d4 dpow(const d4& a, double b) {  // a^b, a > 0
  d4 r; r.v = pow(a.v, b);
  const double dr = b * r.v / a.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = a.t[j] * dr;
  return r;
}

struct x4 {
  d4 v, d;
};
__device__ __forceinline__ x4 mkx(const d4& v, const d4& d) { x4 r; r.v = v; r.d = d; return r; }
__device__ __forceinline__ x4 operator+(const x4& a, const x4& b) { return mkx(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ x4 operator-(const x4& a, const x4& b) { return mkx(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ x4 operator-(const x4& a) { return mkx(-a.v, -a.d); }
__device__ __forceinline__ x4 operator*(const x4& a, const x4& b) { return mkx(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ x4 operator*(const x4& a, const d4& b) { return mkx(a.v * b, a.d * b); }
__device__ __forceinline__ x4 operator*(const d4& b, const x4& a) { return mkx(a.v * b, a.d * b); }
__device__ __forceinline__ x4 operator*(const x4& a, double b) { return mkx(a.v * b, a.d * b); }
__device__ __forceinline__ x4 operator*(double b, const x4& a) { return mkx(a.v * b, a.d * b); }
__device__ __forceinline__ x4 operator+(const x4& a, const d4& b) { return mkx(a.v + b, a.d); }
__device__ __forceinline__ x4 operator+(const d4& b, const x4& a) { return mkx(a.v + b, a.d); }
__device__ __forceinline__ x4 operator-(const x4& a, const d4& b) { return mkx(a.v - b, a.d); }
__device__ __forceinline__ x4 operator-(const d4& b, const x4& a) { return mkx(b - a.v, -a.d); }
__device__ __forceinline__ x4 operator+(const x4& a, double b) { return mkx(a.v + b, a.d); }
__device__ __forceinline__ x4 operator+(double b, const x4& a) { return mkx(a.v + b, a.d); }
__device__ __forceinline__ x4 operator-(const x4& a, double b) { return mkx(a.v - b, a.d); }
__device__ __forceinline__ x4 operator-(double b, const x4& a) { return mkx(b - a.v, -a.d); }
__device__ __forceinline__ x4 operator/(const x4& a, const x4& b) {
  d4 q = a.v / b.v;
  return mkx(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ x4 operator/(double a, const x4& b) {
  d4 q = a / b.v;
  return mkx(q, -(q * b.d) / b.v);
}
__device__ __forceinline__ double vof(const x4& a) { return a.v.v; }
template <> __device__ __forceinline__ x4 cst<x4>(double v) { return mkx(c4(v), c4(0.0)); }

// ------------------------------------------------------- spline evaluation
// Cubic B-spline on the uniform grid with Interpolations.jl's OnGrid
// indexing: interval i = clamp(floor(u), 0, n-2), t = u - i.
struct SplW {
  int i;
  double w0, w1, w2, w3;     // values
  double d0, d1, d2, d3;     // first derivative weights (per unit x)
};

__device__ __forceinline__ void spl_locate(const CosmoDev& c, double x, int& i, double& t) {
  double u = (x - c.x0) * c.inv_hx;
  double f = floor(u);
  f = fmin(fmax(f, 0.0), double(c.n - 2));
  i = int(f);
  t = u - f;
}

__device__ __forceinline__ void spl_weights(const CosmoDev& c, double x, SplW& w, bool deriv) {
  double t;
  spl_locate(c, x, w.i, t);
  double s = 1.0 - t, t2 = t * t, s2 = s * s;
  const double sixth = 1.0 / 6.0;
  w.w0 = s2 * s * sixth;
  w.w3 = t2 * t * sixth;
  w.w1 = (4.0 - 6.0 * t2 + 3.0 * t2 * t) * sixth;
  w.w2 = 1.0 - w.w0 - w.w1 - w.w3;
  if (deriv) {
    double ih = c.inv_hx;
    w.d0 = -0.5 * s2 * ih;
    w.d3 = 0.5 * t2 * ih;
    w.d1 = (-2.0 * t + 1.5 * t2) * ih;
    w.d2 = -(w.d0 + w.d1 + w.d3);
  }
}

__device__ __forceinline__ double spl_cold(const CosmoDev& c, int id, double x) {
  const double* p = c.cold + (size_t)id * (c.n + 2);
  double t;
  int i;
  spl_locate(c, x, i, t);
  double s = 1.0 - t, t2 = t * t, s2 = s * s;
  return (p[i] * s2 * s + p[i + 1] * (4.0 - 6.0 * t2 + 3.0 * t2 * t) + p[i + 2] * (4.0 - 6.0 * s2 + 3.0 * s2 * s) +
          p[i + 3] * t2 * t) * (1.0 / 6.0);
}

// Arguments of the line-of-sight kernels (los.cu): the C_l reduction of
// cltt / clte / clee (spectra.jl:70-160) over ncz cosmologies, and the C_l^TT
// reduction with its tangent along six parameter directions.
struct LosArgs {
  int nb, nslots, nrow, nm;
  const int* ells;          // [nslots]
  const double* coef;       // [ncz][nslots][nb+2]
  const double* inv_dg;     // [ncz]
  const double* yv;         // [ncz][nrow]  eta0 - eta(x_i)
  const double* kmid;       // [ncz][nm]
  const double* wts;        // [ncz][nm]
  const double* SdT;        // [ncz][nrow][nm]
  const double* SdE;        // [ncz][nrow][nm] or null
  double* tt;               // [ncz][nslots]
  double* te;
  double* ee;
  unsigned long long* terms;  // (l, k, x) terms evaluated, accumulated (null: not counted)
};

struct LosGradArgs {
  int nb, nslots, nrow, nm;
  const int* ells;
  const double* coef;   // [nslots][nb+2]
  const double* inv_dg; // [1]
  const double* yv;     // [nrow]
  const double* dyv;    // [6][dstride]
  const double* kmid;   // [nm]
  const double* wts;    // [nm]
  const double* dwts;   // [6][dstride]
  int dstride;          // stride of dwts and dyv per direction
  const double* Sd;     // [nrow][nm]
  const double* dSd;    // [6][nrow][nm]
  double* tt;           // [nslots]
  double* dtt;          // [6][nslots]
  unsigned long long* terms;  // (l, k, x) terms evaluated, accumulated (null: not counted)
  // the line of sight's adjoint (dSd null: the derivatives at fixed
  // sources): 2 w_m Delta_l(k_m) per slot [nslots][nm], and the slot's
  // zero-skip bound on the Bessel argument [nslots] (null: not written)
  double* cbar;
  double* ulo;
};

// The adjoint of the C_l^TT projection for one cotangent ybar[nslots]:
// Sbar_d[i][m] = 4 pi sum_l ybar_l cbar[l][m] j_l(k_m y_i) over the terms
// the forward reduction evaluated, then back through the resampling to the
// sources' cotangent Sbar[nk][nx] at the nodes i0 .. i0 + nrow - 1.
struct LosAdjArgs {
  int nb, nslots, nrow, nm, nk, nx, i0;
  const double* coef;   // [nslots][nb+2]
  const double* inv_dg; // [1]
  const double* yv;     // [nrow]
  const double* kmid;   // [nm]
  const double* kgrid;  // [nk]
  const double* dxs;    // [nrow]
  const double* ybar;   // [nslots]
  const double* cbar;   // [nslots][nm]
  const double* ulo;    // [nslots]
  double* Sbd;          // [nrow][nm] (zeroed by the launcher)
  double* Sbar;         // [nk][nx] (zeroed by the launcher)
};

// 8-point Gauss-Legendre rule on [-1, 1] (nodes ascending).
struct GL8 {
  double x[8], w[8];
};

// A spherical-Bessel moment table (order moments m = 0..order-1 of j_n on N
// uniform nodes of [kmin, kmax], step h) and its B-spline coefficients
// coef[(N + 2) * order] in HBM.
struct MomTabDev {
  double* coef;
  int n, order, N;
  double kmin, kmax, h;
  GL8 g;
};

}  // namespace bolt
