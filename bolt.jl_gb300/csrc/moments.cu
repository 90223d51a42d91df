// Moments of the spherical Bessel functions, I_m(x) = int_0^x t^m j_n(t) dt,
// their cubic B-spline table and the Filon-type integrals over it (Bolt.jl
// src/bessel/):
//
//   sph_j_moment_maclaurin_1F2 / _asymp / _weniger_1F2  moments.jl:56-92  -> moment_direct_kernel
//   sph_bessel_interpolator(nu, order, kmin, kmax, N)   interpolator.jl:81-110
//        -> moment_seg_kernel + moment_prefix_kernel (nodes) + bspline_fir_kernel / bspline_ends_kernel
//   MomentTable call (x)                                interpolator.jl:67-75 -> moment_eval_kernel
//   integrate_sph_bessel_filon                          integrator.jl:7-19    -> filon_kernel
//   _loop_integrate_sph_bessel_filon, summed            integrator.jl:25-38   -> filon_piecewise_kernel
//     (one integrand per k, the line-of-sight shape)                          -> filon_batched_kernel
//
// Methods.  The Maclaurin series of the moment below x = 2 (and below the
// table), the Lommel-function form above x_c = max(50, 4n) (and above the
// table): I_m = P_m + (m+n-1) x^{m-1} j_n(x) s(m-3/2, n-1/2) - x^m j_{n-1}(x)
// s(m-1/2, n+1/2), with s(p, q) = S_{p,q}(x) / x^{p-1} by its large-argument
// expansion and P_m = sqrt(pi) 2^{m-1} Gamma((n+m+1)/2) / Gamma((n-m)/2+1).
// Between them the reference evaluates a Weniger transform of 1F2 in
// Double64; here table nodes below x_c are prefix sums (compensated, one
// block) of 8-point Gauss-Legendre integrals over the node intervals, which
// every node computes independently; the direct evaluation integrates from 0
// (the first unit of t in u = sqrt(t), where t^m for half-integer m is not
// smooth).  All arithmetic is FP64.
//
// Table layout in HBM: coef[(N + 2) * order], the orders of one B-spline
// coefficient adjacent (one evaluation reads 4 * order consecutive-ish
// doubles).  The prefilter of the constant (1, 4, 1) system is the
// convolution c_j = sqrt(3) sum_d (-r)^|d| y_{j+d}, r = 2 - sqrt(3),
// truncated at |d| <= 32 (r^33 < 1e-18), one thread per coefficient; the
// coefficients within 32 of each end are solved exactly by a short
// sequential sweep between the known end value and the first convolved
// coefficient.
#include <cuda_runtime.h>

#include "bolt_dev.cuh"

namespace bolt {

// j_n(t) of one order (n = -1: cos t / t).  Power series below t = 1, upward
// recurrence where t >= n, otherwise the ratios j_l / j_{l+1} by the
// backward recurrence anchored on j_floor(t).
__host__ __device__ double sphj_dev(int n, double t) {
  if (n < 0) return cos(t) / t;
  if (t == 0.0) return n == 0 ? 1.0 : 0.0;
  if (t < 1.0) {
    double pre = 1.0;
    for (int i = 1; i <= n; ++i) pre *= t / (2.0 * i + 1.0);
    double term = 1.0, s = 1.0;
    for (int k = 1; k < 80; ++k) {
      term *= -t * t / (2.0 * k * (2.0 * n + 2.0 * k + 1.0));
      s += term;
      if (fabs(term) < 1e-18 * fabs(s)) break;
    }
    return pre * s;
  }
  double sn, cs;
  sincos(t, &sn, &cs);
  const double it = 1.0 / t;
  const double j0 = sn * it, j1 = (sn * it - cs) * it;
  if (n == 0) return j0;
  if (n == 1) return j1;
  double a = j0, b = j1;
  const int lt = t >= n ? n : (int)floor(t);
  for (int l = 1; l < lt; ++l) {
    double c = (2.0 * l + 1.0) * it * b - a;
    a = b;
    b = c;
  }
  if (t >= n) return b;
  const int ls = n + 20 + (int)ceil(10.0 * cbrt(t));
  double r = (2.0 * ls + 3.0) * it, prod = 1.0;
  for (int l = ls - 1; l >= lt; --l) {
    r = (2.0 * l + 3.0) * it - 1.0 / r;
    if (l < n) prod /= r;
  }
  return b * prod;
}

__host__ __device__ double mom_maclaurin(int n, double m, double x) {
  const double a = n + m;
  double pre;
  if (n <= 100) {
    double df = 1.0;
    for (int i = 1; i <= n; ++i) df *= 2.0 * i + 1.0;
    pre = pow(x, a + 1.0) / ((a + 1.0) * df);
  } else {
    double ldf = lgamma(2.0 * n + 2.0) - n * 0.69314718055994530942 - lgamma(n + 1.0);
    pre = exp((a + 1.0) * log(x) - log(a + 1.0) - ldf);
  }
  double term = 1.0, s = 1.0;
  for (int k = 1; k < 2000; ++k) {
    term *= -x * x * (a + 2.0 * k - 1.0) / (2.0 * k * (a + 2.0 * k + 1.0) * (2.0 * n + 2.0 * k + 1.0));
    s += term;
    if (fabs(term) < 1e-17 * fabs(s)) break;
  }
  return pre * s;
}

// S_{p,q}(x) / x^{p-1}, cut at the smallest term.
__host__ __device__ double lommel_ser(double p, double q, double x) {
  const double ix2 = 1.0 / (x * x);
  double s = 1.0, c = 1.0;
  for (int j = 0; j < 80; ++j) {
    double f = p - 1.0 - 2.0 * j;
    double cn = c * (q * q - f * f) * ix2;
    if (cn == 0.0 || fabs(cn) >= fabs(c)) break;
    c = cn;
    s += c;
    if (fabs(c) < 1e-18 * fabs(s)) break;
  }
  return s;
}

__host__ __device__ double gamma_ratio_dev(double a, double b) {
  if (b <= 0.0 && b == floor(b)) return 0.0;
  if (a < 150.0 && fabs(b) < 150.0) return tgamma(a) / tgamma(b);
  double sg = 1.0;
  if (b < 0.0) sg = (((long long)ceil(-b)) % 2 == 1) ? -1.0 : 1.0;
  return sg * exp(lgamma(a) - lgamma(b));
}

__host__ __device__ double mom_asymp(int n, double m, double x) {
  const double P = 1.7724538509055160273 * pow(2.0, m - 1.0) * gamma_ratio_dev(0.5 * (n + m + 1.0), 0.5 * (n - m) + 1.0);
  const double s1 = lommel_ser(m - 1.5, n - 0.5, x);
  const double s2 = lommel_ser(m - 0.5, n + 0.5, x);
  const double xm = pow(x, m);
  return P + (m + n - 1.0) * (xm / x) * sphj_dev(n, x) * s1 - xm * sphj_dev(n - 1, x) * s2;
}

__host__ __device__ __forceinline__ double mom_cut(int n) { return fmax(50.0, 4.0 * n); }

__device__ __forceinline__ double mom_warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// int_a^b t^m j_n(t) dt, 8-point Gauss-Legendre on consecutive panels of
// width min(1, 2 max(t, (n+1)/60) / (n+m+1)) at their left end t: below the
// turning point the integrand grows like t^(n+m), and a panel spans about
// two of its e-folds (the integrand smooth on [a, b]).
__host__ __device__ double mom_panels(int n, double m, double a, double b, const GL8& g) {
  if (!(b > a)) return 0.0;
  const double tfl = (n + 1.0) / 60.0, rate = 2.0 / (n + fabs(m) + 1.0);
  double s = 0.0, lo = a;
  while (lo < b) {
    const double w = fmin(1.0, rate * fmax(lo, tfl));
    const double hi = (b - lo <= 1.5 * w) ? b : lo + w;
    const double h = hi - lo, mid = lo + 0.5 * h;
    lo = hi;
    double ps = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const double t = fma(0.5 * h, g.x[q], mid);
      const double tm = m == 0.0 ? 1.0 : (m == 1.0 ? t : (m == 2.0 ? t * t : pow(t, m)));
      ps = fma(g.w[q], tm * sphj_dev(n, t), ps);
    }
    s = fma(0.5 * h, ps, s);
  }
  return s;
}

// int_0^x t^m j_n(t) dt: [0, min(x, 1)] as int 2 u^{2m+1} j_n(u^2) du, then t.
__host__ __device__ double mom_quad(int n, double m, double x, const GL8& g) {
  const double x1 = fmin(x, 1.0), u1 = sqrt(x1);
  double s = 0.0;
  const int npu = 4;
  const double hu = u1 / npu;
  for (int p = 0; p < npu; ++p) {
    const double mid = (p + 0.5) * hu;
    double ps = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const double u = fma(0.5 * hu, g.x[q], mid);
      ps = fma(g.w[q], 2.0 * pow(u, 2.0 * m + 1.0) * sphj_dev(n, u * u), ps);
    }
    s = fma(0.5 * hu, ps, s);
  }
  return s + mom_panels(n, m, x1, x, g);
}

__host__ __device__ double mom_direct(int n, double m, double x, const GL8& g) {
  if (x <= 2.0) return mom_maclaurin(n, m, x);
  if (x < mom_cut(n)) return mom_quad(n, m, x, g);
  return mom_asymp(n, m, x);
}

__global__ void moment_direct_kernel(int n, double m, const double* __restrict__ x, int nx, double* __restrict__ out,
                                     GL8 g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nx) out[i] = mom_direct(n, m, x[i], g);
}

__host__ __device__ __forceinline__ double node_x(const MomTabDev& T, int i) {
  return i == T.N - 1 ? T.kmax : fma((double)i, T.h, T.kmin);
}

// Node i: from nc on (the nodes at or above the cut) the Lommel form into
// y; below it the integral over [x_{i-1}, x_i] (from 0 for i = 0) into seg.
__host__ __device__ __forceinline__ void seg_node(const MomTabDev& T, int nc, int i, double* y, double* seg) {
  const double x = node_x(T, i);
  for (int m = 0; m < T.order; ++m) {
    if (i >= nc) {
      y[(size_t)i * T.order + m] = mom_asymp(T.n, m, x);
    } else {
      const double lo = i == 0 ? 0.0 : node_x(T, i - 1);
      seg[(size_t)i * T.order + m] = mom_panels(T.n, m, lo, x, T.g);
    }
  }
}

__global__ void moment_seg_kernel(MomTabDev T, int nc, double* __restrict__ y, double* __restrict__ seg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < T.N) seg_node(T, nc, i, y, seg);
}

__host__ __device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// y_i = sum_{j <= i} seg_j for the nodes below the cut (nc of them), one
// block: compensated (value, error) pairs, per-thread chunks, a block scan.
__global__ void __launch_bounds__(1024) moment_prefix_kernel(MomTabDev T, int nc, const double* __restrict__ seg,
                                                            double* __restrict__ y) {
  __shared__ double ss[1024], se[1024];
  const int tid = threadIdx.x, nth = blockDim.x;
  const int chunk = (nc + nth - 1) / nth;
  const int i0 = tid * chunk, i1 = min(nc, i0 + chunk);
  for (int m = 0; m < T.order; ++m) {
    double s = 0.0, c = 0.0;
    for (int i = i0; i < i1; ++i) {
      double e;
      two_sum(s, seg[(size_t)i * T.order + m], s, e);
      c += e;
    }
    ss[tid] = s;
    se[tid] = c;
    __syncthreads();
    // inclusive Hillis-Steele scan of the pairs
    for (int off = 1; off < nth; off <<= 1) {
      double os = 0.0, oc = 0.0;
      if (tid >= off) { os = ss[tid - off]; oc = se[tid - off]; }
      __syncthreads();
      if (tid >= off) {
        double s2, e;
        two_sum(os, ss[tid], s2, e);
        ss[tid] = s2;
        se[tid] = oc + se[tid] + e;
      }
      __syncthreads();
    }
    double ps = tid > 0 ? ss[tid - 1] : 0.0, pc = tid > 0 ? se[tid - 1] : 0.0;
    for (int i = i0; i < i1; ++i) {
      double e;
      two_sum(ps, seg[(size_t)i * T.order + m], ps, e);
      pc += e;
      y[(size_t)i * T.order + m] = ps + pc;
    }
    __syncthreads();
  }
}

constexpr int kFir = 32;

// Interior B-spline coefficients c[j], j = kFir + 1 .. N - kFir (1-based on
// the data: c[j] pairs with y[j - 1]), one thread per (j, order).
__host__ __device__ __forceinline__ void fir_coef(const MomTabDev& T, const double* y, const double* w, double* coef,
                                                  long long t) {
  const int j = kFir + 1 + (int)(t / T.order), m = (int)(t % T.order);
  const double* yc = y + (size_t)(j - 1) * T.order + m;
  double s = w[0] * yc[0];
#pragma unroll 8
  for (int d = 1; d <= kFir; ++d) s = fma(w[d], yc[(long long)d * T.order] + yc[-(long long)d * T.order], s);
  coef[(size_t)j * T.order + m] = s;
}

__global__ void bspline_fir_kernel(MomTabDev T, const double* __restrict__ y, const double* __restrict__ w,
                                   double* __restrict__ coef) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nj = T.N - 2 * kFir;
  if (t < (long long)nj * T.order) fir_coef(T, y, w, coef, t);
}

// The coefficients next to the ends (or all of them for short tables): the
// (1, 4, 1) system between c[1] = y[0] and the convolved c[kFir + 1] (left
// side), and between the convolved c[N - kFir] and c[N] = y[N - 1] (right
// side), by a sequential sweep; then the padding c[0], c[N + 1].  Thread
// t = side * order + m; below 2 kFir + 4 nodes one thread per order sweeps
// the whole table.
__host__ __device__ __forceinline__ void ends_thread(const MomTabDev& T, const double* y, double* coef, double* work,
                                                    int t) {
  const bool whole = T.N < 2 * kFir + 4;
  const int sides = whole ? 1 : 2;
  if (t >= sides * T.order) return;
  const int side = t / T.order, m = t % T.order, o = T.order, N = T.N;
  auto C = [&](int j) -> double& { return coef[(size_t)j * o + m]; };
  auto Y = [&](int i) { return y[(size_t)i * o + m]; };
  int j0, j1;  // unknowns c[j0..j1], c[j0 - 1] and c[j1 + 1] known
  if (whole) {
    C(1) = Y(0);
    C(N) = Y(N - 1);
    j0 = 2;
    j1 = N - 1;
  } else if (side == 0) {
    C(1) = Y(0);
    j0 = 2;
    j1 = kFir;
  } else {
    C(N) = Y(N - 1);
    j0 = N - kFir + 1;
    j1 = N - 1;
  }
  if (j1 >= j0) {
    double* cp = work + (size_t)t * (whole ? N : kFir + 2);
    // rows j: c[j-1] + 4 c[j] + c[j+1] = 6 y[j-1]
    double prev = 0.0;
    for (int j = j0; j <= j1; ++j) {
      double rhs = 6.0 * Y(j - 1);
      if (j == j0) rhs -= C(j0 - 1);
      if (j == j1) rhs -= C(j1 + 1);
      double den = 4.0 - (j == j0 ? 0.0 : cp[j - j0 - 1]);
      double inv = 1.0 / den;
      cp[j - j0] = inv;  // super-diagonal 1 / den
      prev = (rhs - (j == j0 ? 0.0 : prev)) * inv;
      C(j) = prev;
    }
    for (int j = j1 - 1; j >= j0; --j) C(j) = C(j) - cp[j - j0] * C(j + 1);
  }
  if (whole || side == 0) coef[0 * o + m] = 2.0 * C(1) - C(2);
  if (whole || side == 1) coef[(size_t)(N + 1) * o + m] = 2.0 * C(N) - C(N - 1);
}

__global__ void bspline_ends_kernel(MomTabDev T, const double* __restrict__ y, double* __restrict__ coef,
                                    double* __restrict__ work) {
  ends_thread(T, y, coef, work, threadIdx.x);
}

// MomentTable call: inside [kmin, kmax] the splines, above the Lommel form,
// below the series.
__host__ __device__ __forceinline__ void mom_eval(const MomTabDev& T, double x, double* out) {
  if (x >= T.kmin && x <= T.kmax) {
    double u = (x - T.kmin) / T.h;
    double fl = floor(u);
    fl = fmin(fmax(fl, 0.0), (double)(T.N - 2));
    const double t = u - fl, s = 1.0 - t, t2 = t * t, s2 = s * s;
    const double w0 = s2 * s * (1.0 / 6.0);
    const double w3 = t2 * t * (1.0 / 6.0);
    const double w1 = fma(t2, fma(0.5, t, -1.0), 2.0 / 3.0);  // 2/3 - t^2 + t^3/2
    const double w2 = fma(s2, fma(0.5, s, -1.0), 2.0 / 3.0);  // 2/3 - s^2 + s^3/2
    const double* c = T.coef + (size_t)fl * T.order;
    for (int m = 0; m < T.order; ++m)
      out[m] = c[m] * w0 + c[T.order + m] * w1 + c[2 * T.order + m] * w2 + c[3 * T.order + m] * w3;
  } else if (x > T.kmax) {
    for (int m = 0; m < T.order; ++m) out[m] = mom_asymp(T.n, m, x);
  } else {
    for (int m = 0; m < T.order; ++m) out[m] = mom_maclaurin(T.n, m, x);
  }
}

__global__ void moment_eval_kernel(MomTabDev T, const double* __restrict__ x, int nx, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx) return;
  double v[4];
  mom_eval(T, x[i], v);
  for (int m = 0; m < T.order; ++m) out[(size_t)i * T.order + m] = v[m];
}

// Polynomial coefficients of the quadratic with p(a) = f, p'(a) = f',
// p'' = f'': p(t) = c0 + c1 t + c2 t^2.
__host__ __device__ __forceinline__ void quad_coefs(double f, double fp, double fpp, double a, double& c0, double& c1,
                                           double& c2) {
  c2 = 0.5 * fpp;
  c1 = fp - a * fpp;
  c0 = f - a * fp + 0.5 * a * a * fpp;
}

// int_a^b p(t) j_n(k t) dt = sum_j c_j k^{-j-1} (I_j(k b) - I_j(k a)).
__host__ __device__ __forceinline__ double filon_one(const MomTabDev& T, double f, double fp, double fpp, double k,
                                                    double a, double b) {
  double c0, c1, c2;
  quad_coefs(f, fp, fpp, a, c0, c1, c2);
  const double ik = 1.0 / k;
  double Ia[4], Ib[4];
  mom_eval(T, k * a, Ia);
  mom_eval(T, k * b, Ib);
  return c0 * ik * (Ib[0] - Ia[0]) + c1 * ik * ik * (Ib[1] - Ia[1]) + c2 * ik * ik * ik * (Ib[2] - Ia[2]);
}

__global__ void filon_kernel(MomTabDev T, int n, const double* __restrict__ f, const double* __restrict__ fp,
                             const double* __restrict__ fpp, const double* __restrict__ k,
                             const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = filon_one(T, f[i], fp[i], fpp[i], k[i], a[i], b[i]);
}

// Node weights of the piecewise sum: the moments at t_i enter with
// D_j(i) = c_j(segment i - 1) - c_j(segment i) (c of the missing segments 0),
// so every node's moments are evaluated once (the reuse of
// _loop_integrate_sph_bessel_filon).  D[i * 4 + j], j < 3.
__host__ __device__ __forceinline__ void filon_weights(int nt, const double* t, const double* f, const double* fp,
                                                      const double* fpp, double* D, int i) {
  double l0 = 0.0, l1 = 0.0, l2 = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0;
  if (i > 0) quad_coefs(f[i - 1], fp[i - 1], fpp[i - 1], t[i - 1], l0, l1, l2);
  if (i < nt - 1) quad_coefs(f[i], fp[i], fpp[i], t[i], r0, r1, r2);
  D[(size_t)i * 4 + 0] = l0 - r0;
  D[(size_t)i * 4 + 1] = l1 - r1;
  D[(size_t)i * 4 + 2] = l2 - r2;
  D[(size_t)i * 4 + 3] = t[i];
}

__global__ void filon_weights_kernel(int nt, const double* __restrict__ t, const double* __restrict__ f,
                                     const double* __restrict__ fp, const double* __restrict__ fpp,
                                     double* __restrict__ D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nt) filon_weights(nt, t, f, fp, fpp, D, i);
}

// out[ik] = sum_i sum_j D_j(i) k^{-j-1} I_j(k t_i): one block per k (grid
// stride over k), threads over the nodes, a block reduction.
__global__ void __launch_bounds__(256) filon_piecewise_kernel(MomTabDev T, int nt, const double* __restrict__ D,
                                                              int nk, const double* __restrict__ k,
                                                              double* __restrict__ out) {
  __shared__ double red[32];
  for (int ik = blockIdx.x; ik < nk; ik += gridDim.x) {
    const double kk = k[ik], i1 = 1.0 / kk, i2 = i1 * i1, i3 = i2 * i1;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;  // sum_i D_j(i) I_j(k t_i), scaled by k^{-j-1} once
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
      const double2 d01 = reinterpret_cast<const double2*>(D)[2 * i];
      const double2 d23 = reinterpret_cast<const double2*>(D)[2 * i + 1];
      double v[4];
      mom_eval(T, kk * d23.y, v);
      a0 = fma(d01.x, v[0], a0);
      a1 = fma(d01.y, v[1], a1);
      a2 = fma(d23.x, v[2], a2);
    }
    double acc = fma(a0, i1, fma(a1, i2, a2 * i3));
    acc = mom_warp_sum(acc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = acc;
    __syncthreads();
    if (wid == 0) {
      double s = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
      s = mom_warp_sum(s);
      if (lane == 0) out[ik] = s;
    }
    __syncthreads();
  }
}

// The line-of-sight shape of the same sum: one integrand per k (f, f', f''
// [nk][nt] on shared nodes t), out[ik] = sum_i int_{t_i}^{t_{i+1}} p_{ik,i}(t)
// j_nu(k t) dt.  One block per k (grid-stride), threads over nodes; each
// node forms its weights from the quadratics of the segments on either side.
__global__ void __launch_bounds__(256) filon_batched_kernel(MomTabDev T, int nt, const double* __restrict__ t,
                                                            const double* __restrict__ f,
                                                            const double* __restrict__ fp,
                                                            const double* __restrict__ fpp, int nk,
                                                            const double* __restrict__ k, double* __restrict__ out) {
  __shared__ double red[32];
  for (int ik = blockIdx.x; ik < nk; ik += gridDim.x) {
    const double kk = k[ik], i1 = 1.0 / kk, i2 = i1 * i1, i3 = i2 * i1;
    const double* fk = f + (size_t)ik * nt;
    const double* fpk = fp + (size_t)ik * nt;
    const double* fppk = fpp + (size_t)ik * nt;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
      double l0 = 0.0, l1 = 0.0, l2 = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0;
      if (i > 0) quad_coefs(fk[i - 1], fpk[i - 1], fppk[i - 1], t[i - 1], l0, l1, l2);
      if (i < nt - 1) quad_coefs(fk[i], fpk[i], fppk[i], t[i], r0, r1, r2);
      double v[4];
      mom_eval(T, kk * t[i], v);
      a0 = fma(l0 - r0, v[0], a0);
      a1 = fma(l1 - r1, v[1], a1);
      a2 = fma(l2 - r2, v[2], a2);
    }
    double acc = fma(a0, i1, fma(a1, i2, a2 * i3));
    acc = mom_warp_sum(acc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = acc;
    __syncthreads();
    if (wid == 0) {
      double s = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
      s = mom_warp_sum(s);
      if (lane == 0) out[ik] = s;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- launchers ---
int launch_moment_direct(int n, double m, const double* d_x, int nx, double* d_out, const GL8& g, cudaStream_t st) {
  if (nx <= 0) return 0;
  moment_direct_kernel<<<(nx + 127) / 128, 128, 0, st>>>(n, m, d_x, nx, d_out, g);
  return (int)cudaGetLastError();
}

// Builds T.coef (N + 2) * order from scratch buffers y, seg ((N) * order
// each), the FIR weights w[kFir + 1] and work (2 * order * (kFir + 2), or
// order * N for short tables).
int launch_moment_table(const MomTabDev& T, double* d_y, double* d_seg, const double* d_w, double* d_work,
                        cudaStream_t st) {
  const int N = T.N;
  // the nodes below the cut are the first nc (node_x increases with i)
  const double cut = fmax(50.0, 4.0 * T.n);
  int nc = 0;
  if (cut > T.kmin) nc = (int)fmin((double)N, ceil((cut - T.kmin) / T.h));
  while (nc > 0 && node_x(T, nc - 1) >= cut) --nc;
  while (nc < N && node_x(T, nc) < cut) ++nc;
  moment_seg_kernel<<<(N + 127) / 128, 128, 0, st>>>(T, nc, d_y, d_seg);
  if (nc > 0) moment_prefix_kernel<<<1, 1024, 0, st>>>(T, nc, d_seg, d_y);
  if (N >= 2 * kFir + 4) {
    long long nthr = (long long)(N - 2 * kFir) * T.order;
    bspline_fir_kernel<<<(unsigned)((nthr + 255) / 256), 256, 0, st>>>(T, d_y, d_w, T.coef);
  }
  bspline_ends_kernel<<<1, 32, 0, st>>>(T, d_y, T.coef, d_work);
  return (int)cudaGetLastError();
}

int launch_moment_eval(const MomTabDev& T, const double* d_x, int nx, double* d_out, cudaStream_t st) {
  if (nx <= 0) return 0;
  moment_eval_kernel<<<(nx + 127) / 128, 128, 0, st>>>(T, d_x, nx, d_out);
  return (int)cudaGetLastError();
}

int launch_filon(const MomTabDev& T, int n, const double* f, const double* fp, const double* fpp, const double* k,
                 const double* a, const double* b, double* out, cudaStream_t st) {
  if (n <= 0) return 0;
  filon_kernel<<<(n + 127) / 128, 128, 0, st>>>(T, n, f, fp, fpp, k, a, b, out);
  return (int)cudaGetLastError();
}

int launch_filon_piecewise(const MomTabDev& T, int nt, const double* t, const double* f, const double* fp,
                           const double* fpp, double* D, int nk, const double* k, double* out, int nblocks,
                           cudaStream_t st) {
  if (nt <= 0 || nk <= 0) return 0;
  filon_weights_kernel<<<(nt + 255) / 256, 256, 0, st>>>(nt, t, f, fp, fpp, D);
  filon_piecewise_kernel<<<nblocks > 0 ? nblocks : nk, 256, 0, st>>>(T, nt, D, nk, k, out);
  return (int)cudaGetLastError();
}

int launch_filon_batched(const MomTabDev& T, int nt, const double* t, const double* f, const double* fp,
                         const double* fpp, int nk, const double* k, double* out, int nblocks, cudaStream_t st) {
  if (nt <= 0 || nk <= 0) return 0;
  filon_batched_kernel<<<nblocks > 0 ? nblocks : nk, 256, 0, st>>>(T, nt, t, f, fp, fpp, nk, k, out);
  return (int)cudaGetLastError();
}

}  // namespace bolt
