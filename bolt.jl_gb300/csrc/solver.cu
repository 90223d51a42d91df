// Persistent Rosenbrock (Rodas4) solver for the Newtonian-gauge Boltzmann
// hierarchy, one warp per k-mode.
//
// Restates, on the GPU, boltsolve + hierarchy! + initial_conditions +
// source_function(_P) + plin from Bolt.jl (src/perturbations.jl:25-33,
// 161-271, 274-338, 343-404; src/spectra.jl:163-198).  The reference
// integrates with OrdinaryDiffEq's KenCarp4; this kernel integrates the same
// linear ODE u' = A(x) u with Rodas4 (Hairer & Wanner, RODAS coefficient
// set 1), landing exactly on every output node.
//
// Linear algebra.  A(x) = L(x) + U(x) W(x)^T where L is block diagonal with
// one tridiagonal chain per species (photon temperature with the baryon pair
// (delta_b, v_b) hanging off Theta_1, photon polarization, massless
// neutrinos, one chain per massive-neutrino momentum bin, the CDM pair and
// Phi) and U W^T holds the three global couplings Phi', Psi and Pi.  Each
// chain is eliminated from its highest multipole down to l = 0, so the
// rank-3 border only touches the last few rows of every chain: a stage
// solve is one forward sweep, a 3x3 capacitance solve on the chain tails,
// and one back substitution -- O(N) FP64 work, one lane per chain.
//
// Memory.  Everything the serial chain sweeps and the right-hand side touch
// (stage state, the vector being solved, the chain factors, border tails,
// stage scalars) lives in shared memory; the state, the six stage increments
// and the previous step for dense output live in a per-warp global slab that
// stays L2-resident, so eight modes fit on an SM.  Warps pull modes from a
// device work queue so modes with very different step counts balance across
// the 152 SMs.
//
// Outputs.  Trajectory nodes and source nodes at x >= x_dense are landed on
// exactly; source nodes below x_dense (before recombination, where the
// line-of-sight integral never reads them) come from cubic Hermite dense
// output between accepted steps, as the reference's KenCarp4 dense output
// does for every node.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "bolt_dev.cuh"

namespace bolt {

namespace rodas {
__constant__ double kA[5][4] = {{1.544, 0, 0, 0},
                                {0.9466785280815826, 0.2557011698983284, 0, 0},
                                {3.314825187068521, 2.896124015972201, 0.9986419139977817, 0},
                                {1.221224509226641, 6.019134481288629, 12.53708332932087, -0.687886036105895},
                                {0, 0, 0, 0}};
__constant__ double kC[6][5] = {{0, 0, 0, 0, 0},
                                {-5.6688, 0, 0, 0, 0},
                                {-2.430093356833875, -0.2063599157091915, 0, 0, 0},
                                {-0.1073529058151375, -9.594562251023355, -20.47028614809616, 0, 0},
                                {7.496443313967647, -10.24680431464352, -33.99990352819905, 11.7089089320616, 0},
                                {8.083246795921522, -7.981132988064893, -31.52159432874371, 16.31930543123136,
                                 -6.058818238834054}};
__constant__ double kCx[6] = {0.0, 0.386, 0.21, 0.63, 1.0, 1.0};
__constant__ double kD[6] = {0.25, -0.1043, 0.1035, -0.0362, 0.0, 0.0};
constexpr double kGamma = 0.25;
}  // namespace rodas

constexpr int kTail = 5;   // tail slots per chain
constexpr int kBorder = 3; // Phi', Psi, Pi

// Shared memory per warp (mode): the stage state yt and the vector being
// solved b (both read at random by the chain sweeps and the right-hand
// side), the chain factors, the border tails and the per-stage scalars.
// The state y, the stage increments K_1..K_6, df/dx and the previous step
// (for dense output) live in a per-warp global scratch slab that stays
// resident in L2; they are only touched by row-parallel, coalesced loops.
constexpr int kStages = 6;   // slots: 0..4 the distinct stage abscissae, 5 any other x
constexpr int kScal = 12;    // scalars per slot

struct Shared {
  double *yt, *b, *fl, *fi, *fc;
  double *q, *df0, *Aq, *Bq, *qe, *eq, *qe_d, *eq_d;
  double *Uf, *Wt, *cl1, *cl2, *sc, *sc_d, *misc;
  // tangent-linear modes only (null otherwise): tangents [..][kTD] of the
  // stage scalars (slots 0..5, and d/dx at slot 0), q / eps and eps / q,
  // the perturbed sets' momenta, the tangents of the per-mode q constants
  // and of the cosmology constants; the tangent stage states yd and
  // right-hand sides bd ([kTD][N]) and the border partials of the tangent
  // solves
  double *sct, *sct_d, *qet, *eqt, *qet_d, *eqt_d, *qpj, *dq, *ddf0, *dAq, *dBq, *cstn, *yd, *bd, *part4;
};

struct Scratch {
  double *y, *fx, *K, *yp, *fp;  // K: 6 x N
};

constexpr int kMiscDoubles = 32 + 9 * 32;  // capacitance, reductions, per-chain partials

// Lane packing of the chains (chains.cuh): seg + chain per thread, the
// element lists (768 ints for every variant), owners and three counters.
__host__ __device__ inline int pack_ints(int threads) { return 2 * threads + 768 + 32 + 4; }

// The coefficient tangents of a tangent or adjoint mode: stage-scalar
// tangents (6 slots and d/dx), q/eps and eps/q tangents, the perturbed sets'
// momenta and the momentum-bin constants' tangents, the cosmology
// constants' tangents -- at most kCoefTanMax doubles (nq <= 27).
__host__ __device__ inline int coef_tan_doubles(int nq) {
  return (kStages + 1) * kScal * kTD + 2 * (kStages + 1) * nq * kTD + 5 * nq * kTD + 8 * kTD;
}
constexpr int kCoefTanMax = (kStages + 1) * kScal * kTD + 2 * (kStages + 1) * 27 * kTD + 5 * 27 * kTD + 8 * kTD;
// A tangent mode keeps them in shared memory with the tangent solves' border
// partials and its tangent stage state and right-hand sides (kTD x N each);
// an adjoint mode keeps them in its global slab (read through L1), so that
// as many adjoint CTAs fit an SM as plain ones.  (Measured: the tangent
// kernel with its stage vectors in the global slab instead runs 0.27 vs
// 0.33 served spectra/s -- its solves then read global memory.)
__host__ __device__ inline int tan_doubles(int N, int nq) {
  return coef_tan_doubles(nq) + 32 * kBorder * kTD + 2 * kTD * N;
}
// Kernel kinds: 0 plain (and recorded / replayed / checkpointed) modes,
// 1 tangent-linear modes, 2 adjoint (reverse-sweep) modes.
__host__ __device__ inline int per_mode_doubles(int N, int nq, int Lmax, int threads, int kind = 0) {
  int nch = nq + 5;
  return 5 * N + 4 * nq + 2 * kStages * nq + 2 * nq + 2 * nch * kTail * kBorder + 2 * (Lmax + 1) + kStages * kScal +
         kScal + kMiscDoubles + (kind == 1 ? tan_doubles(N, nq) : 0) +
         (pack_ints(threads) + 1) / 2;
}
// Global scratch of an adjoint mode after the base slab (adjoint.cuh).
__host__ __device__ inline int adj_scratch_doubles(int N) { return (15 + 2 * kTD + 7 * kCkptEvery + 1) * N; }
__host__ __device__ inline int scratch_per_warp(int N, int kind = 0) {
  return 10 * N + (kind == 1 ? 9 * kTD * N : (kind == 2 ? adj_scratch_doubles(N) + kCoefTanMax : 0));
}

struct Mode {
  const CosmoDev* C;
  double k;
  int N, lg, lnu, lmnu, nq, iTp, iN, iM, iPhi, nch;
  // tangent-linear modes: the cosmologies of the kTD perturbed parameter
  // sets and 1 / their parameter steps (coefficient tangents are their
  // differences from C over the step)
  const CosmoDev* tc[kTD];
  double tinv[kTD];
};

// The four interleaved hot tables at node j (H, eta, tau', csb2).
struct HotCoef {
  double x, y, z, w;
};
__device__ __forceinline__ void load_hot(const CosmoDev& C, int i, HotCoef& c0, HotCoef& c1, HotCoef& c2, HotCoef& c3) {
  const double2* p = reinterpret_cast<const double2*>(C.hot + 4 * (size_t)i);
  double2 a0 = __ldg(p), b0 = __ldg(p + 1), a1 = __ldg(p + 2), b1 = __ldg(p + 3);
  double2 a2 = __ldg(p + 4), b2 = __ldg(p + 5), a3 = __ldg(p + 6), b3 = __ldg(p + 7);
  c0.x = a0.x; c0.y = a0.y; c0.z = b0.x; c0.w = b0.y;
  c1.x = a1.x; c1.y = a1.y; c1.z = b1.x; c1.w = b1.y;
  c2.x = a2.x; c2.y = a2.y; c2.z = b2.x; c2.w = b2.y;
  c3.x = a3.x; c3.y = a3.y; c3.z = b3.x; c3.w = b3.y;
}

// Stage scalars: everything in the right-hand side that depends on x only.
template <class T>
struct Scal {
  T Hc, eta, tp, cs2, a, kH, iHe, R, cpsi, dphi, k2H2;
};

// The eleven stage scalars (and their x-derivatives into d, when d is not
// null) of cosmology C at x for wavenumber k.
__device__ __forceinline__ void stage_scalars_vals(const CosmoDev& C, double k, double x, double* o, double* od) {
  SplW w;
  spl_weights(C, x, w, true);
  HotCoef c0, c1, c2, c3;
  load_hot(C, w.i, c0, c1, c2, c3);
  dd Hc = mk(c0.x * w.w0 + c1.x * w.w1 + c2.x * w.w2 + c3.x * w.w3, c0.x * w.d0 + c1.x * w.d1 + c2.x * w.d2 + c3.x * w.d3);
  dd eta = mk(c0.y * w.w0 + c1.y * w.w1 + c2.y * w.w2 + c3.y * w.w3, c0.y * w.d0 + c1.y * w.d1 + c2.y * w.d2 + c3.y * w.d3);
  dd tp = mk(c0.z * w.w0 + c1.z * w.w1 + c2.z * w.w2 + c3.z * w.w3, c0.z * w.d0 + c1.z * w.d1 + c2.z * w.d2 + c3.z * w.d3);
  dd cs2 = mk(c0.w * w.w0 + c1.w * w.w1 + c2.w * w.w2 + c3.w * w.w3, c0.w * w.d0 + c1.w * w.d1 + c2.w * w.d2 + c3.w * w.d3);
  double ea = exp(x);
  dd a = mk(ea, ea);
  dd iH = 1.0 / Hc;
  dd v[11];
  v[0] = Hc; v[1] = eta; v[2] = tp; v[3] = cs2; v[4] = a;
  v[5] = k * iH;
  v[6] = iH / eta;
  v[7] = (4.0 * C.Omega_r / (3.0 * C.Omega_b)) / a;
  v[8] = (12.0 * C.H0 * C.H0 / (k * k)) / (a * a);
  v[9] = (C.H0 * C.H0 * 0.5) * iH * iH;
  v[10] = (k * k / 3.0) * iH * iH;
  for (int f = 0; f < 11; ++f) o[f] = v[f].v;
  if (od)
    for (int f = 0; f < 11; ++f) od[f] = v[f].d;
}

// Scalars (and their x-derivatives) at x, one lane per abscissa, written to
// shared-memory slot `slot`; derivatives are kept for slot 0 only.
__device__ __forceinline__ void stage_scalars_to(const Mode& m, const Shared& S, double x, int slot) {
  stage_scalars_vals(*m.C, m.k, x, S.sc + slot * kScal, slot == 0 ? S.sc_d : nullptr);
}

// Momentum-bin constants of cosmology C for bin q (background.jl:21-30,
// perturbations.jl:127-158): the momentum q, dlnf0/dlnq, and the weights of
// the rho / sigma (Aq) and theta (Bq) integrals.
__device__ __forceinline__ void qconst(const CosmoDev& C, int q, double& qq, double& df0, double& Aq, double& Bq) {
  double xq = C.qx[q];
  double lq = C.logqmin + (C.logqmax - C.logqmin) / 2.0 * (xq + 1.0);
  qq = pow(10.0, lq);
  double dxdq = (1.0 + (-1.0 + 2.0 / (C.logqmax - C.logqmin) * ((1.0 + C.logqmin) - C.logqmin))) / (qq * log(10.0));
  double f0 = 2.0 / pow(2.0 * M_PI, 3.0) / (exp(qq / C.Tnu) + 1.0);
  df0 = -qq / C.Tnu / (1.0 + exp(-qq / C.Tnu));
  Aq = 4.0 * M_PI * qq * qq * f0 / dxdq * C.qw[q];  // rho: Aq eps M0, sigma: Aq q^2/eps M2
  Bq = 4.0 * M_PI * qq * qq * qq * f0 / dxdq * C.qw[q];
}

// Massive-neutrino energies q/eps, eps/q for (slot, q) pairs spread over the CTA.
__device__ __forceinline__ void nu_energies_slots(const Mode& m, const Shared& S, int s0, int s1, int tid, int nth) {
  const int nq = m.nq, tot = (s1 - s0) * nq;
  for (int t = tid; t < tot; t += nth) {
    int sl = s0 + t / nq, q = t - (t / nq) * nq;
    double a = S.sc[sl * kScal + 4];
    double am = a * m.C->Sigma_m_nu, qq = S.q[q];
    double eps = sqrt(qq * qq + am * am);
    S.qe[sl * nq + q] = qq / eps;
    S.eq[sl * nq + q] = eps / qq;
    if (sl == 0) {
      double deps = am * am / eps;  // d eps / dx
      S.qe_d[q] = -qq * deps / (eps * eps);
      S.eq_d[q] = deps / qq;
    }
  }
}

// All stage abscissae of one step at once (slots 0..4: x, x + c2 h, x + c3 h,
// x + c4 h, x_new), one thread per abscissa.
__device__ __forceinline__ void prepare_stages(const Mode& m, const Shared& S, double x, double h, double xn, int tid,
                                               int nth) {
  if (tid < 5) {
    double xs = tid == 0 ? x : (tid == 4 ? xn : x + rodas::kCx[tid] * h);
    stage_scalars_to(m, S, xs, tid);
  }
  __syncthreads();
  nu_energies_slots(m, S, 0, 5, tid, nth);
  __syncthreads();
}

// One extra abscissa in slot 5 (dense-output and final nodes).
__device__ __forceinline__ void prepare_other(const Mode& m, const Shared& S, double x, int tid, int nth) {
  if (tid == 0) stage_scalars_to(m, S, x, 5);
  __syncthreads();
  nu_energies_slots(m, S, 5, 6, tid, nth);
  __syncthreads();
}

template <class T> __device__ __forceinline__ Scal<T> get_scal(const Shared& S, int slot);
template <> __device__ __forceinline__ Scal<double> get_scal<double>(const Shared& S, int slot) {
  const double* o = S.sc + slot * kScal;
  Scal<double> s;
  s.Hc = o[0]; s.eta = o[1]; s.tp = o[2]; s.cs2 = o[3]; s.a = o[4]; s.kH = o[5]; s.iHe = o[6]; s.R = o[7];
  s.cpsi = o[8]; s.dphi = o[9]; s.k2H2 = o[10];
  return s;
}
template <> __device__ __forceinline__ Scal<dd> get_scal<dd>(const Shared& S, int slot) {
  const double* o = S.sc + slot * kScal;
  const double* d = S.sc_d;
  Scal<dd> s;
  s.Hc = mk(o[0], d[0]); s.eta = mk(o[1], d[1]); s.tp = mk(o[2], d[2]); s.cs2 = mk(o[3], d[3]); s.a = mk(o[4], d[4]);
  s.kH = mk(o[5], d[5]); s.iHe = mk(o[6], d[6]); s.R = mk(o[7], d[7]); s.cpsi = mk(o[8], d[8]);
  s.dphi = mk(o[9], d[9]); s.k2H2 = mk(o[10], d[10]);
  return s;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Number types of a right-hand-side evaluation: T, the type of its stage
// scalars (double; dd for d/dx; d4 for the tangents along kTD parameter
// directions; x4 for both), and KT<T>, the type of its per-mode and
// per-cosmology constants (double, or d4 with their tangents).
template <class T> struct KT { using type = double; };
template <> struct KT<d4> { using type = d4; };
template <> struct KT<x4> { using type = d4; };

// A per-mode constant v[i] (with its tangents t[i * kTD + j] for K = d4).
template <class K> __device__ __forceinline__ K kval(const double* v, const double* t, int i);
template <> __device__ __forceinline__ double kval<double>(const double* v, const double*, int i) { return v[i]; }
template <> __device__ __forceinline__ d4 kval<d4>(const double* v, const double* t, int i) {
  d4 r;
  r.v = v[i];
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = t[i * kTD + j];
  return r;
}

// Per-cosmology constants: 0.25 / rho_crit, 1 / rho_crit, Omega_c, Omega_b,
// H0, rho_crit, Sigma_m_nu, h (tangents in S.cstn[id * kTD + j]).
constexpr int kCosN = 8;
__device__ __forceinline__ double cos_const(const CosmoDev& C, int id) {
  switch (id) {
    case 0: return 0.25 / C.rho_crit;
    case 1: return 1.0 / C.rho_crit;
    case 2: return C.Omega_c;
    case 3: return C.Omega_b;
    case 4: return C.H0;
    case 5: return C.rho_crit;
    case 6: return C.Sigma_m_nu;
    default: return C.h;
  }
}
template <class K> __device__ __forceinline__ K kcos(const Mode& m, const Shared& S, int id);
template <> __device__ __forceinline__ double kcos<double>(const Mode& m, const Shared&, int id) {
  return cos_const(*m.C, id);
}
template <> __device__ __forceinline__ d4 kcos<d4>(const Mode& m, const Shared& S, int id) {
  d4 r;
  r.v = kcos<double>(m, S, id);
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = S.cstn[id * kTD + j];
  return r;
}

template <class T> __device__ __forceinline__ T qe_of(const Shared& S, int sl, int nq, int q);
template <> __device__ __forceinline__ double qe_of<double>(const Shared& S, int sl, int nq, int q) { return S.qe[sl * nq + q]; }
template <> __device__ __forceinline__ dd qe_of<dd>(const Shared& S, int sl, int nq, int q) { return mk(S.qe[q], S.qe_d[q]); }
template <> __device__ __forceinline__ d4 qe_of<d4>(const Shared& S, int sl, int nq, int q) {
  return kval<d4>(S.qe, S.qet, sl * nq + q);
}
template <> __device__ __forceinline__ x4 qe_of<x4>(const Shared& S, int sl, int nq, int q) {
  return mkx(kval<d4>(S.qe, S.qet, q), kval<d4>(S.qe_d, S.qet_d, q));
}
template <class T> __device__ __forceinline__ T eq_of(const Shared& S, int sl, int nq, int q);
template <> __device__ __forceinline__ double eq_of<double>(const Shared& S, int sl, int nq, int q) { return S.eq[sl * nq + q]; }
template <> __device__ __forceinline__ dd eq_of<dd>(const Shared& S, int sl, int nq, int q) { return mk(S.eq[q], S.eq_d[q]); }
template <> __device__ __forceinline__ d4 eq_of<d4>(const Shared& S, int sl, int nq, int q) {
  return kval<d4>(S.eq, S.eqt, sl * nq + q);
}
template <> __device__ __forceinline__ x4 eq_of<x4>(const Shared& S, int sl, int nq, int q) {
  return mkx(kval<d4>(S.eq, S.eqt, q), kval<d4>(S.eq_d, S.eqt_d, q));
}

template <> __device__ __forceinline__ Scal<d4> get_scal<d4>(const Shared& S, int slot) {
  const int o = slot * kScal;
  Scal<d4> s;
  s.Hc = kval<d4>(S.sc, S.sct, o + 0); s.eta = kval<d4>(S.sc, S.sct, o + 1); s.tp = kval<d4>(S.sc, S.sct, o + 2);
  s.cs2 = kval<d4>(S.sc, S.sct, o + 3); s.a = kval<d4>(S.sc, S.sct, o + 4); s.kH = kval<d4>(S.sc, S.sct, o + 5);
  s.iHe = kval<d4>(S.sc, S.sct, o + 6); s.R = kval<d4>(S.sc, S.sct, o + 7); s.cpsi = kval<d4>(S.sc, S.sct, o + 8);
  s.dphi = kval<d4>(S.sc, S.sct, o + 9); s.k2H2 = kval<d4>(S.sc, S.sct, o + 10);
  return s;
}
template <> __device__ __forceinline__ Scal<x4> get_scal<x4>(const Shared& S, int) {
  Scal<x4> s;
#define XS(f, i) s.f = mkx(kval<d4>(S.sc, S.sct, i), kval<d4>(S.sc_d, S.sct_d, i))
  XS(Hc, 0); XS(eta, 1); XS(tp, 2); XS(cs2, 3); XS(a, 4); XS(kH, 5); XS(iHe, 6); XS(R, 7); XS(cpsi, 8);
  XS(dphi, 9); XS(k2H2, 10);
#undef XS
  return s;
}

// Where a right-hand side goes: values (and d/dx for dd) into v (d); the
// tangents of a d4 evaluation into t[j * N + i]; an x4 evaluation writes its
// value to v, its tangents to t and the tangents of its x-derivative to td.
struct Sink {
  double *v, *d, *t, *td;
  int N;
};
template <class T> __device__ __forceinline__ void put(const Sink& o, int i, const T& x);
template <> __device__ __forceinline__ void put<double>(const Sink& o, int i, const double& x) { o.v[i] = x; }
template <> __device__ __forceinline__ void put<dd>(const Sink& o, int i, const dd& x) { o.v[i] = x.v; o.d[i] = x.d; }
template <> __device__ __forceinline__ void put<d4>(const Sink& o, int i, const d4& x) {
#pragma unroll
  for (int j = 0; j < kTD; ++j) o.t[j * o.N + i] = x.t[j];
}
template <> __device__ __forceinline__ void put<x4>(const Sink& o, int i, const x4& x) {
  o.v[i] = x.v.v;
#pragma unroll
  for (int j = 0; j < kTD; ++j) {
    o.t[j * o.N + i] = x.v.t[j];
    o.td[j * o.N + i] = x.d.t[j];
  }
}
__device__ __forceinline__ Sink sink(double* v, double* d = nullptr) { Sink o; o.v = v; o.d = d; o.t = o.td = nullptr; o.N = 0; return o; }

// State read by a right-hand side: plain values, or values with their
// tangents du[j * N + i].
struct StP {
  const double* u;
  __device__ __forceinline__ double operator[](int i) const { return u[i]; }
};
struct StD4 {
  const double* u;
  const double* du;
  int N;
  __device__ __forceinline__ d4 operator[](int i) const {
    d4 r;
    r.v = u[i];
#pragma unroll
    for (int j = 0; j < kTD; ++j) r.t[j] = du[j * N + i];
    return r;
  }
};

template <class T> __device__ __forceinline__ T warp_sum_t(T v);
template <> __device__ __forceinline__ double warp_sum_t<double>(double v) { return warp_sum(v); }
template <> __device__ __forceinline__ dd warp_sum_t<dd>(dd v) { return mk(warp_sum(v.v), warp_sum(v.d)); }
template <> __device__ __forceinline__ d4 warp_sum_t<d4>(d4 v) {
  v.v = warp_sum(v.v);
#pragma unroll
  for (int j = 0; j < kTD; ++j) v.t[j] = warp_sum(v.t[j]);
  return v;
}
template <> __device__ __forceinline__ x4 warp_sum_t<x4>(x4 v) { return mkx(warp_sum_t<d4>(v.v), warp_sum_t<d4>(v.d)); }

// The radiation-streaming switch of hierarchy! (perturbations.jl:216) from
// the stage scalars: k eta > 240 and -tau' H / eta > 100.
template <class T>
__device__ __forceinline__ bool rsa_switch(const Mode& m, const Scal<T>& s) {
  return (m.k * vof(s.eta) > 240.0) && (-vof(s.tp) * vof(s.Hc) / vof(s.eta) > 100.0);
}

// Metric potentials Psi and Phi' (perturbations.jl:182-194) from the state u.
template <class T, class U>
__device__ __forceinline__ void metric(const Mode& m, const Shared& S, int sl, const Scal<T>& s, const U& u,
                                       int lane, T& Psi, T& Phip) {
  using K = typename KT<T>::type;
  const CosmoDev& C = *m.C;
  T rho = cst<T>(0.0), sig = cst<T>(0.0);
  for (int q = lane; q < m.nq; q += 32) {
    T qe = qe_of<T>(S, sl, m.nq, q), eq = eq_of<T>(S, sl, m.nq, q);
    K qq = kval<K>(S.q, S.dq, q);
    // eps = q * eq ; q^2/eps = q * qe
    rho = rho + (kval<K>(S.Aq, S.dAq, q) * qq) * eq * u[m.iM + q];
    sig = sig + (kval<K>(S.Aq, S.dAq, q) * qq) * qe * u[m.iM + 2 * m.nq + q];
  }
  rho = warp_sum_t<T>(rho);
  sig = warp_sum_t<T>(sig);
  const double Omega_nu = C.Omega_nu;
  const auto Phi = u[m.iPhi];
  Psi = -Phi - s.cpsi * (C.Omega_r * u[2] + Omega_nu * u[m.iN + 2] + sig * kcos<K>(m, S, 0));
  T ia = 1.0 / s.a;
  Phip = Psi - s.k2H2 * Phi +
         s.dphi * ((kcos<K>(m, S, 2) * u[m.iPhi + 1] + kcos<K>(m, S, 3) * u[m.iPhi + 3]) * ia +
                   (4.0 * C.Omega_r * u[0] + 4.0 * Omega_nu * u[m.iN] + rho * kcos<K>(m, S, 1)) * (ia * ia));
}

// The state overwrite of hierarchy!'s radiation-streaming branch
// (perturbations.jl:217-227), applied to the accepted state u at the step's
// end abscissa (stage slot 4; OrdinaryDiffEq hands the integrator's own
// state to the right-hand side at the end of a step, so the reference's
// accepted state carries these values): Theta_0, Theta_1 from the metric and
// the baryons, Theta_2 = 0, N_0 = Phi, N_1 = -2 H Phi' / k, N_2 = 0, with
// Phi' formed from u before the overwrite.  One warp; lane 0 writes.
__device__ void rsa_overwrite(const Mode& m, const Shared& S, double x, double* u, int lane) {
  const Scal<double> s = get_scal<double>(S, 4);
  double Psi, Phip;
  metric<double>(m, S, 4, s, StP{u}, lane, Psi, Phip);
  if (lane != 0) return;
  const double Phi = u[m.iPhi], delb = u[m.iPhi + 3], vb = u[m.iPhi + 4];
  const double Hk = s.Hc / m.k, tpp = spl_cold(*m.C, C_TAUPP, x);
  u[0] = Phi - Hk * s.tp * vb;
  u[1] = Hk * (-2.0 * Phip + s.tp * (Phi - s.cs2 * delb) + Hk * (tpp - s.tp) * vb);
  u[2] = 0.0;
  u[m.iN] = Phi;
  u[m.iN + 1] = -2.0 * Hk * Phip;
  u[m.iN + 2] = 0.0;
}

// hierarchy! (perturbations.jl:161-271): writes f into out (and df/dx into
// out_d for T = dd), one row per thread over the whole CTA.  Every warp
// forms the metric potentials itself (two nq-term sums), so no barrier is
// needed before the rows.  Returns true when the radiation-streaming switch
// is on.
template <class T, class U>
__device__ bool rhs_rows(const Mode& m, const Shared& S, int sl, const U& u, const Sink& out, int tid, int nth) {
  using K = typename KT<T>::type;
  using E = decltype(u[0]);
  const int lane = tid & 31;
  const Scal<T> s = get_scal<T>(S, sl);
  T Psi, Phip;
  metric<T>(m, S, sl, s, u, lane, Psi, Phip);
  const int lg = m.lg, lnu = m.lnu, lmnu = m.lmnu, nq = m.nq;
  const double* cl1 = S.cl1;
  const double* cl2 = S.cl2;
  const bool rsa = rsa_switch(m, s);
  const E Pi = u[2] + u[m.iTp + 2] + u[m.iTp];
  const E vb = u[m.iPhi + 4];
  const E zero = cst<E>(0.0);
  for (int i = tid; i < m.N; i += nth) {
    T f;
    if (i < m.iM) {
      if (rsa) {
        f = cst<T>(0.0);
      } else if (i < m.iTp) {  // photon temperature
        const int l = i;
        if (l < lg) {
          E lo = l > 0 ? u[l - 1] : zero;
          f = s.kH * (cl1[l] * lo - cl2[l] * u[l + 1]);
          if (l >= 1) f = f + s.tp * u[l];
          if (l == 0) f = f - Phip;
          if (l == 1) f = f + (1.0 / 3.0) * s.kH * Psi + s.tp * (vb / 3.0);
          if (l == 2) f = f - s.tp * (Pi / 10.0);
        } else {
          f = s.kH * u[lg - 1] - ((lg + 1.0) * s.iHe - s.tp) * u[lg];
        }
      } else if (i < m.iN) {  // photon polarization
        const int l = i - m.iTp, P = m.iTp;
        if (l < lg) {
          E lo = l > 0 ? u[P + l - 1] : zero;
          f = s.kH * (cl1[l] * lo - cl2[l] * u[P + l + 1]) + s.tp * u[P + l];
          if (l == 0) f = f - s.tp * (Pi / 2.0);
          if (l == 2) f = f - s.tp * (Pi / 10.0);
        } else {
          f = s.kH * u[P + lg - 1] - ((lg + 1.0) * s.iHe - s.tp) * u[P + lg];
        }
      } else {  // massless neutrinos
        const int l = i - m.iN, Nn = m.iN;
        if (l < lnu) {
          E lo = l > 0 ? u[Nn + l - 1] : zero;
          f = s.kH * (cl1[l] * lo - cl2[l] * u[Nn + l + 1]);
          if (l == 0) f = f - Phip;
          if (l == 1) f = f + (1.0 / 3.0) * s.kH * Psi;
        } else {
          f = s.kH * u[Nn + lnu - 1] - (lnu + 1.0) * s.iHe * u[Nn + lnu];
        }
      }
    } else if (i < m.iPhi) {  // massive neutrinos (MB 57)
      const int j = i - m.iM;
      const int l = j / nq, q = j - l * nq;
      const int Mm = m.iM;
      T qe = qe_of<T>(S, sl, nq, q);
      if (l < lmnu) {
        E lo = l > 0 ? u[Mm + j - nq] : zero;
        f = (s.kH * qe) * (cl1[l] * lo - cl2[l] * u[Mm + j + nq]);
        if (l == 0) f = f + Phip * kval<K>(S.df0, S.ddf0, q);
        if (l == 1) f = f - (1.0 / 3.0) * s.kH * eq_of<T>(S, sl, nq, q) * Psi * kval<K>(S.df0, S.ddf0, q);
      } else {
        f = qe * s.kH * u[Mm + j - nq] - (lmnu + 1.0) * s.iHe * u[Mm + j];
      }
    } else {  // metric and matter
      const int r = i - m.iPhi;
      const E v = u[m.iPhi + 2], delb = u[m.iPhi + 3];
      if (r == 0) f = Phip;
      else if (r == 1) f = s.kH * v - 3.0 * Phip;
      else if (r == 2) f = -v - s.kH * Psi;
      else if (r == 3) f = s.kH * vb - 3.0 * Phip;
      else f = -vb - s.kH * (Psi + s.cs2 * delb) + s.tp * s.R * (3.0 * u[1] + vb);
    }
    put<T>(out, i, f);
  }
  return rsa;
}

// ------------------------------------------------------------ factorize ----
// Chains: 0 photon temperature (+ baryon pair), 1 polarization, 2 massless
// neutrinos, 3..3+nq-1 massive-neutrino bins, 3+nq CDM pair, 4+nq Phi.
// Tail slots per chain: [l=0, l=1, l=2, extra0, extra1]; chain 0 uses the
// extras for (v_b, delta_b); the CDM chain uses slots (delta, v) = (0, 1);
// Phi uses slot 0.
__device__ __forceinline__ int tail_index(const Mode& m, int c, int slot) {
  if (c == 0) {
    if (slot < 3) return slot;
    return slot == 3 ? m.iPhi + 4 : m.iPhi + 3;
  }
  if (c == 1) return m.iTp + slot;
  if (c == 2) return m.iN + slot;
  if (c < 3 + m.nq) return m.iM + slot * m.nq + (c - 3);
  if (c == 3 + m.nq) return m.iPhi + 1 + slot;  // delta, v
  return m.iPhi;
}

__device__ __forceinline__ int tail_slots(const Mode& m, int c) {
  if (c == 0) return 5;
  if (c < 3 + m.nq) return 3;
  if (c == 3 + m.nq) return 2;
  return 1;
}

// ------------------------------------------------------------- outputs ----
// Table `id` at x: the spline value (double), or the value with its
// tangents from the perturbed parameter sets' tables (d4).
template <class T> __device__ __forceinline__ T tabv(const Mode& m, int id, double x);
template <> __device__ __forceinline__ double tabv<double>(const Mode& m, int id, double x) { return spl_cold(*m.C, id, x); }
template <> __device__ __forceinline__ d4 tabv<d4>(const Mode& m, int id, double x) {
  d4 r;
  r.v = spl_cold(*m.C, id, x);
#pragma unroll
  for (int j = 0; j < kTD; ++j) r.t[j] = (spl_cold(*m.tc[j], id, x) - r.v) * m.tinv[j];
  return r;
}
__device__ __forceinline__ double dexp_t(double a) { return exp(a); }
__device__ __forceinline__ d4 dexp_t(const d4& a) { return dexp(a); }

// source_function and source_function_P (perturbations.jl:343-404) at a
// grid node, from u and du = hierarchy!(u); T = d4 gives their tangents
// (u and du then carry theirs).  Lane 0 writes outT / outE (wantE).
template <class T, class U>
__device__ void emit_sources_t(const Mode& m, const Shared& S, double x, const U& u, const U& du, int lane, T& outT,
                               T& outE, bool wantE) {
  using K = typename KT<T>::type;
  const CosmoDev& C = *m.C;
  double a = exp(x);
  T sig = cst<T>(0.0), sigp = cst<T>(0.0);
  const K msum = kcos<K>(m, S, 6);
  for (int q = lane; q < m.nq; q += 32) {
    K am = a * msum, qq = kval<K>(S.q, S.dq, q);
    K eps = dsqrt(qq * qq + am * am);
    K w = kval<K>(S.Aq, S.dAq, q) * qq * qq / eps;
    sig = sig + w * u[m.iM + 2 * m.nq + q];
    sigp = sigp + w * du[m.iM + 2 * m.nq + q];
  }
  sig = warp_sum_t<T>(sig);
  sigp = warp_sum_t<T>(sigp);
  if (lane != 0) return;
  const K H0 = kcos<K>(m, S, 4), rho_crit = kcos<K>(m, S, 5);
  const K H0sq = H0 * H0;
  const double k = m.k;
  T Hc = tabv<T>(m, C_H, x), Hcp = tabv<T>(m, C_HP, x), Hcpp = tabv<T>(m, C_HPP, x);
  T tau = tabv<T>(m, C_TAU, x), tp = tabv<T>(m, C_TAUP, x), tpp = tabv<T>(m, C_TAUPP, x);
  T g = tabv<T>(m, C_G, x), gp = tabv<T>(m, C_GP, x), gpp = tabv<T>(m, C_GPP, x);
  T eta = tabv<T>(m, C_ETA, x);
  const double Omega_nu = C.Omega_nu;
  const int Tp = m.iTp;
  const auto Phi = u[m.iPhi], Phip = du[m.iPhi], vb = u[m.iPhi + 4], vbp = du[m.iPhi + 4];
  T c = 12.0 * H0sq / (k * k) / (a * a);
  T Psi = -Phi - c * (C.Omega_r * u[2] + Omega_nu * u[m.iN + 2] + sig / rho_crit / 4.0);
  T Psip = -Phip - c * (C.Omega_r * (du[2] - 2.0 * u[2]) + Omega_nu * (du[m.iN + 2] - 2.0 * u[m.iN + 2]) +
                        (sigp - 2.0 * sig) / rho_crit / 4.0);
  const auto Pi = u[2] + u[Tp + 2] + u[Tp];
  const auto Pip = du[2] + du[Tp + 2] + du[Tp];
  T term1 = g * (u[0] + Psi + Pi / 4.0) + dexp_t(-tau) * (Psip - Phip);
  T term2 = (-1.0 / k) * (Hcp * g * vb + Hc * gp * vb + Hc * g * vbp);
  T Pipp = 2.0 * k / (5.0 * Hc) * (-Hcp / Hc * u[1] + du[1]) + (3.0 / 10.0) * (tpp * Pi + tp * Pip) -
           3.0 * k / (5.0 * Hc) * (-Hcp / Hc * (u[3] + u[Tp + 1] + u[Tp + 3]) + (du[3] + du[Tp + 1] + du[Tp + 3]));
  T term3 = (3.0 / (4.0 * k * k)) * ((Hcp * Hcp + Hc * Hcpp) * g * Pi + 3.0 * Hc * Hcp * (gp * Pi + g * Pip) +
                                     Hc * Hc * (gpp * Pi + 2.0 * gp * Pip + g * Pipp));
  outT = term1 + term2 + term3;
  // same spline, same evaluation as eta(x): y is exactly 0 at the last node,
  // where the reference's 3 / (4 y^2) is infinite (perturbations.jl:401-403)
  if (wantE) {
    T y = (x == C.x_last) ? cst<T>(0.0) : k * (tabv<T>(m, C_ETA, C.x_last) - eta);
    outE = (3.0 / (4.0 * y * y)) * g * Pi;
  }
}

__device__ void emit_sources(const Mode& m, const Shared& S, double x, const double* u, const double* du, int lane,
                             double* outT, double* outE) {
  double t = 0.0, e = 0.0;
  emit_sources_t<double>(m, S, x, StP{u}, StP{du}, lane, t, e, outE != nullptr);
  if (lane == 0) {
    *outT = t;
    if (outE) *outE = e;
  }
}

// plin (spectra.jl:163-198) at the final node x; T = d4 gives its tangents
// (u then carries theirs).  Lane 0 writes out.
__device__ __forceinline__ double dpow_t(double a, double b) { return pow(a, b); }
__device__ __forceinline__ d4 dpow_t(const d4& a, double b) { return dpow(a, b); }
template <class T, class U>
__device__ void emit_plin_t(const Mode& m, const Shared& S, double x, const U& u, int lane, T& out) {
  using K = typename KT<T>::type;
  const CosmoDev& C = *m.C;
  double a = exp(x);
  T rho = cst<T>(0.0), th = cst<T>(0.0);
  const K msum = kcos<K>(m, S, 6);
  for (int q = lane; q < m.nq; q += 32) {
    K am = a * msum, qq = kval<K>(S.q, S.dq, q);
    K eps = dsqrt(qq * qq + am * am);
    rho = rho + kval<K>(S.Aq, S.dAq, q) * eps * u[m.iM + q];
    th = th + kval<K>(S.Bq, S.dBq, q) * u[m.iM + m.nq + q];
  }
  rho = warp_sum_t<T>(rho);
  th = warp_sum_t<T>(th);
  if (lane != 0) return;
  double k = m.k;
  const K rho_crit = kcos<K>(m, S, 5), h = kcos<K>(m, S, 7), Omega_c = kcos<K>(m, S, 2), Omega_b = kcos<K>(m, S, 3);
  T r0 = tabv<T>(m, C_RHO0M, x);
  T Mrho = rho / r0, Mth = k * th / r0;
  const auto dcN = u[m.iPhi + 1], vcN = u[m.iPhi + 2], dbN = u[m.iPhi + 3], vbN = u[m.iPhi + 4];
  T vmnu = -Mth / k;
  K Tg = dpow_t(15.0 / (M_PI * M_PI) * rho_crit * C.Omega_r, 0.25);
  K nufac = (90.0 * 1.2020569 / (11.0 * pow(M_PI, 4))) * (C.Omega_r * h * h / Tg) * pow(C.N_nu / 3.0, 0.75);
  K Omega_nu = msum * nufac / (h * h);
  K Om = Omega_c + Omega_b + Omega_nu;
  T Hc = tabv<T>(m, C_H, x);
  T dc = dcN - 3.0 * Hc * vcN / k, db = dbN - 3.0 * Hc * vbN / k, dn = Mrho - 3.0 * Hc * vmnu / k;
  T dm = (Omega_c * dc + Omega_b * db + Omega_nu * dn) / Om;
  double Pp = C.A * pow(k / 0.05, C.n_s - 1.0);
  out = (2.0 * M_PI * M_PI / (k * k * k)) * dm * dm * Pp;
}

__device__ void emit_plin(const Mode& m, const Shared& S, double x, const double* u, int lane, double* out) {
  double v = 0.0;
  emit_plin_t<double>(m, S, x, StP{u}, lane, v);
  if (lane == 0) *out = v;
}

// initial_conditions (perturbations.jl:274-338) of cosmology C with the
// momentum-bin constants q, df0, lane 0 serial (once per mode).
__device__ void initial_state(const Mode& m, const CosmoDev& C, const double* qv, const double* df0v, double xi,
                              double* u, int lane) {
  for (int i = lane; i < m.N; i += 32) u[i] = 0.0;
  __syncwarp();
  if (lane == 0) {
    double k = m.k;
    double Hc = spl_cold(C, C_H, xi), eta = spl_cold(C, C_ETA, xi), tp = spl_cold(C, C_TAUP, xi);
    double ai = exp(xi);
    double fnu = 1.0 / (1.0 + 1.0 / (7.0 * C.N_nu / 8.0 * pow(4.0 / 11.0, 4.0 / 3.0)));
    double Phi = (4.0 * fnu + 10.0) / (4.0 * fnu + 15.0);
    double Cc = -((15.0 + 4.0 * fnu) / (20.0 + 8.0 * fnu)) * Phi;
    double* Th = u;
    double* Tp = u + m.iTp;
    double* Nn = u + m.iN;
    Th[0] = -40.0 * Cc / (15.0 + 4.0 * fnu) / 4.0;
    Th[1] = 10.0 * Cc / (15.0 + 4.0 * fnu) * (k * k * eta) / (3.0 * k);
    Th[2] = -8.0 * k / (15.0 * Hc * tp) * Th[1];
    Tp[0] = (5.0 / 4.0) * Th[2];
    Tp[1] = -k / (4.0 * Hc * tp) * Th[2];
    Tp[2] = (1.0 / 4.0) * Th[2];
    for (int l = 3; l <= m.lg; ++l) {
      Th[l] = -l / (2.0 * l + 1.0) * k / (Hc * tp) * Th[l - 1];
      Tp[l] = -l / (2.0 * l + 1.0) * k / (Hc * tp) * Tp[l - 1];
    }
    double del = 3.0 * Th[0];
    double v = -3.0 * k * Th[1];
    Nn[0] = Th[0];
    Nn[1] = Th[1];
    Nn[2] = -(k * k * eta * eta) / 15.0 * 1.0 / (1.0 + 2.0 / 5.0 * fnu) * Phi / 2.0;
    for (int l = 3; l <= m.lnu; ++l) Nn[l] = k / ((2.0 * l + 1.0) * Hc) * Nn[l - 1];
    for (int q = 0; q < m.nq; ++q) {
      double qq = qv[q], am = ai * C.Sigma_m_nu;
      double eps = sqrt(qq * qq + am * am), df0 = df0v[q];
      u[m.iM + q] = -Nn[0] * df0;
      u[m.iM + m.nq + q] = -eps / qq * Nn[1] * df0;
      u[m.iM + 2 * m.nq + q] = -Nn[2] * df0;
      for (int l = 3; l <= m.lmnu; ++l)
        u[m.iM + l * m.nq + q] = qq / eps * k / ((2.0 * l + 1.0) * Hc) * u[m.iM + (l - 1) * m.nq + q];
    }
    u[m.iPhi] = Phi;
    u[m.iPhi + 1] = del;
    u[m.iPhi + 2] = v;
    u[m.iPhi + 3] = del;
    u[m.iPhi + 4] = v;
  }
  __syncwarp();
}

#include "chains.cuh"
#include "tangent.cuh"

// --------------------------------------------------------------- driver ----
// Optional per-phase cycle counters (compile with -DBOLT_PHASE_TIMERS): thread
// 0 accumulates clock64() deltas between phase boundaries, which include the
// barrier waits, i.e. the CTA's critical path per phase.
#ifdef BOLT_PHASE_TIMERS
__device__ unsigned long long g_phase_cycles[16];
#define PT_DECL long long pt_last_ = clock64(); long long pt_acc_[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
#define PT(k) if (tid == 0) { long long n_ = clock64(); pt_acc_[k] += n_ - pt_last_; pt_last_ = n_; }
#define PT_FLUSH if (tid == 0) for (int i_ = 0; i_ < 12; ++i_) atomicAdd(&g_phase_cycles[i_], (unsigned long long)pt_acc_[i_]);
#else
#define PT_DECL
#define PT(k)
#define PT_FLUSH
#endif

// One CTA of WPM warps integrates one mode.  Row-parallel work (the
// right-hand sides, the stage combinations, the error norm, dense output) is
// spread over all threads; the chain recurrences run as segmented scans over
// all lanes (chains.cuh).  WPM = 4 spreads a mode's FP64 work over the four
// SM sub-partitions (lowest latency per step); WPM = 1 issues the fewest
// FP64 instructions per step (no per-warp duplicated scalar work, longer
// per-lane scans) and fits more modes on an SM (highest throughput when
// many modes are in flight).

// Cubic Hermite interpolation on [x0, x1] from (y0, f0, y1, f1) into u.
__device__ __forceinline__ void hermite(int N, double x0, double x1, double xq, const double* y0, const double* f0,
                                        const double* y1, const double* f1, double* u, int tid, int nth) {
  double hh = x1 - x0, t = (xq - x0) / hh, t2 = t * t, t3 = t2 * t;
  double h00 = 2.0 * t3 - 3.0 * t2 + 1.0, h10 = (t3 - 2.0 * t2 + t) * hh, h01 = -2.0 * t3 + 3.0 * t2,
         h11 = (t3 - t2) * hh;
  for (int i = tid; i < N; i += nth) u[i] = h00 * y0[i] + h10 * f0[i] + h01 * y1[i] + h11 * f1[i];
  __syncthreads();
}

__device__ __forceinline__ void copy_vec(int N, const double* src, double* dst, int tid, int nth) {
  for (int i = tid; i < N; i += nth) dst[i] = src[i];
}

// Block sum of one value per thread (red: >= WPM doubles of smem).
template <int WPM>
__device__ __forceinline__ double block_sum(double v, double* red, int tid) {
  v = warp_sum(v);
  if (WPM == 1) return v;
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < WPM; ++w) t += red[w];
  __syncthreads();
  return t;
}

// Per-mode set-up shared by the solver kinds (0 plain, 1 tangent, 2
// adjoint): the mode's dimensions and tangent cosmologies, the shared-memory
// layout per_mode_doubles() sizes, the chain packing, the global slab and
// the per-mode constants.  All threads; returns false when the chains do
// not fit the CTA (ends with a barrier).
template <int WPM, int KIND>
__device__ bool setup_mode(const ModeDev& md, const CosmoDev* cosmos, double* base, double* gscr, int tid, Mode& m,
                           Shared& S, Pack& PK, Scratch& G) {
  constexpr int nth = 32 * WPM;
  m.C = cosmos + md.cosmo;
  m.k = md.k;
  m.lg = md.lg; m.lnu = md.lnu; m.lmnu = md.lmnu; m.nq = md.nq;
  m.N = 2 * (m.lg + 1) + (m.lnu + 1) + (m.lmnu + 1) * m.nq + 5;
  m.iTp = m.lg + 1;
  m.iN = 2 * (m.lg + 1);
  m.iM = m.iN + m.lnu + 1;
  m.iPhi = m.iM + (m.lmnu + 1) * m.nq;
  m.nch = m.nq + 5;
  for (int j = 0; j < kTD; ++j) {
    m.tc[j] = KIND ? cosmos + md.tcos[j] : m.C;
    m.tinv[j] = KIND ? md.tinv[j] : 0.0;
  }
  const CosmoDev& C = *m.C;
  const int N = m.N, nq = m.nq;
  int Lmax = max(m.lg, max(m.lnu, m.lmnu));
  S.sct = S.sct_d = S.qet = S.eqt = S.qet_d = S.eqt_d = S.qpj = S.dq = S.ddf0 = S.dAq = S.dBq = S.cstn = nullptr;
  S.yd = S.bd = S.part4 = nullptr;
  double* p = base;
  S.yt = p; p += N;
  S.b = p; p += N;
  S.fl = p; p += N;
  S.fi = p; p += N;
  S.fc = p; p += N;
  S.q = p; p += nq;
  S.df0 = p; p += nq;
  S.Aq = p; p += nq;
  S.Bq = p; p += nq;
  S.qe = p; p += kStages * nq;
  S.eq = p; p += kStages * nq;
  S.qe_d = p; p += nq;
  S.eq_d = p; p += nq;
  S.Uf = p; p += m.nch * kTail * kBorder;
  S.Wt = p; p += m.nch * kTail * kBorder;
  S.cl1 = p; p += Lmax + 1;
  S.cl2 = p; p += Lmax + 1;
  S.sc = p; p += kStages * kScal;
  S.sc_d = p; p += kScal;
  S.misc = p;                 // [0..8] capacitance inverse, [16..23] block reductions, [24] flags, [32..] partials
  p += kMiscDoubles;
  if (KIND) {  // tangent: tan_doubles() of shared memory; adjoint: the coefficient tangents in the
              // global slab after its scratch
    double* keep = p;
    if (KIND == 2) p = gscr + 10 * N + adj_scratch_doubles(N);
    S.sct = p; p += kStages * kScal * kTD;
    S.sct_d = p; p += kScal * kTD;
    S.qet = p; p += kStages * nq * kTD;
    S.eqt = p; p += kStages * nq * kTD;
    S.qet_d = p; p += nq * kTD;
    S.eqt_d = p; p += nq * kTD;
    S.qpj = p; p += kTD * nq;
    S.dq = p; p += nq * kTD;
    S.ddf0 = p; p += nq * kTD;
    S.dAq = p; p += nq * kTD;
    S.dBq = p; p += nq * kTD;
    S.cstn = p; p += 8 * kTD;
    if (KIND == 1) {
      S.part4 = p; p += 32 * kBorder * kTD;
      S.yd = p; p += kTD * N;
      S.bd = p; p += kTD * N;
    } else {
      p = keep;
    }
  }
  {
    int* ip = reinterpret_cast<int*>(p);
    PK.seg = ip; ip += nth;
    PK.chain = ip; ip += nth;
    PK.idx = ip; ip += kLaneElems;
    PK.owner = ip; ip += 32;
    PK.E = ip;
    PK.em = kLaneElems / nth;
    PK.nt = nth;
  }
  G.y = gscr;
  G.fx = gscr + N;
  G.K = gscr + 2 * N;
  G.yp = gscr + 8 * N;
  G.fp = gscr + 9 * N;
  // per-mode constants (perturbations.jl:164-166; background.jl:21-30)
  for (int l = tid; l <= Lmax; l += nth) {
    S.cl1[l] = double(l) / (2.0 * l + 1.0);
    S.cl2[l] = (l + 1.0) / (2.0 * l + 1.0);
  }
  for (int q = tid; q < nq; q += nth) qconst(C, q, S.q[q], S.df0[q], S.Aq[q], S.Bq[q]);
  if (tid == 0) S.misc[25] = build_pack(m, PK, nth) ? 1.0 : 0.0;
  __syncthreads();
  return S.misc[25] != 0.0;
}

template <int WPM, bool TAN>
__device__ void solve_one(const ModeDev& md, const CosmoDev* cosmos, const SolverCfg& cfg, double* base,
                          double* gscr, int tid) {
  constexpr int nth = 32 * WPM;
  const int lane = tid & 31, warp = tid >> 5;
  Mode m;
  Shared S;
  Pack PK;
  Scratch G;
  const bool packed = setup_mode<WPM, TAN ? 1 : 0>(md, cosmos, base, gscr, tid, m, S, PK, G);
  const CosmoDev& C = *m.C;
  const int N = m.N;
  double* red = S.misc + 16;
  TanScratch T;
  T.dy = gscr + 10 * N;
  T.dK = T.dy + kTD * N;
  T.fxt = T.dK + 6 * kTD * N;
  T.tmp = T.fxt + kTD * N;
  double x = C.x0;
  const double xend = md.xout[md.nout - 1];
  if (!packed) {
    if (tid == 0) { *md.status = ST_BAD_INPUT; if (md.counters) { md.counters[0] = 0; md.counters[1] = 0; } }
    return;
  }
  if (warp == 0) initial_state(m, C, S.q, S.df0, x, S.yt, lane);
  __syncthreads();
  copy_vec(N, S.yt, G.y, tid, nth);
  __syncthreads();
  if (TAN) {
    tan_setup(m, S, tid, nth);
    tan_initial(m, S, x, G.y, T.dy, S.bd, tid, nth);
  }
  int status = ST_OK;
  bool rsa_any = false;
  long long nacc = 0, nrej = 0;
  int jo = 0;
  while (jo < md.nout && md.xout[jo] < x) ++jo;
  int jtan = jo;  // next node of the tangent outputs (tangent modes land on every node)
  // nodes below x_dense are produced by dense output (sources only)
  const bool ckpt = (md.flags & MODE_CKPT) != 0;  // lands on every node; steps replayable bit for bit
  const bool dense_ok = (md.flags & MODE_SOURCES) && !(md.flags & MODE_TRAJ) && !TAN && !ckpt;
  if (ckpt) copy_vec(N, G.y, md.ckpt, tid, nth);
  int jd = 0;
  if (dense_ok)
    while (jd < md.nout - 1 && md.xout[jd] < cfg.x_dense) ++jd;
  double h = cfg.h0;
  const double rtol = cfg.reltol, atol = cfg.abstol;
  const bool record = (md.flags & MODE_RECORD) != 0, replay = (md.flags & MODE_REPLAY) != 0;
  bool rec_over = false;
  double xprev = x;
  bool have_prev = false;
  double x_done = -1e300;  // last abscissa whose outputs were emitted
  PT_DECL
  while (true) {
    if (x >= xend) {
      const bool pend = (jo < md.nout);
      if (pend) {
        prepare_other(m, S, x, tid, nth);
        double* Kf = G.K + N;
        copy_vec(N, G.y, S.yt, tid, nth);
        __syncthreads();
        rhs_rows<double>(m, S, 5, StP{S.yt}, sink(Kf), tid, nth);
        __syncthreads();
        if (dense_ok && have_prev) {
          while (jo < md.nout && md.xout[jo] < x) {
            double xq = md.xout[jo];
            hermite(N, xprev, x, xq, G.yp, G.fp, G.y, Kf, S.yt, tid, nth);
            prepare_other(m, S, xq, tid, nth);
            rhs_rows<double>(m, S, 5, StP{S.yt}, sink(G.K), tid, nth);
            __syncthreads();
            if (warp == 0) emit_sources(m, S, xq, S.yt, G.K, lane, md.src_T + jo, md.src_E ? md.src_E + jo : nullptr);
            __syncthreads();
            ++jo;
          }
          prepare_other(m, S, x, tid, nth);
          copy_vec(N, G.y, S.yt, tid, nth);
          __syncthreads();
        }
        if (jo < md.nout && md.xout[jo] == x) {
          if ((md.flags & MODE_SOURCES) && warp == 0)
            emit_sources(m, S, x, S.yt, Kf, lane, md.src_T + jo, md.src_E ? md.src_E + jo : nullptr);
          if (md.flags & MODE_TRAJ)
            for (int i = tid; i < N; i += nth) md.traj[(size_t)jo * N + i] = G.y[i];
          ++jo;
        }
        __syncthreads();
        if (TAN && (md.flags & MODE_SOURCES) && jtan < md.nout && md.xout[jtan] == x) {
          double xs[kStages];
          xs[5] = x;
          tan_prepare(m, S, xs, 5, 6, tid, nth);
          Sink o;
          o.v = nullptr; o.d = nullptr; o.t = S.bd; o.td = nullptr; o.N = N;
          rhs_rows<d4>(m, S, 5, StD4{S.yt, T.dy, N}, o, tid, nth);
          __syncthreads();
          if (warp == 0) tan_emit_sources(m, S, md, x, S.yt, T.dy, Kf, S.bd, jtan, lane);
          ++jtan;
          __syncthreads();
        }
      }
      if (md.flags & MODE_PLIN) {
        copy_vec(N, G.y, S.yt, tid, nth);
        __syncthreads();
        if (warp == 0) emit_plin(m, S, x, S.yt, lane, md.plin);
        if (TAN && warp == 0) {
          d4 dP = c4(0.0);
          emit_plin_t<d4>(m, S, x, StD4{S.yt, T.dy, N}, lane, dP);
          if (lane == 0)
            for (int j = 0; j < kTD; ++j)
              if (md.tplin[j]) *md.tplin[j] = dP.t[j];
        }
      }
      break;
    }
    // next landing target: the first node at or above x_dense strictly past x
    // whose index from the first such node is a multiple of the stride (or
    // the last node); nodes passed on the way come from dense output
    int jt = max(jo, jd);
    while (jt < md.nout && md.xout[jt] <= x) ++jt;
    if (dense_ok && cfg.land_stride > 1)
      while (jt < md.nout - 1 && (jt - jd) % cfg.land_stride != 0) ++jt;
    double target = jt < md.nout ? md.xout[jt] : xend;
    bool landing = false;
    double hs = h;
    if (x + hs >= target - 1e-14 * fabs(target)) { hs = target - x; landing = true; }
    double xn = landing ? target : x + hs;
    if (ckpt) hs = xn - x;  // the step a replay from the record takes
    if (replay) {
      if (nacc >= md.rec_cap) { status = ST_REPLAY_SHORT; break; }
      xn = md.rec[nacc];
      hs = xn - x;
      landing = (xn == target);
    }
    if (!(hs > 0.0)) { status = ST_DT_UNDERFLOW; break; }
    PT(9)
    prepare_stages(m, S, x, hs, xn, tid, nth);
    PT(0)
    const bool fok = factorize_scan(m, S, PK, hs * rodas::kGamma, tid, nth);
    // stage 1: f and df/dx at (x, y) into b / fx
    copy_vec(N, G.y, S.yt, tid, nth);
    __syncthreads();
    if (!fok) { status = ST_LU_FAIL; break; }
    PT(1)
    bool r = rhs_rows<dd>(m, S, 0, StP{S.yt}, sink(S.b, G.fx), tid, nth);
    rsa_any |= r;
    __syncthreads();
    PT(2)
    double* K0 = G.K;
    if (x != x_done) {
      // outputs that fall on this abscissa or inside the last accepted step
      if (dense_ok && have_prev && jo < md.nout && md.xout[jo] < x) {
        copy_vec(N, S.b, K0, tid, nth);  // f at x, kept while interpolating
        __syncthreads();
        while (jo < md.nout && md.xout[jo] < x) {
          double xq = md.xout[jo];
          hermite(N, xprev, x, xq, G.yp, G.fp, G.y, K0, S.yt, tid, nth);
          prepare_other(m, S, xq, tid, nth);
          rhs_rows<double>(m, S, 5, StP{S.yt}, sink(G.K + N), tid, nth);
          __syncthreads();
          if (warp == 0) emit_sources(m, S, xq, S.yt, G.K + N, lane, md.src_T + jo, md.src_E ? md.src_E + jo : nullptr);
          __syncthreads();
          ++jo;
        }
        copy_vec(N, G.y, S.yt, tid, nth);
        __syncthreads();
      }
      if (jo < md.nout && md.xout[jo] == x) {
        if ((md.flags & MODE_SOURCES) && warp == 0)
          emit_sources(m, S, x, S.yt, S.b, lane, md.src_T + jo, md.src_E ? md.src_E + jo : nullptr);
        if (md.flags & MODE_TRAJ)
          for (int i = tid; i < N; i += nth) md.traj[(size_t)jo * N + i] = G.y[i];
        ++jo;
      }
      if (dense_ok) {
        for (int i = tid; i < N; i += nth) { G.yp[i] = G.y[i]; G.fp[i] = S.b[i]; }
        xprev = x;
        have_prev = true;
      }
      x_done = x;
      __syncthreads();
    }
    PT(3)
    const double ih = 1.0 / hs;
    for (int i = tid; i < N; i += nth) S.b[i] += hs * rodas::kD[0] * G.fx[i];
    __syncthreads();
    wsolve_scan(m, S, PK, S.b, tid, nth);
    copy_vec(N, S.b, K0, tid, nth);
    PT(4)
    for (int st = 1; st < 6; ++st) {
      // stage state
      if (st < 5) {
        for (int i = tid; i < N; i += nth) {
          double acc = G.y[i];
          for (int j = 0; j < st; ++j) acc += rodas::kA[st - 1][j] * G.K[j * N + i];
          S.yt[i] = acc;
        }
      } else {
        for (int i = tid; i < N; i += nth) S.yt[i] += G.K[4 * N + i];
      }
      __syncthreads();
      PT(5)
      const int sl = st < 4 ? st : 4;
      r = rhs_rows<double>(m, S, sl, StP{S.yt}, sink(S.b), tid, nth);
      rsa_any |= r;
      // each thread combines the rows it produced (same row assignment)
      const double hd = hs * rodas::kD[st];
      for (int i = tid; i < N; i += nth) {
        double acc = S.b[i];
        if (st < 4) acc += hd * G.fx[i];
        double cs = 0.0;
        for (int j = 0; j < st; ++j) cs += rodas::kC[st][j] * G.K[j * N + i];
        S.b[i] = acc + ih * cs;
      }
      __syncthreads();
      PT(6)
      wsolve_scan(m, S, PK, S.b, tid, nth);
      if (st < 5) copy_vec(N, S.b, G.K + st * N, tid, nth);
      PT(7)
    }
    // error estimate: the last stage increment (in b)
    double en = 0.0, fac = 1.0;
    bool fin = true;
    if (replay) {  // the recorded step is taken as it is: only check the state
      for (int i = tid; i < N; i += nth) fin = fin && isfinite(S.yt[i] + S.b[i]);
      fin = __syncthreads_and(fin);
      if (!fin) { status = ST_NONFINITE; break; }
    } else {
      for (int i = tid; i < N; i += nth) {
        double yn = S.yt[i] + S.b[i];
        double sc = atol + rtol * fmax(fabs(G.y[i]), fabs(yn));
        double e = S.b[i] / sc;
        en += e * e;
        fin = fin && isfinite(yn);
      }
      en = sqrt(block_sum<WPM>(en, red, tid) / N);
      fin = __syncthreads_and(fin);
      if (!fin || !(en == en)) en = 1e10;
      fac = 0.9 * pow(fmax(en, 1e-12), -0.25);
      fac = fmin(6.0, fmax(0.2, fac));
    }
    if (en <= 1.0) {
      if (TAN) tan_step<WPM>(m, S, PK, G, T, md, x, hs, xn, jtan, tid, nth);
      else
        for (int i = tid; i < N; i += nth) G.y[i] = S.yt[i] + S.b[i];
      if (record && tid == 0) {
        if (nacc < md.rec_cap) md.rec[nacc] = xn;
        else rec_over = true;
      }
      if (ckpt && (nacc + 1) % kCkptEvery == 0 && nacc + 1 <= md.rec_cap)
        copy_vec(N, G.y, md.ckpt + size_t((nacc + 1) / kCkptEvery) * N, tid, nth);
      __syncthreads();
      if (rsa_switch(m, get_scal<double>(S, 4))) {  // uniform over the CTA
        if (TAN) { status = ST_TANGENT_RSA; break; }
        if (warp == 0) rsa_overwrite(m, S, xn, G.y, lane);
        __syncthreads();
      }
      x = xn;
      ++nacc;
      double hp = hs * fac;
      h = landing ? fmax(h, hp) : hp;
    } else {
      ++nrej;
      h = hs * fmin(1.0, fac);
      if (!(h >= 1e-14 * fmax(1.0, fabs(x)))) { status = fin ? ST_DT_UNDERFLOW : ST_NONFINITE; break; }
    }
    if (nacc + nrej > cfg.max_steps) { status = ST_MAXITERS; break; }
    PT(8)
  }
  PT_FLUSH
  if (tid == 0) {
    *md.status = status | (rsa_any ? ST_RSA_FIRED : 0) | (rec_over ? ST_REC_OVERFLOW : 0);
    if (md.counters) { md.counters[0] = nacc; md.counters[1] = nrej; }
  }
}

// boltsolve_rsa's post-processing (perturbations.jl:35-111): on the nodes
// past each mode's RSA switch, the photon and massless-neutrino multipoles of
// the stored trajectory are replaced by their radiation-streaming values
// (rsa_perts!, perturbations.jl:35-88): Theta_0, Theta_1, N_0, N_1 from the
// metric, baryons and opacity; Theta_2 = N_2 = 0; Theta_2..Theta_{lg-1},
// Theta^P_2..Theta^P_{lg-1}, N_2..N_{l_nu-1} zeroed (the reference's loops
// leave the top multipoles and Theta^P_0,1 as they are).  One thread per
// (mode, node); first[mode] is the first node replaced.
__global__ void rsa_post_kernel(const ModeDev* __restrict__ modes, int nmodes, const CosmoDev* __restrict__ cosmos,
                                const int* __restrict__ first) {
  const int r = blockIdx.y;
  if (r >= nmodes) return;
  const ModeDev& md = modes[r];
  const int j = first[r] + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= md.nout) return;
  const CosmoDev& C = cosmos[md.cosmo];
  const int lg = md.lg, lnu = md.lnu, lmnu = md.lmnu, nq = md.nq;
  const int N = 2 * (lg + 1) + (lnu + 1) + (lmnu + 1) * nq + 5;
  const int iTp = lg + 1, iN = 2 * (lg + 1), iM = iN + lnu + 1, iPhi = iM + (lmnu + 1) * nq;
  double* u = md.traj + (size_t)j * N;
  const double x = md.xout[j], k = md.k, a = exp(x);
  const double Hc = spl_cold(C, C_H, x), tp = spl_cold(C, C_TAUP, x), tpp = spl_cold(C, C_TAUPP, x);
  const double cs2 = spl_cold(C, C_CSB2, x);
  // rho_sigma (perturbations.jl:127-143): 4 pi sum w q^2 f0 / (dx/dq) {eps M_0, q^2/eps M_2}
  double rho = 0.0, sig = 0.0;
  for (int q = 0; q < nq; ++q) {
    double lq = C.logqmin + (C.logqmax - C.logqmin) / 2.0 * (C.qx[q] + 1.0);
    double qq = pow(10.0, lq);
    double dxdq = (1.0 + (-1.0 + 2.0 / (C.logqmax - C.logqmin) * ((1.0 + C.logqmin) - C.logqmin))) / (qq * log(10.0));
    double f0 = 2.0 / pow(2.0 * M_PI, 3.0) / (exp(qq / C.Tnu) + 1.0);
    double Aq = 4.0 * M_PI * qq * qq * f0 / dxdq * C.qw[q];
    double am = a * C.Sigma_m_nu, eps = sqrt(qq * qq + am * am);
    rho += Aq * eps * u[iM + q];
    sig += Aq * qq * qq / eps * u[iM + 2 * nq + q];
  }
  const double H0sq = C.H0 * C.H0, Phi = u[iPhi], delta = u[iPhi + 1], delb = u[iPhi + 3], vb = u[iPhi + 4];
  const double Psi = -Phi - 12.0 * H0sq / (k * k) / (a * a) *
                                (C.Omega_r * u[2] + C.Omega_nu * u[iN + 2] + sig / C.rho_crit / 4.0);
  const double Phip = Psi - k * k / (3.0 * Hc * Hc) * Phi +
                      H0sq / (2.0 * Hc * Hc) *
                          (C.Omega_c / a * delta + C.Omega_b / a * delb + 4.0 * C.Omega_r / (a * a) * u[0] +
                           4.0 * C.Omega_nu / (a * a) * u[iN] + rho / (a * a) / C.rho_crit);
  const double Hk = Hc / k;
  u[0] = Phi - Hk * tp * vb;
  u[1] = Hk * (-2.0 * Phip + tp * (Phi - cs2 * delb) + Hk * (tpp - tp) * vb);
  u[2] = 0.0;
  u[iN] = Phi;
  u[iN + 1] = -2.0 * Hk * Phip;
  u[iN + 2] = 0.0;
  for (int l = 2; l < lg; ++l) { u[l] = 0.0; u[iTp + l] = 0.0; }
  for (int l = 2; l < lnu; ++l) u[iN + l] = 0.0;
}

int launch_rsa_post(const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const int* d_first, int nout,
                    cudaStream_t stream) {
  if (nmodes <= 0) return 0;
  dim3 g((nout + 127) / 128, nmodes);
  rsa_post_kernel<<<g, 128, 0, stream>>>(d_modes, nmodes, d_cosmos, d_first);
  return cudaGetLastError();
}

#include "adjoint.cuh"

// The reverse sweep of one adjoint mode (MODE_ADJOINT, adjoint.cuh): the
// forward mode's checkpoints and step record, the cotangents of its outputs
// in md.sbar; writes the parameter cotangent's four partials to md.tbar.
template <int WPM>
__device__ void adjoint_one(const ModeDev& md, const CosmoDev* cosmos, double* base, double* gscr, int tid) {
  constexpr int nth = 32 * WPM;
  Mode m;
  Shared S;
  Pack PK;
  Scratch G;
  const bool packed = setup_mode<WPM, 2>(md, cosmos, base, gscr, tid, m, S, PK, G);
  const CosmoDev& C = *m.C;
  const int N = m.N;
  double* red = S.misc + 16;
  AdjScratch A;
  {
    double* p = gscr + 10 * N;
    A.lam = p; p += N;
    A.yb = p; p += N;
    A.Kb = p; p += 6 * N;
    A.Yb = p; p += N;
    A.Fb = p; p += N;
    A.u1 = p; p += N;
    A.du = p; p += N;
    A.gu = p; p += N;
    A.gdu = p; p += N;
    A.tmp = p; p += N;
    A.t4 = p; p += kTD * N;
    A.t4b = p; p += kTD * N;
    A.seg = p; p += size_t(kCkptEvery + 1) * N;
    A.segK = p;
  }
  double tb[kTD] = {0.0, 0.0, 0.0, 0.0};
  int status = ST_OK;
  const long long nf = md.nfwd ? (long long)md.nfwd[0] : 0;
  if (!packed) status = ST_BAD_INPUT;
  else if (nf <= 0 || nf > md.rec_cap) status = ST_REPLAY_SHORT;
  if (status == ST_OK) {
    tan_setup(m, S, tid, nth);
    for (int i = tid; i < N; i += nth) A.lam[i] = 0.0;
    __syncthreads();
    const bool src = (md.flags & MODE_SOURCES) != 0, plin = (md.flags & MODE_PLIN) != 0;
    int jo = md.nout - 1;  // the next output node from the top
    const int nseg = int((nf + kCkptEvery - 1) / kCkptEvery);
    for (int sg = nseg - 1; sg >= 0 && status == ST_OK; --sg) {
      const long long n0 = (long long)sg * kCkptEvery, n1 = min(n0 + (long long)kCkptEvery, nf);
      // replay the segment from its checkpoint, keeping the states y_n0 .. y_n1
      // and every step's stage increments
      copy_vec(N, md.ckpt + size_t(sg) * N, G.y, tid, nth);
      __syncthreads();
      double x = n0 == 0 ? C.x0 : md.rec[n0 - 1];
      for (long long n = n0; n < n1; ++n) {
        copy_vec(N, G.y, A.seg + size_t(n - n0) * N, tid, nth);
        const double xn = md.rec[n];
        const int rc = replay_stages<WPM>(m, S, PK, G, x, xn - x, xn, tid, nth);
        if (rc != ST_OK) { status = rc; break; }
        double* kk = A.segK + size_t(n - n0) * 6 * N;
        for (int i = tid; i < N; i += nth) {
          for (int j = 0; j < 6; ++j) kk[j * N + i] = G.K[j * N + i];
          G.y[i] = S.yt[i] + S.b[i];
        }
        __syncthreads();
        x = xn;
      }
      if (status != ST_OK) break;
      copy_vec(N, G.y, A.seg + size_t(n1 - n0) * N, tid, nth);
      __syncthreads();
      // backwards through the segment: step n's factorisation again, its
      // stored stages, the cotangent of its end node, lam pulled back
      for (long long n = n1 - 1; n >= n0; --n) {
        const double xs = n == 0 ? C.x0 : md.rec[n - 1], xn = md.rec[n], hs = xn - xs;
        const double* kk = A.segK + size_t(n - n0) * 6 * N;
        for (int i = tid; i < N; i += nth) {
          G.y[i] = A.seg[size_t(n - n0) * N + i];
          A.u1[i] = A.seg[size_t(n + 1 - n0) * N + i];
          for (int j = 0; j < 6; ++j) G.K[j * N + i] = kk[j * N + i];
        }
        prepare_stages(m, S, xs, hs, xn, tid, nth);
        if (!factorize_scan(m, S, PK, hs * rodas::kGamma, tid, nth)) { status = ST_LU_FAIL; break; }
        double xsl[5];
        xsl[0] = xs;
        for (int sl = 1; sl < 4; ++sl) xsl[sl] = xs + rodas::kCx[sl] * hs;
        xsl[4] = xn;
        tan_prepare(m, S, xsl, 0, 5, tid, nth);  // ends with a barrier
        bool at_node = false;
        double sbT = 0.0;
        if (src && jo >= 0 && md.xout[jo] == xn) {
          at_node = true;
          sbT = md.sbar[jo];
          --jo;
        }
        const bool last = (n == nf - 1);
        const double pb = (plin && last) ? md.sbar[0] : 0.0;
        if ((at_node && sbT != 0.0) || pb != 0.0)
          adjoint_seed<WPM>(m, S, A, 4, xn, at_node, sbT, plin && last, pb, tb, tid, nth);
        adjoint_step<WPM>(m, S, PK, G, A, hs, tb, tid, nth);
      }
    }
    if (status == ST_OK) {
      copy_vec(N, md.ckpt, A.u1, tid, nth);  // the initial state
      __syncthreads();
      if (src && jo >= 0 && md.xout[jo] == C.x0 && md.sbar[jo] != 0.0) {
        prepare_other(m, S, C.x0, tid, nth);
        double xsl[kStages];
        xsl[5] = C.x0;
        tan_prepare(m, S, xsl, 5, 6, tid, nth);
        adjoint_seed<WPM>(m, S, A, 5, C.x0, true, md.sbar[jo], false, 0.0, tb, tid, nth);
      }
      // the initial conditions' tangents: tb[j] += lam . d y_0 / d theta_j
      tan_initial(m, S, C.x0, A.u1, A.t4, A.tmp, tid, nth);
      for (int i = tid; i < N; i += nth)
#pragma unroll
        for (int j = 0; j < kTD; ++j) tb[j] = fma(A.lam[i], A.t4[j * N + i], tb[j]);
    }
  }
  for (int j = 0; j < kTD; ++j) {
    const double v = block_sum<WPM>(tb[j], red, tid);
    if (tid == 0 && md.tbar) md.tbar[j] = status == ST_OK ? v : 0.0;
  }
  if (tid == 0) {
    *md.status = status;
    if (md.counters) { md.counters[0] = nf; md.counters[1] = 0; }
  }
}

// Self-check of the adjoint's building blocks on one mode at (x, hs), one
// warp, pseudo-random vectors u, lam, du: out[sl] (sl = 0..4) = |lam.(A u) -
// (A^T lam).u| over sum |lam_i (A u)_i| at stage slot sl; out[5] the same
// for A' (d/dx); out[6] = max |M^T z - lam| / max |lam| for z = M^-T lam,
// M^T z formed as z / (h gamma) - A_0^T z; out[7] = max |M x - u| / max |u|
// for x = M^-1 u (the forward solve, M x = x / (h gamma) - A_0 x); out[8] =
// |S_T(u, du) - (g_u.u + g_du.du)| over the sum of the terms' magnitudes
// (source_grad); out[9] = |(P(u + e v) - P(u - e v)) / 2e - g.v| / |g.v|
// (plin_grad, P quadratic in u); out[10] = 1 if the streaming switch is on;
// out[11] = |lam.(M^-1 u) - (M^-T lam).u| / sum |lam_i (M^-1 u)_i|;
// out[12] = the largest over the stage slots and tangent directions of
// |coef_dot - dA_dot| / sum_i |lam_i (dA u)_i| on pseudo-random tangents;
// out[13] the same for the x-derivative variant against x4 arithmetic.
__device__ __forceinline__ double prand(int i, int seed) {
  unsigned x = unsigned(i) * 2654435761u ^ (unsigned(seed) * 40503u + 12345u);
  x ^= x >> 13;
  x *= 0x5bd1e995u;
  x ^= x >> 15;
  return double(x & 0xFFFFFFu) / double(0x800000) - 1.0;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__global__ void __launch_bounds__(32) adjoint_check_kernel(ModeDev md, const CosmoDev* __restrict__ cosmos,
                                                           double x, double hs, double* __restrict__ gscr,
                                                           double* __restrict__ out) {
  extern __shared__ double smem[];
  const int tid = threadIdx.x, lane = tid, nth = 32;
  Mode m;
  Shared S;
  Pack PK;
  Scratch G;
  if (!setup_mode<1, 2>(md, cosmos, smem, gscr, tid, m, S, PK, G)) {
    if (tid == 0) out[15] = -1.0;
    return;
  }
  const int N = m.N;
  double* u = gscr + 10 * N;
  double* lam = u + N;
  double* du = lam + N;
  double* w1 = du + N;
  double* w2 = w1 + N;
  double* w3 = w2 + N;
  double* gu = w3 + N;
  double* gdu = gu + N;
  for (int i = tid; i < N; i += nth) {
    u[i] = prand(i, 1);
    lam[i] = prand(i, 2);
    du[i] = prand(i, 3);
  }
  tan_setup(m, S, tid, nth);
  prepare_stages(m, S, x, hs, x + hs, tid, nth);
  const bool fok = factorize_scan(m, S, PK, hs * rodas::kGamma, tid, nth);
  const double ig = 1.0 / (hs * rodas::kGamma);
  bool rsa = false;
  for (int sl = 0; sl < 5; ++sl) {
    rsa |= rhs_rows<double>(m, S, sl, StP{u}, sink(w1), tid, nth);
    rhs_cols<double>(m, S, sl, lam, sink(w2), tid, nth);
    double d1 = 0.0, d2 = 0.0, sc = 0.0;
    for (int i = tid; i < N; i += nth) {
      d1 += lam[i] * w1[i];
      d2 += w2[i] * u[i];
      sc += fabs(lam[i] * w1[i]);
    }
    d1 = warp_sum(d1); d2 = warp_sum(d2); sc = warp_sum(sc);
    if (tid == 0) out[sl] = fabs(d1 - d2) / sc;
    __syncthreads();
  }
  {
    rhs_rows<dd>(m, S, 0, StP{u}, sink(w1, w3), tid, nth);          // w3 = A' u
    rhs_cols<dd>(m, S, 0, lam, sink(w1, w2), tid, nth);             // w2 = A'^T lam
    double d1 = 0.0, d2 = 0.0, sc = 0.0;
    for (int i = tid; i < N; i += nth) {
      d1 += lam[i] * w3[i];
      d2 += w2[i] * u[i];
      sc += fabs(lam[i] * w3[i]);
    }
    d1 = warp_sum(d1); d2 = warp_sum(d2); sc = warp_sum(sc);
    if (tid == 0) out[5] = fabs(d1 - d2) / sc;
    __syncthreads();
  }
  {  // transposed solve
    copy_vec(N, lam, S.b, tid, nth);
    __syncthreads();
    wsolve_scan_T(m, S, PK, S.b, tid, nth);
    copy_vec(N, S.b, w3, tid, nth);
    __syncthreads();
    // the two solves are each other's transposes: lam.(M^-1 u) = (M^-T lam).u
    copy_vec(N, u, S.b, tid, nth);
    __syncthreads();
    wsolve_scan(m, S, PK, S.b, tid, nth);
    {
      double d1 = 0.0, d2 = 0.0, sc = 0.0;
      for (int i = tid; i < N; i += nth) {
        d1 += lam[i] * S.b[i];
        d2 += w3[i] * u[i];
        sc += fabs(lam[i] * S.b[i]);
      }
      d1 = warp_sum(d1); d2 = warp_sum(d2); sc = warp_sum(sc);
      if (tid == 0) out[11] = fabs(d1 - d2) / sc;
    }
    __syncthreads();
    rhs_cols<double>(m, S, 0, w3, sink(w2), tid, nth);
    double e = 0.0, sc = 0.0;
    for (int i = tid; i < N; i += nth) {
      e = fmax(e, fabs(ig * w3[i] - w2[i] - lam[i]));
      sc = fmax(sc, fabs(lam[i]));
    }
    e = warp_max(e); sc = warp_max(sc);
    if (tid == 0) out[6] = fok ? e / sc : -1.0;
    __syncthreads();
  }
  {  // forward solve
    copy_vec(N, u, S.b, tid, nth);
    __syncthreads();
    wsolve_scan(m, S, PK, S.b, tid, nth);
    copy_vec(N, S.b, w3, tid, nth);
    __syncthreads();
    rhs_rows<double>(m, S, 0, StP{w3}, sink(w2), tid, nth);
    double e = 0.0, sc = 0.0;
    for (int i = tid; i < N; i += nth) {
      e = fmax(e, fabs(ig * w3[i] - w2[i] - u[i]));
      sc = fmax(sc, fabs(u[i]));
    }
    e = warp_max(e); sc = warp_max(sc);
    if (tid == 0) out[7] = fok ? e / sc : -1.0;
    __syncthreads();
  }
  {  // source gradient: S_T is linear in (u, du)
    for (int i = tid; i < N; i += nth) { gu[i] = 0.0; gdu[i] = 0.0; }
    __syncthreads();
    double sT = 0.0, sE = 0.0;
    emit_sources_t<double>(m, S, x, StP{u}, StP{du}, lane, sT, sE, false);
    source_grad(m, S, x, 1.0, gu, gdu, lane);
    __syncwarp();
    double lin = 0.0, mag = 0.0;
    for (int i = tid; i < N; i += nth) {
      lin += gu[i] * u[i] + gdu[i] * du[i];
      mag += fabs(gu[i] * u[i]) + fabs(gdu[i] * du[i]);
    }
    lin = warp_sum(lin); mag = warp_sum(mag);
    if (tid == 0) out[8] = fabs(sT - lin) / mag;
    __syncthreads();
  }
  {  // coefficient cotangents against the tangent-number right-hand side, on
     // pseudo-random tangents of every coefficient
    double* T1[9] = {S.sct, S.sct_d, S.qet, S.eqt, S.qet_d, S.eqt_d, S.dq, S.ddf0, S.dAq};
    const int L1[9] = {kStages * kScal * kTD, kScal * kTD, kStages * m.nq * kTD, kStages * m.nq * kTD,
                       m.nq * kTD, m.nq * kTD, m.nq * kTD, m.nq * kTD, m.nq * kTD};
    for (int a = 0; a < 9; ++a)
      for (int t = tid; t < L1[a]; t += nth) T1[a][t] = prand(t, 10 + a);
    for (int t = tid; t < m.nq * kTD; t += nth) S.dBq[t] = prand(t, 19);
    for (int t = tid; t < 8 * kTD; t += nth) S.cstn[t] = prand(t, 20);
    __syncthreads();
    double worst = 0.0;
    for (int sl = 0; sl < 5; ++sl) {
      double t1[kTD] = {0.0, 0.0, 0.0, 0.0}, t2[kTD] = {0.0, 0.0, 0.0, 0.0};
      double* t4 = gu;  // kTD * N doubles: gu, gdu and the scratch after them
      dA_dot(m, S, sl, u, lam, t4, t1, tid, nth);
      coef_dot<double>(m, S, sl, u, lam, t2, tid, nth);
      for (int j = 0; j < kTD; ++j) {
        const double a1 = warp_sum(t1[j]), a2 = warp_sum(t2[j]);
        double mag = 0.0;
        for (int i = tid; i < N; i += nth) mag += fabs(lam[i] * t4[j * N + i]);
        mag = warp_sum(mag);
        worst = fmax(worst, fabs(a1 - a2) / mag);
      }
      __syncthreads();
    }
    if (tid == 0) out[12] = worst;
    // the x-derivative variant against x4 arithmetic: lam . (dA'_0 u)
    {
      double t2[kTD] = {0.0, 0.0, 0.0, 0.0};
      Sink o;
      o.v = w1; o.d = nullptr; o.t = gu; o.td = gu + kTD * N; o.N = N;
      rhs_rows<x4>(m, S, 0, StC{u}, o, tid, nth);
      coef_dot<dd>(m, S, 0, u, lam, t2, tid, nth);
      double wx = 0.0;
      for (int j = 0; j < kTD; ++j) {
        double a1 = 0.0, mag = 0.0;
        for (int i = tid; i < N; i += nth) {
          a1 += lam[i] * o.td[j * N + i];
          mag += fabs(lam[i] * o.td[j * N + i]);
        }
        a1 = warp_sum(a1);
        mag = warp_sum(mag);
        wx = fmax(wx, fabs(a1 - warp_sum(t2[j])) / mag);
      }
      if (tid == 0) out[13] = wx;
    }
    __syncthreads();
  }
  {  // P_lin gradient: quadratic in u, so the central difference is exact
    for (int i = tid; i < N; i += nth) gu[i] = 0.0;
    __syncthreads();
    plin_grad(m, S, x, u, 1.0, gu, lane);
    __syncwarp();
    const double e = 1e-3;
    for (int i = tid; i < N; i += nth) { w1[i] = u[i] + e * du[i]; w2[i] = u[i] - e * du[i]; }
    __syncwarp();
    double pp = 0.0, pm = 0.0;
    emit_plin_t<double>(m, S, x, StP{w1}, lane, pp);
    emit_plin_t<double>(m, S, x, StP{w2}, lane, pm);
    pp = __shfl_sync(0xffffffffu, pp, 0);
    pm = __shfl_sync(0xffffffffu, pm, 0);
    double gv = 0.0;
    for (int i = tid; i < N; i += nth) gv += gu[i] * du[i];
    gv = warp_sum(gv);
    if (tid == 0) {
      out[9] = fabs((pp - pm) / (2.0 * e) - gv) / fabs(gv);
      out[10] = rsa ? 1.0 : 0.0;
      out[15] = N;
    }
  }
}

int launch_adjoint_check(const CosmoDev* d_cos, int id, double k, int lg, int lnu, int lmnu, int nq, double x,
                         double hs, double* d_scr, double* d_out, cudaStream_t st) {
  ModeDev md;
  std::memset(&md, 0, sizeof(md));
  md.k = k;
  md.cosmo = id;
  md.lg = lg; md.lnu = lnu; md.lmnu = lmnu; md.nq = nq;
  for (int j = 0; j < kTD; ++j) { md.tcos[j] = id; md.tinv[j] = 0.0; }
  const int N = 2 * (lg + 1) + (lnu + 1) + (lmnu + 1) * nq + 5;
  const int Lmax = std::max(lg, std::max(lnu, lmnu));
  const size_t smem = size_t(per_mode_doubles(N, nq, Lmax, 32, 2)) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(adjoint_check_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return e;
  adjoint_check_kernel<<<1, 32, smem, st>>>(md, d_cos, x, hs, d_scr, d_out);
  return cudaGetLastError();
}
size_t adjoint_check_scratch_bytes(int N) { return size_t(scratch_per_warp(N, 2) + 8 * N) * sizeof(double); }

// Persistent CTAs: the first wave takes modes blockIdx.x (modes arrive sorted
// by decreasing cost, and consecutive blocks land on different SMs, so the
// longest modes spread one per SM); later modes come from a device queue.
// KIND: every mode of the launch is plain (0, including recorded, replayed
// and checkpointed modes), tangent-linear (1, MODE_TANGENT) or adjoint (2,
// MODE_ADJOINT).
template <int WPM, int KIND>
__global__ void __launch_bounds__(32 * WPM) rodas_kernel(const ModeDev* __restrict__ modes, int nmodes,
                                                         const CosmoDev* __restrict__ cosmos, SolverCfg cfg,
                                                         int* __restrict__ queue, double* __restrict__ scratch,
                                                         int scr_per_mode) {
  extern __shared__ double smem[];
  __shared__ int s_mode;
  const int tid = threadIdx.x;
  double* gscr = scratch + (size_t)blockIdx.x * scr_per_mode;
  int mi = blockIdx.x;
  while (mi < nmodes) {
    if (KIND == 2) adjoint_one<WPM>(modes[mi], cosmos, smem, gscr, tid);
    else solve_one<WPM, KIND == 1>(modes[mi], cosmos, cfg, smem, gscr, tid);
    __syncthreads();
    if (tid == 0) s_mode = gridDim.x + atomicAdd(queue, 1);
    __syncthreads();
    mi = s_mode;
  }
}

namespace {
// The kernel variant: warps per mode 1, 2 or 4; tangent and adjoint modes
// with one warp.
const void* kernel_of(int wpm, int kind) {
  if (kind == 1) return (const void*)rodas_kernel<1, 1>;
  if (kind == 2) return (const void*)rodas_kernel<1, 2>;
  return wpm == 1 ? (const void*)rodas_kernel<1, 0>
                  : (wpm == 2 ? (const void*)rodas_kernel<2, 0> : (const void*)rodas_kernel<4, 0>);
}
int norm_wpm(int wpm, int kind) { return kind ? 1 : ((wpm == 1 || wpm == 2) ? wpm : 4); }
size_t smem_of(int maxN, int maxnq, int maxL, int wpm, int kind) {
  return size_t(per_mode_doubles(maxN, maxnq, maxL, 32 * wpm, kind)) * sizeof(double);
}
}  // namespace

// Host helpers.  wpm: warps per mode (1, 2 or 4; anything else means 4;
// tangent and adjoint launches use one); kind as rodas_kernel's KIND.
// Writes the number of persistent CTAs to launch (one mode each at a time).
int rodas_grid_warps(int nmodes, int maxN, int maxnq, int maxL, int wpm, int kind, int* blocks) {
  wpm = norm_wpm(wpm, kind);
  const size_t smem = smem_of(maxN, maxnq, maxL, wpm, kind);
  const void* f = kernel_of(wpm, kind);
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return -int(e);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int bps = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, f, 32 * wpm, smem);
  if (e != cudaSuccess) return -int(e);
  if (bps < 1) return -int(cudaErrorInvalidConfiguration);
  *blocks = std::min(nmodes, nsm * bps);
  return 0;
}
int rodas_grid_warps(int nmodes, int maxN, int maxnq, int maxL, int wpm, int* blocks) {
  return rodas_grid_warps(nmodes, maxN, maxnq, maxL, wpm, 0, blocks);
}

int launch_rodas(const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const SolverCfg& cfg, int* d_queue,
                 int maxN, int maxnq, int maxL, int wpm, int kind, int blocks, double* d_scratch, cudaStream_t stream) {
  wpm = norm_wpm(wpm, kind);
  const size_t smem = smem_of(maxN, maxnq, maxL, wpm, kind);
  cudaError_t e = cudaMemsetAsync(d_queue, 0, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  const int spm = scratch_per_warp(maxN, kind);
  if (kind == 1)
    rodas_kernel<1, 1><<<blocks, 32, smem, stream>>>(d_modes, nmodes, d_cosmos, cfg, d_queue, d_scratch, spm);
  else if (kind == 2)
    rodas_kernel<1, 2><<<blocks, 32, smem, stream>>>(d_modes, nmodes, d_cosmos, cfg, d_queue, d_scratch, spm);
  else if (wpm == 1)
    rodas_kernel<1, 0><<<blocks, 32, smem, stream>>>(d_modes, nmodes, d_cosmos, cfg, d_queue, d_scratch, spm);
  else if (wpm == 2)
    rodas_kernel<2, 0><<<blocks, 64, smem, stream>>>(d_modes, nmodes, d_cosmos, cfg, d_queue, d_scratch, spm);
  else
    rodas_kernel<4, 0><<<blocks, 128, smem, stream>>>(d_modes, nmodes, d_cosmos, cfg, d_queue, d_scratch, spm);
  return cudaGetLastError();
}
int launch_rodas(const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const SolverCfg& cfg, int* d_queue,
                 int maxN, int maxnq, int maxL, int wpm, int blocks, double* d_scratch, cudaStream_t stream) {
  return launch_rodas(d_modes, nmodes, d_cosmos, cfg, d_queue, maxN, maxnq, maxL, wpm, 0, blocks, d_scratch,
                      stream);
}

// Kernel-node description of one solver launch, for CUDA graphs whose
// node parameters are updated per batch.  args must stay alive until the
// node parameters have been set (the values are copied then).
int rodas_node_params(int wpm, int kind, const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos,
                      const SolverCfg& cfg, int* d_queue, int maxN, int maxnq, int maxL, int blocks, double* d_scratch,
                      RodasNodeArgs* args, cudaKernelNodeParams* p) {
  wpm = norm_wpm(wpm, kind);
  args->modes = d_modes;
  args->nmodes = nmodes;
  args->cosmos = d_cosmos;
  args->cfg = cfg;
  args->queue = d_queue;
  args->scratch = d_scratch;
  args->spm = scratch_per_warp(maxN, kind);
  args->ptrs[0] = &args->modes;
  args->ptrs[1] = &args->nmodes;
  args->ptrs[2] = &args->cosmos;
  args->ptrs[3] = &args->cfg;
  args->ptrs[4] = &args->queue;
  args->ptrs[5] = &args->scratch;
  args->ptrs[6] = &args->spm;
  p->func = const_cast<void*>(kernel_of(wpm, kind));
  p->gridDim = dim3(blocks);
  p->blockDim = dim3(32 * wpm);
  p->sharedMemBytes = unsigned(smem_of(maxN, maxnq, maxL, wpm, kind));
  p->kernelParams = args->ptrs;
  p->extra = nullptr;
  return 0;
}
int rodas_node_params(int wpm, const ModeDev* d_modes, int nmodes, const CosmoDev* d_cosmos, const SolverCfg& cfg,
                      int* d_queue, int maxN, int maxnq, int maxL, int blocks, double* d_scratch, RodasNodeArgs* args,
                      cudaKernelNodeParams* p) {
  return rodas_node_params(wpm, 0, d_modes, nmodes, d_cosmos, cfg, d_queue, maxN, maxnq, maxL, blocks, d_scratch,
                           args, p);
}

size_t rodas_smem_per_mode(int maxN, int maxnq, int maxL, int wpm, int kind) {
  return smem_of(maxN, maxnq, maxL, norm_wpm(wpm, kind), kind);
}
size_t rodas_smem_per_mode(int maxN, int maxnq, int maxL, int wpm) {
  return rodas_smem_per_mode(maxN, maxnq, maxL, wpm, 0);
}
size_t rodas_smem_per_warp(int maxN, int maxnq, int maxL) { return rodas_smem_per_mode(maxN, maxnq, maxL, 4); }
size_t rodas_scratch_per_warp(int maxN, int kind) { return size_t(scratch_per_warp(maxN, kind)) * sizeof(double); }
size_t rodas_scratch_per_warp(int maxN) { return rodas_scratch_per_warp(maxN, 0); }

#ifdef BOLT_PHASE_TIMERS
int rodas_phase_cycles(unsigned long long* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_phase_cycles, sizeof(unsigned long long) * 16);
  if (reset) {
    unsigned long long z[16] = {0};
    cudaMemcpyToSymbol(g_phase_cycles, z, sizeof(z));
  }
  return int(e);
}
#endif

}  // namespace bolt
