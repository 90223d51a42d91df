// Chain linear algebra for the Rosenbrock step matrix M - U W^T, with
// M = I/(h gamma) - L block diagonal (one tridiagonal chain per species) and
// a rank-3 border U W^T (Phi', Psi, Pi).
//
// On GB300 a dependent FP64 operation costs ~250 cycles, so a sequential
// Thomas sweep over a 51-element multipole chain is latency bound.  Here
// every chain is spread over a segment of lanes (E consecutive elements per
// lane, in elimination order from the highest multipole down to l = 0) and
// the three recurrences are evaluated as segmented warp scans:
//   pivots      piv_j = d_j - lo_j up_{j-1} / piv_{j-1}
//               as products of normalised 2x2 Moebius matrices,
//   forward     b'_j = b_j - fl_j b'_{j-1}           (affine scan),
//   backward    x_j  = fi_j b'_j - fc_j x_{j+1}      (reverse affine scan).
// The sequential depth drops from the chain length to E + log2(lanes).
// The border only touches the last rows of every chain (l <= 2), so after the
// forward scan the chain's tail owner forms W^T y on a few rows, the CTA sums
// the per-chain partials, and the owner corrects its tail before the
// backward scan.
// Included inside namespace bolt by solver.cu, after the Mode / Shared /
// tail helpers it uses.
#pragma once

constexpr int kLaneElems = 768;  // threads x elements-per-lane budget of every variant
constexpr int kMaxChains = 32;

// Packing of chains onto the CTA's lanes (shared memory, built per mode).
struct Pack {
  int* seg;      // [threads] segment start lane within the warp, -1 = idle lane
  int* chain;    // [threads] chain id of the lane
  int* idx;      // [em][threads] state indices in elimination order, -1 = pad (at the end); element e of
                 // thread t at idx[e * nt + t], so a warp reading its lanes' e-th elements touches 32
                 // consecutive words (no bank conflicts)
  int* owner;    // [kMaxChains] thread holding the chain's l = 0 element
  int* E;        // [0] elements per lane, [1] thread for the CDM pair + Phi, [2] lanes of the longest segment
  int em;        // largest elements per lane (kLaneElems / threads)
  int nt;        // threads
};

// Thread tid's element list, read as idx[e].
struct LaneIdx {
  const int* p;
  int s;
  __device__ __forceinline__ int operator[](int e) const { return p[e * s]; }
};
__device__ __forceinline__ LaneIdx lane_idx(const Pack& P, int tid) { return LaneIdx{P.idx + tid, P.nt}; }

struct ChainDesc {
  int L, base, stride;  // top multipole, state index of l = 0, index stride
};

__device__ __forceinline__ ChainDesc chain_desc(const Mode& m, int c) {
  ChainDesc d;
  if (c == 0) { d.L = m.lg; d.base = 0; d.stride = 1; }
  else if (c == 1) { d.L = m.lg; d.base = m.iTp; d.stride = 1; }
  else if (c == 2) { d.L = m.lnu; d.base = m.iN; d.stride = 1; }
  else { d.L = m.lmnu; d.base = m.iM + (c - 3); d.stride = m.nq; }
  return d;
}

// Thread 0: first-fit-decreasing packing of the multipole chains into the
// CTA's warps for the smallest E that fits (segments never cross a warp);
// one idle thread is kept for the CDM pair and Phi.
__device__ bool build_pack(const Mode& m, const Pack& P, int nthreads) {
  const int nw = nthreads / 32, nc = 3 + m.nq;
  for (int E = 2; E <= P.em; ++E) {
    int used[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int place[kMaxChains];
    bool ok = true;
    for (int c = 0; c < nc && ok; ++c) {  // chains come longest first (T, P, N, then M)
      int len = chain_desc(m, c).L + 1;
      int need = (len + E - 1) / E;
      int w = 0;
      while (w < nw && used[w] + need > 32) ++w;
      if (w == nw) ok = false;
      else { place[c] = w * 32 + used[w]; used[w] += need; }
    }
    if (!ok) continue;
    int spare = -1;
    for (int w = nw - 1; w >= 0 && spare < 0; --w)
      if (used[w] < 32) spare = w * 32 + 31;
    if (spare < 0) continue;
    for (int t = 0; t < nthreads; ++t) {
      P.seg[t] = -1;
      P.chain[t] = -1;
      for (int e = 0; e < P.em; ++e) P.idx[e * nthreads + t] = -1;
    }
    for (int c = 0; c < nc; ++c) {
      ChainDesc d = chain_desc(m, c);
      int len = d.L + 1, need = (len + E - 1) / E, t0 = place[c];
      for (int g = 0; g < need; ++g) {
        int t = t0 + g;
        P.seg[t] = t0 & 31;
        P.chain[t] = c;
        for (int e = 0; e < E; ++e) {
          int j = g * E + e;
          if (j < len) P.idx[e * nthreads + t] = d.base + (d.L - j) * d.stride;
        }
      }
      P.owner[c] = t0 + (len - 1) / E;
    }
    int maxseg = 1;  // lanes of the longest segment: the scan levels needed
    for (int c = 0; c < nc; ++c) maxseg = max(maxseg, (chain_desc(m, c).L + E) / E);
    P.E[0] = E;
    P.E[1] = spare;
    P.E[2] = maxseg;
    return true;
  }
  return false;
}

// Matrix entries of one multipole element (state index i, multipole l of
// chain c): diagonal d, coupling to the previous element (l + 1) lo and to
// the next element (l - 1) up, all of M = I/(h gamma) - L.
struct ElemC {
  double d, lo, up, upPrev;  // upPrev = up of element l + 1 (the previous one)
};

__device__ __forceinline__ ElemC elem_coef(const Mode& m, const Shared& S, const Scal<double>& s, double ig, int c,
                                           int l, int L, bool rsa) {
  ElemC e;
  if (rsa && c <= 2) {  // radiation streaming: the photon and massless-nu rows of f are zero
    e.d = ig;
    e.lo = 0.0;
    e.up = 0.0;
    e.upPrev = 0.0;
    return e;
  }
  double mu = c >= 3 ? S.qe[c - 3] : 1.0;  // slot 0 (q / eps at x)
  double mk = mu * s.kH;
  double jd;
  if (l == L) jd = -(L + 1.0) * s.iHe + (c <= 1 ? s.tp : 0.0);
  else jd = (c == 1 || (c == 0 && l >= 1)) ? s.tp : 0.0;
  e.d = ig - jd;
  e.lo = l < L ? mk * S.cl2[l] : 0.0;
  e.up = l == L ? -mk : (l >= 1 ? -mk * S.cl1[l] : 0.0);
  e.upPrev = l + 1 == L ? -mk : (l + 1 < L ? -mk * S.cl1[l + 1] : 0.0);
  return e;
}

struct M2 {
  double a, b, c, d;  // [[a, b], [c, d]]
};
__device__ __forceinline__ M2 mmul(const M2& x, const M2& y) {  // x * y
  M2 r;
  r.a = fma(x.a, y.a, x.b * y.c);
  r.b = fma(x.a, y.b, x.b * y.d);
  r.c = fma(x.c, y.a, x.d * y.c);
  r.d = fma(x.c, y.b, x.d * y.d);
  return r;
}
__device__ __forceinline__ M2 shfl_up_m2(const M2& v, int off) {
  M2 r;
  r.a = __shfl_up_sync(0xffffffffu, v.a, off);
  r.b = __shfl_up_sync(0xffffffffu, v.b, off);
  r.c = __shfl_up_sync(0xffffffffu, v.c, off);
  r.d = __shfl_up_sync(0xffffffffu, v.d, off);
  return r;
}

// Baryon pair (delta_b, v_b) hanging off Theta_1: eliminated first.  Returns
// lb = M[Theta1][vb] / piv_vb and the correction to Theta_1's diagonal.
__device__ __forceinline__ double baryon_pair(const Mode& m, const Shared& S, const Scal<double>& s, double ig,
                                              double hg, bool rsa, double& dT1_corr) {
  int idb = m.iPhi + 3, ivb = m.iPhi + 4;
  double Mdb_vb = -s.kH;               // M[db][vb]
  double Mvb_db = s.kH * s.cs2;        // M[vb][db]
  double dvb = ig + 1.0 - s.tp * s.R;  // M[vb][vb]
  double Mvb_T1 = -3.0 * s.tp * s.R;   // M[vb][Theta1]
  double l_vb = Mvb_db * hg;
  double piv_vb = dvb - l_vb * Mdb_vb;
  double ipvb = 1.0 / piv_vb;
  S.fl[ivb] = l_vb;
  S.fi[ivb] = ipvb;
  S.fc[ivb] = Mvb_T1 * ipvb;
  S.fi[idb] = hg;
  S.fc[idb] = Mdb_vb * hg;
  double lb = rsa ? 0.0 : (-s.tp / 3.0) * ipvb;  // M[Theta1][vb] / piv_vb (no Theta_1 row under streaming)
  S.fl[idb] = lb;                     // stored in delta_b's unused multiplier slot
  dT1_corr = -lb * Mvb_T1;
  return lb;
}

// Border tails of chain c, written to shared memory: U (coefficients of
// Phi', Psi, Pi in the chain's last rows) into uf, W (gradients of Phi', Psi,
// Pi on those rows) into wt; slots as in tail_index().
__device__ __forceinline__ void border_tails(const Mode& m, const Shared& S, const Scal<double>& s, int c, bool rsa,
                                             double* U, double* W) {
  const CosmoDev& C = *m.C;
  for (int a = 0; a < kTail * kBorder; ++a) { U[a] = 0.0; W[a] = 0.0; }
  double ia = 1.0 / s.a;
#define UU(a, b) U[(a) * kBorder + (b)]
#define WW(a, b) W[(a) * kBorder + (b)]
  if (c == 0) {
    UU(0, 0) = -1.0; UU(1, 1) = s.kH / 3.0; UU(2, 2) = -s.tp / 10.0; UU(3, 1) = -s.kH; UU(4, 0) = -3.0;
    WW(0, 0) = s.dphi * 4.0 * C.Omega_r * ia * ia;
    WW(2, 1) = -s.cpsi * C.Omega_r; WW(2, 0) = WW(2, 1); WW(2, 2) = 1.0;
    WW(4, 0) = s.dphi * C.Omega_b * ia;
    if (rsa) { UU(0, 0) = 0.0; UU(1, 1) = 0.0; UU(2, 2) = 0.0; }  // photon rows are zero; baryon rows stay
  } else if (c == 1) {
    if (!rsa) { UU(0, 2) = -s.tp / 2.0; UU(2, 2) = -s.tp / 10.0; }
    WW(0, 2) = 1.0; WW(2, 2) = 1.0;
  } else if (c == 2) {
    if (!rsa) { UU(0, 0) = -1.0; UU(1, 1) = s.kH / 3.0; }
    WW(0, 0) = s.dphi * 4.0 * C.Omega_nu * ia * ia;
    WW(2, 1) = -s.cpsi * C.Omega_nu; WW(2, 0) = WW(2, 1);
  } else if (c < 3 + m.nq) {
    int q = c - 3;
    UU(0, 0) = S.df0[q]; UU(1, 1) = -s.kH / 3.0 * S.eq[q] * S.df0[q];
    double qq = S.q[q];
    WW(0, 0) = s.dphi * S.Aq[q] * qq * S.eq[q] * ia * ia / C.rho_crit;
    WW(2, 1) = -s.cpsi * S.Aq[q] * qq * S.qe[q] * 0.25 / C.rho_crit; WW(2, 0) = WW(2, 1);
  } else if (c == 3 + m.nq) {
    UU(0, 0) = -3.0; UU(1, 1) = -s.kH;
    WW(0, 0) = s.dphi * C.Omega_c * ia;
  } else {
    UU(0, 0) = 1.0;
    WW(0, 1) = -1.0; WW(0, 0) = -1.0 - s.k2H2;
  }
#undef UU
#undef WW
}

// For border column b: forward sweep of U over the tail (in place, U -> Uf)
// and partial back substitution; returns W^T M^{-1} U_b into cap[r*3+b].
__device__ __forceinline__ void tail_minv_u(const Mode& m, const Shared& S, int c, double* U, const double* W, int b,
                                            double* cap) {
  double X[kTail] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (c < 3 + m.nq) {
    int i0 = tail_index(m, c, 0), i1 = tail_index(m, c, 1), i2 = tail_index(m, c, 2);
    double u2 = U[2 * kBorder + b];
    double u1 = U[1 * kBorder + b] - S.fl[i1] * u2;
    double uvb = 0.0, udb = 0.0;
    if (c == 0) {
      udb = U[4 * kBorder + b];
      uvb = U[3 * kBorder + b] - S.fl[m.iPhi + 4] * udb;
      u1 -= S.fl[m.iPhi + 3] * uvb;  // lb
    }
    double u0 = U[0 * kBorder + b] - S.fl[i0] * u1;
    U[0 * kBorder + b] = u0; U[1 * kBorder + b] = u1; U[2 * kBorder + b] = u2;
    U[3 * kBorder + b] = uvb; U[4 * kBorder + b] = udb;
    X[0] = u0 * S.fi[i0];
    X[1] = u1 * S.fi[i1] - S.fc[i1] * X[0];
    X[2] = u2 * S.fi[i2] - S.fc[i2] * X[1];
    if (c == 0) {
      int ivb = m.iPhi + 4, idb = m.iPhi + 3;
      X[3] = uvb * S.fi[ivb] - S.fc[ivb] * X[1];
      X[4] = udb * S.fi[idb] - S.fc[idb] * X[3];
    }
  } else if (c == 3 + m.nq) {
    double uv = U[1 * kBorder + b];
    double ud = U[0 * kBorder + b] - S.fl[m.iPhi + 1] * uv;
    U[0 * kBorder + b] = ud;
    X[0] = ud * S.fi[m.iPhi + 1];
    X[1] = uv * S.fi[m.iPhi + 2];
  } else {
    X[0] = U[0 * kBorder + b] * S.fi[m.iPhi];
  }
  for (int r = 0; r < kBorder; ++r) {
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < kTail; ++a) acc += W[a * kBorder + r] * X[a];
    cap[r * 3 + b] = acc;
  }
}

// Sum over the CTA of per-chain partials stored in part[c * stride + r]:
// every warp reduces the nch partials with shuffles (no extra barrier).
__device__ __forceinline__ double chain_sum(const double* part, int nch, int stride, int r, int lane) {
  double v = lane < nch ? part[lane * stride + r] : 0.0;
  return warp_sum(v);
}

// Factorisation of M chain by chain (segmented Moebius scans), border tails
// and the 3x3 capacitance inverse (misc[0..8]).  All threads call it; returns
// false on a zero or non-finite pivot.
__device__ bool factorize_scan(const Mode& m, const Shared& S, const Pack& P, double hg, int tid, int nth) {
  const int lane = tid & 31;
  const Scal<double> s = get_scal<double>(S, 0);
  const double ig = 1.0 / hg;
  const bool rsa = rsa_switch(m, s);
  const int E = P.E[0];
  const int c = P.chain[tid];
  const int seg = P.seg[tid];
  const int own_c = (tid == P.E[1]) ? 3 + m.nq : ((c >= 0 && P.owner[c] == tid) ? c : -1);
  const int own_c2 = (tid == P.E[1]) ? 4 + m.nq : -1;
  bool ok = true;
  const LaneIdx idx = lane_idx(P, tid);
  // ---- local Moebius products; the per-element factors wait in fl / fi
  // (multipliers) and yt / b (couplings), which are free during the
  // factorisation
  M2 loc = {1.0, 0.0, 0.0, 1.0};
  if (c >= 0) {
    ChainDesc cd = chain_desc(m, c);
    for (int e = 0; e < E; ++e) {
      const int i = idx[e];
      if (i < 0) break;
      int l = (i - cd.base) / cd.stride;
      ElemC ec = elem_coef(m, S, s, ig, c, l, cd.L, rsa);
      if (c == 0 && l == 1) {
        double corr;
        baryon_pair(m, S, s, ig, hg, rsa, corr);
        ec.d += corr;
      }
      double p = ec.lo * ec.upPrev;  // 0 for the chain's first element
      double id = frcp(ec.d);
      double am = -p * id;
      S.fl[i] = am;
      S.fi[i] = id;
      S.yt[i] = ec.lo;
      S.b[i] = ec.up;
      M2 t = {1.0, am, id, 0.0};
      loc = mmul(t, loc);
    }
  }
  // ---- segmented inclusive scan over lanes: pre = loc * pre(previous)
  M2 inc = loc;
  for (int off = 1; off < P.E[2]; off <<= 1) {
    M2 o = shfl_up_m2(inc, off);
    if (seg >= 0 && lane - off >= seg) inc = mmul(inc, o);
  }
  M2 ex = shfl_up_m2(inc, 1);
  if (!(seg >= 0 && lane > seg)) ex = M2{1.0, 0.0, 0.0, 1.0};
  if (c >= 0) {
    double vn = ex.a, vm = ex.c;  // ex * (1, 0)
    double fi_prev = vm / vn;     // 0 at the chain's first element
    for (int e = 0; e < E; ++e) {
      const int i = idx[e];
      if (i < 0) break;
      double am = S.fl[i], bm = S.fi[i], lo = S.yt[i], up = S.b[i];
      double n2 = fma(am, vm, vn), m2 = bm * vn;
      double fi = m2 * frcp(n2);
      S.fi[i] = fi;
      S.fl[i] = lo * fi_prev;
      S.fc[i] = up * fi;
      ok = ok && isfinite(fi) && n2 != 0.0;
      fi_prev = fi;
      vn = n2;
      vm = m2;
    }
  }
  // ---- CDM pair and Phi (spare thread)
  if (tid == P.E[1]) {
    int idl = m.iPhi + 1, iv = m.iPhi + 2;
    double ipv = 1.0 / (ig + 1.0);
    S.fl[iv] = 0.0; S.fi[iv] = ipv; S.fc[iv] = 0.0;
    S.fl[idl] = -s.kH * ipv; S.fi[idl] = hg; S.fc[idl] = 0.0;
    S.fl[m.iPhi] = 0.0; S.fi[m.iPhi] = hg; S.fc[m.iPhi] = 0.0;
  }
  ok = __syncthreads_and(ok);
  // ---- border tails and capacitance contributions (tail owners)
  double* part = S.misc + 32;  // [nch][9]
  for (int k2 = 0; k2 < 2; ++k2) {
    const int cc = k2 == 0 ? own_c : own_c2;  // each owner handles its own chain(s) concurrently
    if (cc < 0) continue;
    double* uf = S.Uf + cc * kTail * kBorder;
    double* wt = S.Wt + cc * kTail * kBorder;
    border_tails(m, S, s, cc, rsa, uf, wt);
    for (int b = 0; b < kBorder; ++b) tail_minv_u(m, S, cc, uf, wt, b, part + cc * 9);
  }
  __syncthreads();
  double Cm[9];
  for (int r = 0; r < 9; ++r) Cm[r] = ((r % 4) == 0 ? 1.0 : 0.0) - chain_sum(part, m.nch, 9, r, lane);
  double det = Cm[0] * (Cm[4] * Cm[8] - Cm[5] * Cm[7]) - Cm[1] * (Cm[3] * Cm[8] - Cm[5] * Cm[6]) +
               Cm[2] * (Cm[3] * Cm[7] - Cm[4] * Cm[6]);
  double id = 1.0 / det;
  if (tid == 0) {
    S.misc[0] = (Cm[4] * Cm[8] - Cm[5] * Cm[7]) * id;
    S.misc[1] = (Cm[2] * Cm[7] - Cm[1] * Cm[8]) * id;
    S.misc[2] = (Cm[1] * Cm[5] - Cm[2] * Cm[4]) * id;
    S.misc[3] = (Cm[5] * Cm[6] - Cm[3] * Cm[8]) * id;
    S.misc[4] = (Cm[0] * Cm[8] - Cm[2] * Cm[6]) * id;
    S.misc[5] = (Cm[2] * Cm[3] - Cm[0] * Cm[5]) * id;
    S.misc[6] = (Cm[3] * Cm[7] - Cm[4] * Cm[6]) * id;
    S.misc[7] = (Cm[1] * Cm[6] - Cm[0] * Cm[7]) * id;
    S.misc[8] = (Cm[0] * Cm[4] - Cm[1] * Cm[3]) * id;
  }
  __syncthreads();
  return ok && isfinite(id) && det != 0.0;
}

// In-place solve b <- (M - U W^T)^{-1} b (all threads).
__device__ void wsolve_scan(const Mode& m, const Shared& S, const Pack& P, double* b, int tid, int nth) {
  const int lane = tid & 31;
  const int E = P.E[0];
  const int c = P.chain[tid];
  const int seg = P.seg[tid];
  const int own_c = (tid == P.E[1]) ? 3 + m.nq : ((c >= 0 && P.owner[c] == tid) ? c : -1);
  const int own_c2 = (tid == P.E[1]) ? 4 + m.nq : -1;
  // ---- forward: b'_j = b_j - fl_j b'_{j-1}
  const LaneIdx idx = lane_idx(P, tid);
  double A = 1.0, B = 0.0;
  int cnt = 0;  // valid elements of this lane
  if (c >= 0) {
    for (int e = 0; e < E; ++e) {
      const int i = idx[e];
      if (i < 0) break;
      double bi = b[i];
      if (c == 0 && i == 1) {  // Theta_1 <- baryon pair (eliminated first)
        double bdb = b[m.iPhi + 3];
        double bvb = b[m.iPhi + 4] - S.fl[m.iPhi + 4] * bdb;
        bi -= S.fl[m.iPhi + 3] * bvb;
        b[m.iPhi + 4] = bvb;
        b[i] = bi;
      }
      double al = -S.fl[i];
      A = al * A;
      B = fma(al, B, bi);
      cnt = e + 1;
    }
  }
  for (int off = 1; off < P.E[2]; off <<= 1) {
    double oA = __shfl_up_sync(0xffffffffu, A, off), oB = __shfl_up_sync(0xffffffffu, B, off);
    if (seg >= 0 && lane - off >= seg) { B = fma(A, oB, B); A = A * oA; }
  }
  double prev = __shfl_up_sync(0xffffffffu, B, 1);
  if (!(seg >= 0 && lane > seg)) prev = 0.0;
  for (int e = 0; e < cnt; ++e) {
    const int i = idx[e];
    double v = fma(-S.fl[i], prev, b[i]);
    b[i] = v;
    prev = v;
  }
  if (tid == P.E[1]) b[m.iPhi + 1] -= S.fl[m.iPhi + 1] * b[m.iPhi + 2];
  __syncthreads();
  // ---- border: t = W^T y at the tails, s = C^{-1} t, tail correction
  double* part = S.misc + 32;
  for (int k2 = 0; k2 < 2; ++k2) {
    const int cc = k2 == 0 ? own_c : own_c2;  // each owner handles its own chain(s) concurrently
    if (cc < 0) continue;
    double xt[kTail] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (cc < 3 + m.nq) {
      int i0 = tail_index(m, cc, 0), i1 = tail_index(m, cc, 1), i2 = tail_index(m, cc, 2);
      xt[0] = b[i0] * S.fi[i0];
      xt[1] = b[i1] * S.fi[i1] - S.fc[i1] * xt[0];
      xt[2] = b[i2] * S.fi[i2] - S.fc[i2] * xt[1];
      if (cc == 0) {
        int ivb = m.iPhi + 4, idb = m.iPhi + 3;
        xt[3] = b[ivb] * S.fi[ivb] - S.fc[ivb] * xt[1];
        xt[4] = b[idb] * S.fi[idb] - S.fc[idb] * xt[3];
      }
    } else if (cc == 3 + m.nq) {
      xt[0] = b[m.iPhi + 1] * S.fi[m.iPhi + 1];
      xt[1] = b[m.iPhi + 2] * S.fi[m.iPhi + 2];
    } else {
      xt[0] = b[m.iPhi] * S.fi[m.iPhi];
    }
    const double* wt = S.Wt + cc * kTail * kBorder;
    for (int r = 0; r < kBorder; ++r) {
      double acc = 0.0;
      for (int a = 0; a < kTail; ++a) acc += wt[a * kBorder + r] * xt[a];
      part[cc * 9 + r] = acc;
    }
  }
  __syncthreads();
  double t0 = chain_sum(part, m.nch, 9, 0, lane), t1 = chain_sum(part, m.nch, 9, 1, lane),
         t2 = chain_sum(part, m.nch, 9, 2, lane);
  double sv[kBorder];
  for (int r = 0; r < kBorder; ++r) sv[r] = S.misc[r * 3 + 0] * t0 + S.misc[r * 3 + 1] * t1 + S.misc[r * 3 + 2] * t2;
  for (int k2 = 0; k2 < 2; ++k2) {
    const int cc = k2 == 0 ? own_c : own_c2;  // each owner handles its own chain(s) concurrently
    if (cc < 0) continue;
    const double* uf = S.Uf + cc * kTail * kBorder;
    int ns = tail_slots(m, cc);
    for (int a = 0; a < ns; ++a) {
      int i = tail_index(m, cc, a);
      b[i] += uf[a * kBorder + 0] * sv[0] + uf[a * kBorder + 1] * sv[1] + uf[a * kBorder + 2] * sv[2];
    }
  }
  __syncthreads();
  // ---- backward: x_j = fi_j b'_j - fc_j x_{j+1} (reverse scan)
  A = 1.0;
  B = 0.0;
  for (int e = cnt - 1; e >= 0; --e) {
    const int i = idx[e];
    double ga = b[i] * S.fi[i], de = -S.fc[i];
    B = fma(de, B, ga);
    A = de * A;
  }
  int segend = 31;
  {
    // last lane of this lane's segment: lanes of one chain are contiguous
    int ch = c;
    int l2 = lane;
    while (l2 < 31 && P.chain[(tid - lane) + l2 + 1] == ch && P.seg[(tid - lane) + l2 + 1] == seg) ++l2;
    segend = l2;
  }
  for (int off = 1; off < P.E[2]; off <<= 1) {
    double oA = __shfl_down_sync(0xffffffffu, A, off), oB = __shfl_down_sync(0xffffffffu, B, off);
    if (seg >= 0 && lane + off <= segend) { B = fma(A, oB, B); A = A * oA; }
  }
  double nxt = __shfl_down_sync(0xffffffffu, B, 1);
  if (!(seg >= 0 && lane < segend)) nxt = 0.0;
  for (int e = cnt - 1; e >= 0; --e) {
    const int i = idx[e];
    double v = fma(-S.fc[i], nxt, b[i] * S.fi[i]);
    b[i] = v;
    nxt = v;
    if (c == 0 && i == 1) {  // baryon pair after Theta_1
      int ivb = m.iPhi + 4, idb = m.iPhi + 3;
      double xvb = b[ivb] * S.fi[ivb] - S.fc[ivb] * v;
      b[ivb] = xvb;
      b[idb] = b[idb] * S.fi[idb] - S.fc[idb] * xvb;
    }
  }
  if (tid == P.E[1]) {
    b[m.iPhi + 1] = b[m.iPhi + 1] * S.fi[m.iPhi + 1];
    b[m.iPhi + 2] = b[m.iPhi + 2] * S.fi[m.iPhi + 2];
    b[m.iPhi] = b[m.iPhi] * S.fi[m.iPhi];
  }
  __syncthreads();
}
