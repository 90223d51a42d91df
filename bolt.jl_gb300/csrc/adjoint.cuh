// Discrete adjoint of the Rodas4 solve (mode flags MODE_CKPT, MODE_ADJOINT).
//
// The forward solve of a mode (MODE_RECORD | MODE_CKPT) records the end
// abscissa of every accepted step and keeps the state at the start of every
// kCkptEvery-th one.  The reverse sweep (MODE_ADJOINT) walks the segments
// between checkpoints from the last to the first: it replays the segment's
// steps from its checkpoint (states and stage increments kept in global
// scratch), then runs through them backwards, refactorising each step and
// pulling the cotangent lambda of the state back through it.  For the
// linear ODE u' = A(x) u the step is
//   M K_i = A_i Y_i + h d_i A'_0 y + (1/h) sum_{j<i} C_ij K_j,
//   Y_i = y + sum_{j<i} a_ij K_j,  y_new = Y_6 + K_6,  M = I/(h gamma) - A_0,
// and its adjoint, stage by stage from the last,
//   rbar_i = M^-T Kbar_i,
//   Ybar_i += A_i^T rbar_i,  Fbar += h d_i rbar_i,  Kbar_j += (C_ij / h) rbar_i,
//   ybar += Ybar_i,  Kbar_j += a_ij Ybar_i,
// then ybar += A'_0^T Fbar.  The parameter cotangent collects, per stage,
// rbar_i . (dA_i Y_i + dA_0 K_i) and, per step, Fbar . dA'_0 y, with the
// coefficient tangents dA of the tangent-linear mode (the differences of the
// perturbed parameter sets' coefficients over their steps), so the two modes
// differentiate the same discrete pipeline.  The outputs' cotangents enter
// at their nodes (S_T: the gradient of source_function with respect to the
// state and its derivative; P_lin: the gradient of plin), the initial
// conditions' tangents close the sweep.  A^T lambda comes from the column
// form of hierarchy! (rhs_cols), M^-T from the step's chain factorisation
// read in transposed order (wsolve_scan_T).
//
// Included inside namespace bolt by solver.cu, after tangent.cuh.
#pragma once

// State read as d4 numbers with zero tangents (the coefficients' tangents
// alone: dA u).
struct StC {
  const double* u;
  __device__ __forceinline__ d4 operator[](int i) const { return c4(u[i]); }
};
// State read as d4 numbers with tangents du[j * N + i], or none (du null).
struct StM {
  const double* u;
  const double* du;
  int N;
  __device__ __forceinline__ d4 operator[](int i) const {
    d4 r = c4(u[i]);
    if (du)
#pragma unroll
      for (int j = 0; j < kTD; ++j) r.t[j] = du[j * N + i];
    return r;
  }
};

// (A^T lam)_i of one chain column j (multipole j of a chain with top L and
// state indices base + l * stride): mk = the chain's streaming factor
// (k / H, times q / eps for massive neutrinos), dlo the diagonal of rows
// l < L, dtop that of row L.
template <class T>
__device__ __forceinline__ T chain_col(const T& mk, const T& dlo, const T& dtop, const double* cl1, const double* cl2,
                                       int j, int L, const double* lam, int base, int stride) {
  T g = (j < L ? dlo : dtop) * lam[base + j * stride];
  if (j >= 1) g = g - mk * (cl2[j - 1] * lam[base + (j - 1) * stride]);
  if (j + 1 <= L) g = g + (j + 1 < L ? mk * cl1[j + 1] : mk) * lam[base + (j + 1) * stride];
  return g;
}

// Column form of rhs_rows: out = A(x_sl)^T lam (T = double), and for T = dd
// also out.d = A'(x_sl)^T lam.  A = L + U W^T: the direct couplings of
// hierarchy! (perturbations.jl:196-270) transposed, plus the metric border
// (Phi', Psi, Pi) as W (U^T lam).  Rows that the radiation-streaming switch
// zeroes contribute nothing.  All threads; returns the switch.
template <class T>
__device__ bool rhs_cols(const Mode& m, const Shared& S, int sl, const double* lam, const Sink& out, int tid, int nth) {
  using K = typename KT<T>::type;
  const int lane = tid & 31;
  const Scal<T> s = get_scal<T>(S, sl);
  const bool rsa = rsa_switch(m, s);
  const int lg = m.lg, lnu = m.lnu, lmnu = m.lmnu, nq = m.nq;
  const double* cl1 = S.cl1;
  const double* cl2 = S.cl2;
  const CosmoDev& C = *m.C;
  const double Omega_nu = C.Omega_nu;
  // ---- border rows: bP = sum_r U[r][Phi'] lam_r, bS (Psi), bPi (Pi)
  T bP = cst<T>(0.0), bS = cst<T>(0.0), bPi = cst<T>(0.0);
  for (int q = lane; q < nq; q += 32) {
    const K df0 = kval<K>(S.df0, S.ddf0, q);
    bP = bP + df0 * lam[m.iM + q];                                                       // M_0q: + Phi' df0
    bS = bS - ((1.0 / 3.0) * s.kH * eq_of<T>(S, sl, nq, q) * df0) * lam[m.iM + nq + q];  // M_1q
  }
  bP = warp_sum_t<T>(bP);
  bS = warp_sum_t<T>(bS);
  if (!rsa) {
    bP = bP - (lam[0] + lam[m.iN]);                                  // Theta_0, N_0: - Phi'
    bS = bS + (1.0 / 3.0) * s.kH * (lam[1] + lam[m.iN + 1]);          // Theta_1, N_1: + k/H Psi / 3
    bPi = -s.tp * (lam[2] / 10.0 + lam[m.iTp] / 2.0 + lam[m.iTp + 2] / 10.0);
  }
  bP = bP + (lam[m.iPhi] - 3.0 * (lam[m.iPhi + 1] + lam[m.iPhi + 3]));  // Phi: + Phi'; delta_c, delta_b: - 3 Phi'
  bS = bS - s.kH * (lam[m.iPhi + 2] + lam[m.iPhi + 4]);                 // v_c, v_b: - k/H Psi
  // Psi enters Phi' with weight one: the gradient of Psi carries bS + bP
  const T gS = bS + bP;
  const K rc0 = kcos<K>(m, S, 0), rc1 = kcos<K>(m, S, 1), Oc = kcos<K>(m, S, 2), Ob = kcos<K>(m, S, 3);
  const T ia = 1.0 / s.a;
  const T dP = s.dphi * bP;  // the explicit part of Phi'
  const T zero = cst<T>(0.0);
  for (int i = tid; i < m.N; i += nth) {
    T g = zero;
    if (i < m.iM) {
      if (i < m.iTp) {  // photon temperature
        const int l = i;
        if (!rsa) g = chain_col<T>(s.kH, l >= 1 ? s.tp : zero, s.tp - (lg + 1.0) * s.iHe, cl1, cl2, l, lg, lam, 0, 1);
        if (l == 1) g = g + 3.0 * s.tp * s.R * lam[m.iPhi + 4];  // v_b row: + tau' R 3 Theta_1
        if (l == 0) g = g + (4.0 * C.Omega_r) * ia * ia * dP;
        if (l == 2) g = g - (s.cpsi * C.Omega_r) * gS + bPi;
      } else if (i < m.iN) {  // photon polarization
        const int l = i - m.iTp;
        if (!rsa) g = chain_col<T>(s.kH, s.tp, s.tp - (lg + 1.0) * s.iHe, cl1, cl2, l, lg, lam, m.iTp, 1);
        if (l == 0 || l == 2) g = g + bPi;
      } else {  // massless neutrinos
        const int l = i - m.iN;
        if (!rsa) g = chain_col<T>(s.kH, zero, -(lnu + 1.0) * s.iHe, cl1, cl2, l, lnu, lam, m.iN, 1);
        if (l == 0) g = g + (4.0 * Omega_nu) * ia * ia * dP;
        if (l == 2) g = g - (s.cpsi * Omega_nu) * gS;
      }
    } else if (i < m.iPhi) {  // massive neutrinos
      const int j = i - m.iM;
      const int l = j / nq, q = j - l * nq;
      const T mk = qe_of<T>(S, sl, nq, q) * s.kH;
      g = chain_col<T>(mk, zero, -(lmnu + 1.0) * s.iHe, cl1, cl2, l, lmnu, lam, m.iM + q, nq);
      const K wq = kval<K>(S.Aq, S.dAq, q) * kval<K>(S.q, S.dq, q);
      if (l == 0) g = g + (wq * eq_of<T>(S, sl, nq, q) * rc1) * (ia * ia) * dP;   // rho / rho_crit in Phi'
      if (l == 2) g = g - (s.cpsi * (wq * qe_of<T>(S, sl, nq, q) * rc0)) * gS;    // sigma / (4 rho_crit) in Psi
    } else {  // metric and matter
      const int r = i - m.iPhi;
      if (r == 0) g = -gS - s.k2H2 * bP;                                         // Phi
      else if (r == 1) g = (Oc * ia) * dP;                                       // delta_c
      else if (r == 2) g = s.kH * lam[m.iPhi + 1] - lam[m.iPhi + 2];              // v_c
      else if (r == 3) g = (Ob * ia) * dP - s.kH * s.cs2 * lam[m.iPhi + 4];       // delta_b
      else {                                                                     // v_b
        g = s.kH * lam[m.iPhi + 3] + (s.tp * s.R - 1.0) * lam[m.iPhi + 4];
        if (!rsa) g = g + (s.tp / 3.0) * lam[1];
      }
    }
    put<T>(out, i, g);
  }
  return rsa;
}

// In-place transposed solve b <- (M - U W^T)^-T b with the step's
// factorisation (all threads).  With M = L U (L unit lower, U upper in the
// elimination order of factorize_scan) and the capacitance C = I - W^T M^-1 U:
//   U^T: v_j = b_j - fc_{j-1} v_{j-1}, w_j = fi_j v_j   (forward scan),
//   border: t = (L^-1 U)^T w (the stored tails), s = C^-T t,
//           w_tail += (U^-T W)_tail s,
//   L^T: z_j = w_j - fl_{j+1} z_{j+1}                 (reverse scan).
__device__ void wsolve_scan_T(const Mode& m, const Shared& S, const Pack& P, double* b, int tid, int nth) {
  const int lane = tid & 31;
  const int E = P.E[0];
  const int c = P.chain[tid];
  const int seg = P.seg[tid];
  const int own_c = (tid == P.E[1]) ? 3 + m.nq : ((c >= 0 && P.owner[c] == tid) ? c : -1);
  const int own_c2 = (tid == P.E[1]) ? 4 + m.nq : -1;
  const int idb = m.iPhi + 3, ivb = m.iPhi + 4;
  const LaneIdx idx = lane_idx(P, tid);
  int cnt = 0;
  if (c >= 0)
    for (int e = 0; e < E; ++e) {
      if (idx[e] < 0) break;
      cnt = e + 1;
    }
  int segend = 31;
  {
    int l2 = lane;
    while (l2 < 31 && P.chain[(tid - lane) + l2 + 1] == c && P.seg[(tid - lane) + l2 + 1] == seg) ++l2;
    segend = l2;
  }
  // fc of the element before this lane's first, fl of the one after its last
  const double fc_in = (c >= 0 && lane > seg) ? S.fc[P.idx[(E - 1) * P.nt + tid - 1]] : 0.0;
  const double fl_out = (c >= 0 && lane < segend) ? S.fl[P.idx[tid + 1]] : 0.0;
  // ---- forward (U^T): v_j = b_j - fc_{j-1} v_{j-1}; the baryon pair (delta_b,
  // v_b, eliminated before Theta_1) folds into Theta_1's right-hand side
  double A = 1.0, B = 0.0;
  {
    double fcp = fc_in;
    for (int e = 0; e < cnt; ++e) {
      const int i = idx[e];
      double ci = b[i];
      if (c == 0 && i == 1) {
        const double vdb = b[idb];
        const double vvb = fma(-S.fc[idb], vdb, b[ivb]);
        ci = fma(-S.fc[ivb], vvb, ci);
        b[idb] = vdb * S.fi[idb];
        b[ivb] = vvb * S.fi[ivb];
        b[i] = ci;
      }
      const double al = -fcp;
      A = al * A;
      B = fma(al, B, ci);
      fcp = S.fc[i];
    }
  }
  for (int off = 1; off < P.E[2]; off <<= 1) {
    double oA = __shfl_up_sync(0xffffffffu, A, off), oB = __shfl_up_sync(0xffffffffu, B, off);
    if (seg >= 0 && lane - off >= seg) { B = fma(A, oB, B); A = A * oA; }
  }
  double prev = __shfl_up_sync(0xffffffffu, B, 1);
  if (!(seg >= 0 && lane > seg)) prev = 0.0;
  {
    double fcp = fc_in;
    for (int e = 0; e < cnt; ++e) {
      const int i = idx[e];
      const double v = fma(-fcp, prev, b[i]);
      fcp = S.fc[i];
      b[i] = v * S.fi[i];
      prev = v;
    }
  }
  if (tid == P.E[1]) {  // CDM pair (v_c eliminated first; fc[v_c] = 0) and Phi
    const int idl = m.iPhi + 1, iv = m.iPhi + 2;
    const double vv = b[iv];
    const double vd = fma(-S.fc[iv], vv, b[idl]);
    b[iv] = vv * S.fi[iv];
    b[idl] = vd * S.fi[idl];
    b[m.iPhi] = b[m.iPhi] * S.fi[m.iPhi];
  }
  __syncthreads();
  // ---- border: t = Uf^T w over the tails, s = C^-T t, w_tail += (U^-T W) s
  double* part = S.misc + 32;
  for (int k2 = 0; k2 < 2; ++k2) {
    const int cc = k2 == 0 ? own_c : own_c2;
    if (cc < 0) continue;
    const double* uf = S.Uf + cc * kTail * kBorder;
    const int ns = tail_slots(m, cc);
    for (int r = 0; r < kBorder; ++r) {
      double acc = 0.0;
      for (int a = 0; a < ns; ++a) acc = fma(uf[a * kBorder + r], b[tail_index(m, cc, a)], acc);
      part[cc * 9 + r] = acc;
    }
  }
  __syncthreads();
  const double t0 = chain_sum(part, m.nch, 9, 0, lane), t1 = chain_sum(part, m.nch, 9, 1, lane),
               t2 = chain_sum(part, m.nch, 9, 2, lane);
  double sv[kBorder];
  for (int r = 0; r < kBorder; ++r) sv[r] = S.misc[0 * 3 + r] * t0 + S.misc[1 * 3 + r] * t1 + S.misc[2 * 3 + r] * t2;
  for (int k2 = 0; k2 < 2; ++k2) {
    const int cc = k2 == 0 ? own_c : own_c2;
    if (cc < 0) continue;
    const double* wt = S.Wt + cc * kTail * kBorder;
    double add[kTail] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int r = 0; r < kBorder; ++r) {
      double vw[kTail] = {0.0, 0.0, 0.0, 0.0, 0.0};
      if (cc < 3 + m.nq) {  // tail order of elimination: l = 2, (delta_b, v_b), l = 1, l = 0
        const int i1 = tail_index(m, cc, 1), i2 = tail_index(m, cc, 2);
        vw[2] = wt[2 * kBorder + r];
        vw[1] = fma(-S.fc[i2], vw[2], wt[1 * kBorder + r]);
        if (cc == 0) {
          vw[4] = wt[4 * kBorder + r];
          vw[3] = fma(-S.fc[idb], vw[4], wt[3 * kBorder + r]);
          vw[1] = fma(-S.fc[ivb], vw[3], vw[1]);
        }
        vw[0] = fma(-S.fc[i1], vw[1], wt[0 * kBorder + r]);
      } else if (cc == 3 + m.nq) {  // slots (delta_c, v_c); v_c eliminated first
        vw[1] = wt[1 * kBorder + r];
        vw[0] = fma(-S.fc[m.iPhi + 2], vw[1], wt[0 * kBorder + r]);
      } else {
        vw[0] = wt[r];
      }
      for (int a = 0; a < kTail; ++a) add[a] = fma(vw[a], sv[r], add[a]);
    }
    const int ns = tail_slots(m, cc);
    for (int a = 0; a < ns; ++a) {
      const int i = tail_index(m, cc, a);
      b[i] = fma(S.fi[i], add[a], b[i]);
    }
  }
  __syncthreads();
  // ---- backward (L^T): z_j = w_j - fl_{j+1} z_{j+1}; the pair after Theta_1
  A = 1.0;
  B = 0.0;
  for (int e = cnt - 1; e >= 0; --e) {
    const int i = idx[e];
    const double be = -(e == cnt - 1 ? fl_out : S.fl[idx[e + 1]]);
    B = fma(be, B, b[i]);
    A = be * A;
  }
  for (int off = 1; off < P.E[2]; off <<= 1) {
    double oA = __shfl_down_sync(0xffffffffu, A, off), oB = __shfl_down_sync(0xffffffffu, B, off);
    if (seg >= 0 && lane + off <= segend) { B = fma(A, oB, B); A = A * oA; }
  }
  double nxt = __shfl_down_sync(0xffffffffu, B, 1);
  if (!(seg >= 0 && lane < segend)) nxt = 0.0;
  for (int e = cnt - 1; e >= 0; --e) {
    const int i = idx[e];
    const double be = -(e == cnt - 1 ? fl_out : S.fl[idx[e + 1]]);
    const double z = fma(be, nxt, b[i]);
    b[i] = z;
    nxt = z;
    if (c == 0 && i == 1) {  // L[Theta_1][v_b] = lb (kept in fl[delta_b]), L[v_b][delta_b] = fl[v_b]
      const double zvb = fma(-S.fl[idb], z, b[ivb]);
      b[ivb] = zvb;
      b[idb] = fma(-S.fl[ivb], zvb, b[idb]);
    }
  }
  if (tid == P.E[1]) b[m.iPhi + 2] = fma(-S.fl[m.iPhi + 1], b[m.iPhi + 1], b[m.iPhi + 2]);
  __syncthreads();
}

// Gradient of source_function (perturbations.jl:343-389, emit_sources_t's
// T part) with respect to the state u and its derivative du at node x,
// times sb: gu += sb dS_T/du, gdu += sb dS_T/d(du).  S_T is linear in
// (u, du); the coefficients are those of emit_sources_t.  Warp 0 (lane 0
// the scalar rows, every lane its momentum bins).  gu / gdu are added to.
__device__ void source_grad(const Mode& m, const Shared& S, double x, double sb, double* gu, double* gdu, int lane) {
  const CosmoDev& C = *m.C;
  const double a = exp(x), k = m.k;
  const double H0 = C.H0, rho_crit = C.rho_crit;
  const double Hc = spl_cold(C, C_H, x), Hcp = spl_cold(C, C_HP, x), Hcpp = spl_cold(C, C_HPP, x);
  const double tau = spl_cold(C, C_TAU, x), tp = spl_cold(C, C_TAUP, x), tpp = spl_cold(C, C_TAUPP, x);
  const double g = spl_cold(C, C_G, x), gp = spl_cold(C, C_GP, x), gpp = spl_cold(C, C_GPP, x);
  const double Omega_nu = C.Omega_nu;
  const double c = 12.0 * H0 * H0 / (k * k) / (a * a);
  const double et = exp(-tau);
  const double aPsi = g, aPsip = et;
  const double f34 = 3.0 / (4.0 * k * k);
  const double cPP = f34 * Hc * Hc * g;  // coefficient of Pi''
  const double aPi = g / 4.0 + f34 * ((Hcp * Hcp + Hc * Hcpp) * g + 3.0 * Hc * Hcp * gp + Hc * Hc * gpp) +
                     cPP * (3.0 / 10.0) * tpp;
  const double aPip = f34 * (3.0 * Hc * Hcp * g + 2.0 * Hc * Hc * gp) + cPP * (3.0 / 10.0) * tp;
  const double aS = -c / (4.0 * rho_crit) * aPsi + 2.0 * c / (4.0 * rho_crit) * aPsip;  // d/d sigma
  const double aSp = -c / (4.0 * rho_crit) * aPsip;                                       // d/d sigma'
  for (int q = lane; q < m.nq; q += 32) {
    const double am = a * C.Sigma_m_nu, qq = S.q[q];
    const double eps = sqrt(qq * qq + am * am);
    const double w = S.Aq[q] * qq * qq / eps;
    gu[m.iM + 2 * m.nq + q] += sb * w * aS;
    gdu[m.iM + 2 * m.nq + q] += sb * w * aSp;
  }
  if (lane != 0) return;
  const int Tp = m.iTp;
  const double a1 = cPP * (2.0 * k / (5.0 * Hc)) * (-Hcp / Hc), ad1 = cPP * 2.0 * k / (5.0 * Hc);
  const double a3 = cPP * (-3.0 * k / (5.0 * Hc)) * (-Hcp / Hc), ad3 = cPP * (-3.0 * k / (5.0 * Hc));
  gu[0] += sb * g;
  gu[1] += sb * a1;
  gu[2] += sb * (-c * C.Omega_r * aPsi + 2.0 * c * C.Omega_r * aPsip + aPi);
  gu[3] += sb * a3;
  gu[Tp] += sb * aPi;
  gu[Tp + 1] += sb * a3;
  gu[Tp + 2] += sb * aPi;
  gu[Tp + 3] += sb * a3;
  gu[m.iN + 2] += sb * (-c * Omega_nu * aPsi + 2.0 * c * Omega_nu * aPsip);
  gu[m.iPhi] += sb * (-aPsi);
  gu[m.iPhi + 4] += sb * (-(1.0 / k) * (Hcp * g + Hc * gp));
  gdu[1] += sb * ad1;
  gdu[2] += sb * (-c * C.Omega_r * aPsip + aPip);
  gdu[3] += sb * ad3;
  gdu[Tp] += sb * aPip;
  gdu[Tp + 1] += sb * ad3;
  gdu[Tp + 2] += sb * aPip;
  gdu[Tp + 3] += sb * ad3;
  gdu[m.iN + 2] += sb * (-c * Omega_nu * aPsip);
  gdu[m.iPhi] += sb * (-2.0 * et);
  gdu[m.iPhi + 4] += sb * (-(1.0 / k) * Hc * g);
}

// Gradient of plin (spectra.jl:163-198, emit_plin_t) with respect to the
// state u at x, times pb, added to gu.  Warp 0.
__device__ void plin_grad(const Mode& m, const Shared& S, double x, const double* u, double pb, double* gu, int lane) {
  const CosmoDev& C = *m.C;
  const double a = exp(x), k = m.k;
  double rho = 0.0, th = 0.0;
  for (int q = lane; q < m.nq; q += 32) {
    const double am = a * C.Sigma_m_nu, qq = S.q[q];
    const double eps = sqrt(qq * qq + am * am);
    rho += S.Aq[q] * eps * u[m.iM + q];
    th += S.Bq[q] * u[m.iM + m.nq + q];
  }
  rho = warp_sum(rho);
  th = warp_sum(th);
  const double r0 = spl_cold(C, C_RHO0M, x), Hc = spl_cold(C, C_H, x);
  const double h = C.h, Omega_c = C.Omega_c, Omega_b = C.Omega_b;
  const double Tg = pow(15.0 / (M_PI * M_PI) * C.rho_crit * C.Omega_r, 0.25);
  const double nufac = (90.0 * 1.2020569 / (11.0 * pow(M_PI, 4))) * (C.Omega_r * h * h / Tg) * pow(C.N_nu / 3.0, 0.75);
  const double Omega_nu = C.Sigma_m_nu * nufac / (h * h);
  const double Om = Omega_c + Omega_b + Omega_nu;
  const double dc = u[m.iPhi + 1] - 3.0 * Hc * u[m.iPhi + 2] / k, db = u[m.iPhi + 3] - 3.0 * Hc * u[m.iPhi + 4] / k;
  const double dn = rho / r0 + 3.0 * Hc * th / (r0 * k);
  const double dm = (Omega_c * dc + Omega_b * db + Omega_nu * dn) / Om;
  const double Pp = C.A * pow(k / 0.05, C.n_s - 1.0);
  const double g0 = pb * 2.0 * (2.0 * M_PI * M_PI / (k * k * k)) * dm * Pp / Om;  // d P / d(Om dm), times pb
  for (int q = lane; q < m.nq; q += 32) {
    const double am = a * C.Sigma_m_nu, qq = S.q[q];
    const double eps = sqrt(qq * qq + am * am);
    gu[m.iM + q] += g0 * Omega_nu * S.Aq[q] * eps / r0;
    gu[m.iM + m.nq + q] += g0 * Omega_nu * 3.0 * Hc * S.Bq[q] / (r0 * k);
  }
  if (lane != 0) return;
  gu[m.iPhi + 1] += g0 * Omega_c;
  gu[m.iPhi + 2] += g0 * Omega_c * (-3.0 * Hc / k);
  gu[m.iPhi + 3] += g0 * Omega_b;
  gu[m.iPhi + 4] += g0 * Omega_b * (-3.0 * Hc / k);
}

// Global scratch of an adjoint mode after the base slab: lam, ybar, Kbar
// [6], Ybar, Fbar, the state at the step's end u1, its derivative du, the
// output gradients gu / gdu, a vector tmp, two tangent blocks [kTD][N]
// (t4, t4b), the segment's states [kCkptEvery + 1][N] and its steps' stage
// increments [kCkptEvery][6][N].  (adj_scratch_doubles() in solver.cu
// sizes it.)
struct AdjScratch {
  double *lam, *yb, *Kb, *Yb, *Fb, *u1, *du, *gu, *gdu, *tmp, *t4, *t4b, *seg, *segK;
};

// rhs_rows in d4 numbers of a constant state u at slot sl: t4[j][i] =
// (dA_sl u)_i; the calling thread then adds rb . t4[j] to tb[j] over its own
// rows (rhs_rows' row assignment).
__device__ __forceinline__ void dA_dot(const Mode& m, const Shared& S, int sl, const double* u, const double* rb,
                                       double* t4, double* tb, int tid, int nth) {
  Sink o;
  o.v = nullptr; o.d = nullptr; o.t = t4; o.td = nullptr; o.N = m.N;
  rhs_rows<d4>(m, S, sl, StC{u}, o, tid, nth);
  for (int i = tid; i < m.N; i += nth)
#pragma unroll
    for (int j = 0; j < kTD; ++j) tb[j] = fma(rb[i], t4[j * m.N + i], tb[j]);
}

// rb . (dA_sl u) along the kTD tangent directions, added to tb[j], from the
// cotangents of hierarchy!'s coefficients: the reverse of rhs_rows (and of
// metric) over its coefficients -- the stage scalars, q/eps and eps/q of
// slot sl, the momentum-bin constants and the cosmology constants -- each
// cotangent times its tangents (S.sct, S.qet, S.eqt, S.dq, S.dAq, S.ddf0,
// S.cstn).  One pass whatever the number of directions; the same products
// as dA_dot.  T = dd (slot 0): rb . (dA'_0 u), the tangents of the
// x-derivative: with coefficients c carrying c' = dc/dx, each cotangent
// cbar = (d(rb.A u)/dc, its x-derivative) contributes cbar' dc + cbar dc'
// (dc' the tangents of c', S.sct_d / S.qet_d / S.eqt_d; the momentum-bin
// and cosmology constants do not depend on x).  Every thread adds its own
// rows' share (the metric's share on lane 0 and the momentum bins' on their
// lanes).  One warp.
template <class T>
__device__ __forceinline__ void addc(double* tb, const T& bar, const double* t0, const double* td);
template <>
__device__ __forceinline__ void addc<double>(double* tb, const double& bar, const double* t0, const double*) {
#pragma unroll
  for (int j = 0; j < kTD; ++j) tb[j] = fma(bar, t0[j], tb[j]);
}
template <>
__device__ __forceinline__ void addc<dd>(double* tb, const dd& bar, const double* t0, const double* td) {
#pragma unroll
  for (int j = 0; j < kTD; ++j) tb[j] = fma(bar.d, t0[j], td ? fma(bar.v, td[j], tb[j]) : tb[j]);
}

template <class T>
__device__ void coef_dot(const Mode& m, const Shared& S, int sl, const double* u, const double* rb, double* tb,
                         int tid, int nth) {
  const int lane = tid & 31;
  const int nq = m.nq, lg = m.lg, lnu = m.lnu, lmnu = m.lmnu;
  const bool X = sizeof(T) != sizeof(double);  // the x-derivative variant (slot 0)
  const Scal<T> s = get_scal<T>(S, sl);
  const bool rsa = rsa_switch(m, s);
  const double* cl1 = S.cl1;
  const double* cl2 = S.cl2;
  const CosmoDev& C = *m.C;
  const double Omega_nu = C.Omega_nu;
  const T zero = cst<T>(0.0);
  // the metric's values, as metric() forms them
  T rho = zero, sig = zero;
  for (int q = lane; q < nq; q += 32) {
    rho = rho + (S.Aq[q] * S.q[q]) * eq_of<T>(S, sl, nq, q) * u[m.iM + q];
    sig = sig + (S.Aq[q] * S.q[q]) * qe_of<T>(S, sl, nq, q) * u[m.iM + 2 * nq + q];
  }
  rho = warp_sum_t<T>(rho);
  sig = warp_sum_t<T>(sig);
  const double rc0 = cos_const(C, 0), rc1 = cos_const(C, 1), Oc = cos_const(C, 2), Ob = cos_const(C, 3);
  const double Phi = u[m.iPhi];
  const T Psi = -Phi - s.cpsi * (C.Omega_r * u[2] + Omega_nu * u[m.iN + 2] + sig * rc0);
  const T ia = 1.0 / s.a;
  const double X1 = Oc * u[m.iPhi + 1] + Ob * u[m.iPhi + 3];
  const T X2 = 4.0 * C.Omega_r * u[0] + 4.0 * Omega_nu * u[m.iN] + rho * rc1;
  const T Phip = Psi - s.k2H2 * Phi + s.dphi * (X1 * ia + X2 * (ia * ia));
  const double Pi = u[2] + u[m.iTp + 2] + u[m.iTp];
  const double vb = u[m.iPhi + 4];
  // tangents of slot sl's scalars and of their x-derivatives (slot 0)
  const double* st = S.sct + (sl * kScal) * kTD;
  const double* sd = X ? S.sct_d : nullptr;
  auto sct = [&](int f) { return st + f * kTD; };
  auto scd = [&](int f) { return X ? sd + f * kTD : nullptr; };
  // ---- rows: cotangents of the scalars (this thread's share), of Psi and
  // Phi', and the momentum-bin ones added at once
  T bkH = zero, btp = zero, biHe = zero, bcs2 = zero, bR = zero, bPsi = zero, bPhip = zero;
  for (int i = tid; i < m.N; i += nth) {
    const double r = rb[i];
    if (i < m.iM) {
      if (rsa) continue;
      if (i < m.iN) {  // photon temperature (T) and polarization (P)
        const bool P = i >= m.iTp;
        const int b0 = P ? m.iTp : 0, l = i - b0;
        if (l < lg) {
          const double lo = l > 0 ? u[b0 + l - 1] : 0.0;
          bkH = bkH + r * (cl1[l] * lo - cl2[l] * u[b0 + l + 1]);
          if (P || l >= 1) btp = btp + r * u[i];
          if (!P) {
            if (l == 0) bPhip = bPhip - r;
            if (l == 1) { bkH = bkH + r * (Psi / 3.0); bPsi = bPsi + r * (s.kH / 3.0); btp = btp + r * (vb / 3.0); }
            if (l == 2) btp = btp - r * (Pi / 10.0);
          } else {
            if (l == 0) btp = btp - r * (Pi / 2.0);
            if (l == 2) btp = btp - r * (Pi / 10.0);
          }
        } else {
          bkH = bkH + r * u[b0 + lg - 1];
          biHe = biHe - r * (lg + 1.0) * u[i];
          btp = btp + r * u[i];
        }
      } else {  // massless neutrinos
        const int l = i - m.iN, b0 = m.iN;
        if (l < lnu) {
          const double lo = l > 0 ? u[b0 + l - 1] : 0.0;
          bkH = bkH + r * (cl1[l] * lo - cl2[l] * u[b0 + l + 1]);
          if (l == 0) bPhip = bPhip - r;
          if (l == 1) { bkH = bkH + r * (Psi / 3.0); bPsi = bPsi + r * (s.kH / 3.0); }
        } else {
          bkH = bkH + r * u[b0 + lnu - 1];
          biHe = biHe - r * (lnu + 1.0) * u[i];
        }
      }
    } else if (i < m.iPhi) {  // massive neutrinos
      const int jm = i - m.iM;
      const int l = jm / nq, q = jm - l * nq;
      const int iq = sl * nq + q;
      const T qe = qe_of<T>(S, sl, nq, q), eq = eq_of<T>(S, sl, nq, q);
      const double* qet = S.qet + iq * kTD;
      const double* qetd = X ? S.qet_d + q * kTD : nullptr;
      const double* eqt = S.eqt + iq * kTD;
      const double* eqtd = X ? S.eqt_d + q * kTD : nullptr;
      const double df0 = S.df0[q];
      if (l < lmnu) {
        const double lo = l > 0 ? u[i - nq] : 0.0;
        const double B = cl1[l] * lo - cl2[l] * u[i + nq];
        bkH = bkH + r * qe * B;
        addc<T>(tb, r * s.kH * B, qet, qetd);
        if (l == 0) {
          bPhip = bPhip + r * df0;
          addc<T>(tb, r * Phip, S.ddf0 + q * kTD, nullptr);
        }
        if (l == 1) {
          const double c = r * (1.0 / 3.0);
          bkH = bkH - c * eq * Psi * df0;
          addc<T>(tb, -c * s.kH * Psi * df0, eqt, eqtd);
          bPsi = bPsi - c * s.kH * eq * df0;
          addc<T>(tb, -c * s.kH * eq * Psi, S.ddf0 + q * kTD, nullptr);
        }
      } else {
        const double lo = u[i - nq];
        addc<T>(tb, r * s.kH * lo, qet, qetd);
        bkH = bkH + r * qe * lo;
        biHe = biHe - r * (lmnu + 1.0) * u[i];
      }
    } else {  // metric and matter
      const int rr = i - m.iPhi;
      if (rr == 0) bPhip = bPhip + r;
      else if (rr == 1) { bkH = bkH + r * u[m.iPhi + 2]; bPhip = bPhip - 3.0 * r; }
      else if (rr == 2) { bkH = bkH - r * Psi; bPsi = bPsi - r * s.kH; }
      else if (rr == 3) { bkH = bkH + r * vb; bPhip = bPhip - 3.0 * r; }
      else {
        const double d = u[m.iPhi + 3];
        bkH = bkH - r * (Psi + s.cs2 * d);
        bPsi = bPsi - r * s.kH;
        bcs2 = bcs2 - r * s.kH * d;
        btp = btp + r * s.R * (3.0 * u[1] + vb);
        bR = bR + r * s.tp * (3.0 * u[1] + vb);
      }
    }
  }
  // the scalars' cotangents (this thread's share) times their tangents
  addc<T>(tb, bkH, sct(5), scd(5));
  addc<T>(tb, btp, sct(2), scd(2));
  addc<T>(tb, biHe, sct(6), scd(6));
  addc<T>(tb, bcs2, sct(3), scd(3));
  addc<T>(tb, bR, sct(7), scd(7));
  // ---- the metric, backwards: Phi' = Psi - k2H2 Phi + dphi (X1 ia + X2 ia^2),
  // Psi = -Phi - cpsi (Omega_r Theta_2 + Omega_nu N_2 + sigma rc0)
  bPhip = warp_sum_t<T>(bPhip);
  bPsi = warp_sum_t<T>(bPsi) + bPhip;
  const T brho = bPhip * s.dphi * (ia * ia) * rc1;
  const T bsig = -bPsi * s.cpsi * rc0;
  if (lane == 0) {
    addc<T>(tb, -bPhip * Phi, sct(10), scd(10));                                    // k2H2
    addc<T>(tb, bPhip * (X1 * ia + X2 * (ia * ia)), sct(9), scd(9));                // dphi
    addc<T>(tb, -(bPhip * s.dphi * (X1 + 2.0 * X2 * ia)) * (ia * ia), sct(4), scd(4));  // a, through 1/a
    addc<T>(tb, -bPsi * (C.Omega_r * u[2] + Omega_nu * u[m.iN + 2] + sig * rc0), sct(8), scd(8));  // cpsi
    addc<T>(tb, -bPsi * s.cpsi * sig, S.cstn + 0 * kTD, nullptr);                  // 0.25 / rho_crit
    addc<T>(tb, bPhip * s.dphi * (ia * ia) * rho, S.cstn + 1 * kTD, nullptr);       // 1 / rho_crit
    addc<T>(tb, bPhip * s.dphi * ia * u[m.iPhi + 1], S.cstn + 2 * kTD, nullptr);    // Omega_c
    addc<T>(tb, bPhip * s.dphi * ia * u[m.iPhi + 3], S.cstn + 3 * kTD, nullptr);    // Omega_b
  }
  for (int q = lane; q < nq; q += 32) {  // rho = sum Aq q eq M_0q, sigma = sum Aq q qe M_2q
    const double m0 = u[m.iM + q], m2 = u[m.iM + 2 * nq + q];
    const double Aq = S.Aq[q], qq = S.q[q];
    const T qe = qe_of<T>(S, sl, nq, q), eq = eq_of<T>(S, sl, nq, q);
    addc<T>(tb, brho * qq * eq * m0 + bsig * qq * qe * m2, S.dAq + q * kTD, nullptr);
    addc<T>(tb, brho * Aq * eq * m0 + bsig * Aq * qe * m2, S.dq + q * kTD, nullptr);
    addc<T>(tb, brho * Aq * qq * m0, S.eqt + (sl * nq + q) * kTD, X ? S.eqt_d + q * kTD : nullptr);
    addc<T>(tb, bsig * Aq * qq * m2, S.qet + (sl * nq + q) * kTD, X ? S.qet_d + q * kTD : nullptr);
  }
}

// Stages of one replayed step from (x, G.y) with size hs to xn: the
// arithmetic of solve_one's step (no error control, no outputs).  Leaves
// K_1..K_5 in G.K[0..4], K_6 in S.b and G.K[5], Y_6 in S.yt, the
// factorisation and the stage scalars (slots 0..4) in shared memory.
// Returns ST_OK, ST_LU_FAIL or ST_TANGENT_RSA.  All threads.
template <int WPM>
__device__ int replay_stages(const Mode& m, const Shared& S, const Pack& PK, const Scratch& G, double x, double hs,
                             double xn, int tid, int nth) {
  const int N = m.N;
  prepare_stages(m, S, x, hs, xn, tid, nth);
  const bool fok = factorize_scan(m, S, PK, hs * rodas::kGamma, tid, nth);
  copy_vec(N, G.y, S.yt, tid, nth);
  __syncthreads();
  if (!fok) return ST_LU_FAIL;
  bool rsa = rhs_rows<dd>(m, S, 0, StP{S.yt}, sink(S.b, G.fx), tid, nth);
  __syncthreads();
  const double ih = 1.0 / hs;
  for (int i = tid; i < N; i += nth) S.b[i] += hs * rodas::kD[0] * G.fx[i];
  __syncthreads();
  wsolve_scan(m, S, PK, S.b, tid, nth);
  copy_vec(N, S.b, G.K, tid, nth);
  for (int st = 1; st < 6; ++st) {
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
    const int sl = st < 4 ? st : 4;
    rsa |= rhs_rows<double>(m, S, sl, StP{S.yt}, sink(S.b), tid, nth);
    const double hd = hs * rodas::kD[st];
    for (int i = tid; i < N; i += nth) {
      double acc = S.b[i];
      if (st < 4) acc += hd * G.fx[i];
      double cs = 0.0;
      for (int j = 0; j < st; ++j) cs += rodas::kC[st][j] * G.K[j * N + i];
      S.b[i] = acc + ih * cs;
    }
    __syncthreads();
    wsolve_scan(m, S, PK, S.b, tid, nth);
    copy_vec(N, S.b, G.K + st * N, tid, nth);
  }
  __syncthreads();
  return rsa ? ST_TANGENT_RSA : ST_OK;
}

// One step of the reverse sweep (the adjoint of replay_stages' step, see the
// top of this file).  On entry: G.y = y, G.K[0..5] = K_1..K_6, the step's
// factorisation, stage scalars and their tangents (slots 0..4); A.lam = the
// cotangent of y_new.  On exit A.lam = the cotangent of y; tb[j] gains the
// step's share of the parameter cotangent.  All threads.
template <int WPM>
__device__ void adjoint_step(const Mode& m, const Shared& S, const Pack& PK, const Scratch& G, const AdjScratch& A,
                             double hs, double* tb, int tid, int nth) {
  const int N = m.N;
  const double ih = 1.0 / hs;
  for (int i = tid; i < N; i += nth) {
    for (int j = 0; j < 5; ++j) A.Kb[j * N + i] = 0.0;
    A.Kb[5 * N + i] = A.lam[i];  // y_new = Y_6 + K_6
    A.Yb[i] = A.lam[i];
    A.yb[i] = 0.0;
    A.Fb[i] = 0.0;
  }
  __syncthreads();
  for (int st = 5; st >= 0; --st) {
    copy_vec(N, A.Kb + st * N, S.b, tid, nth);
    __syncthreads();
    wsolve_scan_T(m, S, PK, S.b, tid, nth);  // rbar_st in S.b
    const int sl = st == 0 ? 0 : (st < 4 ? st : 4);
    rhs_cols<double>(m, S, sl, S.b, sink(A.tmp), tid, nth);  // A_sl^T rbar
    // this stage's state Y_st (into S.yt): y, y + sum a K, or Y_5 + K_5
    if (st == 0) {
      copy_vec(N, G.y, S.yt, tid, nth);
    } else if (st < 5) {
      for (int i = tid; i < N; i += nth) {
        double acc = G.y[i];
        for (int j = 0; j < st; ++j) acc += rodas::kA[st - 1][j] * G.K[j * N + i];
        S.yt[i] = acc;
      }
    } else {
      for (int i = tid; i < N; i += nth) {
        double acc = G.y[i];
        for (int j = 0; j < 4; ++j) acc += rodas::kA[3][j] * G.K[j * N + i];
        S.yt[i] = acc + G.K[4 * N + i];
      }
    }
    __syncthreads();
    coef_dot<double>(m, S, sl, S.yt, S.b, tb, tid, nth);         // rbar . dA_sl Y_st
    coef_dot<double>(m, S, 0, G.K + st * N, S.b, tb, tid, nth);  // rbar . dA_0 K_st (M depends on A_0)
    const double hd = hs * rodas::kD[st];
    for (int i = tid; i < N; i += nth) {
      const double rb = S.b[i];
      if (st < 4) A.Fb[i] = fma(hd, rb, A.Fb[i]);
      for (int j = 0; j < st; ++j) A.Kb[j * N + i] = fma(ih * rodas::kC[st][j], rb, A.Kb[j * N + i]);
      if (st == 5) {  // Ybar_6 = lam + A_4^T rbar_6; Y_6 = Y_5 + K_5
        const double y6 = A.Yb[i] + A.tmp[i];
        A.Kb[4 * N + i] += y6;
        A.Yb[i] = y6;  // carried into Ybar_5
      } else if (st >= 1) {
        const double ys = (st == 4 ? A.Yb[i] : 0.0) + A.tmp[i];
        A.yb[i] += ys;
        for (int j = 0; j < st; ++j) A.Kb[j * N + i] = fma(rodas::kA[st - 1][j], ys, A.Kb[j * N + i]);
      } else {
        A.yb[i] += A.tmp[i];
      }
    }
    __syncthreads();
  }
  // the d/dx term of stage 1..4: Fbar . A'_0 y
  {
    Sink o;
    o.v = A.tmp; o.d = A.gu; o.t = nullptr; o.td = nullptr; o.N = N;
    rhs_cols<dd>(m, S, 0, A.Fb, o, tid, nth);  // A.gu = A'_0^T Fbar
    coef_dot<dd>(m, S, 0, G.y, A.Fb, tb, tid, nth);  // Fbar . dA'_0 y
    for (int i = tid; i < N; i += nth) A.lam[i] = A.yb[i] + A.gu[i];
  }
  __syncthreads();
}

// Cotangent of the outputs at node x (slot sl holds x's stage scalars and
// their tangents; A.u1 the state there): S_T with cotangent sbT (if
// sources) and P_lin with cotangent pb (if plin).  lam += the state
// gradient; tb[j] += the partials at fixed state.  All threads.
template <int WPM>
__device__ void adjoint_seed(const Mode& m, const Shared& S, const AdjScratch& A, int sl, double x, bool src,
                             double sbT, bool plin, double pb, double* tb, int tid, int nth) {
  const int N = m.N, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < N; i += nth) { A.gu[i] = 0.0; A.gdu[i] = 0.0; }
  __syncthreads();
  if (warp == 0) {
    if (src && sbT != 0.0) source_grad(m, S, x, sbT, A.gu, A.gdu, lane);
    __syncwarp();
    if (plin && pb != 0.0) plin_grad(m, S, x, A.u1, pb, A.gu, lane);
  }
  __syncthreads();
  if (src && sbT != 0.0) {
    rhs_cols<double>(m, S, sl, A.gdu, sink(A.tmp), tid, nth);  // A^T d S / d(du)
    for (int i = tid; i < N; i += nth) A.gu[i] += A.tmp[i];
    // partials at fixed state, S_T(u, du) with du = A u: those of the
    // source's own coefficients, and (sbT dS/d(du)) . dA u from the
    // hierarchy's coefficient cotangents
    coef_dot<double>(m, S, sl, A.u1, A.gdu, tb, tid, nth);
    rhs_rows<double>(m, S, sl, StP{A.u1}, sink(A.du), tid, nth);
    __syncthreads();
    if (warp == 0) {
      d4 oT = c4(0.0), oE = c4(0.0);
      emit_sources_t<d4>(m, S, x, StM{A.u1, nullptr, N}, StM{A.du, nullptr, N}, lane, oT, oE, false);
      if (lane == 0)
        for (int j = 0; j < kTD; ++j) tb[j] += sbT * oT.t[j];
    }
  }
  if (plin && pb != 0.0 && warp == 0) {
    d4 dP = c4(0.0);
    emit_plin_t<d4>(m, S, x, StC{A.u1}, lane, dP);
    if (lane == 0)
      for (int j = 0; j < kTD; ++j) tb[j] += pb * dP.t[j];
  }
  __syncthreads();
  for (int i = tid; i < N; i += nth) A.lam[i] += A.gu[i];
  __syncthreads();
}
