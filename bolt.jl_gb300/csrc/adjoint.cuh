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
  const int* idx = P.idx + tid * P.em;
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
  const double fc_in = (c >= 0 && lane > seg) ? S.fc[P.idx[(tid - 1) * P.em + E - 1]] : 0.0;
  const double fl_out = (c >= 0 && lane < segend) ? S.fl[P.idx[(tid + 1) * P.em]] : 0.0;
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
// as dA_dot.  Every thread adds its own rows' share (the metric's share on
// lane 0 and the momentum bins' on their lanes).  One warp.
__device__ void coef_dot(const Mode& m, const Shared& S, int sl, const double* u, const double* rb, double* tb,
                         int tid, int nth) {
  const int lane = tid & 31;
  const int nq = m.nq, lg = m.lg, lnu = m.lnu, lmnu = m.lmnu;
  const Scal<double> s = get_scal<double>(S, sl);
  const bool rsa = rsa_switch(m, s);
  const double* cl1 = S.cl1;
  const double* cl2 = S.cl2;
  const CosmoDev& C = *m.C;
  const double Omega_nu = C.Omega_nu;
  const double* qe = S.qe + sl * nq;
  const double* eq = S.eq + sl * nq;
  // the metric's values, as metric() forms them
  double rho = 0.0, sig = 0.0;
  for (int q = lane; q < nq; q += 32) {
    rho = rho + (S.Aq[q] * S.q[q]) * eq[q] * u[m.iM + q];
    sig = sig + (S.Aq[q] * S.q[q]) * qe[q] * u[m.iM + 2 * nq + q];
  }
  rho = warp_sum(rho);
  sig = warp_sum(sig);
  const double rc0 = cos_const(C, 0), rc1 = cos_const(C, 1), Oc = cos_const(C, 2), Ob = cos_const(C, 3);
  const double Phi = u[m.iPhi];
  const double Psi = -Phi - s.cpsi * (C.Omega_r * u[2] + Omega_nu * u[m.iN + 2] + sig * rc0);
  const double ia = 1.0 / s.a;
  const double X1 = Oc * u[m.iPhi + 1] + Ob * u[m.iPhi + 3];
  const double X2 = 4.0 * C.Omega_r * u[0] + 4.0 * Omega_nu * u[m.iN] + rho * rc1;
  const double Phip = Psi - s.k2H2 * Phi + s.dphi * (X1 * ia + X2 * (ia * ia));
  const double Pi = u[2] + u[m.iTp + 2] + u[m.iTp];
  const double vb = u[m.iPhi + 4];
  // ---- rows: cotangents of the scalars (this thread's share), of Psi and
  // Phi', and the momentum-bin ones added at once
  double bkH = 0.0, btp = 0.0, biHe = 0.0, bcs2 = 0.0, bR = 0.0, bPsi = 0.0, bPhip = 0.0;
  auto add_q = [&](const double* t, int idx, double bar) {  // tb[j] += bar * t[idx * kTD + j]
#pragma unroll
    for (int j = 0; j < kTD; ++j) tb[j] = fma(bar, t[idx * kTD + j], tb[j]);
  };
  for (int i = tid; i < m.N; i += nth) {
    const double r = rb[i];
    if (i < m.iM) {
      if (rsa) continue;
      if (i < m.iN) {  // photon temperature (T) and polarization (P)
        const bool P = i >= m.iTp;
        const int b0 = P ? m.iTp : 0, l = i - b0;
        if (l < lg) {
          const double lo = l > 0 ? u[b0 + l - 1] : 0.0;
          bkH += r * (cl1[l] * lo - cl2[l] * u[b0 + l + 1]);
          if (P || l >= 1) btp += r * u[i];
          if (!P) {
            if (l == 0) bPhip -= r;
            if (l == 1) { bkH += r * (Psi / 3.0); bPsi += r * (s.kH / 3.0); btp += r * (vb / 3.0); }
            if (l == 2) btp -= r * (Pi / 10.0);
          } else {
            if (l == 0) btp -= r * (Pi / 2.0);
            if (l == 2) btp -= r * (Pi / 10.0);
          }
        } else {
          bkH += r * u[b0 + lg - 1];
          biHe -= r * (lg + 1.0) * u[i];
          btp += r * u[i];
        }
      } else {  // massless neutrinos
        const int l = i - m.iN, b0 = m.iN;
        if (l < lnu) {
          const double lo = l > 0 ? u[b0 + l - 1] : 0.0;
          bkH += r * (cl1[l] * lo - cl2[l] * u[b0 + l + 1]);
          if (l == 0) bPhip -= r;
          if (l == 1) { bkH += r * (Psi / 3.0); bPsi += r * (s.kH / 3.0); }
        } else {
          bkH += r * u[b0 + lnu - 1];
          biHe -= r * (lnu + 1.0) * u[i];
        }
      }
    } else if (i < m.iPhi) {  // massive neutrinos
      const int jm = i - m.iM;
      const int l = jm / nq, q = jm - l * nq;
      const int iq = sl * nq + q;
      if (l < lmnu) {
        const double lo = l > 0 ? u[i - nq] : 0.0;
        const double B = cl1[l] * lo - cl2[l] * u[i + nq];
        bkH += r * qe[q] * B;
        add_q(S.qet, iq, r * s.kH * B);
        if (l == 0) {
          bPhip += r * S.df0[q];
          add_q(S.ddf0, q, r * Phip);
        }
        if (l == 1) {
          const double c = r * (1.0 / 3.0);
          bkH -= c * eq[q] * Psi * S.df0[q];
          add_q(S.eqt, iq, -c * s.kH * Psi * S.df0[q]);
          bPsi -= c * s.kH * eq[q] * S.df0[q];
          add_q(S.ddf0, q, -c * s.kH * eq[q] * Psi);
        }
      } else {
        const double lo = u[i - nq];
        add_q(S.qet, iq, r * s.kH * lo);
        bkH += r * qe[q] * lo;
        biHe -= r * (lmnu + 1.0) * u[i];
      }
    } else {  // metric and matter
      const int rr = i - m.iPhi;
      if (rr == 0) bPhip += r;
      else if (rr == 1) { bkH += r * u[m.iPhi + 2]; bPhip -= 3.0 * r; }
      else if (rr == 2) { bkH -= r * Psi; bPsi -= r * s.kH; }
      else if (rr == 3) { bkH += r * vb; bPhip -= 3.0 * r; }
      else {
        const double d = u[m.iPhi + 3];
        bkH -= r * (Psi + s.cs2 * d);
        bPsi -= r * s.kH;
        bcs2 -= r * s.kH * d;
        btp += r * s.R * (3.0 * u[1] + vb);
        bR += r * s.tp * (3.0 * u[1] + vb);
      }
    }
  }
  // the scalars' cotangents (this thread's share) times their tangents
  {
    const double* st = S.sct + (sl * kScal) * kTD;
#pragma unroll
    for (int j = 0; j < kTD; ++j) {
      double acc = tb[j];
      acc = fma(bkH, st[5 * kTD + j], acc);
      acc = fma(btp, st[2 * kTD + j], acc);
      acc = fma(biHe, st[6 * kTD + j], acc);
      acc = fma(bcs2, st[3 * kTD + j], acc);
      acc = fma(bR, st[7 * kTD + j], acc);
      tb[j] = acc;
    }
  }
  // ---- the metric, backwards: Phi' = Psi - k2H2 Phi + dphi (X1 ia + X2 ia^2),
  // Psi = -Phi - cpsi (Omega_r Theta_2 + Omega_nu N_2 + sigma rc0)
  bPhip = warp_sum(bPhip);
  bPsi = warp_sum(bPsi) + bPhip;
  const double brho = bPhip * s.dphi * (ia * ia) * rc1;
  const double bsig = -bPsi * s.cpsi * rc0;
  if (lane == 0) {
    const double* st = S.sct + (sl * kScal) * kTD;
    const double bk2H2 = -bPhip * Phi;
    const double bdphi = bPhip * (X1 * ia + X2 * (ia * ia));
    const double bia = bPhip * s.dphi * (X1 + 2.0 * X2 * ia);
    const double ba = -bia * (ia * ia);
    const double bcpsi = -bPsi * (C.Omega_r * u[2] + Omega_nu * u[m.iN + 2] + sig * rc0);
    const double bOc = bPhip * s.dphi * ia * u[m.iPhi + 1], bOb = bPhip * s.dphi * ia * u[m.iPhi + 3];
    const double brc1 = bPhip * s.dphi * (ia * ia) * rho, brc0 = -bPsi * s.cpsi * sig;
#pragma unroll
    for (int j = 0; j < kTD; ++j) {
      double acc = tb[j];
      acc = fma(bk2H2, st[10 * kTD + j], acc);
      acc = fma(bdphi, st[9 * kTD + j], acc);
      acc = fma(ba, st[4 * kTD + j], acc);
      acc = fma(bcpsi, st[8 * kTD + j], acc);
      acc = fma(brc0, S.cstn[0 * kTD + j], acc);
      acc = fma(brc1, S.cstn[1 * kTD + j], acc);
      acc = fma(bOc, S.cstn[2 * kTD + j], acc);
      acc = fma(bOb, S.cstn[3 * kTD + j], acc);
      tb[j] = acc;
    }
  }
  for (int q = lane; q < nq; q += 32) {  // rho = sum Aq q eq M_0q, sigma = sum Aq q qe M_2q
    const double m0 = u[m.iM + q], m2 = u[m.iM + 2 * nq + q];
    const double Aq = S.Aq[q], qq = S.q[q];
    add_q(S.dAq, q, brho * qq * eq[q] * m0 + bsig * qq * qe[q] * m2);
    add_q(S.dq, q, brho * Aq * eq[q] * m0 + bsig * Aq * qe[q] * m2);
    add_q(S.eqt, sl * nq + q, brho * Aq * qq * m0);
    add_q(S.qet, sl * nq + q, bsig * Aq * qq * m2);
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
    coef_dot(m, S, sl, S.yt, S.b, tb, tid, nth);         // rbar . dA_sl Y_st
    coef_dot(m, S, 0, G.K + st * N, S.b, tb, tid, nth);  // rbar . dA_0 K_st (M depends on A_0)
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
    Sink x;
    x.v = A.tmp; x.d = nullptr; x.t = A.t4; x.td = A.t4b; x.N = N;
    rhs_rows<x4>(m, S, 0, StC{G.y}, x, tid, nth);  // t4b = dA'_0 y
    for (int i = tid; i < N; i += nth) {
      A.lam[i] = A.yb[i] + A.gu[i];
#pragma unroll
      for (int j = 0; j < kTD; ++j) tb[j] = fma(A.Fb[i], A.t4b[j * N + i], tb[j]);
    }
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
    coef_dot(m, S, sl, A.u1, A.gdu, tb, tid, nth);
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
