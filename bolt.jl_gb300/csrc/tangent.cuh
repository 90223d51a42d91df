// Tangent-linear Rosenbrock steps (mode flag MODE_TANGENT).
//
// A tangent mode integrates the state y and, along with it, its derivatives
// dy_j with respect to kTD parameters (h, omega_b, omega_c, Sigma m_nu), the
// derivative of the discrete Rodas4 solution at fixed steps -- the
// derivative the reference's ForwardDiff gradient takes through one
// discretisation.  For a linear ODE u' = A(x) u the stages
//   M K_i = A_i Y_i + h d_i A'_0 y + (1/h) sum_j C_ij K_j,  M = I/(h gamma) - A_0
// differentiate to
//   M dK_i = A_i dY_i + dA_i Y_i + dA_0 K_i + h d_i (A'_0 dy + dA'_0 y)
//            + (1/h) sum_j C_ij dK_j,
// so every step solves kTD more right-hand sides with the step's own
// factorisation: no new factorisation, no second solve of the state.  The
// right-hand-side tangents come from one evaluation of hierarchy! in tangent
// numbers (d4: a value and its kTD derivatives; x4 adds d/dx for A'_0),
// whose coefficient tangents dA are the differences of the coefficients of
// the kTD perturbed parameter sets (frozen-step tables, see the engine)
// over their steps.  The tangents are propagated only through accepted
// steps, after the step is accepted.
//
// Included inside namespace bolt by solver.cu, after chains.cuh.
#pragma once

// In-place solve of the kTD right-hand sides b[j * N + i] with the step's
// factorisation: wsolve_scan's recurrences, interleaved over the directions
// (each lane carries kTD independent chains of dependent operations).
__device__ void wsolve_scan4(const Mode& m, const Shared& S, const Pack& P, double* b, int tid, int nth) {
  const int N = m.N;
  const int lane = tid & 31;
  const int E = P.E[0];
  const int c = P.chain[tid];
  const int seg = P.seg[tid];
  const int own_c = (tid == P.E[1]) ? 3 + m.nq : ((c >= 0 && P.owner[c] == tid) ? c : -1);
  const int own_c2 = (tid == P.E[1]) ? 4 + m.nq : -1;
  const int idb = m.iPhi + 3, ivb = m.iPhi + 4;
  // ---- forward: b'_j = b_j - fl_j b'_{j-1}
  const LaneIdx idx = lane_idx(P, tid);
  double A = 1.0, B[kTD];
#pragma unroll
  for (int d = 0; d < kTD; ++d) B[d] = 0.0;
  int cnt = 0;
  if (c >= 0) {
    for (int e = 0; e < E; ++e) {
      const int i = idx[e];
      if (i < 0) break;
      const double al = -S.fl[i];
#pragma unroll
      for (int d = 0; d < kTD; ++d) {
        double bi = b[d * N + i];
        if (c == 0 && i == 1) {  // Theta_1 <- baryon pair (eliminated first)
          double bdb = b[d * N + idb];
          double bvb = b[d * N + ivb] - S.fl[ivb] * bdb;
          bi -= S.fl[idb] * bvb;
          b[d * N + ivb] = bvb;
          b[d * N + i] = bi;
        }
        B[d] = fma(al, B[d], bi);
      }
      A = al * A;
      cnt = e + 1;
    }
  }
  for (int off = 1; off < P.E[2]; off <<= 1) {
    double oA = __shfl_up_sync(0xffffffffu, A, off), oB[kTD];
#pragma unroll
    for (int d = 0; d < kTD; ++d) oB[d] = __shfl_up_sync(0xffffffffu, B[d], off);
    if (seg >= 0 && lane - off >= seg) {
#pragma unroll
      for (int d = 0; d < kTD; ++d) B[d] = fma(A, oB[d], B[d]);
      A = A * oA;
    }
  }
  double prev[kTD];
#pragma unroll
  for (int d = 0; d < kTD; ++d) {
    prev[d] = __shfl_up_sync(0xffffffffu, B[d], 1);
    if (!(seg >= 0 && lane > seg)) prev[d] = 0.0;
  }
  for (int e = 0; e < cnt; ++e) {
    const int i = idx[e];
    const double fl = S.fl[i];
#pragma unroll
    for (int d = 0; d < kTD; ++d) {
      double v = fma(-fl, prev[d], b[d * N + i]);
      b[d * N + i] = v;
      prev[d] = v;
    }
  }
  if (tid == P.E[1])
#pragma unroll
    for (int d = 0; d < kTD; ++d) b[d * N + m.iPhi + 1] -= S.fl[m.iPhi + 1] * b[d * N + m.iPhi + 2];
  __syncthreads();
  // ---- border: t = W^T y at the tails, s = C^{-1} t, tail correction
  double* part = S.part4;  // [chain][3][kTD]
  for (int k2 = 0; k2 < 2; ++k2) {
    const int cc = k2 == 0 ? own_c : own_c2;
    if (cc < 0) continue;
    double xt[kTail][kTD];
#pragma unroll
    for (int a = 0; a < kTail; ++a)
#pragma unroll
      for (int d = 0; d < kTD; ++d) xt[a][d] = 0.0;
#pragma unroll
    for (int d = 0; d < kTD; ++d) {
      const double* bd = b + d * N;
      if (cc < 3 + m.nq) {
        int i0 = tail_index(m, cc, 0), i1 = tail_index(m, cc, 1), i2 = tail_index(m, cc, 2);
        xt[0][d] = bd[i0] * S.fi[i0];
        xt[1][d] = bd[i1] * S.fi[i1] - S.fc[i1] * xt[0][d];
        xt[2][d] = bd[i2] * S.fi[i2] - S.fc[i2] * xt[1][d];
        if (cc == 0) {
          xt[3][d] = bd[ivb] * S.fi[ivb] - S.fc[ivb] * xt[1][d];
          xt[4][d] = bd[idb] * S.fi[idb] - S.fc[idb] * xt[3][d];
        }
      } else if (cc == 3 + m.nq) {
        xt[0][d] = bd[m.iPhi + 1] * S.fi[m.iPhi + 1];
        xt[1][d] = bd[m.iPhi + 2] * S.fi[m.iPhi + 2];
      } else {
        xt[0][d] = bd[m.iPhi] * S.fi[m.iPhi];
      }
    }
    const double* wt = S.Wt + cc * kTail * kBorder;
    for (int r = 0; r < kBorder; ++r)
#pragma unroll
      for (int d = 0; d < kTD; ++d) {
        double acc = 0.0;
        for (int a = 0; a < kTail; ++a) acc += wt[a * kBorder + r] * xt[a][d];
        part[(cc * kBorder + r) * kTD + d] = acc;
      }
  }
  __syncthreads();
  double sv[kBorder][kTD];
  {
    double t[kBorder][kTD];
    for (int r = 0; r < kBorder; ++r)
#pragma unroll
      for (int d = 0; d < kTD; ++d)
        t[r][d] = warp_sum(lane < m.nch ? part[(lane * kBorder + r) * kTD + d] : 0.0);
    for (int r = 0; r < kBorder; ++r)
#pragma unroll
      for (int d = 0; d < kTD; ++d)
        sv[r][d] = S.misc[r * 3 + 0] * t[0][d] + S.misc[r * 3 + 1] * t[1][d] + S.misc[r * 3 + 2] * t[2][d];
  }
  for (int k2 = 0; k2 < 2; ++k2) {
    const int cc = k2 == 0 ? own_c : own_c2;
    if (cc < 0) continue;
    const double* uf = S.Uf + cc * kTail * kBorder;
    int ns = tail_slots(m, cc);
    for (int a = 0; a < ns; ++a) {
      int i = tail_index(m, cc, a);
#pragma unroll
      for (int d = 0; d < kTD; ++d)
        b[d * N + i] += uf[a * kBorder + 0] * sv[0][d] + uf[a * kBorder + 1] * sv[1][d] + uf[a * kBorder + 2] * sv[2][d];
    }
  }
  __syncthreads();
  // ---- backward: x_j = fi_j b'_j - fc_j x_{j+1} (reverse scan)
  A = 1.0;
#pragma unroll
  for (int d = 0; d < kTD; ++d) B[d] = 0.0;
  for (int e = cnt - 1; e >= 0; --e) {
    const int i = idx[e];
    const double fi = S.fi[i], de = -S.fc[i];
#pragma unroll
    for (int d = 0; d < kTD; ++d) B[d] = fma(de, B[d], b[d * N + i] * fi);
    A = de * A;
  }
  int segend = 31;
  {
    int l2 = lane;
    while (l2 < 31 && P.chain[(tid - lane) + l2 + 1] == c && P.seg[(tid - lane) + l2 + 1] == seg) ++l2;
    segend = l2;
  }
  for (int off = 1; off < P.E[2]; off <<= 1) {
    double oA = __shfl_down_sync(0xffffffffu, A, off), oB[kTD];
#pragma unroll
    for (int d = 0; d < kTD; ++d) oB[d] = __shfl_down_sync(0xffffffffu, B[d], off);
    if (seg >= 0 && lane + off <= segend) {
#pragma unroll
      for (int d = 0; d < kTD; ++d) B[d] = fma(A, oB[d], B[d]);
      A = A * oA;
    }
  }
  double nxt[kTD];
#pragma unroll
  for (int d = 0; d < kTD; ++d) {
    nxt[d] = __shfl_down_sync(0xffffffffu, B[d], 1);
    if (!(seg >= 0 && lane < segend)) nxt[d] = 0.0;
  }
  for (int e = cnt - 1; e >= 0; --e) {
    const int i = idx[e];
    const double fi = S.fi[i], fc = S.fc[i];
#pragma unroll
    for (int d = 0; d < kTD; ++d) {
      double v = fma(-fc, nxt[d], b[d * N + i] * fi);
      b[d * N + i] = v;
      nxt[d] = v;
      if (c == 0 && i == 1) {  // baryon pair after Theta_1
        double xvb = b[d * N + ivb] * S.fi[ivb] - S.fc[ivb] * v;
        b[d * N + ivb] = xvb;
        b[d * N + idb] = b[d * N + idb] * S.fi[idb] - S.fc[idb] * xvb;
      }
    }
  }
  if (tid == P.E[1])
#pragma unroll
    for (int d = 0; d < kTD; ++d) {
      b[d * N + m.iPhi + 1] = b[d * N + m.iPhi + 1] * S.fi[m.iPhi + 1];
      b[d * N + m.iPhi + 2] = b[d * N + m.iPhi + 2] * S.fi[m.iPhi + 2];
      b[d * N + m.iPhi] = b[d * N + m.iPhi] * S.fi[m.iPhi];
    }
  __syncthreads();
}

// Per-mode set-up of a tangent mode: the perturbed sets' momentum-bin
// constants (qpj) and the tangents of the q constants and of the metric's
// cosmology constants.  All threads; ends with a barrier.
__device__ void tan_setup(const Mode& m, const Shared& S, int tid, int nth) {
  const int nq = m.nq;
  for (int t = tid; t < nq * kTD; t += nth) {
    const int q = t / kTD, j = t - q * kTD;
    double qq, df0, Aq, Bq;
    qconst(*m.tc[j], q, qq, df0, Aq, Bq);
    const double inv = m.tinv[j];
    S.qpj[j * nq + q] = qq;
    S.dq[q * kTD + j] = (qq - S.q[q]) * inv;
    S.ddf0[q * kTD + j] = (df0 - S.df0[q]) * inv;
    S.dAq[q * kTD + j] = (Aq - S.Aq[q]) * inv;
    S.dBq[q * kTD + j] = (Bq - S.Bq[q]) * inv;
  }
  for (int t = tid; t < kCosN * kTD; t += nth) {
    const int id = t / kTD, j = t - id * kTD;
    S.cstn[id * kTD + j] = (cos_const(*m.tc[j], id) - cos_const(*m.C, id)) * m.tinv[j];
  }
  __syncthreads();
}

// Tangents of the stage scalars and of q/eps, eps/q at slots s0..s1-1 with
// abscissae xs[slot]; slot 0 also those of their x-derivatives.  Needs the
// base values in S.sc / S.qe / S.eq of the same slots.  All threads; ends
// with a barrier.
__device__ void tan_prepare(const Mode& m, const Shared& S, const double* xs, int s0, int s1, int tid, int nth) {
  for (int t = tid; t < (s1 - s0) * kTD; t += nth) {
    const int sl = s0 + t / kTD, j = t % kTD;
    double v[kScal], vd[kScal];
    stage_scalars_vals(*m.tc[j], m.k, xs[sl], v, sl == 0 ? vd : nullptr);
    const double inv = m.tinv[j];
    for (int f = 0; f < 11; ++f) S.sct[(sl * kScal + f) * kTD + j] = (v[f] - S.sc[sl * kScal + f]) * inv;
    if (sl == 0)
      for (int f = 0; f < 11; ++f) S.sct_d[f * kTD + j] = (vd[f] - S.sc_d[f]) * inv;
  }
  const int nq = m.nq;
  for (int t = tid; t < (s1 - s0) * nq * kTD; t += nth) {
    const int sl = s0 + t / (nq * kTD), r = t % (nq * kTD), q = r / kTD, j = r % kTD;
    const double a = S.sc[sl * kScal + 4];
    const double am = a * m.tc[j]->Sigma_m_nu, qq = S.qpj[j * nq + q];
    const double eps = sqrt(qq * qq + am * am);
    const double inv = m.tinv[j];
    S.qet[(sl * nq + q) * kTD + j] = (qq / eps - S.qe[sl * nq + q]) * inv;
    S.eqt[(sl * nq + q) * kTD + j] = (eps / qq - S.eq[sl * nq + q]) * inv;
    if (sl == 0) {
      const double deps = am * am / eps;  // d eps / dx
      S.qet_d[q * kTD + j] = (-qq * deps / (eps * eps) - S.qe_d[q]) * inv;
      S.eqt_d[q * kTD + j] = (deps / qq - S.eq_d[q]) * inv;
    }
  }
  __syncthreads();
}

// Tangent initial state dy[j] = d initial_conditions / d theta_j (y the
// base state); S.yt and qs (nq doubles) serve as scratch.  All threads.
__device__ void tan_initial(const Mode& m, const Shared& S, double xi, const double* y, double* dy, double* qs,
                            int tid, int nth) {
  const int N = m.N, nq = m.nq, lane = tid & 31, warp = tid >> 5;
  for (int j = 0; j < kTD; ++j) {
    double* df0j = qs;  // perturbed dlnf0/dlnq
    for (int q = tid; q < nq; q += nth) {
      double qq, df0, Aq, Bq;
      qconst(*m.tc[j], q, qq, df0, Aq, Bq);
      df0j[q] = df0;
    }
    __syncthreads();
    if (warp == 0) initial_state(m, *m.tc[j], S.qpj + j * nq, df0j, xi, S.yt, lane);
    __syncthreads();
    const double inv = m.tinv[j];
    for (int i = tid; i < N; i += nth) dy[j * N + i] = (S.yt[i] - y[i]) * inv;
    __syncthreads();
  }
}

// Global scratch of a tangent mode (after the base slab): dy [kTD][N], the
// stage tangents dK [6][kTD][N], d(f_x) [kTD][N] and dA_0 K [kTD][N].
struct TanScratch {
  double *dy, *dK, *fxt, *tmp;
};
__host__ __device__ inline int tan_scratch_doubles(int N) { return 9 * kTD * N; }

// Tangent outputs at node jt: sources at x from (y, dy) and (f, df).  Warp 0.
__device__ void tan_emit_sources(const Mode& m, const Shared& S, const ModeDev& md, double x, const double* y,
                                 const double* dy, const double* f, const double* df, int jt, int lane) {
  d4 oT = c4(0.0), oE = c4(0.0);
  const bool wantE = md.tsrc_E[0] != nullptr;
  emit_sources_t<d4>(m, S, x, StD4{y, dy, m.N}, StD4{f, df, m.N}, lane, oT, oE, wantE);
  if (lane == 0)
    for (int j = 0; j < kTD; ++j) {
      if (md.tsrc_T[j]) md.tsrc_T[j][jt] = oT.t[j];
      if (wantE && md.tsrc_E[j]) md.tsrc_E[j][jt] = oE.t[j];
    }
}

// One accepted Rodas4 step of the tangents (see the top of this file), then
// the state update y <- Y_6 + K_6 (the base step's own arithmetic).  On
// entry: G.y = y, G.K[0..4] = K_1..K_5, S.b = K_6, the step's factorisation
// and stage scalars (slots 0..4) in shared memory.  Emits the tangent
// outputs at x when node jt lies there.  All threads.
template <int WPM>
__device__ void tan_step(const Mode& m, const Shared& S, const Pack& PK, const Scratch& G, const TanScratch& T,
                         const ModeDev& md, double x, double hs, double xn, int& jt, int tid, int nth) {
  const int N = m.N, lane = tid & 31, warp = tid >> 5;
  const size_t TN = size_t(kTD) * N;
  for (int i = tid; i < N; i += nth) G.K[5 * N + i] = S.b[i];  // K_6
  double xs[5];
  xs[0] = x;
  for (int sl = 1; sl < 4; ++sl) xs[sl] = x + rodas::kCx[sl] * hs;
  xs[4] = xn;
  tan_prepare(m, S, xs, 0, 5, tid, nth);
  // ---- stage 1 (x): df, d(f_x) of the state; the value f for the outputs
  for (int i = tid; i < N; i += nth) S.yt[i] = G.y[i];
  for (int t = tid; t < int(TN); t += nth) S.yd[t] = T.dy[t];
  __syncthreads();
  {
    Sink o;
    o.v = S.b; o.d = nullptr; o.t = S.bd; o.td = T.fxt; o.N = N;
    rhs_rows<x4>(m, S, 0, StD4{S.yt, S.yd, N}, o, tid, nth);
  }
  __syncthreads();
  while (jt < md.nout && md.xout[jt] < x) ++jt;
  if (jt < md.nout && md.xout[jt] == x) {
    if (warp == 0) tan_emit_sources(m, S, md, x, S.yt, S.yd, S.b, S.bd, jt, lane);
    ++jt;
    __syncthreads();
  }
  const double ih = 1.0 / hs;
  for (int st = 0; st < 6; ++st) {
    if (st > 0) {
      if (st < 5) {
        for (int i = tid; i < N; i += nth) {
          double acc = G.y[i];
          for (int j = 0; j < st; ++j) acc += rodas::kA[st - 1][j] * G.K[j * N + i];
          S.yt[i] = acc;
        }
        for (int t = tid; t < int(TN); t += nth) {
          double acc = T.dy[t];
          for (int j = 0; j < st; ++j) acc += rodas::kA[st - 1][j] * T.dK[j * TN + t];
          S.yd[t] = acc;
        }
      } else {
        for (int i = tid; i < N; i += nth) S.yt[i] += G.K[4 * N + i];
        for (int t = tid; t < int(TN); t += nth) S.yd[t] += T.dK[4 * TN + t];
      }
      __syncthreads();
      Sink o;
      o.v = nullptr; o.d = nullptr; o.t = S.bd; o.td = nullptr; o.N = N;
      rhs_rows<d4>(m, S, st < 4 ? st : 4, StD4{S.yt, S.yd, N}, o, tid, nth);
    }
    {  // dA_0 K_st (K_st of the base step, at the step's start)
      Sink o;
      o.v = nullptr; o.d = nullptr; o.t = T.tmp; o.td = nullptr; o.N = N;
      rhs_rows<d4>(m, S, 0, StP{G.K + st * N}, o, tid, nth);
    }
    // each thread combines the rows it produced (same row assignment)
    const double hd = hs * rodas::kD[st];
    for (int i = tid; i < N; i += nth)
      for (int d = 0; d < kTD; ++d) {
        const size_t t = size_t(d) * N + i;
        double acc = S.bd[t] + T.tmp[t];
        if (st < 4) acc += hd * T.fxt[t];
        double cs = 0.0;
        for (int j = 0; j < st; ++j) cs += rodas::kC[st][j] * T.dK[j * TN + t];
        S.bd[t] = acc + ih * cs;
      }
    __syncthreads();
    wsolve_scan4(m, S, PK, S.bd, tid, nth);
    if (st < 5)
      for (int t = tid; t < int(TN); t += nth) T.dK[st * TN + t] = S.bd[t];
  }
  // y, dy at xn (S.yt = Y_6, S.yd = dY_6; K_6 in G.K[5], dK_6 in S.bd)
  for (int i = tid; i < N; i += nth) G.y[i] = S.yt[i] + G.K[5 * N + i];
  for (int t = tid; t < int(TN); t += nth) T.dy[t] = S.yd[t] + S.bd[t];
  __syncthreads();
}
