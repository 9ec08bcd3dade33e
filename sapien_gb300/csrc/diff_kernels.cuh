// Differentiation kernels: RNEA / ABA / FK adjoints, dense derivative matrices and the
// checkpointed semi-implicit-Euler rollout (forward and reverse). One environment per
// thread; every kernel recomputes the spatial intermediates it needs instead of reading a
// stored tape, except the rollout backward, which recomputes one checkpoint segment at a
// time and keeps that segment's intermediates in caller-provided scratch.
#pragma once
#include "diff_core.cuh"

namespace sgdyn {

template <int MAXJ>
struct Ext {
  static constexpr int MAXV = MAXJ + 5;
  static constexpr int MAXQ = MAXJ + 6;
};

template <int MAXJ>
__device__ __forceinline__ void load_row(const Arr& a, int64_t e, int cols, double* out) {
  for (int c = 0; c < cols; c++) out[c] = ldv(a, e, c);
}
__device__ __forceinline__ void store_row(const Arr& a, int64_t e, int cols, const double* in) {
  for (int c = 0; c < cols; c++) stv(a, e, c, in[c]);
}

template <int MAXJ, class Tab>
__device__ __forceinline__ void rnea_vjp_env(const Tab& T, const VjpArgs& a, const int64_t e) {
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const int nv = T.nv(), nq = T.nq_ext();
  double q[MAXQ], qd[MAXV], qdd[MAXV], tb[MAXV], o1[MAXV], o2[MAXV], o3[MAXV];
  load_row<MAXJ>(a.q, e, nq, q);
  load_row<MAXJ>(a.qd, e, nv, qd);
  load_row<MAXJ>(a.x, e, nv, qdd);
  load_row<MAXJ>(a.bar, e, nv, tb);
  DynWork<MAXJ> W;
  AdjScratch<MAXJ> A;
  rnea_forward<MAXJ>(T, q, qd, qdd, W);
  rnea_subtree_forces<MAXJ>(T, W, A.F);
  rnea_adjoint<MAXJ>(T, W, A, tb, a.o1.p ? o1 : nullptr, a.o2.p ? o2 : nullptr, a.o3.p ? o3 : nullptr, 1.0);
  if (a.o1.p) store_row(a.o1, e, nv, o1);
  if (a.o2.p) store_row(a.o2, e, nv, o2);
  if (a.o3.p) store_row(a.o3, e, nv, o3);
}

template <int MAXJ>
__global__ void __launch_bounds__(32) rnea_vjp_kernel(const DModel* __restrict__ model, const VjpArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  rnea_vjp_env<MAXJ>(RuntimeTab{model}, a, e);
}

template <int MAXJ, class Tab>
__device__ __forceinline__ void aba_vjp_env(const Tab& T, const VjpArgs& a, const int64_t e) {
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const int nv = T.nv(), nq = T.nq_ext();
  double q[MAXQ], qd[MAXV], tau[MAXV], qb[MAXV], qdd[MAXV], lam[MAXV], o1[MAXV], o2[MAXV];
  load_row<MAXJ>(a.q, e, nq, q);
  load_row<MAXJ>(a.qd, e, nv, qd);
  load_row<MAXJ>(a.x, e, nv, tau);
  load_row<MAXJ>(a.bar, e, nv, qb);
  DynWork<MAXJ> W;
  AdjScratch<MAXJ> A;
  aba_forward<MAXJ>(T, q, qd, tau, qdd, W);
  rnea_subtree_forces<MAXJ>(T, W, A.F);
  minv_solve<MAXJ>(T, W, qb, lam);
  rnea_adjoint<MAXJ>(T, W, A, lam, a.o1.p ? o1 : nullptr, a.o2.p ? o2 : nullptr, nullptr, -1.0);
  if (a.o1.p) store_row(a.o1, e, nv, o1);
  if (a.o2.p) store_row(a.o2, e, nv, o2);
  if (a.o3.p) store_row(a.o3, e, nv, lam);
}

template <int MAXJ>
__global__ void __launch_bounds__(32) aba_vjp_kernel(const DModel* __restrict__ model, const VjpArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  aba_vjp_env<MAXJ>(RuntimeTab{model}, a, e);
}

// Link pose adjoint: a link at p with rotation R receives the world force
// (pbar, p x pbar + n_R), n_R = axial part of R Rbar^T (so that tr(Rbar^T [w]x R) = w . n_R);
// forces are summed over subtrees and projected on the world motion subspaces.
template <int MAXJ>
__global__ void __launch_bounds__(32) fk_vjp_kernel(const DModel* __restrict__ model, const FkVjpArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  constexpr int MAXQ = Ext<MAXJ>::MAXQ;
  const int nj = model->nj, nq = model->nq_ext, nl = model->nlinks;
  const DJoint* __restrict__ JT = model_joints(model);
  const DLink* __restrict__ LT = model_links(model);
  double q[MAXQ];
  load_row<MAXJ>(a.q, e, nq, q);
  DynWork<MAXJ> W;
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  Mot* F = W.pA;
  for (int i = 1; i < nj; i++) {
    pose_and_S<MAXJ>(JT[i], i, q, W);
    F[i] = zero;
  }
  for (int l = 0; l < nl; l++) {
    const DLink& L = LT[l];
    const int j = L.joint;
    if (j == 0) continue;  // links welded to the base do not move
    M3 Rl;
    for (int k = 0; k < 9; k++) Rl.a[k] = L.R[k];
    const M3 R = mul(W.oR[j], Rl);
    const V3 p = mul_add(W.oR[j], mk(L.p[0], L.p[1], L.p[2]), W.op[j]);
    const V3 pb = mk(ldv(a.pbar, e, 3 * l), ldv(a.pbar, e, 3 * l + 1), ldv(a.pbar, e, 3 * l + 2));
    Mot f{pb, cross(p, pb)};
    if (a.Rbar.p) {
      M3 Rb;
      for (int k = 0; k < 9; k++) Rb.a[k] = ldv(a.Rbar, e, 9 * l + k);
      const M3 A = mul(R, transpose(Rb));
      f.w = f.w + mk(A.a[5] - A.a[7], A.a[6] - A.a[2], A.a[1] - A.a[3]);
    }
    F[j] = add6(F[j], f);
  }
  for (int i = nj - 1; i >= 1; i--) {
    const DJoint& J = JT[i];
    for (int k = 0; k < J.nv; k++) stv(a.qbar, e, J.vcol + k, dot6(W.Sw[J.ivx + k], F[i]));
    if (J.parent > 0) F[J.parent] = add6(F[J.parent], F[i]);
  }
}

// Analytic RNEA derivatives, column by column (forward mode over the subtree composites).
// Perturbing tree column c = (joint j, coordinate l), s = S_c, moves subtree(j) rigidly by
// s; with lambda = parent(j), u = v_lambda x s, alpha = a_lambda x s (a_0 = -gravity,
// v_0 = 0), beta = alpha - u x v_lambda and gamma = (v_lambda + v_j) x s, the columns are
//   rows of a strict ancestor i of j (S_i fixed):
//     dtau_i/dq_c   = S_i . (s x* F_j + Ib_j beta + Db_j u + u x* H_j)
//     dtau_i/dqd_c  = S_i . (Db_j s + s x* H_j + Ib_j gamma)
//     dtau_i/dqdd_c = S_i . Ib_j s
//   rows of i in subtree(j) (S_i moves with the subtree; the s x* F term cancels):
//     dtau_i/dq_c   = P_i . beta + Q_i . u
//     dtau_i/dqd_c  = Q_i . s + P_i . gamma
//     dtau_i/dqdd_c = P_i . s
//   and 0 elsewhere (composites: deriv_composites). From tau_i = S_i . F_i with
// v_k = v_lambda + (rigidly moved part), a_k likewise, and d(v x* I v)/dv, whose subtree
// sum is the rate Db plus the momentum term. Subtrees are contiguous in the table's joint
// order, so "i in subtree(j)" is j <= i < subtree_end(j). A thread writes the columns
// c = g, g + G, ... (G = a.groups) of one environment, whole columns including zeros.
// The per-column vectors of the formulas above for tree column t = J.ivx + l of joint j.
struct ColumnTerms {
  Mot s, u, beta, gam, Phi, Psi;
};

template <int MAXJ, class Tab>
__device__ __forceinline__ ColumnTerms column_terms(const Tab& T, const DynWork<MAXJ>& W,
                                                    const DerivComposites<MAXJ>& C, int j, int t) {
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  const Mot a0{mk(-T.gravity(0), -T.gravity(1), -T.gravity(2)), mk(0, 0, 0)};
  const int p = T.joint(j).parent;
  const Mot vl = (p == 0) ? zero : W.vel[p];
  const Mot al = (p == 0) ? a0 : W.acc[p];
  ColumnTerms ct;
  ct.s = W.Sw[t];
  ct.u = add_crossm(zero, vl, ct.s);
  ct.beta = add_crossm(add_crossm(zero, al, ct.s), vl, ct.u);  // alpha - u x v_lambda
  ct.gam = add_crossm(zero, add6(vl, W.vel[j]), ct.s);
  ct.Phi = rbi_mul_add(C.Ib[j], ct.beta, add_crossf(zero, ct.s, C.F[j]));
  ct.Phi = add_crossf(rbi_mul_add(C.Db[j], ct.u, ct.Phi), ct.u, C.H[j]);
  ct.Psi = rbi_mul_add(C.Ib[j], ct.gam, rbi_mul_add(C.Db[j], ct.s, add_crossf(zero, ct.s, C.H[j])));
  return ct;
}

// Entry (row column ti of joint i, column t of joint j) of dtau/dq, dtau/dqd, dtau/dqdd.
template <int MAXJ>
__device__ __forceinline__ void column_entry(const DynWork<MAXJ>& W, const DerivComposites<MAXJ>& C,
                                             const ColumnTerms& ct, bool anc, bool sub, int t, int ti, double& dq,
                                             double& dqd, double& dqdd) {
  dq = dqd = dqdd = 0;
  if (anc) {
    const Mot Si = W.Sw[ti];
    dq = dot6(Si, ct.Phi);
    dqd = dot6(Si, ct.Psi);
    dqdd = dot6(Si, C.P[t]);
  } else if (sub) {
    const Mot P = C.P[ti], Q = C.Q[ti];
    dq = dot6(P, ct.beta) + dot6(Q, ct.u);
    dqd = dot6(Q, ct.s) + dot6(P, ct.gam);
    dqdd = dot6(P, ct.s);
  }
}

template <int MAXJ, class Tab>
__device__ __forceinline__ void rnea_derivative_columns(const Tab& T, const DynWork<MAXJ>& W,
                                                        const DerivComposites<MAXJ>& C, const DerivArgs& a,
                                                        const int64_t e, const int g) {
  const int nj = T.nj(), nv = T.nv();
  for (int j = 1; j < nj; j++) {
    const DJoint& J = T.joint(j);
    for (int l = 0; l < J.nv; l++) {
      const int t = J.ivx + l;
      if (t % a.groups != g) continue;
      const int c = J.vcol + l;
      const ColumnTerms ct = column_terms<MAXJ>(T, W, C, j, t);
      for (int i = 1; i < nj; i++) {
        const DJoint& I = T.joint(i);
        const bool anc = i < j && j < I.subtree_end;
        const bool sub = i >= j && i < J.subtree_end;
        for (int k = 0; k < I.nv; k++) {
          const int r = I.vcol + k;
          double dq, dqd, dqdd;
          column_entry<MAXJ>(W, C, ct, anc, sub, t, I.ivx + k, dq, dqd, dqdd);
          stv(a.d_q, e, r * nv + c, dq);
          stv(a.d_qd, e, r * nv + c, dqd);
          if (a.d_x.p) stv(a.d_x, e, r * nv + c, dqdd);
        }
      }
    }
  }
}

template <int MAXJ>
__global__ void __launch_bounds__(32) rnea_derivatives_kernel(const DModel* __restrict__ model, const DerivArgs a) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= a.n * a.groups) return;
  const int64_t e = idx % a.n;
  const int g = int(idx / a.n);
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const RuntimeTab T{model};
  const int nv = T.nv(), nq = T.nq_ext();
  double q[MAXQ], qd[MAXV], qdd[MAXV];
  load_row<MAXJ>(a.q, e, nq, q);
  load_row<MAXJ>(a.qd, e, nv, qd);
  load_row<MAXJ>(a.x, e, nv, qdd);
  DynWork<MAXJ> W;
  DerivComposites<MAXJ> C;
  rnea_forward<MAXJ>(T, q, qd, qdd, W);
  deriv_composites<MAXJ>(T, W, C);
  rnea_derivative_columns<MAXJ>(T, W, C, a, e, g);
}

// Joint-space inertia in tree-column order factored as M = L^T D L with the tree's
// sparsity (Featherstone, "Rigid Body Dynamics Algorithms", 2008, sec. 6.5): column a's
// parent lam[a] is the previous column of its joint, else the last column of the parent
// joint, else -1; L is unit lower triangular with nonzeros only at (a, ancestor of a), so
// the factorisation costs sum depth^2 and a solve 2 sum depth. H holds M's lower triangle
// (packed by rows: entry (a, b <= a) at ltdl_at(a, b)) on entry and L below the diagonal
// on exit; Dinv = 1 / D.
__device__ __forceinline__ int ltdl_at(int a, int b) { return a * (a + 1) / 2 + b; }

__device__ __forceinline__ void ltdl_factor(double* H, const int* lam, double* Dinv, int n) {
  for (int k = n - 1; k >= 0; k--) {
    const double rk = 1.0 / H[ltdl_at(k, k)];
    Dinv[k] = rk;
    for (int i = lam[k]; i >= 0; i = lam[i]) {
      const double f = H[ltdl_at(k, i)] * rk;
      for (int j = i; j >= 0; j = lam[j]) H[ltdl_at(i, j)] -= f * H[ltdl_at(k, j)];
      H[ltdl_at(k, i)] = f;
    }
  }
}
// B <- M^-1 B in place for R right-hand sides at once (B row-major [n][R]), M = L^T D L
// from ltdl_factor; end[i] = one past the last descendant column of column i (subtrees are
// contiguous in tree-column order). L^T y = b runs in pull form over each column's
// descendant range, L x = z over its ancestor chain; each step has R independent updates.
template <int R>
__device__ __forceinline__ void ltdl_solve_many(const double* H, const int* lam, const int* end, const double* Dinv,
                                                int n, double* B) {
  for (int i = n - 1; i >= 0; i--) {
    double y[R];
#pragma unroll
    for (int r = 0; r < R; r++) y[r] = B[i * R + r];
    for (int k = i + 1; k < end[i]; k++) {
      const double h = H[ltdl_at(k, i)];
#pragma unroll
      for (int r = 0; r < R; r++) y[r] -= h * B[k * R + r];
    }
#pragma unroll
    for (int r = 0; r < R; r++) B[i * R + r] = y[r];
  }
  for (int k = 0; k < n; k++) {
    double x[R];
    const double d = Dinv[k];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = B[k * R + r] * d;
    for (int i = lam[k]; i >= 0; i = lam[i]) {
      const double h = H[ltdl_at(k, i)];
#pragma unroll
      for (int r = 0; r < R; r++) x[r] -= h * B[i * R + r];
    }
#pragma unroll
    for (int r = 0; r < R; r++) B[k * R + r] = x[r];
  }
}

// ABA derivatives from the RNEA ones at qdd = ABA(q, qd, tau): dqdd/dq = -M^-1 dtau/dq,
// dqdd/dqd = -M^-1 dtau/dqd, dqdd/dtau = M^-1 (Carpentier & Mansard, RSS 2018). The tau
// columns come from the analytic column formulas above, M from the same composites
// (M_ab = P_a . S_b for b an ancestor-or-self column of a), and every M^-1 product is an
// LTDL solve. A thread writes the columns c = g, g + G, ... of one environment, solving
// them in batches of CB columns (3 CB right-hand sides); the launch picks CB >= the
// columns per thread where it can, so no batch runs half empty.
template <int MAXJ, int CB>
__global__ void __launch_bounds__(32) aba_derivatives_kernel(const DModel* __restrict__ model, const DerivArgs a) {
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const RuntimeTab T{model};
  const int nj = T.nj(), nv = T.nv(), nq = T.nq_ext();
  // the column tree, shared by the block (one model): parent column, external index,
  // one past the last descendant column
  __shared__ int lam[MAXV], ext[MAXV], cend[MAXV];
  for (int i = 1 + int(threadIdx.x); i < nj; i += blockDim.x) {
    const DJoint& J = T.joint(i);
    const int p = J.parent;
    const int last = J.subtree_end < nj ? T.joint(J.subtree_end).ivx : nv;
    for (int k = 0; k < J.nv; k++) {
      const int t = J.ivx + k;
      lam[t] = k > 0 ? t - 1 : (p > 0 ? T.joint(p).ivx + T.joint(p).nv - 1 : -1);
      ext[t] = J.vcol + k;
      cend[t] = last;
    }
  }
  __syncthreads();
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= a.n * a.groups) return;
  const int64_t e = idx % a.n;
  const int g = int(idx / a.n);
  double q[MAXQ], qd[MAXV], tau[MAXV], qdd[MAXV];
  load_row<MAXJ>(a.q, e, nq, q);
  load_row<MAXJ>(a.qd, e, nv, qd);
  load_row<MAXJ>(a.x, e, nv, tau);
  DynWork<MAXJ> W;
  DerivComposites<MAXJ> C;
  // forward dynamics through the factorisation built anyway: the RNEA sweep at qdd = 0
  // gives the bias accelerations and forces, qdd = M^-1 (tau - tau_bias), then the
  // accelerations and subtree forces take the qdd terms (a_i += sum_{m <= i} S_m qdd_m,
  // F_i += sum_{k in subtree(i)} I_k da_k)
  for (int c = 0; c < nv; c++) qdd[c] = 0.0;
  rnea_forward<MAXJ>(T, q, qd, qdd, W);
  deriv_composites<MAXJ>(T, W, C);
  double H[MAXV * (MAXV + 1) / 2], Dinv[MAXV];
  for (int t = 0; t < nv; t++)
    for (int b = t; b >= 0; b = lam[b]) H[ltdl_at(t, b)] = dot6(C.P[t], W.Sw[b]);
  ltdl_factor(H, lam, Dinv, nv);
  {
    double x[MAXV];
    for (int i = 1; i < nj; i++) {
      const DJoint& J = T.joint(i);
      for (int k = 0; k < J.nv; k++) x[J.ivx + k] = tau[J.vcol + k] - dot6(W.Sw[J.ivx + k], C.F[i]);
    }
    ltdl_solve_many<1>(H, lam, cend, Dinv, nv, x);
    const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
    Mot da[MAXJ];
    for (int i = 1; i < nj; i++) {
      const DJoint& J = T.joint(i);
      Mot d = J.parent > 0 ? da[J.parent] : zero;
      for (int k = 0; k < J.nv; k++) d = axpy6(x[J.ivx + k], W.Sw[J.ivx + k], d);
      da[i] = d;
      W.acc[i] = add6(W.acc[i], d);
    }
    for (int i = 1; i < nj; i++) da[i] = rbi_mul(W.Iw[i], da[i]);  // now I_i da_i, summed over subtrees below
    for (int i = nj - 1; i >= 1; i--) {
      const int p = T.joint(i).parent;
      if (p > 0) da[p] = add6(da[p], da[i]);
      C.F[i] = add6(C.F[i], da[i]);
    }
  }
  // right-hand sides per batch: [dtau/dq columns | dtau/dqd columns | unit vectors]
  constexpr int RB = 3 * CB;
  double B[MAXV * RB];
  int cols[CB], ncols = 0;
  auto flush = [&]() {
    ltdl_solve_many<RB>(H, lam, cend, Dinv, nv, B);
    for (int m = 0; m < ncols; m++) {
      const int c = ext[cols[m]];
      for (int r = 0; r < nv; r++) {
        stv(a.d_q, e, ext[r] * nv + c, -B[r * RB + m]);
        stv(a.d_qd, e, ext[r] * nv + c, -B[r * RB + CB + m]);
        if (a.d_x.p) stv(a.d_x, e, ext[r] * nv + c, B[r * RB + 2 * CB + m]);
      }
    }
    ncols = 0;
  };
  for (int j = 1; j < nj; j++) {
    const DJoint& J = T.joint(j);
    for (int l = 0; l < J.nv; l++) {
      const int t = J.ivx + l;
      if (t % a.groups != g) continue;
      if (ncols == 0)
        for (int k = 0; k < nv * RB; k++) B[k] = 0.0;
      const int m = ncols++;
      cols[m] = t;
      const ColumnTerms ct = column_terms<MAXJ>(T, W, C, j, t);
      for (int i = 1; i < nj; i++) {
        const DJoint& I = T.joint(i);
        const bool anc = i < j && j < I.subtree_end;
        const bool sub = i >= j && i < J.subtree_end;
        if (!anc && !sub) continue;
        for (int k = 0; k < I.nv; k++) {
          const int ti = I.ivx + k;
          double dqdd;
          column_entry<MAXJ>(W, C, ct, anc, sub, t, ti, B[ti * RB + m], B[ti * RB + CB + m], dqdd);
        }
      }
      B[t * RB + 2 * CB + m] = 1.0;
      if (ncols == CB) flush();
    }
  }
  if (ncols > 0) flush();
}

// ---- rollouts ---------------------------------------------------------------------

// q <- q + dt qd for angle / slide coordinates (models without free flyers).
template <class Tab>
__device__ __forceinline__ void euler_positions(const Tab& T, double* q, const double* qd, double dt) {
#pragma unroll
  for (int i = 1; i < T.nj(); i++) {
    const DJoint& J = T.joint(i);
    q[J.qcol] = fma(dt, qd[J.vcol], q[J.qcol]);
  }
}

template <int MAXJ, class Tab>
__device__ __forceinline__ void rollout_forward_env(const Tab& T, const RolloutArgs& a, const int64_t e) {
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const int nv = T.nv(), nq = T.nq_ext();
  const int64_t n = a.n;
  double q[MAXQ], qd[MAXV], tau[MAXV], qdd[MAXV];
  for (int c = 0; c < nq; c++) q[c] = a.q0[e * nq + c];
  for (int c = 0; c < nv; c++) qd[c] = a.qd0[e * nv + c];
  DynWork<MAXJ> W;
  for (int t = 0; t < a.T; t++) {
    if (a.q_ckpt && t % a.K == 0) {
      const int64_t s = t / a.K;
      for (int c = 0; c < nq; c++) a.q_ckpt[(s * n + e) * nq + c] = q[c];
      for (int c = 0; c < nv; c++) a.qd_ckpt[(s * n + e) * nv + c] = qd[c];
    }
    for (int c = 0; c < nv; c++) tau[c] = a.tau[(int64_t(t) * n + e) * nv + c];
    aba_forward<MAXJ>(T, q, qd, tau, qdd, W);
    for (int c = 0; c < nv; c++) qd[c] = fma(a.dt, qdd[c], qd[c]);
    euler_positions(T, q, qd, a.dt);
  }
  for (int c = 0; c < nq; c++) a.qT[e * nq + c] = q[c];
  for (int c = 0; c < nv; c++) a.qdT[e * nv + c] = qd[c];
}

template <int MAXJ>
__global__ void __launch_bounds__(32) rollout_forward_kernel(const DModel* __restrict__ model, const RolloutArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  rollout_forward_env<MAXJ>(RuntimeTab{model}, a, e);
}

// Per step of a segment the scratch holds, structure-of-arrays over environments:
// S (6 per velocity), U (6 per velocity), then per joint D^-1 (1), v (6), a (6), I v (6),
// world inertia (10), subtree force (6); plus the free-flyer factor (21).
__host__ __device__ inline int64_t stash_doubles_per_step(int nj, int nq, int nv) {
  (void)nq;
  return 12 * int64_t(nv) + int64_t(nj) * 35 + 21;
}

template <int MAXJ, class Tab>
__device__ __forceinline__ void stash_io(const Tab& T, DynWork<MAXJ>& W, Mot* F, double* base, int64_t n,
                                         int64_t e, bool store) {
  const int nj = T.nj(), nv = T.nv();
  int64_t f = 0;
  auto io = [&](double& x) {
    if (store) base[f * n + e] = x;
    else x = base[f * n + e];
    f++;
  };
  auto io6 = [&](Mot& m) {
    io(m.v.x); io(m.v.y); io(m.v.z); io(m.w.x); io(m.w.y); io(m.w.z);
  };
#pragma unroll
  for (int k = 0; k < nv; k++) io6(W.Sw[k]);
#pragma unroll
  for (int k = 0; k < nv; k++) io6(W.Uv[k]);
#pragma unroll
  for (int i = 1; i < nj; i++) {
    io(W.Dinv[i]);
    io6(W.vel[i]);
    io6(W.acc[i]);
    io6(W.hY[i]);
    RBI& Y = W.Iw[i];
    io(Y.m); io(Y.h.x); io(Y.h.y); io(Y.h.z);
    for (int k = 0; k < 6; k++) io(Y.I[k]);
    io6(F[i]);
  }
  for (int k = 0; k < 21; k++) io(W.Lff[k]);
}

// Backward, part 1. Segments are independent given their checkpoints, so one thread per
// (segment of the group, environment) re-runs its segment and keeps every step's
// intermediates in the scratch: [segment of group][step of segment][field][env].
template <int MAXJ, class Tab>
__device__ __forceinline__ void rollout_recompute_env(const Tab& T, const RolloutArgs& a, const int64_t idx) {
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const int nv = T.nv(), nq = T.nq_ext(), nj = T.nj();
  const int64_t n = a.n;
  const int64_t e = idx % n;
  const int g = int(idx / n), s = a.s_lo + g;
  const int64_t per_step = stash_doubles_per_step(nj, nq, nv);
  double q[MAXQ], qd[MAXV], tau[MAXV], qdd[MAXV];
  for (int c = 0; c < nq; c++) q[c] = a.q_ckpt[(int64_t(s) * n + e) * nq + c];
  for (int c = 0; c < nv; c++) qd[c] = a.qd_ckpt[(int64_t(s) * n + e) * nv + c];
  DynWork<MAXJ> W;
  const int t0 = s * a.K, t1 = min(a.T, t0 + a.K);
  for (int t = t0; t < t1; t++) {
    double* base = a.scratch + (int64_t(g) * a.K + (t - t0)) * per_step * n;
    for (int c = 0; c < nv; c++) tau[c] = a.tau[(int64_t(t) * n + e) * nv + c];
    aba_forward<MAXJ>(T, q, qd, tau, qdd, W);
    rnea_subtree_forces<MAXJ>(T, W, W.pA);  // ABA's bias forces are no longer needed
    stash_io<MAXJ>(T, W, W.pA, base, n, e, true);
    for (int c = 0; c < nv; c++) qd[c] = fma(a.dt, qdd[c], qd[c]);
    euler_positions(T, q, qd, a.dt);
  }
}

// Backward, part 2: one thread per environment walks the group's steps in reverse from
// the stored intermediates. The adjoint of the state enters from qT_bar / qdT_bar for the
// last group and from q0_bar / qd0_bar (the previous group's result) otherwise, and
// leaves through q0_bar / qd0_bar.
template <int MAXJ, class Tab>
__device__ __forceinline__ void rollout_reverse_env(const Tab& T, const RolloutArgs& a, const int64_t e) {
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const int nv = T.nv(), nq = T.nq_ext(), nj = T.nj();
  const int64_t n = a.n;
  const int64_t per_step = stash_doubles_per_step(nj, nq, nv);
  const int nseg = (a.T + a.K - 1) / a.K;
  const bool last = a.s_lo + a.s_cnt == nseg;
  const double* qin = last ? a.qT_bar : a.q0_bar;
  const double* qdin = last ? a.qdT_bar : a.qd0_bar;
  double qb[MAXQ], qdb[MAXV], qddb[MAXV], lam[MAXV], o1[MAXV], o2[MAXV];
  for (int c = 0; c < nq; c++) qb[c] = qin ? qin[e * nq + c] : 0.0;
  for (int c = 0; c < nv; c++) qdb[c] = qdin ? qdin[e * nv + c] : 0.0;
  DynWork<MAXJ> W;
  AdjScratch<MAXJ> A;
  for (int s = a.s_lo + a.s_cnt - 1; s >= a.s_lo; s--) {
    const int t0 = s * a.K, t1 = min(a.T, t0 + a.K);
    // q' = q + dt qd' and qd' = qd + dt qdd, reversed
    for (int t = t1 - 1; t >= t0; t--) {
      double* base = a.scratch + (int64_t(s - a.s_lo) * a.K + (t - t0)) * per_step * n;
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
        qdb[J.vcol] = fma(a.dt, qb[J.qcol], qdb[J.vcol]);
      }
      for (int c = 0; c < nv; c++) qddb[c] = a.dt * qdb[c];
      stash_io<MAXJ>(T, W, A.F, base, n, e, false);
      minv_solve<MAXJ>(T, W, qddb, lam);
      for (int c = 0; c < nv; c++) a.tau_bar[(int64_t(t) * n + e) * nv + c] = lam[c];
      rnea_adjoint<MAXJ>(T, W, A, lam, o1, o2, nullptr, -1.0);
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
        qb[J.qcol] += o1[J.vcol];
      }
      for (int c = 0; c < nv; c++) qdb[c] += o2[c];
    }
  }
  for (int c = 0; c < nq; c++) a.q0_bar[e * nq + c] = qb[c];
  for (int c = 0; c < nv; c++) a.qd0_bar[e * nv + c] = qdb[c];
}

template <int MAXJ>
__global__ void __launch_bounds__(32) rollout_recompute_kernel(const DModel* __restrict__ model, const RolloutArgs a) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= a.n * a.s_cnt) return;
  rollout_recompute_env<MAXJ>(RuntimeTab{model}, a, idx);
}

template <int MAXJ>
__global__ void __launch_bounds__(32) rollout_reverse_kernel(const DModel* __restrict__ model, const RolloutArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  rollout_reverse_env<MAXJ>(RuntimeTab{model}, a, e);
}

}  // namespace sgdyn
