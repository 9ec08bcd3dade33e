// Differentiation kernels: RNEA / ABA / FK adjoints, dense derivative matrices and the
// checkpointed semi-implicit-Euler rollout (forward and reverse). One environment per
// thread; every kernel recomputes the spatial intermediates it needs instead of reading a
// stored tape, except the rollout backward, which recomputes one checkpoint segment at a
// time and keeps that segment's intermediates in caller-provided scratch.
#pragma once
#include "diff_core.cuh"
#include "se3.cuh"

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
// order, so "i in subtree(j)" is j <= i < subtree_end(j).
// The per-column vectors of the formulas above for tree column s = S_t of joint j, parent
// velocity / acceleration vl, al (v_0 = 0, a_0 = -gravity) and v_j.
struct ColumnTerms {
  Mot s, u, beta, gam, Phi, Psi;
};

__device__ __forceinline__ ColumnTerms column_terms(Mot s, Mot vl, Mot al, Mot vj, Mot Fj, Mot Hj, const RBI& Ibj,
                                                    const RBI& Dbj) {
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  ColumnTerms ct;
  ct.s = s;
  ct.u = add_crossm(zero, vl, s);
  ct.beta = add_crossm(add_crossm(zero, al, s), vl, ct.u);  // alpha - u x v_lambda
  ct.gam = add_crossm(zero, add6(vl, vj), s);
  ct.Phi = rbi_mul_add(Ibj, ct.beta, add_crossf(zero, s, Fj));
  ct.Phi = add_crossf(rbi_mul_add(Dbj, ct.u, ct.Phi), ct.u, Hj);
  ct.Psi = rbi_mul_add(Ibj, ct.gam, rbi_mul_add(Dbj, s, add_crossf(zero, s, Hj)));
  return ct;
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
// with L(k, i) and Dinv(k) read through the accessors; end[i] = one past the last
// descendant column of column i (subtrees are contiguous in tree-column order). L^T y = b
// runs in pull form over each column's descendant range, L x = z over its ancestor chain.
template <int R, class LF, class DF>
__device__ __forceinline__ void ltdl_solve_many(LF Lk, DF Dk, const int* lam, const int* end, int n, double* B) {
  for (int i = n - 1; i >= 0; i--) {
    double y[R];
#pragma unroll
    for (int r = 0; r < R; r++) y[r] = B[i * R + r];
    for (int k = i + 1; k < end[i]; k++) {
      const double h = Lk(k, i);
#pragma unroll
      for (int r = 0; r < R; r++) y[r] -= h * B[k * R + r];
    }
#pragma unroll
    for (int r = 0; r < R; r++) B[i * R + r] = y[r];
  }
  for (int k = 0; k < n; k++) {
    double x[R];
    const double d = Dk(k);
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = B[k * R + r] * d;
    for (int i = lam[k]; i >= 0; i = lam[i]) {
      const double h = Lk(k, i);
#pragma unroll
      for (int r = 0; r < R; r++) x[r] -= h * B[i * R + r];
    }
#pragma unroll
    for (int r = 0; r < R; r++) B[k * R + r] = x[r];
  }
}

// The tree of velocity columns, built by every block in shared memory (one model per
// launch): parent column, external index, one past the last descendant column.
template <class Tab>
__device__ __forceinline__ void column_tree(const Tab& T, int* lam, int* ext, int* cend) {
  const int nj = T.nj(), nv = T.nv();
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
}

// Scratch of the derivative kernels: field f of environment e at scratch[f n + e].
struct DerivScratch {
  double* p;
  int64_t n, e;
  __device__ __forceinline__ double& at(int f) const { return p[int64_t(f) * n + e]; }
  __device__ __forceinline__ Mot mot(int f) const {
    return Mot{mk(at(f), at(f + 1), at(f + 2)), mk(at(f + 3), at(f + 4), at(f + 5))};
  }
  __device__ __forceinline__ void put(int f, Mot m) const {
    at(f) = m.v.x; at(f + 1) = m.v.y; at(f + 2) = m.v.z;
    at(f + 3) = m.w.x; at(f + 4) = m.w.y; at(f + 5) = m.w.z;
  }
  __device__ __forceinline__ RBI rbi(int f) const {
    RBI Y;
    Y.m = at(f);
    Y.h = mk(at(f + 1), at(f + 2), at(f + 3));
#pragma unroll
    for (int k = 0; k < 6; k++) Y.I[k] = at(f + 4 + k);
    return Y;
  }
  __device__ __forceinline__ void put(int f, const RBI& Y) const {
    at(f) = Y.m;
    at(f + 1) = Y.h.x; at(f + 2) = Y.h.y; at(f + 3) = Y.h.z;
#pragma unroll
    for (int k = 0; k < 6; k++) at(f + 4 + k) = Y.I[k];
  }
};

// Preparation, one thread per environment: the forward sweep and the subtree composites
// into the scratch. ABA: the sweep at qdd = 0 gives the bias accelerations and forces; M
// (M_ab = P_a . S_b for b an ancestor-or-self column of a) is factored, qdd = M^-1 (tau -
// tau_bias), and the accelerations and subtree forces take the qdd terms (a_i += sum_{m <=
// i} S_m qdd_m, F_i += sum_{k in subtree(i)} I_k da_k); the factor goes to the scratch too.
template <int MAXJ, bool ABA>
__global__ void __launch_bounds__(32) deriv_prepare_kernel(const DModel* __restrict__ model, const DerivArgs a) {
  constexpr int MAXV = Ext<MAXJ>::MAXV, MAXQ = Ext<MAXJ>::MAXQ;
  const RuntimeTab T{model};
  const int nj = T.nj(), nv = T.nv(), nq = T.nq_ext();
  __shared__ int lam[MAXV], ext[MAXV], cend[MAXV];
  if (ABA) column_tree(T, lam, ext, cend);
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  double q[MAXQ], qd[MAXV], x[MAXV], qdd[MAXV];
  load_row<MAXJ>(a.q, e, nq, q);
  load_row<MAXJ>(a.qd, e, nv, qd);
  load_row<MAXJ>(a.x, e, nv, x);
  DynWork<MAXJ> W;
  DerivComposites<MAXJ> C;
  const DerivScratch D{a.scratch, a.n, e};
  const DerivLayout& L = a.lay;
  if (!ABA) {
    rnea_forward<MAXJ>(T, q, qd, x, W);
    deriv_composites<MAXJ>(T, W, C);
  } else {
    for (int c = 0; c < nv; c++) qdd[c] = 0.0;
    rnea_forward<MAXJ>(T, q, qd, qdd, W);
    deriv_composites<MAXJ>(T, W, C);
    double H[MAXV * (MAXV + 1) / 2], Dinv[MAXV];
    for (int t = 0; t < nv; t++)
      for (int b = t; b >= 0; b = lam[b]) H[ltdl_at(t, b)] = dot6(C.P[t], W.Sw[b]);
    ltdl_factor(H, lam, Dinv, nv);
    for (int i = 1; i < nj; i++) {
      const DJoint& J = T.joint(i);
      for (int k = 0; k < J.nv; k++) qdd[J.ivx + k] = x[J.vcol + k] - dot6(W.Sw[J.ivx + k], C.F[i]);
    }
    ltdl_solve_many<1>([&](int k, int i) { return H[ltdl_at(k, i)]; }, [&](int k) { return Dinv[k]; }, lam, cend, nv,
                       qdd);
    const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
    Mot da[MAXJ];
    for (int i = 1; i < nj; i++) {
      const DJoint& J = T.joint(i);
      Mot d = J.parent > 0 ? da[J.parent] : zero;
      for (int k = 0; k < J.nv; k++) d = axpy6(qdd[J.ivx + k], W.Sw[J.ivx + k], d);
      da[i] = d;
      W.acc[i] = add6(W.acc[i], d);
    }
    for (int i = 1; i < nj; i++) da[i] = rbi_mul(W.Iw[i], da[i]);  // now I_i da_i, summed over subtrees below
    for (int i = nj - 1; i >= 1; i--) {
      const int p = T.joint(i).parent;
      if (p > 0) da[p] = add6(da[p], da[i]);
      C.F[i] = add6(C.F[i], da[i]);
    }
    for (int k = 0; k < nv * (nv + 1) / 2; k++) D.at(L.L + k) = H[k];
    for (int k = 0; k < nv; k++) D.at(L.Dinv + k) = Dinv[k];
  }
  for (int t = 0; t < nv; t++) {
    D.put(L.S + 6 * t, W.Sw[t]);
    D.put(L.P + 6 * t, C.P[t]);
    D.put(L.Q + 6 * t, C.Q[t]);
  }
  for (int i = 1; i < nj; i++) {
    D.put(L.v + 6 * i, W.vel[i]);
    D.put(L.a + 6 * i, W.acc[i]);
    D.put(L.F + 6 * i, C.F[i]);
    D.put(L.H + 6 * i, C.H[i]);
    D.put(L.Ib + 10 * i, C.Ib[i]);
    D.put(L.Db + 10 * i, C.Db[i]);
  }
}

// One column, one environment: the column terms of tree column t (joint j) and the entries
// of the ancestor rows (S_i . Phi, S_i . Psi, S_i . P_t) and subtree rows (P_i . beta +
// Q_i . u, Q_i . s + P_i . gamma, P_i . s); others are 0. Calls f(tree row, dq, dqd, dqdd).
template <class Tab, class F>
__device__ __forceinline__ void derivative_column(const Tab& T, const DerivScratch& D, const DerivLayout& L,
                                                  int t, F&& f) {
  const int nj = T.nj();
  int j = 1;
  while (t >= T.joint(j).ivx + T.joint(j).nv) j++;
  const DJoint& J = T.joint(j);
  const int p = J.parent;
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  const Mot a0{mk(-T.gravity(0), -T.gravity(1), -T.gravity(2)), mk(0, 0, 0)};
  const ColumnTerms ct = column_terms(D.mot(L.S + 6 * t), p ? D.mot(L.v + 6 * p) : zero, p ? D.mot(L.a + 6 * p) : a0,
                                      D.mot(L.v + 6 * j), D.mot(L.F + 6 * j), D.mot(L.H + 6 * j),
                                      D.rbi(L.Ib + 10 * j), D.rbi(L.Db + 10 * j));
  const Mot Pt = D.mot(L.P + 6 * t);
  for (int i = 1; i < nj; i++) {
    const DJoint& I = T.joint(i);
    const bool anc = i < j && j < I.subtree_end;
    const bool sub = i >= j && i < J.subtree_end;
    for (int k = 0; k < I.nv; k++) {
      const int ti = I.ivx + k;
      if (anc) {
        const Mot Si = D.mot(L.S + 6 * ti);
        f(ti, dot6(Si, ct.Phi), dot6(Si, ct.Psi), dot6(Si, Pt));
      } else if (sub) {
        const Mot P = D.mot(L.P + 6 * ti), Q = D.mot(L.Q + 6 * ti);
        f(ti, dot6(P, ct.beta) + dot6(Q, ct.u), dot6(Q, ct.s) + dot6(P, ct.gam), dot6(P, ct.s));
      } else {
        f(ti, 0.0, 0.0, 0.0);
      }
    }
  }
}

// RNEA derivatives: thread (tree column t, environment e) writes column ext(t) of the three
// matrices of environment e.
template <int MAXJ>
__global__ void __launch_bounds__(128) rnea_deriv_columns_kernel(const DModel* __restrict__ model, const DerivArgs a) {
  constexpr int MAXV = Ext<MAXJ>::MAXV;
  const RuntimeTab T{model};
  const int nv = T.nv();
  __shared__ int lam[MAXV], ext[MAXV], cend[MAXV];
  column_tree(T, lam, ext, cend);
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= a.n * nv) return;
  const int64_t e = idx % a.n;
  const int t = int(idx / a.n);
  const int c = ext[t];
  const DerivScratch D{a.scratch, a.n, e};
  derivative_column(T, D, a.lay, t, [&](int ti, double dq, double dqd, double dqdd) {
    const int r = ext[ti];
    stv(a.d_q, e, r * nv + c, dq);
    stv(a.d_qd, e, r * nv + c, dqd);
    if (a.d_x.p) stv(a.d_x, e, r * nv + c, dqdd);
  });
}

// ABA derivatives (Carpentier & Mansard, RSS 2018): dqdd/dq = -M^-1 dtau/dq, dqdd/dqd =
// -M^-1 dtau/dqd, dqdd/dtau = M^-1, with the dtau columns at qdd = ABA(q, qd, tau) and every
// M^-1 product one solve with the prepared factor: thread (tree column t, environment e)
// solves its three right-hand sides in one walk and writes column ext(t).
template <int MAXJ>
__global__ void __launch_bounds__(128) aba_deriv_columns_kernel(const DModel* __restrict__ model, const DerivArgs a) {
  constexpr int MAXV = Ext<MAXJ>::MAXV;
  const RuntimeTab T{model};
  const int nv = T.nv();
  __shared__ int lam[MAXV], ext[MAXV], cend[MAXV];
  column_tree(T, lam, ext, cend);
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= a.n * nv) return;
  const int64_t e = idx % a.n;
  const int t = int(idx / a.n);
  const DerivScratch D{a.scratch, a.n, e};
  const DerivLayout& L = a.lay;
  double B[MAXV * 3];
  derivative_column(T, D, L, t, [&](int ti, double dq, double dqd, double) {
    B[3 * ti] = dq;
    B[3 * ti + 1] = dqd;
    B[3 * ti + 2] = ti == t ? 1.0 : 0.0;
  });
  ltdl_solve_many<3>([&](int k, int i) { return D.at(L.L + ltdl_at(k, i)); }, [&](int k) { return D.at(L.Dinv + k); },
                     lam, cend, nv, B);
  const int c = ext[t];
  for (int r = 0; r < nv; r++) {
    stv(a.d_q, e, ext[r] * nv + c, -B[3 * r]);
    stv(a.d_qd, e, ext[r] * nv + c, -B[3 * r + 1]);
    if (a.d_x.p) stv(a.d_x, e, ext[r] * nv + c, B[3 * r + 2]);
  }
}

// ---- rollouts ---------------------------------------------------------------------

// q <- q (+) dt qd: angle / slide coordinates advance by dt qd, a free flyer (the root
// joint) moves on SE(3) by the body twist dt qd (Pinocchio's integrate).
template <class Tab>
__device__ __forceinline__ void euler_positions(const Tab& T, double* q, const double* qd, double dt) {
#pragma unroll
  for (int i = 1; i < T.nj(); i++) {
    const DJoint& J = T.joint(i);
    if (J.kind == JK_FREEFLYER) {
      double d[6];
#pragma unroll
      for (int k = 0; k < 6; k++) d[k] = dt * qd[J.vcol + k];
      free_flyer_integrate(q + J.qcol, d);
    } else {
      q[J.qcol] = fma(dt, qd[J.vcol], q[J.qcol]);
    }
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
// world inertia (10), subtree force (6); plus the free-flyer factor (21) and the step's
// free-flyer displacement dt qd' (6, the body twist its integrate applied).
__host__ __device__ inline int64_t stash_doubles_per_step(int nj, int nq, int nv) {
  (void)nq;
  return 12 * int64_t(nv) + int64_t(nj) * 35 + 21 + 6;
}

template <int MAXJ, class Tab>
__device__ __forceinline__ void stash_io(const Tab& T, DynWork<MAXJ>& W, Mot* F, double* ffd, double* base, int64_t n,
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
  for (int k = 0; k < 6; k++) io(ffd[k]);
}

// The free-flyer joint of a model (0 if none; only the root may be one).
template <class Tab>
__device__ __forceinline__ int free_flyer_joint(const Tab& T) {
#pragma unroll
  for (int i = 1; i < T.nj(); i++)
    if (T.joint(i).kind == JK_FREEFLYER) return i;
  return 0;
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
  const int ff = free_flyer_joint(T);
  const int t0 = s * a.K, t1 = min(a.T, t0 + a.K);
  for (int t = t0; t < t1; t++) {
    double* base = a.scratch + (int64_t(g) * a.K + (t - t0)) * per_step * n;
    for (int c = 0; c < nv; c++) tau[c] = a.tau[(int64_t(t) * n + e) * nv + c];
    aba_forward<MAXJ>(T, q, qd, tau, qdd, W);
    rnea_subtree_forces<MAXJ>(T, W, W.pA);  // ABA's bias forces are no longer needed
    for (int c = 0; c < nv; c++) qd[c] = fma(a.dt, qdd[c], qd[c]);
    double ffd[6] = {0, 0, 0, 0, 0, 0};
    if (ff > 0)
      for (int k = 0; k < 6; k++) ffd[k] = a.dt * qd[T.joint(ff).vcol + k];
    stash_io<MAXJ>(T, W, W.pA, ffd, base, n, e, true);
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
  // A free flyer's block of qb holds its tangent (body-twist) adjoint in the first six of
  // its seven slots, as the caller passes and receives it.
  double qb[MAXQ], qdb[MAXV], qddb[MAXV], lam[MAXV], o1[MAXV], o2[MAXV];
  for (int c = 0; c < nq; c++) qb[c] = qin ? qin[e * nq + c] : 0.0;
  for (int c = 0; c < nv; c++) qdb[c] = qdin ? qdin[e * nv + c] : 0.0;
  DynWork<MAXJ> W;
  AdjScratch<MAXJ> A;
  const int ff = free_flyer_joint(T);
  for (int s = a.s_lo + a.s_cnt - 1; s >= a.s_lo; s--) {
    const int t0 = s * a.K, t1 = min(a.T, t0 + a.K);
    // q' = q (+) dt qd' and qd' = qd + dt qdd, reversed
    for (int t = t1 - 1; t >= t0; t--) {
      double* base = a.scratch + (int64_t(s - a.s_lo) * a.K + (t - t0)) * per_step * n;
      double ffd[6];
      stash_io<MAXJ>(T, W, A.F, ffd, base, n, e, false);
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
        if (J.kind == JK_FREEFLYER) continue;
        qdb[J.vcol] = fma(a.dt, qb[J.qcol], qdb[J.vcol]);
      }
      if (ff > 0) {
        const int qc = T.joint(ff).qcol, vc = T.joint(ff).vcol;
        const Mot g{mk(qb[qc], qb[qc + 1], qb[qc + 2]), mk(qb[qc + 3], qb[qc + 4], qb[qc + 5])};
        Mot vb{mk(qdb[vc], qdb[vc + 1], qdb[vc + 2]), mk(qdb[vc + 3], qdb[vc + 4], qdb[vc + 5])};
        const Mot gq = free_flyer_integrate_adjoint(Mot{mk(ffd[0], ffd[1], ffd[2]), mk(ffd[3], ffd[4], ffd[5])}, g,
                                                    a.dt, vb);
        qb[qc] = gq.v.x; qb[qc + 1] = gq.v.y; qb[qc + 2] = gq.v.z;
        qb[qc + 3] = gq.w.x; qb[qc + 4] = gq.w.y; qb[qc + 5] = gq.w.z;
        qdb[vc] = vb.v.x; qdb[vc + 1] = vb.v.y; qdb[vc + 2] = vb.v.z;
        qdb[vc + 3] = vb.w.x; qdb[vc + 4] = vb.w.y; qdb[vc + 5] = vb.w.z;
      }
      for (int c = 0; c < nv; c++) qddb[c] = a.dt * qdb[c];
      minv_solve<MAXJ>(T, W, qddb, lam);
      for (int c = 0; c < nv; c++) a.tau_bar[(int64_t(t) * n + e) * nv + c] = lam[c];
      rnea_adjoint<MAXJ>(T, W, A, lam, o1, o2, nullptr, -1.0);
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
        for (int k = 0; k < J.nv; k++) qb[J.qcol + k] += o1[J.vcol + k];
      }
      for (int c = 0; c < nv; c++) qdb[c] += o2[c];
    }
  }
  if (ff > 0) qb[T.joint(ff).qcol + 6] = 0.0;
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
