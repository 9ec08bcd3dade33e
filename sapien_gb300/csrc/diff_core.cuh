// Shared device code for the differentiable path: ABA / RNEA forward sweeps that keep
// their intermediates in a per-thread work area, the M^-1 solve that reuses ABA's
// factorisation, and the reverse-mode RNEA sweep.
//
// Reverse-mode RNEA in the world frame. Perturbing joint j's coordinate moves the subtree
// of j rigidly by the world twist xi = S_j. Every world quantity attached to that subtree
// (S, v, a, I, f) transforms covariantly except for the parts inherited from j's parent
// lambda, and the covariant parts cancel in tau_i = S_i . F_i. What remains gives, with
//   w_k = sum_{i in ancestors-or-self(k)} taubar_i S_i          (root to leaves)
//   P_j = sum_{k in subtree(j)} I_k w_k,     Q_j = sum v_k x* (I_k w_k),
//   R_j = sum w_k x* (I_k v_k),              T_j = sum I_k (v_k x w_k),
//   F_j = sum f_k,  W_j = w_lambda,  Z_j = -Q_j + v_lambda x* P_j + R_j + T_j,
// the adjoints per column c of joint j:
//   qbar_c   = S_c . (-a_lambda x* P_j + v_lambda x* Z_j - W_j x* F_j)
//   qdbar_c  = S_c . (Q_j - (v_lambda + v_j) x* P_j - R_j - T_j)
//   qddbar_c = S_c . P_j                                          (= (M taubar)_c)
// (a_0 = -gravity, v_0 = 0). Configuration adjoints are tangent-space adjoints: for a
// free flyer they are with respect to the body twist, as in Pinocchio's derivative API.
// The ABA adjoint uses qdd = M^-1 (tau - h): lambda = M^-1 qddbar, taubar = lambda,
// (qbar, qdbar) = -RNEA-adjoint(q, qd, qdd; lambda) (Carpentier & Mansard, "Analytical
// derivatives of rigid body dynamics algorithms", RSS 2018).
#pragma once
#include "step_kernel.cuh"

namespace sgdyn {

template <int MAXJ>
struct DynWork {
  static constexpr int MAXV = MAXJ + 5;
  M3 oR[MAXJ];
  V3 op[MAXJ];
  Mot Sw[MAXV];
  Mot vel[MAXJ], acc[MAXJ], hY[MAXJ];
  RBI Iw[MAXJ];
  // ABA factorisation
  Sym6 IA[MAXJ];
  Mot pA[MAXJ], cb[MAXJ], Uv[MAXV];
  double uv[MAXV], Dinv[MAXJ];
  double Lff[21];
};

// World pose and motion subspace of joint i from external-order q (thread-local array).
template <int MAXJ>
__device__ __forceinline__ void pose_and_S(const DJoint& J, int i, const double* q, DynWork<MAXJ>& W) {
  const Arr qa{const_cast<double*>(q), 0, 1};
  joint_world_pose(J, qa, 0, W.oR, W.op, W.oR[i], W.op[i]);
  for (int k = 0; k < J.nv; k++) W.Sw[J.ivx + k] = world_S(J, W.oR[i], W.op[i], k);
}

__device__ __forceinline__ RBI local_rbi(const DJoint& J) {
  RBI Y;
  Y.m = J.m;
  Y.h = mk(J.h[0], J.h[1], J.h[2]);
#pragma unroll
  for (int k = 0; k < 6; k++) Y.I[k] = J.I[k];
  return Y;
}

// ABA in the world frame; fills W (acc = world accelerations incl. gravity) and qdd
// (external order).
template <int MAXJ, class Tab>
__device__ void aba_forward(const Tab& T, const double* q, const double* qd, const double* tau,
                            double* qdd, DynWork<MAXJ>& W) {
  const int nj = T.nj();
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, iv = J.ivx;
    pose_and_S(J, i, q, W);
    const RBI Y = rbi_transport(local_rbi(J), W.oR[i], W.op[i]);
    W.Iw[i] = Y;
    Mot vJ = zero;
    for (int k = 0; k < J.nv; k++) vJ = axpy6(qd[J.vcol + k], W.Sw[iv + k], vJ);
    const Mot v = (p == 0) ? vJ : add6(W.vel[p], vJ);
    W.vel[i] = v;
    const Mot h = rbi_mul(Y, v);
    W.hY[i] = h;
    W.cb[i] = add_crossm(zero, v, vJ);
    W.IA[i] = sym6_from_rbi(Y);
    W.pA[i] = add_crossf(zero, v, h);
  }
#pragma unroll
  for (int i = nj - 1; i >= 1; i--) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, iv = J.ivx;
    if (J.nv == 1) {
      const Mot S = W.Sw[iv];
      const Mot U = sym6_mul(W.IA[i], S);
      const double di = 1.0 / dot6(S, U);
      const double u = tau[J.vcol] - dot6(S, W.pA[i]);
      W.Uv[iv] = U;
      W.uv[iv] = u;
      W.Dinv[i] = di;
      if (p > 0) {
        const Mot Ud = scale6(di, U);
        Sym6 Ia = W.IA[i];
        const double ud[6] = {Ud.v.x, Ud.v.y, Ud.v.z, Ud.w.x, Ud.w.y, Ud.w.z};
        const double uu[6] = {U.v.x, U.v.y, U.v.z, U.w.x, U.w.y, U.w.z};
        int t = 0;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
          for (int c = r; c < 3; c++, t++) {
            Ia.A[t] = fma(-ud[r], uu[c], Ia.A[t]);
            Ia.C[t] = fma(-ud[3 + r], uu[3 + c], Ia.C[t]);
          }
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
          for (int c = 0; c < 3; c++) Ia.B[r * 3 + c] = fma(-ud[r], uu[3 + c], Ia.B[r * 3 + c]);
        Mot pa = sym6_mul_add(Ia, W.cb[i], W.pA[i]);
        pa = axpy6(u, Ud, pa);
        Sym6& P = W.IA[p];
#pragma unroll
        for (int k = 0; k < 6; k++) {
          P.A[k] += Ia.A[k];
          P.C[k] += Ia.C[k];
        }
#pragma unroll
        for (int k = 0; k < 9; k++) P.B[k] += Ia.B[k];
        W.pA[p] = add6(W.pA[p], pa);
      }
    } else {
      // free flyer (root only; enforced by the host)
      for (int k = 0; k < 6; k++) {
        W.Uv[iv + k] = sym6_mul(W.IA[i], W.Sw[iv + k]);
        W.uv[iv + k] = tau[J.vcol + k] - dot6(W.Sw[iv + k], W.pA[i]);
      }
      for (int r = 0; r < 6; r++)
        for (int c = 0; c <= r; c++) W.Lff[r * (r + 1) / 2 + c] = dot6(W.Sw[iv + r], W.Uv[iv + c]);
      chol6(W.Lff);
    }
  }
  const Mot a0{mk(-T.gravity(0), -T.gravity(1), -T.gravity(2)), mk(0, 0, 0)};
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, iv = J.ivx;
    Mot a = add6((p == 0) ? a0 : W.acc[p], W.cb[i]);
    if (J.nv == 1) {
      const double x = W.Dinv[i] * (W.uv[iv] - dot6(W.Uv[iv], a));
      a = axpy6(x, W.Sw[iv], a);
      qdd[J.vcol] = x;
    } else {
      double b[6];
      for (int k = 0; k < 6; k++) b[k] = W.uv[iv + k] - dot6(W.Uv[iv + k], a);
      chol6_solve(W.Lff, b);
      for (int k = 0; k < 6; k++) {
        a = axpy6(b[k], W.Sw[iv + k], a);
        qdd[J.vcol + k] = b[k];
      }
    }
    W.acc[i] = a;
  }
}

// y = M^-1 x (external order) from ABA's stored U, D^-1, S: the ABA recursion with zero
// velocity and zero gravity.
template <int MAXJ, class Tab>
__device__ void minv_solve(const Tab& T, DynWork<MAXJ>& W, const double* x, double* y) {
  const int nj = T.nj();
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  Mot* pAs = W.pA;  // reused as scratch: ABA's bias forces are no longer needed
  double* us = W.uv;
  for (int i = 1; i < nj; i++) pAs[i] = zero;
#pragma unroll
  for (int i = nj - 1; i >= 1; i--) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, iv = J.ivx;
    if (J.nv == 1) {
      const double u = x[J.vcol] - dot6(W.Sw[iv], pAs[i]);
      us[iv] = u;
      if (p > 0) pAs[p] = add6(pAs[p], add6(pAs[i], scale6(u * W.Dinv[i], W.Uv[iv])));
    } else {
      for (int k = 0; k < 6; k++) us[iv + k] = x[J.vcol + k] - dot6(W.Sw[iv + k], pAs[i]);
    }
  }
  Mot* as = W.cb;  // scratch accelerations
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, iv = J.ivx;
    Mot a = (p == 0) ? zero : as[p];
    if (J.nv == 1) {
      const double z = W.Dinv[i] * (us[iv] - dot6(W.Uv[iv], a));
      a = axpy6(z, W.Sw[iv], a);
      y[J.vcol] = z;
    } else {
      double b[6];
      for (int k = 0; k < 6; k++) b[k] = us[iv + k] - dot6(W.Uv[iv + k], a);
      chol6_solve(W.Lff, b);
      for (int k = 0; k < 6; k++) {
        a = axpy6(b[k], W.Sw[iv + k], a);
        y[J.vcol + k] = b[k];
      }
    }
    as[i] = a;
  }
}

// RNEA forward quantities (pose, S, v, a, I, I v) for given qdd.
template <int MAXJ, class Tab>
__device__ void rnea_forward(const Tab& T, const double* q, const double* qd, const double* qdd,
                             DynWork<MAXJ>& W) {
  const int nj = T.nj();
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  const Mot a0{mk(-T.gravity(0), -T.gravity(1), -T.gravity(2)), mk(0, 0, 0)};
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, iv = J.ivx;
    pose_and_S(J, i, q, W);
    const RBI Y = rbi_transport(local_rbi(J), W.oR[i], W.op[i]);
    W.Iw[i] = Y;
    Mot vJ = zero;
    Mot a = (p == 0) ? a0 : W.acc[p];
    for (int k = 0; k < J.nv; k++) {
      vJ = axpy6(qd[J.vcol + k], W.Sw[iv + k], vJ);
      a = axpy6(qdd[J.vcol + k], W.Sw[iv + k], a);
    }
    const Mot v = (p == 0) ? vJ : add6(W.vel[p], vJ);
    W.vel[i] = v;
    W.acc[i] = add_crossm(a, v, vJ);
    W.hY[i] = rbi_mul(Y, v);
  }
}

template <int MAXJ>
struct AdjScratch {
  Mot w[MAXJ], F[MAXJ], P[MAXJ], Q[MAXJ], R[MAXJ], T[MAXJ];
};

// Subtree sums of the RNEA body forces f = I a + v x* I v (world frame) into F[1..nj-1].
// They do not depend on the adjoint, so one evaluation serves any number of
// rnea_adjoint calls on the same forward quantities.
template <int MAXJ, class Tab>
__device__ void rnea_subtree_forces(const Tab& T, const DynWork<MAXJ>& W, Mot* F) {
  const int nj = T.nj();
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
#pragma unroll
  for (int i = 1; i < nj; i++) F[i] = rbi_mul_add(W.Iw[i], W.acc[i], add_crossf(zero, W.vel[i], W.hY[i]));
#pragma unroll
  for (int j = nj - 1; j >= 1; j--) {
    const int p = T.joint(j).parent;
    if (p > 0) F[p] = add6(F[p], F[j]);
  }
}

// Time derivative of a world-frame rigid-body inertia moving with twist v,
// Idot = v x* I - I (v x). It has the shape of a rigid-body inertia with zero mass: first
// moment hdot = m v_lin + w x h and rotational part 2 (v_lin . h) 1 - (h v_lin^T + v_lin h^T)
// + K + K^T with K = [w]x Ibar (I = [[m 1, -[h]x], [[h]x, Ibar]]).
__device__ __forceinline__ RBI rbi_rate(const RBI& Y, const Mot& v) {
  const V3 w = v.w, u = v.v, h = Y.h;
  const double* I = Y.I;
  RBI D;
  D.m = 0;
  D.h = add_cross(Y.m * u, w, h);
  const double k00 = -w.z * I[1] + w.y * I[2], k01 = -w.z * I[3] + w.y * I[4], k02 = -w.z * I[4] + w.y * I[5];
  const double k10 = w.z * I[0] - w.x * I[2], k11 = w.z * I[1] - w.x * I[4], k12 = w.z * I[2] - w.x * I[5];
  const double k20 = -w.y * I[0] + w.x * I[1], k21 = -w.y * I[1] + w.x * I[3], k22 = -w.y * I[2] + w.x * I[4];
  const double uh = 2 * dot(u, h);
  D.I[0] = uh - 2 * h.x * u.x + 2 * k00;
  D.I[1] = -(h.x * u.y + u.x * h.y) + k01 + k10;
  D.I[2] = -(h.x * u.z + u.x * h.z) + k02 + k20;
  D.I[3] = uh - 2 * h.y * u.y + 2 * k11;
  D.I[4] = -(h.y * u.z + u.y * h.z) + k12 + k21;
  D.I[5] = uh - 2 * h.z * u.z + 2 * k22;
  return D;
}

// Subtree composites for the analytic RNEA derivatives, per joint i over subtree(i): F the
// RNEA forces, H the momenta I v, Ib the inertias (CRBA's composite), Db their rates
// (rbi_rate); per tree column c of joint i: P_c = Ib_i S_c and Q_c = Db_i S_c - S_c x* H_i.
template <int MAXJ>
struct DerivComposites {
  static constexpr int MAXV = MAXJ + 5;
  Mot F[MAXJ], H[MAXJ];
  RBI Ib[MAXJ], Db[MAXJ];
  Mot P[MAXV], Q[MAXV];
};

template <int MAXJ, class Tab>
__device__ void deriv_composites(const Tab& T, const DynWork<MAXJ>& W, DerivComposites<MAXJ>& C) {
  const int nj = T.nj();
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
#pragma unroll
  for (int i = 1; i < nj; i++) {
    C.F[i] = rbi_mul_add(W.Iw[i], W.acc[i], add_crossf(zero, W.vel[i], W.hY[i]));
    C.H[i] = W.hY[i];
    C.Ib[i] = W.Iw[i];
    C.Db[i] = rbi_rate(W.Iw[i], W.vel[i]);
  }
#pragma unroll
  for (int j = nj - 1; j >= 1; j--) {
    const int p = T.joint(j).parent;
    if (p > 0) {
      C.F[p] = add6(C.F[p], C.F[j]);
      C.H[p] = add6(C.H[p], C.H[j]);
      C.Ib[p] = rbi_add(C.Ib[p], C.Ib[j]);
      C.Db[p] = rbi_add(C.Db[p], C.Db[j]);
    }
  }
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    for (int k = 0; k < J.nv; k++) {
      const Mot S = W.Sw[J.ivx + k];
      C.P[J.ivx + k] = rbi_mul(C.Ib[i], S);
      C.Q[J.ivx + k] = add6(rbi_mul(C.Db[i], S), scale6(-1.0, add_crossf(zero, S, C.H[i])));
    }
  }
}

// Reverse-mode RNEA sweep over the forward quantities in W (acc must be the world
// accelerations the torques were computed with) and the subtree forces in A.F (from
// rnea_subtree_forces; read only). taubar and the outputs are external order; any output
// pointer may be null; outputs are scaled by `sign`. W is not modified.
template <int MAXJ, class Tab>
__device__ void rnea_adjoint(const Tab& T, const DynWork<MAXJ>& W, AdjScratch<MAXJ>& A,
                             const double* taubar, double* qbar, double* qdbar, double* qddbar, double sign) {
  const int nj = T.nj();
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  const Mot a0{mk(-T.gravity(0), -T.gravity(1), -T.gravity(2)), mk(0, 0, 0)};
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, iv = J.ivx;
    Mot wi = (p == 0) ? zero : A.w[p];
    for (int k = 0; k < J.nv; k++) wi = axpy6(taubar[J.vcol + k], W.Sw[iv + k], wi);
    A.w[i] = wi;
    const RBI& Y = W.Iw[i];
    const Mot v = W.vel[i];
    const Mot Pw = rbi_mul(Y, wi);
    A.P[i] = Pw;
    A.Q[i] = add_crossf(zero, v, Pw);
    A.R[i] = add_crossf(zero, wi, W.hY[i]);
    A.T[i] = rbi_mul(Y, add_crossm(zero, v, wi));
  }
#pragma unroll
  for (int j = nj - 1; j >= 1; j--) {
    const DJoint& J = T.joint(j);
    const int p = J.parent, iv = J.ivx;
    const Mot P = A.P[j], Q = A.Q[j], R = A.R[j], T = A.T[j], Fj = A.F[j];
    const Mot vl = (p == 0) ? zero : W.vel[p];
    const Mot al = (p == 0) ? a0 : W.acc[p];
    const Mot Wl = (p == 0) ? zero : A.w[p];
    if (qbar) {
      const Mot Z = add6(add6(scale6(-1.0, Q), add_crossf(zero, vl, P)), add6(R, T));
      Mot G = add_crossf(zero, vl, Z);
      G = add6(G, scale6(-1.0, add_crossf(zero, al, P)));
      G = add6(G, scale6(-1.0, add_crossf(zero, Wl, Fj)));
      for (int k = 0; k < J.nv; k++) qbar[J.vcol + k] = sign * dot6(W.Sw[iv + k], G);
    }
    if (qdbar) {
      const Mot vsum = add6(vl, W.vel[j]);
      Mot G = add6(Q, scale6(-1.0, add_crossf(zero, vsum, P)));
      G = add6(G, scale6(-1.0, add6(R, T)));
      for (int k = 0; k < J.nv; k++) qdbar[J.vcol + k] = sign * dot6(W.Sw[iv + k], G);
    }
    if (qddbar)
      for (int k = 0; k < J.nv; k++) qddbar[J.vcol + k] = sign * dot6(W.Sw[iv + k], P);
    if (p > 0) {
      A.P[p] = add6(A.P[p], P);
      A.Q[p] = add6(A.Q[p], Q);
      A.R[p] = add6(A.R[p], R);
      A.T[p] = add6(A.T[p], T);
    }
  }
}

}  // namespace sgdyn
