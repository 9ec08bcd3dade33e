// Three lanes per environment, one per Cartesian axis ("xyz teams"), for sweeps whose batch
// leaves FP64 schedulers idle.
//
// A warp issues at most one FP64 instruction per ~64 cycles whatever its active lanes, so a
// batch of one environment per thread with fewer warps than FP64 schedulers (the 4096-env
// rollout: 128 warps for 608 schedulers) is bound by each warp's own instruction count.
// Here lane k of a team holds component k of every spatial vector (linear and angular part)
// and row k of every 3x3 block (world rotations, rigid-body and articulated inertias), so
// matrix-vector products, cross products and rank-one updates cost each lane a third of the
// FP64 instructions; a team gathers the other components with warp shuffles, which use no
// FP64 issue slots. Dot products end in a fixed-order sum over the team, and every scalar
// (joint coordinates, D, D^-1, u, q'') is computed identically on the three lanes, so the
// lanes never disagree. Ten teams share a warp; lanes 30 and 31 shadow lanes 27 and 28 and
// store nothing.
//
// The recursions are those of aba_forward (world-frame ABA): pass 1 poses, motion subspaces,
// world inertias, velocities and bias forces; pass 2 articulated inertias
// IA_p += IA - U D^-1 U^T, pA_p += pA + Ia c + U D^-1 u; pass 3 accelerations
// (pinocchio_model.cpp:221-226). Joints with one degree of freedom, plus a free-flyer root:
// its six motion-subspace columns are distributed like any motion, and its 6x6 D = S^T IA S
// is factored (chol6) identically on the three lanes.
#pragma once
#include "kernels.h"
#include "spatial.cuh"
#include "step_kernel.cuh"
#include "diff_kernels.cuh"

namespace sgdyn {

struct Team3 {
  int k, k1, k2;  // this lane's axis and the next two (cyclic)
  int base;       // first lane of the team
  bool valid;     // false on the two shadow lanes of a warp and on teams past the batch

  __device__ __forceinline__ double at(double x, int j) const { return __shfl_sync(0xffffffffu, x, base + j); }
  __device__ __forceinline__ V3 all(double x) const { return mk(at(x, 0), at(x, 1), at(x, 2)); }
  // sum over the team in a fixed order: the same bits on all three lanes
  __device__ __forceinline__ double sum(double x) const { return (at(x, 0) + at(x, 1)) + at(x, 2); }
  // component k of a x b, both distributed
  __device__ __forceinline__ double cross(double a, double b) const {
    return fma(at(a, k1), at(b, k2), -at(a, k2) * at(b, k1));
  }
  // component k of a full 3-vector held by every lane
  __device__ __forceinline__ double pick(V3 v) const { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
};

__device__ __forceinline__ Team3 team3_of_lane(int lane) {
  Team3 t;
  const int l = lane < 30 ? lane : lane - 3;
  t.base = l / 3 * 3;
  t.k = l - t.base;
  t.k1 = t.k == 2 ? 0 : t.k + 1;
  t.k2 = t.k == 0 ? 2 : t.k - 1;
  t.valid = lane < 30;
  return t;
}

// Row k of a row-major 3x3 table matrix.
__device__ __forceinline__ V3 row_of(const double* R, int k) { return mk(R[3 * k], R[3 * k + 1], R[3 * k + 2]); }
// Row k of a symmetric 3x3 stored as xx xy xz yy yz zz.
__device__ __forceinline__ V3 sym_row(const double* S, int k) {
  return k == 0 ? mk(S[0], S[1], S[2]) : (k == 1 ? mk(S[1], S[3], S[4]) : mk(S[2], S[4], S[5]));
}
// Row vector r times the matrix with rows m0, m1, m2.
__device__ __forceinline__ V3 row_mul(V3 r, V3 m0, V3 m1, V3 m2) {
  return mk(fma(r.z, m2.x, fma(r.y, m1.x, r.x * m0.x)), fma(r.z, m2.y, fma(r.y, m1.y, r.x * m0.y)),
            fma(r.z, m2.z, fma(r.y, m1.z, r.x * m0.z)));
}

// Per-lane state of one environment's ABA (component k / row k of every quantity).
template <int MAXJ>
struct Aba3Work {
  V3 oR[MAXJ];                // row k of the joint's world rotation
  double op[MAXJ];            // component k of its world position
  double Sl[MAXJ], Sa[MAXJ];  // motion subspace (one column per joint)
  double vl[MAXJ], va[MAXJ], cl[MAXJ], ca[MAXJ], pl[MAXJ], pa[MAXJ], al[MAXJ], aa[MAXJ];
  V3 A[MAXJ], B[MAXJ], BT[MAXJ], C[MAXJ];  // articulated inertia [[A, B], [B^T, C]], row k
  double Ul[MAXJ], Ua[MAXJ], u[MAXJ], Dinv[MAXJ];
  // free-flyer root: its six subspace columns, U = IA S, u, and the Cholesky factor of D
  double Sl6[6], Sa6[6], Ul6[6], Ua6[6], u6[6], Lff[21];
};

// World-frame ABA of one environment on a team: qdd (external order) from q, qd, tau, all
// three replicated on the lanes.
template <int MAXJ, class Tab>
__device__ __forceinline__ void aba3(const Tab& T, const Team3& tm, const double* q, const double* qd,
                                     const double* tau, double* qdd, Aba3Work<MAXJ>& W) {
  const int nj = T.nj(), k = tm.k;
  const V3 ek = mk(k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0);
  // ---- pass 1: root to leaves ----
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    const int p = J.parent;
    const bool rot_id = (J.flags & JF_ROT_IDENTITY) != 0;
    const V3 ppl = mk(J.p[0], J.p[1], J.p[2]);
    const V3 Rp = p == 0 ? ek : W.oR[p];  // row k of the parent's world rotation
    const double x = q[J.qcol];
    V3 Ro;      // row k of this joint's world rotation
    double po;  // component k of its world position
    double u;   // component k of its world axis
    const bool ff = J.kind == JK_FREEFLYER;  // the root (p == 0), as the host checks
    if (ff) {
      const int c0 = J.qcol;
      const M3 RJ = quat_to_R(q[c0 + 3], q[c0 + 4], q[c0 + 5], q[c0 + 6]);
      const V3 t = mk(q[c0], q[c0 + 1], q[c0 + 2]);
      const V3 rk = rot_id ? ek : row_of(J.R, k);  // row k of the placement rotation
      Ro = row_mul(rk, row_of(RJ.a, 0), row_of(RJ.a, 1), row_of(RJ.a, 2));
      po = fma(rk.z, t.z, fma(rk.y, t.y, fma(rk.x, t.x, tm.pick(ppl))));
      u = 0.0;
    } else if (J.axis_kind == AX_Z) {
      const V3 B = rot_id ? Rp : row_mul(Rp, row_of(J.R, 0), row_of(J.R, 1), row_of(J.R, 2));
      const double o = p == 0 ? tm.pick(ppl) : fma(Rp.z, ppl.z, fma(Rp.y, ppl.y, fma(Rp.x, ppl.x, W.op[p])));
      if (J.kind == JK_PRISMATIC) {
        Ro = B;
        po = fma(x, B.z, o);
      } else {
        double s, c;
        sincos(x, &s, &c);
        Ro = mk(fma(c, B.x, s * B.y), fma(c, B.y, -s * B.x), B.z);
        po = o;
      }
      u = Ro.z;
    } else {
      const V3 ax = mk(J.axis[0], J.axis[1], J.axis[2]);
      V3 pli = ppl;
      M3 Rli;
      if (J.kind == JK_PRISMATIC) {
#pragma unroll
        for (int t = 0; t < 9; t++) Rli.a[t] = J.R[t];
        pli = rot_id ? axpy(x, ax, ppl) : mul_add(Rli, x * ax, ppl);
      } else {
        double s, c;
        sincos(x, &s, &c);
        const M3 RJ = rodrigues(ax, s, c);
        if (rot_id) {
          Rli = RJ;
        } else {
          M3 Rpl;
#pragma unroll
          for (int t = 0; t < 9; t++) Rpl.a[t] = J.R[t];
          Rli = mul(Rpl, RJ);
        }
      }
      Ro = row_mul(Rp, row_of(Rli.a, 0), row_of(Rli.a, 1), row_of(Rli.a, 2));
      po = p == 0 ? tm.pick(pli) : fma(Rp.z, pli.z, fma(Rp.y, pli.y, fma(Rp.x, pli.x, W.op[p])));
      u = fma(Ro.z, ax.z, fma(Ro.y, ax.y, Ro.x * ax.x));
    }
    W.oR[i] = Ro;
    W.op[i] = po;
    double Sl, Sa;
    double vJl, vJa;
    if (ff) {  // columns (Ro e_c, 0) and (po x Ro e_c, Ro e_c); component k of Ro e_c is Ro[k][c]
      const double r[3] = {Ro.x, Ro.y, Ro.z};
      vJl = vJa = 0.0;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        W.Sl6[c] = r[c];
        W.Sa6[c] = 0.0;
        W.Sl6[3 + c] = tm.cross(po, r[c]);
        W.Sa6[3 + c] = r[c];
      }
#pragma unroll
      for (int c = 0; c < 6; c++) {
        vJl = fma(qd[J.vcol + c], W.Sl6[c], vJl);
        vJa = fma(qd[J.vcol + c], W.Sa6[c], vJa);
      }
      Sl = Sa = 0.0;
    } else {
      if (J.kind == JK_PRISMATIC) {
        Sl = u;
        Sa = 0.0;
      } else {
        Sl = tm.cross(po, u);
        Sa = u;
      }
      vJl = qd[J.vcol] * Sl;
      vJa = qd[J.vcol] * Sa;
    }
    W.Sl[i] = Sl;
    W.Sa[i] = Sa;
    // world inertia (m, s = R h + m p, I') with I'_kj = (R I R^T)_kj + d delta_kj - p_k s_j - hr_k p_j,
    // d = m |p|^2 + 2 hr.p, hr = R h (rbi_transport restated per row)
    const double m = J.m;
    const double hr = fma(Ro.z, J.h[2], fma(Ro.y, J.h[1], Ro.x * J.h[0]));
    const double sk = fma(m, po, hr);
    const double d = fma(m, tm.sum(po * po), 2.0 * tm.sum(hr * po));
    const V3 Tk = row_mul(Ro, sym_row(J.I, 0), sym_row(J.I, 1), sym_row(J.I, 2));  // row k of R I
    const V3 R0 = mk(tm.at(Ro.x, 0), tm.at(Ro.y, 0), tm.at(Ro.z, 0));
    const V3 R1 = mk(tm.at(Ro.x, 1), tm.at(Ro.y, 1), tm.at(Ro.z, 1));
    const V3 R2 = mk(tm.at(Ro.x, 2), tm.at(Ro.y, 2), tm.at(Ro.z, 2));
    const V3 sv = tm.all(sk), pv = tm.all(po);
    V3 Ik;
    Ik.x = fma(-hr, pv.x, fma(-po, sv.x, dot(Tk, R0) + (k == 0 ? d : 0.0)));
    Ik.y = fma(-hr, pv.y, fma(-po, sv.y, dot(Tk, R1) + (k == 1 ? d : 0.0)));
    Ik.z = fma(-hr, pv.z, fma(-po, sv.z, dot(Tk, R2) + (k == 2 ? d : 0.0)));
    // velocity, momentum (f, n) = Y v, bias force v x* Y v, velocity-product acceleration
    const double vl = p == 0 ? vJl : W.vl[p] + vJl;
    const double va = p == 0 ? vJa : W.va[p] + vJa;
    W.vl[i] = vl;
    W.va[i] = va;
    const double fl = fma(m, vl, -tm.cross(sk, va));   // m v - s x w
    const double fa = dot(Ik, tm.all(va)) + tm.cross(sk, vl);  // I' w + s x v
    W.pl[i] = tm.cross(va, fl);                         // w x f
    W.pa[i] = tm.cross(va, fa) + tm.cross(vl, fl);      // w x n + v x f
    W.cl[i] = tm.cross(va, vJl) + tm.cross(vl, vJa);    // w x vJ_lin + v x vJ_ang
    W.ca[i] = tm.cross(va, vJa);
    // the articulated inertia starts as the rigid-body inertia [[m 1, -[s]x], [[s]x, I']]
    W.A[i] = m * ek;
    const V3 Bk = k == 0 ? mk(0.0, sv.z, -sv.y) : (k == 1 ? mk(-sv.z, 0.0, sv.x) : mk(sv.y, -sv.x, 0.0));
    W.B[i] = Bk;
    W.BT[i] = -Bk;
    W.C[i] = Ik;
  }
  // ---- pass 2: leaves to root ----
#pragma unroll
  for (int i = nj - 1; i >= 1; i--) {
    const DJoint& J = T.joint(i);
    const int p = J.parent;
    const V3 A = W.A[i], B = W.B[i], BT = W.BT[i], C = W.C[i];
    if (J.kind == JK_FREEFLYER) {  // root: U = IA S per column, D = S^T U factored, u
#pragma unroll
      for (int c = 0; c < 6; c++) {
        const V3 Slv = tm.all(W.Sl6[c]), Sav = tm.all(W.Sa6[c]);
        W.Ul6[c] = dot(A, Slv) + dot(B, Sav);
        W.Ua6[c] = dot(BT, Slv) + dot(C, Sav);
        W.u6[c] = tau[J.vcol + c] - tm.sum(fma(W.Sl6[c], W.pl[i], W.Sa6[c] * W.pa[i]));
      }
#pragma unroll
      for (int r = 0; r < 6; r++)
#pragma unroll
        for (int c = 0; c <= r; c++) W.Lff[r * (r + 1) / 2 + c] = tm.sum(fma(W.Sl6[r], W.Ul6[c], W.Sa6[r] * W.Ua6[c]));
      chol6(W.Lff);
      continue;
    }
    const V3 Slv = tm.all(W.Sl[i]), Sav = tm.all(W.Sa[i]);
    const double Ul = dot(A, Slv) + dot(B, Sav);
    const double Ua = dot(BT, Slv) + dot(C, Sav);
    const double D = tm.sum(fma(W.Sl[i], Ul, W.Sa[i] * Ua));
    const double u = tau[J.vcol] - tm.sum(fma(W.Sl[i], W.pl[i], W.Sa[i] * W.pa[i]));
    const double di = 1.0 / D;
    W.Ul[i] = Ul;
    W.Ua[i] = Ua;
    W.u[i] = u;
    W.Dinv[i] = di;
    if (p > 0) {
      const double Udl = di * Ul, Uda = di * Ua;
      const V3 Ulv = tm.all(Ul), Uav = tm.all(Ua);
      const V3 Ia = mk(fma(-Udl, Ulv.x, A.x), fma(-Udl, Ulv.y, A.y), fma(-Udl, Ulv.z, A.z));
      const V3 Ib = mk(fma(-Udl, Uav.x, B.x), fma(-Udl, Uav.y, B.y), fma(-Udl, Uav.z, B.z));
      const V3 Ibt = mk(fma(-Uda, Ulv.x, BT.x), fma(-Uda, Ulv.y, BT.y), fma(-Uda, Ulv.z, BT.z));
      const V3 Ic = mk(fma(-Uda, Uav.x, C.x), fma(-Uda, Uav.y, C.y), fma(-Uda, Uav.z, C.z));
      const V3 clv = tm.all(W.cl[i]), cav = tm.all(W.ca[i]);
      const double pal = fma(u, Udl, dot(Ia, clv) + dot(Ib, cav) + W.pl[i]);
      const double paa = fma(u, Uda, dot(Ibt, clv) + dot(Ic, cav) + W.pa[i]);
      W.A[p] = W.A[p] + Ia;
      W.B[p] = W.B[p] + Ib;
      W.BT[p] = W.BT[p] + Ibt;
      W.C[p] = W.C[p] + Ic;
      W.pl[p] += pal;
      W.pa[p] += paa;
    }
  }
  // ---- pass 3: root to leaves ----
  const double gk = -T.gravity(k);
#pragma unroll
  for (int i = 1; i < nj; i++) {
    const DJoint& J = T.joint(i);
    const int p = J.parent;
    double al = (p == 0 ? gk : W.al[p]) + W.cl[i];
    double aa = (p == 0 ? 0.0 : W.aa[p]) + W.ca[i];
    if (J.kind == JK_FREEFLYER) {
      double b[6];
#pragma unroll
      for (int c = 0; c < 6; c++) b[c] = W.u6[c] - tm.sum(fma(W.Ul6[c], al, W.Ua6[c] * aa));
      chol6_solve(W.Lff, b);
#pragma unroll
      for (int c = 0; c < 6; c++) {
        al = fma(b[c], W.Sl6[c], al);
        aa = fma(b[c], W.Sa6[c], aa);
        qdd[J.vcol + c] = b[c];
      }
      W.al[i] = al;
      W.aa[i] = aa;
      continue;
    }
    const double x = W.Dinv[i] * (W.u[i] - tm.sum(fma(W.Ul[i], al, W.Ua[i] * aa)));
    al = fma(x, W.Sl[i], al);
    aa = fma(x, W.Sa[i], aa);
    W.al[i] = al;
    W.aa[i] = aa;
    qdd[J.vcol] = x;
  }
}

// Forward rollout (as rollout_forward_env) with a team of three lanes per environment: q,
// qd, tau and the checkpoints are replicated on the lanes; lane 0 stores.
template <int MAXJ, class Tab>
__device__ __forceinline__ void rollout_forward3_env(const Tab& T, const Team3& tm, const RolloutArgs& a,
                                                     const int64_t e) {
  constexpr int MAXV = MAXJ + 5, MAXQ = MAXJ + 6;
  const int nv = T.nv(), nq = T.nq_ext();
  const int64_t n = a.n;
  const bool st = tm.valid && tm.k == 0;
  double q[MAXQ], qd[MAXV], tau[MAXV], qdd[MAXV];
  for (int c = 0; c < nq; c++) q[c] = a.q0[e * nq + c];
  for (int c = 0; c < nv; c++) qd[c] = a.qd0[e * nv + c];
  Aba3Work<MAXJ> W;
  for (int t = 0; t < a.T; t++) {
    if (a.q_ckpt && t % a.K == 0 && st) {
      const int64_t s = t / a.K;
      for (int c = 0; c < nq; c++) a.q_ckpt[(s * n + e) * nq + c] = q[c];
      for (int c = 0; c < nv; c++) a.qd_ckpt[(s * n + e) * nv + c] = qd[c];
    }
    for (int c = 0; c < nv; c++) tau[c] = a.tau[(int64_t(t) * n + e) * nv + c];
    aba3<MAXJ>(T, tm, q, qd, tau, qdd, W);
    for (int c = 0; c < nv; c++) qd[c] = fma(a.dt, qdd[c], qd[c]);
    euler_positions(T, q, qd, a.dt);  // a free flyer moves on SE(3), identically on the lanes
  }
  if (st) {
    for (int c = 0; c < nq; c++) a.qT[e * nq + c] = q[c];
    for (int c = 0; c < nv; c++) a.qdT[e * nv + c] = qd[c];
  }
}

// Batched forward dynamics (computeForwardDynamics, pinocchio_model.cpp:221-226) with a team
// of three lanes per environment: q, qd, tau read through the call's layout, lane 0 writes
// qdd.
template <int MAXJ, class Tab>
__device__ __forceinline__ void aba3_env(const Tab& T, const Team3& tm, const StepArgs& a, const int64_t e) {
  constexpr int MAXV = MAXJ + 5, MAXQ = MAXJ + 6;
  const int nv = T.nv(), nq = T.nq_ext();
  double q[MAXQ], qd[MAXV], tau[MAXV], qdd[MAXV];
  for (int c = 0; c < nq; c++) q[c] = ldv(a.q, e, c);
  for (int c = 0; c < nv; c++) qd[c] = ldv(a.qd, e, c);
  for (int c = 0; c < nv; c++) tau[c] = ldv(a.tau, e, c);
  Aba3Work<MAXJ> W;
  aba3<MAXJ>(T, tm, q, qd, tau, qdd, W);
  if (tm.valid && tm.k == 0)
    for (int c = 0; c < nv; c++) stv(a.qdd_out, e, c, qdd[c]);
}

template <int MAXJ>
__global__ void __launch_bounds__(32) aba3_kernel(const DModel* __restrict__ model, const StepArgs a) {
  Team3 tm = team3_of_lane(threadIdx.x);
  const int64_t e0 = int64_t(blockIdx.x) * 10 + tm.base / 3;
  tm.valid = tm.valid && e0 < a.n;
  aba3_env<MAXJ>(RuntimeTab{model}, tm, a, e0 < a.n ? e0 : a.n - 1);
}

// ---- reverse rollout with three lanes per environment ----------------------------------
// The same reverse step as rollout_reverse_env (M^-1 solve through ABA's factorisation, then
// the world-frame RNEA adjoint of diff_core.cuh, then the semi-implicit Euler adjoint), each
// lane reading its components of the stored intermediates (the stash is one field per
// component, environments contiguous) and computing its components of the adjoint
// quantities w, P = Y w, Q = v x* P, R = w x* Y v, T = Y (v x w).
template <int MAXJ>
struct Rev3Work {
  double Sl[MAXJ], Sa[MAXJ], Ul[MAXJ], Ua[MAXJ], Dinv[MAXJ];
  double vl[MAXJ], va[MAXJ], al[MAXJ], aa[MAXJ], hl[MAXJ], ha[MAXJ], Fl[MAXJ], Fa[MAXJ];
  double m[MAXJ], h[MAXJ];  // mass and component k of the first moment of the world inertia
  V3 I[MAXJ];               // row k of its rotational inertia
  // scratch of the solve and of the adjoint sweep
  double us[MAXJ], xl[MAXJ], xa[MAXJ];
  double wl[MAXJ], wa[MAXJ], Pl[MAXJ], Pa[MAXJ], Ql[MAXJ], Qa[MAXJ], Rl[MAXJ], Ra[MAXJ], Tl[MAXJ], Ta[MAXJ];
  // free-flyer root: its six subspace columns and U, the Cholesky factor of its D, the
  // step's displacement dt qd' and the solve's u
  double Sl6[6], Sa6[6], Ul6[6], Ua6[6], Lff[21], ffd[6], us6[6];
};

// Component k of x x* f = (x_ang x f_lin, x_ang x f_ang + x_lin x f_lin).
__device__ __forceinline__ void crossf3(const Team3& tm, double xl, double xa, double fl, double fa, double& ol,
                                        double& oa) {
  ol = tm.cross(xa, fl);
  oa = tm.cross(xa, fa) + tm.cross(xl, fl);
}
// Component k of Y x for the world inertia (m, h, I): (m x_lin - h x x_ang, I x_ang + h x x_lin).
__device__ __forceinline__ void rbi3(const Team3& tm, double m, double h, V3 Irow, double xl, double xa, double& ol,
                                     double& oa) {
  ol = fma(m, xl, -tm.cross(h, xa));
  oa = dot(Irow, tm.all(xa)) + tm.cross(h, xl);
}

template <int MAXJ, class Tab>
__device__ __forceinline__ void rollout_reverse3_env(const Tab& T, const Team3& tm, const RolloutArgs& a,
                                                     const int64_t e) {
  constexpr int MAXV = MAXJ + 5, MAXQ = MAXJ + 6;
  const int nv = T.nv(), nq = T.nq_ext(), nj = T.nj(), k = tm.k;
  const int64_t n = a.n;
  const int64_t per_step = stash_doubles_per_step(nj, nq, nv);
  const int nseg = (a.T + a.K - 1) / a.K;
  const bool last = a.s_lo + a.s_cnt == nseg;
  const bool st = tm.valid && k == 0;
  const double* qin = last ? a.qT_bar : a.q0_bar;
  const double* qdin = last ? a.qdT_bar : a.qd0_bar;
  double qb[MAXQ], qdb[MAXV], lam[MAXV];
  for (int c = 0; c < nq; c++) qb[c] = qin ? qin[e * nq + c] : 0.0;
  for (int c = 0; c < nv; c++) qdb[c] = qdin ? qdin[e * nv + c] : 0.0;
  Rev3Work<MAXJ> W;
  const double gk = -T.gravity(k);
  for (int s = a.s_lo + a.s_cnt - 1; s >= a.s_lo; s--) {
    const int t0 = s * a.K, t1 = min(a.T, t0 + a.K);
    for (int t = t1 - 1; t >= t0; t--) {
      const double* base = a.scratch + (int64_t(s - a.s_lo) * a.K + (t - t0)) * per_step * n;
      auto ld = [&](int64_t f) { return base[f * n + e]; };
      // this lane's components of the stored intermediates (stash_io's layout)
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const int iv = T.joint(i).ivx;
        const int64_t jb = 12 * int64_t(nv) + int64_t(i - 1) * 35;
        if (T.joint(i).kind == JK_FREEFLYER) {
#pragma unroll
          for (int c = 0; c < 6; c++) {
            W.Sl6[c] = ld(6 * (iv + c) + k);
            W.Sa6[c] = ld(6 * (iv + c) + 3 + k);
            W.Ul6[c] = ld(6 * nv + 6 * (iv + c) + k);
            W.Ua6[c] = ld(6 * nv + 6 * (iv + c) + 3 + k);
          }
          const int64_t tb = 12 * int64_t(nv) + int64_t(nj - 1) * 35;
#pragma unroll
          for (int c = 0; c < 21; c++) W.Lff[c] = ld(tb + c);
#pragma unroll
          for (int c = 0; c < 6; c++) W.ffd[c] = ld(tb + 21 + c);
          W.Sl[i] = W.Sa[i] = W.Ul[i] = W.Ua[i] = 0.0;
        } else {
          W.Sl[i] = ld(6 * iv + k);
          W.Sa[i] = ld(6 * iv + 3 + k);
          W.Ul[i] = ld(6 * nv + 6 * iv + k);
          W.Ua[i] = ld(6 * nv + 6 * iv + 3 + k);
        }
        W.Dinv[i] = ld(jb);
        W.vl[i] = ld(jb + 1 + k);
        W.va[i] = ld(jb + 4 + k);
        W.al[i] = ld(jb + 7 + k);
        W.aa[i] = ld(jb + 10 + k);
        W.hl[i] = ld(jb + 13 + k);
        W.ha[i] = ld(jb + 16 + k);
        W.m[i] = ld(jb + 19);
        W.h[i] = ld(jb + 20 + k);
        const int r0 = k == 0 ? 0 : (k == 1 ? 1 : 2), r1 = k == 0 ? 1 : (k == 1 ? 3 : 4),
                  r2 = k == 0 ? 2 : (k == 1 ? 4 : 5);
        W.I[i] = mk(ld(jb + 23 + r0), ld(jb + 23 + r1), ld(jb + 23 + r2));
        W.Fl[i] = ld(jb + 29 + k);
        W.Fa[i] = ld(jb + 32 + k);
      }
      // q' = q (+) dt qd' and qd' = qd + dt qdd, reversed: qdd_bar = dt qd'_bar; a free
      // flyer's block of qb holds its tangent adjoint (identically on the three lanes)
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
        if (J.kind != JK_FREEFLYER) {
          qdb[J.vcol] = fma(a.dt, qb[J.qcol], qdb[J.vcol]);
          continue;
        }
        const int qc = J.qcol, vc = J.vcol;
        const Mot g{mk(qb[qc], qb[qc + 1], qb[qc + 2]), mk(qb[qc + 3], qb[qc + 4], qb[qc + 5])};
        Mot vb{mk(qdb[vc], qdb[vc + 1], qdb[vc + 2]), mk(qdb[vc + 3], qdb[vc + 4], qdb[vc + 5])};
        const Mot gq = free_flyer_integrate_adjoint(
            Mot{mk(W.ffd[0], W.ffd[1], W.ffd[2]), mk(W.ffd[3], W.ffd[4], W.ffd[5])}, g, a.dt, vb);
        qb[qc] = gq.v.x; qb[qc + 1] = gq.v.y; qb[qc + 2] = gq.v.z;
        qb[qc + 3] = gq.w.x; qb[qc + 4] = gq.w.y; qb[qc + 5] = gq.w.z;
        qdb[vc] = vb.v.x; qdb[vc + 1] = vb.v.y; qdb[vc + 2] = vb.v.z;
        qdb[vc + 3] = vb.w.x; qdb[vc + 4] = vb.w.y; qdb[vc + 5] = vb.w.z;
      }
      // lam = M^-1 (dt qd'_bar): the ABA recursion with zero velocity and gravity
#pragma unroll
      for (int i = 1; i < nj; i++) W.xl[i] = W.xa[i] = 0.0;
#pragma unroll
      for (int i = nj - 1; i >= 1; i--) {
        const DJoint& J = T.joint(i);
        const int p = J.parent;
        if (J.kind == JK_FREEFLYER) {  // the root: no parent to pass to
#pragma unroll
          for (int c = 0; c < 6; c++)
            W.us6[c] = a.dt * qdb[J.vcol + c] - tm.sum(fma(W.Sl6[c], W.xl[i], W.Sa6[c] * W.xa[i]));
          continue;
        }
        const double u = a.dt * qdb[J.vcol] - tm.sum(fma(W.Sl[i], W.xl[i], W.Sa[i] * W.xa[i]));
        W.us[i] = u;
        if (p > 0) {
          const double ud = u * W.Dinv[i];
          W.xl[p] += fma(ud, W.Ul[i], W.xl[i]);
          W.xa[p] += fma(ud, W.Ua[i], W.xa[i]);
        }
      }
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
        const int p = J.parent;
        const double pl = p == 0 ? 0.0 : W.xl[p], pa = p == 0 ? 0.0 : W.xa[p];
        if (J.kind == JK_FREEFLYER) {  // the root: zero parent acceleration
          double b[6];
#pragma unroll
          for (int c = 0; c < 6; c++) b[c] = W.us6[c];
          chol6_solve(W.Lff, b);
          double xl = 0.0, xa = 0.0;
#pragma unroll
          for (int c = 0; c < 6; c++) {
            xl = fma(b[c], W.Sl6[c], xl);
            xa = fma(b[c], W.Sa6[c], xa);
            lam[J.vcol + c] = b[c];
          }
          W.xl[i] = xl;
          W.xa[i] = xa;
          continue;
        }
        const double z = W.Dinv[i] * (W.us[i] - tm.sum(fma(W.Ul[i], pl, W.Ua[i] * pa)));
        W.xl[i] = fma(z, W.Sl[i], pl);  // accelerations of the solve (the bias forces are spent)
        W.xa[i] = fma(z, W.Sa[i], pa);
        lam[J.vcol] = z;
      }
      if (st)
        for (int c = 0; c < nv; c++) a.tau_bar[(int64_t(t) * n + e) * nv + c] = lam[c];
      // RNEA adjoint at lam, scaled by -1 (ABA's adjoint): root to leaves ...
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
        const int p = J.parent;
        double wl, wa;
        if (J.kind == JK_FREEFLYER) {  // the root
          wl = wa = 0.0;
#pragma unroll
          for (int c = 0; c < 6; c++) {
            wl = fma(lam[J.vcol + c], W.Sl6[c], wl);
            wa = fma(lam[J.vcol + c], W.Sa6[c], wa);
          }
        } else {
          const double x = lam[J.vcol];
          wl = p == 0 ? x * W.Sl[i] : fma(x, W.Sl[i], W.wl[p]);
          wa = p == 0 ? x * W.Sa[i] : fma(x, W.Sa[i], W.wa[p]);
        }
        W.wl[i] = wl;
        W.wa[i] = wa;
        double Pl, Pa, Ql, Qa, Rl, Ra, cl, ca, Tl, Ta;
        rbi3(tm, W.m[i], W.h[i], W.I[i], wl, wa, Pl, Pa);
        crossf3(tm, W.vl[i], W.va[i], Pl, Pa, Ql, Qa);
        crossf3(tm, wl, wa, W.hl[i], W.ha[i], Rl, Ra);
        cl = tm.cross(W.va[i], wl) + tm.cross(W.vl[i], wa);  // v x w (motion)
        ca = tm.cross(W.va[i], wa);
        rbi3(tm, W.m[i], W.h[i], W.I[i], cl, ca, Tl, Ta);
        W.Pl[i] = Pl; W.Pa[i] = Pa; W.Ql[i] = Ql; W.Qa[i] = Qa;
        W.Rl[i] = Rl; W.Ra[i] = Ra; W.Tl[i] = Tl; W.Ta[i] = Ta;
      }
      // ... and leaves to root (subtree sums of P, Q, R, T)
#pragma unroll
      for (int j = nj - 1; j >= 1; j--) {
        const DJoint& J = T.joint(j);
        const int p = J.parent;
        const double Pl = W.Pl[j], Pa = W.Pa[j], Ql = W.Ql[j], Qa = W.Qa[j];
        const double Rl = W.Rl[j], Ra = W.Ra[j], Tl = W.Tl[j], Ta = W.Ta[j];
        const double vll = p == 0 ? 0.0 : W.vl[p], vla = p == 0 ? 0.0 : W.va[p];
        const double all = p == 0 ? gk : W.al[p], ala = p == 0 ? 0.0 : W.aa[p];
        const double Wll = p == 0 ? 0.0 : W.wl[p], Wla = p == 0 ? 0.0 : W.wa[p];
        // Z = -Q + v_parent x* P + R + T;  G = v_parent x* Z - a_parent x* P - w_parent x* F
        double xl, xa;
        crossf3(tm, vll, vla, Pl, Pa, xl, xa);
        const double Zl = xl + (Rl + Tl) - Ql, Za = xa + (Ra + Ta) - Qa;
        double Gl, Ga, yl, ya, zl, za;
        crossf3(tm, vll, vla, Zl, Za, Gl, Ga);
        crossf3(tm, all, ala, Pl, Pa, yl, ya);
        crossf3(tm, Wll, Wla, W.Fl[j], W.Fa[j], zl, za);
        Gl = Gl - yl - zl;
        Ga = Ga - ya - za;
        // Gd = Q - (v_parent + v) x* P - R - T
        crossf3(tm, vll + W.vl[j], vla + W.va[j], Pl, Pa, yl, ya);
        const double Gdl = Ql - yl - (Rl + Tl), Gda = Qa - ya - (Ra + Ta);
        if (J.kind == JK_FREEFLYER) {
#pragma unroll
          for (int c = 0; c < 6; c++) {
            qb[J.qcol + c] -= tm.sum(fma(W.Sl6[c], Gl, W.Sa6[c] * Ga));
            qdb[J.vcol + c] -= tm.sum(fma(W.Sl6[c], Gdl, W.Sa6[c] * Gda));
          }
        } else {
          qb[J.qcol] -= tm.sum(fma(W.Sl[j], Gl, W.Sa[j] * Ga));
          qdb[J.vcol] -= tm.sum(fma(W.Sl[j], Gdl, W.Sa[j] * Gda));
        }
        if (p > 0) {
          W.Pl[p] += Pl; W.Pa[p] += Pa; W.Ql[p] += Ql; W.Qa[p] += Qa;
          W.Rl[p] += Rl; W.Ra[p] += Ra; W.Tl[p] += Tl; W.Ta[p] += Ta;
        }
      }
    }
  }
  for (int i = 1; i < nj; i++)
    if (T.joint(i).kind == JK_FREEFLYER) qb[T.joint(i).qcol + 6] = 0.0;
  if (st) {
    for (int c = 0; c < nq; c++) a.q0_bar[e * nq + c] = qb[c];
    for (int c = 0; c < nv; c++) a.qd0_bar[e * nv + c] = qdb[c];
  }
}

template <int MAXJ>
__global__ void __launch_bounds__(32) rollout_reverse3_kernel(const DModel* __restrict__ model, const RolloutArgs a) {
  Team3 tm = team3_of_lane(threadIdx.x);
  const int64_t e0 = int64_t(blockIdx.x) * 10 + tm.base / 3;
  tm.valid = tm.valid && e0 < a.n;
  rollout_reverse3_env<MAXJ>(RuntimeTab{model}, tm, a, e0 < a.n ? e0 : a.n - 1);
}

// Ten environments per warp; teams past the end of the batch repeat the last environment
// and store nothing.
template <int MAXJ>
__global__ void __launch_bounds__(32) rollout_forward3_kernel(const DModel* __restrict__ model, const RolloutArgs a) {
  Team3 tm = team3_of_lane(threadIdx.x);
  const int64_t e0 = int64_t(blockIdx.x) * 10 + tm.base / 3;
  tm.valid = tm.valid && e0 < a.n;
  rollout_forward3_env<MAXJ>(RuntimeTab{model}, tm, a, e0 < a.n ? e0 : a.n - 1);
}

}  // namespace sgdyn
