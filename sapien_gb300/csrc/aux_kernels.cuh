// Link Jacobians, Coriolis matrix and CLIK inverse kinematics, one environment per thread.
// The per-environment bodies are host-device functions: the same code answers
// single-instance calls on the host (host_path.cu).
#pragma once
#include "se3.cuh"
#include "step_kernel.cuh"

namespace sgdyn {

// getLinkJacobian (pinocchio_model.cpp:167-186): WORLD columns oMi.act(S) of the joints
// supporting the link's joint, zero elsewhere; local -> left-multiplied by the inverse
// action of the link pose. computeSingleLinkLocalJacobian (:188-199) is the same matrix
// (link2joint^-1 action of the joint-frame Jacobian = link2world^-1 action of the world one).
template <int MAXJ>
SG_HD void link_jacobian_env(const DModel* __restrict__ model, const LinkJacArgs& a, const int64_t e) {
  const DJoint* __restrict__ JT = model_joints(model);
  const DLink& L = model_links(model)[a.link];
  const int nv = model->nv;
  for (int r = 0; r < 6; r++)
    for (int c = 0; c < nv; c++) stv(a.J, e, r * nv + c, 0.0);
  int chain[MAXJ];
  int depth = 0;
  for (int j = L.joint; j > 0; j = JT[j].parent) chain[depth++] = j;
  M3 oR[MAXJ];
  V3 op[MAXJ];
  for (int d = depth - 1; d >= 0; d--) {
    const int i = chain[d];
    joint_world_pose(JT[i], a.q, e, oR, op, oR[i], op[i]);
  }
  M3 Rl;
#pragma unroll
  for (int k = 0; k < 9; k++) Rl.a[k] = L.R[k];
  M3 R;
  V3 p;
  if (L.joint == 0) {
    R = Rl;
    p = mk(L.p[0], L.p[1], L.p[2]);
  } else {
    R = mul(oR[L.joint], Rl);
    p = mul_add(oR[L.joint], mk(L.p[0], L.p[1], L.p[2]), op[L.joint]);
  }
  for (int d = 0; d < depth; d++) {
    const int i = chain[d];
    const DJoint& J = JT[i];
    for (int k = 0; k < J.nv; k++) {
      Mot S = world_S(J, oR[i], op[i], k);
      if (a.local) {
        S.v = mulT(R, add_cross(S.v, S.w, p));  // R^T (v - p x w)
        S.w = mulT(R, S.w);
      }
      const int c = J.vcol + k;
      stv(a.J, e, 0 * nv + c, S.v.x);
      stv(a.J, e, 1 * nv + c, S.v.y);
      stv(a.J, e, 2 * nv + c, S.v.z);
      stv(a.J, e, 3 * nv + c, S.w.x);
      stv(a.J, e, 4 * nv + c, S.w.y);
      stv(a.J, e, 5 * nv + c, S.w.z);
    }
  }
}

template <int MAXJ>
__global__ void __launch_bounds__(32) link_jacobian_kernel(const DModel* __restrict__ model, const LinkJacArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  link_jacobian_env<MAXJ>(model, a, e);
}

// computeCoriolisMatrix (pinocchio_model.cpp:208-212): the Christoffel-consistent
// factorisation C = sum_b J_b^T (I_b Jdot_b + B_b J_b) with
// B(I, v) = 1/2 ((v x*) I - I (v x) + (I v) xbar*), evaluated with subtree composites:
// for a joint i with composites Ic, Bc over its subtree,
//   C[k, l] = S_k . (Ic Sdot_l + Bc S_l)             l in joint i, k in ancestors-or-self,
//   C[k, l] = (Ic S_k) . Sdot_l + (Bc^T S_k) . S_l   k in joint i, l in strict ancestors,
// where Sdot = v_i x S (world frame) and all other entries vanish.
// For an origin-form inertia (m, h, Ibar) and v = (nu, w), with I v = (f, n), B has a single
// non-zero block column: B = [[0, -[f]x], [0, M]] with
//   M = 1/2 ([w]x Ibar - Ibar [w]x - (h nu^T + nu h^T) + 2 (nu . h) 1 - [n]x),
// so B x = (w_x x f, M w_x) and B^T y = (0, f x y_lin + M^T y_ang). Composites keep the sum
// of f (3 numbers) and of M (9) instead of a dense 6x6.
template <int MAXJ>
SG_HD void coriolis_env(const DModel* __restrict__ model, const CoriolisArgs& a, const int64_t e) {
  constexpr int MAXV = MAXJ + 5;
  const DJoint* __restrict__ JT = model_joints(model);
  const int nj = model->nj, nv = model->nv;
  M3 oR[MAXJ];
  V3 op[MAXJ];
  Mot vel[MAXJ], Sw[MAXV], Sd[MAXV];
  RBI Ic[MAXJ];
  V3 Bf[MAXJ];
  M3 BM[MAXJ];
  const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
  for (int i = 1; i < nj; i++) {
    const DJoint& J = JT[i];
    const int p = J.parent, iv = J.ivx;
    joint_world_pose(J, a.q, e, oR, op, oR[i], op[i]);
    Mot vJ = zero;
    for (int k = 0; k < J.nv; k++) {
      Sw[iv + k] = world_S(J, oR[i], op[i], k);
      vJ = axpy6(ldv(a.qd, e, J.vcol + k), Sw[iv + k], vJ);
    }
    const Mot v = (p == 0) ? vJ : add6(vel[p], vJ);
    vel[i] = v;
    for (int k = 0; k < J.nv; k++) Sd[iv + k] = add_crossm(zero, v, Sw[iv + k]);
    RBI Yl;
    Yl.m = J.m;
    Yl.h = mk(J.h[0], J.h[1], J.h[2]);
    for (int k = 0; k < 6; k++) Yl.I[k] = J.I[k];
    const RBI Y = rbi_transport(Yl, oR[i], op[i]);
    Ic[i] = Y;
    const Mot fn = rbi_mul(Y, v);  // (f, n) = I v
    Bf[i] = fn.v;
    // M = 1/2 (A + A^T - (h nu^T + nu h^T) + 2 (nu . h) 1 - [n]x), A = [w]x Ibar
    const V3 w = v.w, nu = v.v, h = Y.h;
    const double* S = Y.I;  // xx xy xz yy yz zz
    const V3 c0 = cross(w, mk(S[0], S[1], S[2])), c1 = cross(w, mk(S[1], S[3], S[4])),
             c2 = cross(w, mk(S[2], S[4], S[5]));  // columns of A
    const double A[9] = {c0.x, c1.x, c2.x, c0.y, c1.y, c2.y, c0.z, c1.z, c2.z};
    const double hv[3] = {h.x, h.y, h.z}, nv3[3] = {nu.x, nu.y, nu.z};
    const double d2 = 2.0 * dot(nu, h);
    const double N[9] = {0, -fn.w.z, fn.w.y, fn.w.z, 0, -fn.w.x, -fn.w.y, fn.w.x, 0};
    M3 Mi;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        double t = A[r * 3 + c] + A[c * 3 + r] - fma(hv[r], nv3[c], nv3[r] * hv[c]) - N[r * 3 + c];
        if (r == c) t += d2;
        Mi.a[r * 3 + c] = 0.5 * t;
      }
    BM[i] = Mi;
  }
  for (int i = nj - 1; i >= 1; i--) {
    const DJoint& J = JT[i];
    const int p = J.parent, iv = J.ivx;
    const RBI Y = Ic[i];
    const V3 f = Bf[i];
    const M3 Mc = BM[i];
    for (int l = 0; l < J.nv; l++) {
      // Bc S_l = (w_S x f, Mc w_S)
      const Mot Sl = Sw[iv + l];
      const Mot F = add6(rbi_mul(Y, Sd[iv + l]), Mot{cross(Sl.w, f), mul(Mc, Sl.w)});
      const int cl = J.vcol + l;
      for (int j = i; j > 0; j = JT[j].parent) {
        const DJoint& A = JT[j];
        for (int k = 0; k < A.nv; k++) stv(a.C, e, (A.vcol + k) * nv + cl, dot6(Sw[A.ivx + k], F));
      }
    }
    for (int k = 0; k < J.nv; k++) {
      const Mot Sk = Sw[iv + k];
      const Mot H = rbi_mul(Y, Sk);
      // Bc^T S_k = (0, f x S_k,lin + Mc^T S_k,ang)
      const V3 Kw = cross(f, Sk.v) + mulT(Mc, Sk.w);
      const int rk = J.vcol + k;
      for (int j = p; j > 0; j = JT[j].parent) {
        const DJoint& A = JT[j];
        for (int l = 0; l < A.nv; l++) {
          const Mot Sl = Sw[A.ivx + l];
          stv(a.C, e, rk * nv + A.vcol + l, dot6(H, Sd[A.ivx + l]) + dot(Kw, Sl.w));
        }
      }
    }
    // entries with the joints after this joint's subtree (no ancestor relation) vanish
    for (int j = J.subtree_end; j < nj; j++) {
      const int jc = JT[j].vcol, nvj = JT[j].nv;
      for (int k = 0; k < J.nv; k++)
        for (int l = 0; l < nvj; l++) {
          stv(a.C, e, (jc + l) * nv + J.vcol + k, 0.0);
          stv(a.C, e, (J.vcol + k) * nv + jc + l, 0.0);
        }
    }
    if (p > 0) {
      RBI& P = Ic[p];
      P.m += Y.m;
      P.h = P.h + Y.h;
      for (int k = 0; k < 6; k++) P.I[k] += Y.I[k];
      Bf[p] = Bf[p] + f;
      for (int k = 0; k < 9; k++) BM[p].a[k] += Mc.a[k];
    }
  }
}

template <int MAXJ>
__global__ void __launch_bounds__(32) coriolis_kernel(const DModel* __restrict__ model, const CoriolisArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  coriolis_env<MAXJ>(model, a, e);
}

#ifndef __CUDACC_RTC__
// Grid for a grid-stride kernel of one-warp blocks: as few rounds as the resident capacity
// (occupancy x SMs) allows, with the environments spread evenly over the rounds. Without
// it, a batch slightly above one wave (65536 CLIK solves: 2048 warps for ~1800 resident)
// runs a second, nearly empty wave at full per-warp latency.
inline unsigned balanced_grid(int64_t n, int blocks_per_sm) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const int64_t blocks = (n + 31) / 32, cap = int64_t(sms) * (blocks_per_sm > 0 ? blocks_per_sm : 1);
  const int64_t rounds = (blocks + cap - 1) / cap;
  return unsigned(rounds > 0 ? (blocks + rounds - 1) / rounds : 1);
}
#endif

// computeInverseKinematics (pinocchio_model.cpp:228-300): damped-least-squares CLIK on the
// joint-frame log6 error. Loop: FK; iMd = oMi[j]^-1 oMdes; err = log6(iMd); keep the best
// iterate; stop when |err| < eps (success) or after max_iter updates; J = joint-frame
// Jacobian; J = -Jlog6(iMd^-1) J diag(mask); v = -J^T (J J^T + damp 1)^-1 err;
// q = integrate(q, v dt). Returns posP2S(best q), success, best err.
template <int MAXJ>
SG_HD void ik_env(const DModel* __restrict__ model, const IkArgs& a, const int64_t e) {
  constexpr int MAXV = MAXJ + 5;
  const DJoint* __restrict__ JT = model_joints(model);
  const DLink& L = model_links(model)[a.link];
  const int nj = model->nj;
  // per-joint state in internal form: angle / slide; (cos, sin); free flyer x y z qx qy qz qw
  double qs[MAXJ][7], best[MAXJ][7];
  for (int i = 1; i < nj; i++) {
    const DJoint& J = JT[i];
    const int c0 = J.qcol;
    switch (J.kind) {
      case JK_CONTINUOUS: {
        double s, c;
        if (a.has_q0) sincos(ldv(a.q0, e, c0), &s, &c);
        else { s = 0; c = 1; }
        qs[i][0] = c;
        qs[i][1] = s;
        break;
      }
      case JK_FREEFLYER:
        for (int k = 0; k < 7; k++) qs[i][k] = a.has_q0 ? ldv(a.q0, e, c0 + k) : (k == 6 ? 1.0 : 0.0);
        break;
      default:
        qs[i][0] = a.has_q0 ? ldv(a.q0, e, c0) : 0.0;
    }
  }
  int chain[MAXJ];
  int depth = 0;
  for (int j = L.joint; j > 0; j = JT[j].parent) chain[depth++] = j;
  const int jid = L.joint;
  // oMdes = target * l2j^-1
  const V3 pt = mk(ldv(a.target, e, 0), ldv(a.target, e, 1), ldv(a.target, e, 2));
  const M3 Rt = quat_to_R(ldv(a.target, e, 4), ldv(a.target, e, 5), ldv(a.target, e, 6), ldv(a.target, e, 3));
  M3 Rl;
  for (int k = 0; k < 9; k++) Rl.a[k] = L.R[k];
  const M3 Rdes = mul(Rt, transpose(Rl));
  const V3 pdes = pt - mul(Rdes, mk(L.p[0], L.p[1], L.p[2]));
  double mk_[MAXV];
  int ncol = 0;
  for (int d = depth - 1; d >= 0; d--) {
    const DJoint& J = JT[chain[d]];
    for (int k = 0; k < J.nv; k++) mk_[ncol++] = a.has_mask ? double(a.mask[J.vcol + k]) : 1.0;
  }
  for (int i = 1; i < nj; i++)
    for (int k = 0; k < 7; k++) best[i][k] = qs[i][k];
  double minErr = 1e10;
  Mot bestErr{mk(0, 0, 0), mk(0, 0, 0)};
  bool ok = false;
  M3 oR[MAXJ];
  V3 op[MAXJ];
  double Jc[6][MAXV];
  for (int it = 0;; it++) {
    // FK along the chain, root first: B, o = the joint's placement frame in the world, then
    // the joint motion in that frame (a z rotation or slide in a canonical frame)
    for (int d = depth - 1; d >= 0; d--) {
      const int i = chain[d];
      const DJoint& J = JT[i];
      const int p = J.parent;
      M3 Rpl;
      for (int k = 0; k < 9; k++) Rpl.a[k] = J.R[k];
      const V3 ppl = mk(J.p[0], J.p[1], J.p[2]);
      const M3 B = p == 0 ? Rpl : ((J.flags & JF_ROT_IDENTITY) ? oR[p] : mul(oR[p], Rpl));
      const V3 o = p == 0 ? ppl : mul_add(oR[p], ppl, op[p]);
      switch (J.kind) {
        case JK_FREEFLYER:
          oR[i] = mul(B, quat_to_R(qs[i][3], qs[i][4], qs[i][5], qs[i][6]));
          op[i] = mul_add(B, mk(qs[i][0], qs[i][1], qs[i][2]), o);
          break;
        case JK_PRISMATIC: {
          const V3 ax = J.axis_kind == AX_Z ? mk(B.a[2], B.a[5], B.a[8])
                                            : mul(B, mk(J.axis[0], J.axis[1], J.axis[2]));
          oR[i] = B;
          op[i] = axpy(qs[i][0], ax, o);
          break;
        }
        default: {  // revolute (angle) and continuous (cos, sin)
          double s, c;
          if (J.kind == JK_CONTINUOUS) {
            c = qs[i][0];
            s = qs[i][1];
          } else {
            sincos(qs[i][0], &s, &c);
          }
          if (J.axis_kind == AX_Z) {
#pragma unroll
            for (int r = 0; r < 3; r++) {
              const double b0 = B.a[r * 3], b1 = B.a[r * 3 + 1];
              oR[i].a[r * 3 + 0] = fma(c, b0, s * b1);
              oR[i].a[r * 3 + 1] = fma(c, b1, -s * b0);
              oR[i].a[r * 3 + 2] = B.a[r * 3 + 2];
            }
          } else {
            oR[i] = mul(B, rodrigues(mk(J.axis[0], J.axis[1], J.axis[2]), s, c));
          }
          op[i] = o;
        }
      }
    }
    M3 Ro = eye3();
    V3 po = mk(0, 0, 0);
    if (jid > 0) {
      Ro = oR[jid];
      po = op[jid];
    }
    // iMd = oMi^-1 oMdes
    const M3 Re = mul(transpose(Ro), Rdes);
    const V3 pe = mulT(Ro, pdes - po);
    const Mot err = log6(Re, pe);
    const double nrm = sqrt(dot6(err, err));
    if (nrm < minErr) {
      minErr = nrm;
      bestErr = err;
      for (int i = 1; i < nj; i++)
        for (int k = 0; k < 7; k++) best[i][k] = qs[i][k];
    }
    if (nrm < a.eps) {
      ok = true;
      break;
    }
    if (it >= a.max_iter) break;
    // joint-frame Jacobian of the chain columns
    int col = 0;
    for (int d = depth - 1; d >= 0; d--) {
      const int i = chain[d];
      const DJoint& J = JT[i];
      for (int k = 0; k < J.nv; k++, col++) {
        Mot S = world_S(J, oR[i], op[i], k);
        const V3 v = mulT(Ro, add_cross(S.v, S.w, po));
        const V3 w = mulT(Ro, S.w);
        Jc[0][col] = v.x; Jc[1][col] = v.y; Jc[2][col] = v.z;
        Jc[3][col] = w.x; Jc[4][col] = w.y; Jc[5][col] = w.z;
      }
    }
    // Jlog6(iMd^-1) = [[Jinv, -TR], [0, Jinv]], from log6(iMd^-1) = -err
    M3 Jinv, TR;
    jlog6_blocks(Mot{-err.v, -err.w}, Jinv, TR);
    // J2 = -Jlog6 Jc diag(mask), in place column by column
    for (int c = 0; c < ncol; c++) {
      const V3 jv = mk(Jc[0][c], Jc[1][c], Jc[2][c]), jw = mk(Jc[3][c], Jc[4][c], Jc[5][c]);
      const V3 top = mul(Jinv, jv) - mul(TR, jw), bot = mul(Jinv, jw);
      const double m = -mk_[c];
      Jc[0][c] = m * top.x; Jc[1][c] = m * top.y; Jc[2][c] = m * top.z;
      Jc[3][c] = m * bot.x; Jc[4][c] = m * bot.y; Jc[5][c] = m * bot.z;
    }
    // (J J^T + damp) x = err, Cholesky on the packed lower triangle
    double A[21];
    for (int r = 0; r < 6; r++)
      for (int c = 0; c <= r; c++) {
        double s = (r == c) ? a.damp : 0.0;
        for (int k = 0; k < ncol; k++) s = fma(Jc[r][k], Jc[c][k], s);
        A[r * (r + 1) / 2 + c] = s;
      }
    chol6(A);
    double x[6] = {err.v.x, err.v.y, err.v.z, err.w.x, err.w.y, err.w.z};
    chol6_solve(A, x);
    // v = -J^T x ; integrate the chain joints by v dt
    col = 0;
    for (int d = depth - 1; d >= 0; d--) {
      const int i = chain[d];
      const DJoint& J = JT[i];
      double vv[6];
      for (int k = 0; k < J.nv; k++, col++) {
        double s = 0;
        for (int r = 0; r < 6; r++) s = fma(Jc[r][col], x[r], s);
        vv[k] = -s * a.dt;
      }
      switch (J.kind) {
        case JK_CONTINUOUS: {
          double sw, cw;
          sincos(vv[0], &sw, &cw);
          const double c = qs[i][0], s = qs[i][1];
          const double nc = cw * c - sw * s, ns = sw * c + cw * s;
          const double k = (3 - (nc * nc + ns * ns)) / 2;
          qs[i][0] = nc * k;
          qs[i][1] = ns * k;
          break;
        }
        case JK_FREEFLYER:
          free_flyer_integrate(qs[i], vv);
          break;
        default: qs[i][0] += vv[0];
      }
    }
  }
  for (int i = 1; i < nj; i++) {
    const DJoint& J = JT[i];
    switch (J.kind) {
      case JK_CONTINUOUS: stv(a.q_out, e, J.qcol, atan2(best[i][1], best[i][0])); break;
      case JK_FREEFLYER:
        for (int k = 0; k < 7; k++) stv(a.q_out, e, J.qcol + k, best[i][k]);
        break;
      default: stv(a.q_out, e, J.qcol, best[i][0]);
    }
  }
  a.success[e] = ok ? 1 : 0;
  // the error lives in the table's canonical joint frame F' = F C: report it in F
  if (jid > 0) {
    M3 C;
    for (int k = 0; k < 9; k++) C.a[k] = model_frames(model)[jid].C[k];
    bestErr.v = mul(C, bestErr.v);
    bestErr.w = mul(C, bestErr.w);
  }
  stv(a.err, e, 0, bestErr.v.x);
  stv(a.err, e, 1, bestErr.v.y);
  stv(a.err, e, 2, bestErr.v.z);
  stv(a.err, e, 3, bestErr.w.x);
  stv(a.err, e, 4, bestErr.w.y);
  stv(a.err, e, 5, bestErr.w.z);
}

template <int MAXJ>
__global__ void __launch_bounds__(32) ik_kernel(const DModel* __restrict__ model, const IkArgs a) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < a.n; e += int64_t(gridDim.x) * blockDim.x)
    ik_env<MAXJ>(model, a, e);
}

}  // namespace sgdyn
