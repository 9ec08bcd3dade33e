// Fused batched sweep over a kinematic tree, one environment per thread, FP64.
//
// All spatial quantities live in the WORLD frame (the frame Pinocchio's computeJointJacobians
// and crba use). Compared with local-frame recursions this replaces the 6x6 congruence
// transform of articulated inertias (about 220 flops per joint) by one 10-parameter
// rigid-inertia transport shared by CRBA, RNEA and ABA, and the three motion/force
// transforms of RNEA by plain additions. The recursions computed:
//   FK        oMi = oMi[parent] * placement * M_J(q)                 (pinocchio_model.cpp:146-161)
//   Jacobian  J[:, v(i)] = oMi.act(S_i)                               (pinocchio_model.cpp:163-165)
//   CRBA      Ic[i] = sum of world inertias of the subtree;
//             M[j, i] = S_j . (Ic[i] S_i) for j an ancestor of i        (pinocchio_model.cpp:201-206)
//   RNEA      v_i = v_p + S_i qd_i, a_i = a_p + S_i qdd_i + v_i x (S_i qd_i), a_0 = -g,
//             f_i = I_i a_i + v_i x* I_i v_i, tau_i = S_i . f_i, f_p += f_i  (pinocchio_model.cpp:214-219)
//   ABA       Featherstone's three passes with U = IA S, D = S.U, u = tau - S.pA,
//             IA_p += IA - U D^-1 U^T, pA_p += pA + Ia c + U D^-1 u,
//             qdd = D^-1 (u - U.(a_p + c)), a = a_p + c + S qdd        (pinocchio_model.cpp:221-226)
// The SAPIEN<->tree permutation is applied by reading and writing external columns
// directly (DJoint::qcol / vcol); no separate permutation pass exists.
#pragma once
#include "kernels.h"
#include "spatial.cuh"

namespace sgdyn {

// Table policies for the sweep: a table read through a device pointer at run time, or a
// table whose contents are compile-time constants (run-time-compiled per model, so every
// joint loop unrolls into straight-line code with constant parents, axes and inertias).
struct FdLoops;
struct RuntimeTab {
  static constexpr bool kStatic = false;
  using Fd = FdLoops;
  const DModel* m;
  SG_HD int nj() const { return m->nj; }
  SG_HD int nv() const { return m->nv; }
  SG_HD int nq_ext() const { return m->nq_ext; }
  SG_HD int nlinks() const { return m->nlinks; }
  SG_HD double gravity(int k) const { return m->gravity[k]; }
  SG_HD const DJoint& joint(int i) const { return model_joints(m)[i]; }
  SG_HD const DLink& link(int l) const { return model_links(m)[l]; }
};
template <int NJ, int NV, int NL, const DJoint* JT, const DLink* LT, const DModel* M, class FD = FdLoops>
struct StaticTab {
  static constexpr bool kStatic = true;
  using Fd = FD;  // the mass-matrix route's steps (generated per model by the run-time compiler)
  SG_HD static constexpr int nj() { return NJ; }
  SG_HD static constexpr int nv() { return NV; }
  SG_HD int nq_ext() const { return M->nq_ext; }
  SG_HD static constexpr int nlinks() { return NL; }
  SG_HD double gravity(int k) const { return M->gravity[k]; }
  SG_HD const DJoint& joint(int i) const { return JT[i]; }
  SG_HD const DLink& link(int l) const { return LT[l]; }
};

SG_HD double ldv(const Arr& a, int64_t e, int c) { return a.p[e * a.es + int64_t(c) * a.cs]; }
SG_HD void stv(const Arr& a, int64_t e, int c, double v) { a.p[e * a.es + int64_t(c) * a.cs] = v; }

// World pose of joint J from its parent's: (Ro, po) = oMi[parent] * placement * M_J(q).
// A joint in a canonical frame (axis_kind AX_Z) rotates about / slides along z: with
// B = R_parent R_placement, Ro = B Rz(q) mixes two columns of B and keeps the third. Other
// 1-DoF joints keep their axis (Rodrigues), which is cheaper when both the placement and the
// link frames on the joint are unrotated (the table builder decides per joint).
SG_HD void joint_world_pose(const DJoint& J, const Arr& q, int64_t e, const M3* oR, const V3* op,
                                                 M3& Ro, V3& po) {
  const int p = J.parent;
  const bool rot_id = (J.flags & JF_ROT_IDENTITY) != 0;
  M3 Rpl;
#pragma unroll
  for (int k = 0; k < 9; k++) Rpl.a[k] = J.R[k];
  const V3 ppl = mk(J.p[0], J.p[1], J.p[2]);
  if (J.kind == JK_FREEFLYER) {
    const int c0 = J.qcol;
    const V3 t = mk(ldv(q, e, c0), ldv(q, e, c0 + 1), ldv(q, e, c0 + 2));
    const M3 RJ = quat_to_R(ldv(q, e, c0 + 3), ldv(q, e, c0 + 4), ldv(q, e, c0 + 5), ldv(q, e, c0 + 6));
    const M3 Rli = rot_id ? RJ : mul(Rpl, RJ);
    const V3 pli = rot_id ? t + ppl : mul_add(Rpl, t, ppl);
    Ro = (p == 0) ? Rli : mul(oR[p], Rli);
    po = (p == 0) ? pli : mul_add(oR[p], pli, op[p]);
    return;
  }
  if (J.axis_kind == AX_Z) {
    // placement origin in the world
    const V3 o = (p == 0) ? ppl : mul_add(oR[p], ppl, op[p]);
    const M3 B = (p == 0) ? Rpl : (rot_id ? oR[p] : mul(oR[p], Rpl));
    if (J.kind == JK_PRISMATIC) {
      Ro = B;
      po = axpy(ldv(q, e, J.qcol), mk(B.a[2], B.a[5], B.a[8]), o);
    } else {  // revolute and continuous
      double s, c;
      sincos(ldv(q, e, J.qcol), &s, &c);
#pragma unroll
      for (int r = 0; r < 3; r++) {
        const double b0 = B.a[r * 3], b1 = B.a[r * 3 + 1];
        Ro.a[r * 3 + 0] = fma(c, b0, s * b1);
        Ro.a[r * 3 + 1] = fma(c, b1, -s * b0);
        Ro.a[r * 3 + 2] = B.a[r * 3 + 2];
      }
      po = o;
    }
    return;
  }
  const V3 ax = mk(J.axis[0], J.axis[1], J.axis[2]);
  M3 Rli;
  V3 pli;
  if (J.kind == JK_PRISMATIC) {
    const double d = ldv(q, e, J.qcol);
    Rli = Rpl;
    pli = rot_id ? axpy(d, ax, ppl) : mul_add(Rpl, d * ax, ppl);
  } else {
    double s, c;
    sincos(ldv(q, e, J.qcol), &s, &c);
    const M3 RJ = rodrigues(ax, s, c);
    Rli = rot_id ? RJ : mul(Rpl, RJ);
    pli = ppl;
  }
  if (p == 0) {
    Ro = Rli;
    po = pli;
  } else {
    Ro = mul(oR[p], Rli);
    po = mul_add(oR[p], pli, op[p]);
  }
}

// World-frame motion subspace column k of joint J (pose Ro, po): for a joint in a
// canonical frame the z column of Ro, else Ro times the axis.
SG_HD Mot world_S(const DJoint& J, const M3& Ro, V3 po, int k) {
  Mot S;
  if (J.kind == JK_FREEFLYER) {
    V3 r = mk(Ro.a[k % 3], Ro.a[3 + k % 3], Ro.a[6 + k % 3]);  // column of Ro
    if (k < 3) {
      S.v = r;
      S.w = mk(0, 0, 0);
    } else {
      S.v = cross(po, r);
      S.w = r;
    }
    return S;
  }
  const V3 u = (J.axis_kind == AX_Z) ? mk(Ro.a[2], Ro.a[5], Ro.a[8]) : mul(Ro, mk(J.axis[0], J.axis[1], J.axis[2]));
  if (J.kind == JK_PRISMATIC) {
    S.v = u;
    S.w = mk(0, 0, 0);
  } else {
    S.w = u;
    S.v = cross(po, u);
  }
  return S;
}

// Cholesky of a packed symmetric 6x6 (row-major lower triangle, 21 entries) in place; the
// diagonal slots keep the reciprocals 1 / L_jj, so the solves multiply instead of divide.
SG_HD void chol6(double* L) {
  // index of (r, c), c <= r
#define LI(r, c) ((r) * ((r) + 1) / 2 + (c))
  for (int j = 0; j < 6; j++) {
    double d = L[LI(j, j)];
    for (int k = 0; k < j; k++) d = fma(-L[LI(j, k)], L[LI(j, k)], d);
    const double inv = 1.0 / sqrt(d);
    L[LI(j, j)] = inv;
    for (int i = j + 1; i < 6; i++) {
      double s = L[LI(i, j)];
      for (int k = 0; k < j; k++) s = fma(-L[LI(i, k)], L[LI(j, k)], s);
      L[LI(i, j)] = s * inv;
    }
  }
}
SG_HD void chol6_solve(const double* L, double* b) {
  for (int i = 0; i < 6; i++) {
    double s = b[i];
    for (int k = 0; k < i; k++) s = fma(-L[LI(i, k)], b[k], s);
    b[i] = s * L[LI(i, i)];
  }
  for (int i = 5; i >= 0; i--) {
    double s = b[i];
    for (int k = i + 1; k < 6; k++) s = fma(-L[LI(k, i)], b[k], s);
    b[i] = s * L[LI(i, i)];
  }
#undef LI
}

// Several lanes per environment ("team"): L consecutive lanes of a warp share one
// environment. The tree is split into a trunk (a root-connected set of joints that every
// lane of the team computes, identically) and branches (whole subtrees hanging off the
// trunk), each branch owned by one lane. Pass 1 runs the trunk, then each lane its own
// branches side by side; pass 2 runs the branches, sums what they pass up to the trunk
// joints they hang from with a butterfly of warp shuffles (every lane ends with the same
// bits), then runs the trunk; pass 3 runs the trunk, then the branches. The critical path
// per step shrinks from all joints to trunk + heaviest lane. Results are written by a
// joint's owner: the branch's lane, or role 0 for trunk joints.
//
// Team table (ints, per model and L, built on the host):
//   [0] L  [1] ntrunk  [2] smax (longest lane list)  [3] nattach
//   trunk joints [ntrunk] in depth-first order
//   per role, smax joints in depth-first order (0 = idle step)
//   attach joints [nattach]: trunk joints with a child on a branch
//   owner [nj]: -1 for trunk joints, else the owning role
struct NoTeam {
  static constexpr bool kOn = false;
};
struct TeamLanes {
  static constexpr bool kOn = true;
  const int* t;
  int role;
  bool valid;  // false for the lanes of an empty tail slot: they compute but store nothing
  SG_HD int L() const { return t[0]; }
  SG_HD int ntrunk() const { return t[1]; }
  SG_HD int smax() const { return t[2]; }
  SG_HD int nattach() const { return t[3]; }
  SG_HD int trunk(int k) const { return t[4 + k]; }
  SG_HD int sched(int k) const { return t[4 + ntrunk() + role * smax() + k]; }
  SG_HD int attach(int k) const { return t[4 + ntrunk() + L() * smax() + k]; }
  SG_HD int owner(int j) const { return t[4 + ntrunk() + L() * smax() + nattach() + j]; }
  SG_HD double sum(double v) const;
  SG_HD void sum_many(double* v, int n) const;
};

// Sum over the L lanes of a team (L a power of two, teams aligned in the warp).
// (Teams exist only on the device; the host instantiation of the sweep never forms one.)
SG_HD double team_sum(double v, int L) {
#ifdef __CUDA_ARCH__
  for (int m = 1; m < L; m <<= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
#endif
  return v;
}
SG_HD double TeamLanes::sum(double v) const { return team_sum(v, L()); }
SG_HD void TeamLanes::sum_many(double* v, int n) const {
  for (int i = 0; i < n; i++) v[i] = team_sum(v[i], L());
}

// A team whose roles are the warps of a block (L warps, 32 environments; warp r takes role
// r for every lane) with the team table and the role known at compile time (run-time
// compiled per model): each warp's sweep covers the trunk and its own branches with
// constant indices, so its state stays in registers like a one-lane specialised sweep, and
// the warps run different code without diverging. Sums over the team go through shared
// memory (xch: L x kChunk x 32 doubles; sum_many exchanges kChunk values per pair of block
// barriers), in a fixed order, so every warp holds the same bits.
template <int ROLE, const int* TT>
struct RoleTeam {
  static constexpr bool kOn = true;
  static constexpr int role = ROLE;
  static constexpr int kChunk = 8;
  double* xch;
  int lane;
  bool valid;
  SG_HD static constexpr int L() { return TT[0]; }
  SG_HD static constexpr int ntrunk() { return TT[1]; }
  SG_HD static constexpr int smax() { return TT[2]; }
  SG_HD static constexpr int nattach() { return TT[3]; }
  SG_HD static constexpr int trunk(int k) { return TT[4 + k]; }
  SG_HD static constexpr int sched(int k) { return TT[4 + ntrunk() + ROLE * smax() + k]; }
  SG_HD static constexpr int attach(int k) { return TT[4 + ntrunk() + L() * smax() + k]; }
  SG_HD static constexpr int owner(int j) { return TT[4 + ntrunk() + L() * smax() + nattach() + j]; }
  SG_HD double sum(double v) const {
    sum_many(&v, 1);
    return v;
  }
  SG_HD void sum_many(double* v, int n) const {
#ifdef __CUDA_ARCH__
#pragma unroll
    for (int b = 0; b < n; b += kChunk) {
      const int m = n - b < kChunk ? n - b : kChunk;
#pragma unroll
      for (int j = 0; j < m; j++) xch[(ROLE * kChunk + j) * 32 + lane] = v[b + j];
      __syncthreads();
#pragma unroll
      for (int j = 0; j < m; j++) {
        double s = xch[j * 32 + lane];
#pragma unroll
        for (int r = 1; r < L(); r++) s += xch[(r * kChunk + j) * 32 + lane];
        v[b + j] = s;
      }
      __syncthreads();
    }
#else
    (void)v;
    (void)n;
#endif
  }
};

// Entry (a, b <= a) of a symmetric matrix over tree columns, lower triangle packed by rows.
SG_HD constexpr int ltdm_at(int a, int b) { return a * (a + 1) / 2 + b; }

// f(column, joint, dof) for the ancestors of tree column (joint i, dof k), nearest first:
// the joint's earlier degrees of freedom, then each ancestor joint's from its last.
template <class Tab, class F>
SG_HD void ancestor_columns(const Tab& T, int i, int k, const F& f) {
  for (int j = i; j > 0; j = T.joint(j).parent) {
    const DJoint& A = T.joint(j);
    for (int l = (j == i ? k - 1 : A.nv - 1); l >= 0; l--) f(A.ivx + l, j, l);
  }
}

// Forward dynamics from the mass matrix over tree columns (joint i, degree of freedom k,
// numbered ivx + k in depth-first order), whose nonzeros pair a column with its ancestors:
// fill M from the column forces F_a = Y_composite S_a (M_ac = S_c . F_a), store it, y += M x,
// factor M = L^T D L with L unit lower triangular on the same pattern (Featherstone, "Rigid
// Body Dynamics Algorithms", 2008, sec. 6.5: sum depth^2 operations) and solve (2 sum
// depth). These are the loops over run-time tables; the run-time compiler emits the same
// steps per model as straight-line code with constant indices (jit.cpp), so that M stays
// in registers.
struct FdLoops {
  template <class Tab>
  SG_HD static void fill(const Tab& T, double* H, const Mot* S, const Mot* F) {
    for (int i = 1; i < T.nj(); i++)
      for (int k = 0; k < T.joint(i).nv; k++) {
        const int a = T.joint(i).ivx + k;
        H[ltdm_at(a, a)] = dot6(S[a], F[a]);
        ancestor_columns(T, i, k, [&](int c, int, int) { H[ltdm_at(a, c)] = dot6(S[c], F[a]); });
      }
  }
  // st(row, column, value) for every entry of M in external column order
  template <class Tab, class St>
  SG_HD static void store_M(const Tab& T, const double* H, const St& st) {
    for (int i = 1; i < T.nj(); i++) {
      const DJoint& J = T.joint(i);
      for (int k = 0; k < J.nv; k++) {
        const int a = J.ivx + k, ra = J.vcol + k;
        st(ra, ra, H[ltdm_at(a, a)]);
        ancestor_columns(T, i, k, [&](int c, int j, int l) {
          const int rc = T.joint(j).vcol + l;
          st(ra, rc, H[ltdm_at(a, c)]);
          st(rc, ra, H[ltdm_at(a, c)]);
        });
        // joints after this one's subtree are neither its ancestors nor its descendants
        for (int j = J.subtree_end; j < T.nj(); j++)
          for (int l = 0; l < T.joint(j).nv; l++) {
            st(ra, T.joint(j).vcol + l, 0.0);
            st(T.joint(j).vcol + l, ra, 0.0);
          }
      }
    }
  }
  template <class Tab>
  SG_HD static void matvec_add(const Tab& T, const double* H, const double* x, double* y) {
    for (int i = 1; i < T.nj(); i++)
      for (int k = 0; k < T.joint(i).nv; k++) {
        const int a = T.joint(i).ivx + k;
        y[a] = fma(H[ltdm_at(a, a)], x[a], y[a]);
        ancestor_columns(T, i, k, [&](int c, int, int) {
          y[a] = fma(H[ltdm_at(a, c)], x[c], y[a]);
          y[c] = fma(H[ltdm_at(a, c)], x[a], y[c]);
        });
      }
  }
  template <class Tab>
  SG_HD static void factor(const Tab& T, double* H, double* D) {
    for (int i = T.nj() - 1; i >= 1; i--)
      for (int k = T.joint(i).nv - 1; k >= 0; k--) {
        const int a = T.joint(i).ivx + k;
        const double r = 1.0 / H[ltdm_at(a, a)];
        D[a] = r;
        ancestor_columns(T, i, k, [&](int c, int j, int l) {
          const double f = H[ltdm_at(a, c)] * r;
          H[ltdm_at(c, c)] = fma(-f, H[ltdm_at(a, c)], H[ltdm_at(c, c)]);
          ancestor_columns(T, j, l, [&](int d, int, int) { H[ltdm_at(c, d)] = fma(-f, H[ltdm_at(a, d)], H[ltdm_at(c, d)]); });
          H[ltdm_at(a, c)] = f;
        });
      }
  }
  // x <- M^-1 x: L^T y = x (columns descending), then L x = D^-1 y (ascending)
  template <class Tab>
  SG_HD static void solve(const Tab& T, const double* H, const double* D, double* x) {
    for (int i = T.nj() - 1; i >= 1; i--)
      for (int k = T.joint(i).nv - 1; k >= 0; k--) {
        const int a = T.joint(i).ivx + k;
        const double xa = x[a];
        ancestor_columns(T, i, k, [&](int c, int, int) { x[c] = fma(-H[ltdm_at(a, c)], xa, x[c]); });
      }
    for (int i = 1; i < T.nj(); i++)
      for (int k = 0; k < T.joint(i).nv; k++) {
        const int a = T.joint(i).ivx + k;
        double xa = x[a] * D[a];
        ancestor_columns(T, i, k, [&](int c, int, int) { xa = fma(-H[ltdm_at(a, c)], x[c], xa); });
        x[a] = xa;
      }
  }
};

// The whole fused sweep for environment e (rows of the StepArgs arrays).
template <int MAXJ, int OPS, class Tab, class Team = NoTeam>
SG_HD void step_env_t(const Tab& T, const StepArgs& args, const int64_t e, const Team& tm = Team{}) {
  constexpr int MAXV = MAXJ + 5;
  constexpr bool kFK = OPS & OP_FK, kJAC = OPS & OP_JAC, kCRBA = OPS & OP_CRBA, kRNEA = OPS & OP_RNEA,
                 kABA = OPS & OP_ABA;
  // Forward dynamics either by the articulated-body passes (kArt) or from the mass matrix
  // (kFdM: OP_FD_CRBA, chosen per model on the host when it costs fewer FP64 operations).
  // With kFdM the acceleration pass runs at zero joint acceleration (bias forces b, bz) and
  // inverse dynamics reads tau = b + M qdd.
  constexpr bool kFdM = kABA && (OPS & OP_FD_CRBA);
  constexpr bool kArt = kABA && !kFdM;
  constexpr bool kForces = kRNEA || kFdM;  // accelerations and forces of the RNEA pass
  constexpr bool kComposite = kCRBA || kFdM;
  constexpr bool kVel = kRNEA || kABA;
  constexpr bool kInertia = kCRBA || kRNEA || kABA;
  constexpr bool kTeam = Team::kOn;
  static_assert(!(kFdM && kTeam), "teams run the articulated-body passes");
  const int nj = T.nj();

  M3 oR[MAXJ];
  V3 op[MAXJ];
  Mot Sw[MAXV];
  Mot vel[kVel ? MAXJ : 1];
  Mot acc[(kRNEA || kABA) ? MAXJ : 1];
  Mot frc[kForces ? MAXJ : 1];
  // Pass 2 rebuilds each joint's composite (CRBA) and articulated (ABA) inertia as its own
  // body inertia Yb plus what its children passed up (CC, AC). The last child in
  // depth-first order is processed first and initialises its parent's slot, so no slot is
  // zero-filled and only joints with children carry one (teams zero their trunk's slots).
  RBI Yb[(kCRBA || kABA) ? MAXJ : 1];
  RBI CC[kComposite ? MAXJ : 1];
  Sym6 AC[kArt ? MAXJ : 1];
  Mot pA[kArt ? MAXJ : 1], cb[kArt ? MAXJ : 1], Uv[kArt ? MAXV : 1];
  double uv[kArt ? MAXV : 1], Dinv[kArt ? MAXJ : 1];
  double Lff[kArt ? 21 : 1];  // Cholesky factor of D for the (single) free-flyer joint
  // kFdM: the bias forces and the composite-inertia forces F = Y_c S per tree column
  double bz[kFdM ? MAXV : 1];
  Mot Fcol[kFdM ? MAXV : 1];

  const Mot a0{mk(-T.gravity(0), -T.gravity(1), -T.gravity(2)), mk(0, 0, 0)};

  // Each pass reads its inputs in one batch before it starts, so their memory latency is
  // paid once per pass instead of once per joint (most of all when they live in host memory).
  double qin[MAXJ + 6], qdin[kVel ? MAXV : 1], qddin[kRNEA ? MAXV : 1], tauin[kABA ? MAXV : 1];
  {
    const int nq = T.nq_ext(), nv = T.nv();
#pragma unroll
    for (int c = 0; c < nq; c++) qin[c] = ldv(args.q, e, c);
    if constexpr (kVel) {
#pragma unroll
      for (int c = 0; c < nv; c++) qdin[c] = ldv(args.qd, e, c);
    }
    if constexpr (kRNEA) {
#pragma unroll
      for (int c = 0; c < nv; c++) qddin[c] = ldv(args.qdd, e, c);
    }
  }
  const Arr qa{qin, 0, 1};

  // whether this lane writes joint i's results
  auto writes = [&](int i) -> bool {
    if constexpr (kTeam) return tm.valid && (tm.owner(i) < 0 ? tm.role == 0 : tm.owner(i) == tm.role);
    else return true;
  };
  auto in_trunk = [&](int i) -> bool {
    if constexpr (kTeam) return i > 0 && tm.owner(i) < 0;
    else return false;
  };

  // ---------------- pass 1: root to leaves ----------------
  auto pass1 = [&](int i) {
    const DJoint& J = T.joint(i);
    const int p = J.parent;
    M3 Ro;
    V3 po;
    joint_world_pose(J, qa, 0, oR, op, Ro, po);
    oR[i] = Ro;
    op[i] = po;
    const int nvi = J.nv, iv = J.ivx, vc = J.vcol;
    for (int k = 0; k < nvi; k++) Sw[iv + k] = world_S(J, Ro, po, k);
    if constexpr (kJAC) {
      if (writes(i)) {
        const int nv = T.nv();
        for (int k = 0; k < nvi; k++) {
          const Mot S = Sw[iv + k];
          stv(args.J, e, 0 * nv + vc + k, S.v.x);
          stv(args.J, e, 1 * nv + vc + k, S.v.y);
          stv(args.J, e, 2 * nv + vc + k, S.v.z);
          stv(args.J, e, 3 * nv + vc + k, S.w.x);
          stv(args.J, e, 4 * nv + vc + k, S.w.y);
          stv(args.J, e, 5 * nv + vc + k, S.w.z);
        }
      }
    }
    if constexpr (kInertia) {
      RBI Yl;
      Yl.m = J.m;
      Yl.h = mk(J.h[0], J.h[1], J.h[2]);
#pragma unroll
      for (int k = 0; k < 6; k++) Yl.I[k] = J.I[k];
      const RBI Y = rbi_transport(Yl, Ro, po);
      if constexpr (kCRBA || kABA) Yb[i] = Y;
      if constexpr (kVel) {
        Mot vJ{mk(0, 0, 0), mk(0, 0, 0)};
        for (int k = 0; k < nvi; k++) vJ = axpy6(qdin[vc + k], Sw[iv + k], vJ);
        const Mot v = (p == 0) ? vJ : add6(vel[p], vJ);
        vel[i] = v;
        const Mot hY = rbi_mul(Y, v);  // momentum I v
        const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
        const Mot bias = add_crossf(zero, v, hY);  // v x* I v
        if constexpr (kForces) {
          Mot a = (p == 0) ? a0 : acc[p];
          if constexpr (!kFdM)
            for (int k = 0; k < nvi; k++) a = axpy6(qddin[vc + k], Sw[iv + k], a);
          a = add_crossm(a, v, vJ);
          acc[i] = a;
          frc[i] = rbi_mul_add(Y, a, bias);
        }
        if constexpr (kArt) {
          cb[i] = add_crossm(zero, v, vJ);
          pA[i] = bias;
        }
      }
    }
  };

  // ---------------- pass 2: leaves to root ----------------
  auto pass2 = [&](int i) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, nvi = J.nv, iv = J.ivx, vc = J.vcol;
    // a team's trunk joints always carry (zeroed) slots; elsewhere only joints with children
    const bool has_children = in_trunk(i) || J.subtree_end > i + 1;
    // the last child of p in depth-first order ends where p's subtree ends
    const bool first_of_parent = p > 0 && !in_trunk(p) && J.subtree_end == T.joint(p).subtree_end;
    const bool out = writes(i);
    if constexpr (kForces) {
      const Mot f = frc[i];
      if constexpr (kFdM) {
        for (int k = 0; k < nvi; k++) bz[iv + k] = dot6(Sw[iv + k], f);
      } else {
        if (out)
          for (int k = 0; k < nvi; k++) stv(args.tau_out, e, vc + k, dot6(Sw[iv + k], f));
      }
      if (p > 0) frc[p] = add6(frc[p], f);
    }
    if constexpr (kComposite) {
      const int nv = T.nv();
      const RBI Y = has_children ? rbi_add(Yb[i], CC[i]) : Yb[i];
      if constexpr (kFdM) {  // M's entries are formed after the pass
        for (int k = 0; k < nvi; k++) Fcol[iv + k] = rbi_mul(Y, Sw[iv + k]);
      } else if (out) {
        for (int k = 0; k < nvi; k++) {
          const Mot F = rbi_mul(Y, Sw[iv + k]);
          for (int l = 0; l <= k; l++) {  // own block, upper triangle mirrored
            const double m = dot6(Sw[iv + l], F);
            stv(args.M, e, (vc + l) * nv + vc + k, m);
            stv(args.M, e, (vc + k) * nv + vc + l, m);
          }
#pragma unroll
          for (int j = p; j > 0; j = T.joint(j).parent) {
            const int jv = T.joint(j).ivx, jc = T.joint(j).vcol, nvj = T.joint(j).nv;
            for (int l = 0; l < nvj; l++) {
              const double m = dot6(Sw[jv + l], F);
              stv(args.M, e, (jc + l) * nv + vc + k, m);
              stv(args.M, e, (vc + k) * nv + jc + l, m);
            }
          }
        }
        // entries between this joint and the joints after its subtree (neither ancestors
        // nor descendants) are structurally zero; every other entry is written above
#pragma unroll
        for (int j = J.subtree_end; j < nj; j++) {
          const int jc = T.joint(j).vcol, nvj = T.joint(j).nv;
          for (int k = 0; k < nvi; k++)
            for (int l = 0; l < nvj; l++) {
              stv(args.M, e, (jc + l) * nv + vc + k, 0.0);
              stv(args.M, e, (vc + k) * nv + jc + l, 0.0);
            }
        }
      }
      if (p > 0) CC[p] = first_of_parent ? Y : rbi_add(CC[p], Y);
    }
    if constexpr (kArt) {
      const Sym6 IAi = has_children ? sym6_rbi_add(Yb[i], AC[i]) : sym6_from_rbi(Yb[i]);
      if (nvi == 1) {
        const Mot S = Sw[iv];
        const Mot U = sym6_mul(IAi, S);
        const double D = dot6(S, U);
        const double di = 1.0 / D;
        const double u = tauin[vc] - dot6(S, pA[i]);
        Uv[iv] = U;
        uv[iv] = u;
        Dinv[i] = di;
        if (p > 0) {
          const Mot Ud = scale6(di, U);
          Sym6 Ia = IAi;
          const double ud[6] = {Ud.v.x, Ud.v.y, Ud.v.z, Ud.w.x, Ud.w.y, Ud.w.z};
          const double uu[6] = {U.v.x, U.v.y, U.v.z, U.w.x, U.w.y, U.w.z};
          // A -= ud_lin u_lin^T (sym), B -= ud_lin u_ang^T, C -= ud_ang u_ang^T (sym)
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
          Mot pa = sym6_mul_add(Ia, cb[i], pA[i]);
          pa = axpy6(u, Ud, pa);
          if (first_of_parent) AC[p] = Ia;
          else sym6_acc(AC[p], Ia);
          pA[p] = add6(pA[p], pa);
        }
      } else {
        // free flyer: 6x6 D = S^T IA S, Cholesky-factored
        for (int k = 0; k < 6; k++) {
          Uv[iv + k] = sym6_mul(IAi, Sw[iv + k]);
          uv[iv + k] = tauin[vc + k] - dot6(Sw[iv + k], pA[i]);
        }
        for (int r = 0; r < 6; r++)
          for (int c = 0; c <= r; c++) Lff[r * (r + 1) / 2 + c] = dot6(Sw[iv + r], Uv[iv + c]);
        chol6(Lff);
        if (p > 0) {
          // Ia = IA - U D^-1 U^T ; pa = pA + Ia c + U D^-1 u, with D^-1 applied by solves
          Sym6 Ia = IAi;
          double W[6][6];  // W[:, k] = D^-1 e_k
          for (int k = 0; k < 6; k++) {
            for (int r = 0; r < 6; r++) W[r][k] = (r == k) ? 1.0 : 0.0;
            double col[6];
            for (int r = 0; r < 6; r++) col[r] = W[r][k];
            chol6_solve(Lff, col);
            for (int r = 0; r < 6; r++) W[r][k] = col[r];
          }
          Mot UD[6];
          for (int k = 0; k < 6; k++) {
            Mot s{mk(0, 0, 0), mk(0, 0, 0)};
            for (int l = 0; l < 6; l++) s = axpy6(W[l][k], Uv[iv + l], s);
            UD[k] = s;
          }
          for (int k = 0; k < 6; k++) {
            const Mot a = UD[k], b = Uv[iv + k];
            const double ud[6] = {a.v.x, a.v.y, a.v.z, a.w.x, a.w.y, a.w.z};
            const double uu[6] = {b.v.x, b.v.y, b.v.z, b.w.x, b.w.y, b.w.z};
            int t = 0;
            for (int r = 0; r < 3; r++)
              for (int c = r; c < 3; c++, t++) {
                Ia.A[t] = fma(-ud[r], uu[c], Ia.A[t]);
                Ia.C[t] = fma(-ud[3 + r], uu[3 + c], Ia.C[t]);
              }
            for (int r = 0; r < 3; r++)
              for (int c = 0; c < 3; c++) Ia.B[r * 3 + c] = fma(-ud[r], uu[3 + c], Ia.B[r * 3 + c]);
          }
          Mot pa = sym6_mul_add(Ia, cb[i], pA[i]);
          for (int k = 0; k < 6; k++) pa = axpy6(uv[iv + k], UD[k], pa);
          if (first_of_parent) AC[p] = Ia;
          else sym6_acc(AC[p], Ia);
          pA[p] = add6(pA[p], pa);
        }
      }
    }
  };

  // ---------------- pass 3: root to leaves ----------------
  auto pass3 = [&](int i) {
    const DJoint& J = T.joint(i);
    const int p = J.parent, nvi = J.nv, iv = J.ivx, vc = J.vcol;
    const bool out = writes(i);
    Mot a = add6((p == 0) ? a0 : acc[p], cb[i]);
    if (nvi == 1) {
      const double qdd = Dinv[i] * (uv[iv] - dot6(Uv[iv], a));
      a = axpy6(qdd, Sw[iv], a);
      if (out) stv(args.qdd_out, e, vc, qdd);
    } else {
      double b[6];
      for (int k = 0; k < 6; k++) b[k] = uv[iv + k] - dot6(Uv[iv + k], a);
      chol6_solve(Lff, b);
      for (int k = 0; k < 6; k++) {
        a = axpy6(b[k], Sw[iv + k], a);
        if (out) stv(args.qdd_out, e, vc + k, b[k]);
      }
    }
    acc[i] = a;
  };

  auto link_pose = [&](int l) {
    const DLink& L = T.link(l);
    const int j = L.joint;
    {
      M3 R;
      V3 pp;
      M3 Rl;
#pragma unroll
      for (int k = 0; k < 9; k++) Rl.a[k] = L.R[k];
      const V3 pl = mk(L.p[0], L.p[1], L.p[2]);
      if (j == 0) {
        R = Rl;
        pp = pl;
      } else {
        R = (L.flags & JF_ROT_IDENTITY) ? oR[j] : mul(oR[j], Rl);
        pp = mul_add(oR[j], pl, op[j]);
      }
      double qt[4];
      R_to_quat(R, qt);
      stv(args.poses, e, l * 7 + 0, pp.x);
      stv(args.poses, e, l * 7 + 1, pp.y);
      stv(args.poses, e, l * 7 + 2, pp.z);
      stv(args.poses, e, l * 7 + 3, qt[0]);
      stv(args.poses, e, l * 7 + 4, qt[1]);
      stv(args.poses, e, l * 7 + 5, qt[2]);
      stv(args.poses, e, l * 7 + 6, qt[3]);
    }
  };
  auto link_poses = [&]() {
    const int nl = T.nlinks();
#pragma unroll
    for (int l = 0; l < nl; l++) {
      if constexpr (kTeam) {
        if (!writes(T.link(l).joint)) continue;  // another lane holds this joint's pose
      }
      link_pose(l);
    }
  };
  // With compile-time tables and other ops in the same sweep, each link's pose is emitted
  // right after its joint, so the joint's world pose need not stay live to the end of
  // pass 1 (FK alone is faster with the poses written in one run).
  auto links_of = [&](int i) {
    const int nl = T.nlinks();
#pragma unroll
    for (int l = 0; l < nl; l++)
      if (T.link(l).joint == i) link_pose(l);
  };

  // ---------------- forward (and inverse) dynamics from the mass matrix ----------------
  // M over tree columns from the column forces, then tau = b + M qdd and qdd = M^-1 (tau - b)
  // (Tab::Fd: straight-line code per model with compile-time tables, loops otherwise).
  auto mass_matrix_dynamics = [&]() {
    if constexpr (kFdM) {
      using Fd = typename Tab::Fd;
      double Hm[MAXV * (MAXV + 1) / 2], Dm[MAXV], x[MAXV];
      Fd::fill(T, Hm, Sw, Fcol);
      if constexpr (kCRBA) {
        const int nv = T.nv();
        Fd::store_M(T, Hm, [&](int r, int c, double v) { stv(args.M, e, r * nv + c, v); });
      }
      if constexpr (kRNEA) {
        double t[MAXV];
#pragma unroll
        for (int i = 1; i < nj; i++) {
          const DJoint& J = T.joint(i);
#pragma unroll
          for (int k = 0; k < 6; k++)
            if (k < J.nv) {
              t[J.ivx + k] = bz[J.ivx + k];
              x[J.ivx + k] = qddin[J.vcol + k];
            }
        }
        Fd::matvec_add(T, Hm, x, t);
#pragma unroll
        for (int i = 1; i < nj; i++) {
          const DJoint& J = T.joint(i);
#pragma unroll
          for (int k = 0; k < 6; k++)
            if (k < J.nv && writes(i)) stv(args.tau_out, e, J.vcol + k, t[J.ivx + k]);
        }
      }
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
#pragma unroll
        for (int k = 0; k < 6; k++)
          if (k < J.nv) x[J.ivx + k] = tauin[J.vcol + k] - bz[J.ivx + k];
      }
      Fd::factor(T, Hm, Dm);
      Fd::solve(T, Hm, Dm, x);
#pragma unroll
      for (int i = 1; i < nj; i++) {
        const DJoint& J = T.joint(i);
#pragma unroll
        for (int k = 0; k < 6; k++)
          if (k < J.nv && writes(i)) stv(args.qdd_out, e, J.vcol + k, x[J.ivx + k]);
      }
    }
  };

  auto load_tau = [&]() {
    if constexpr (kABA) {
      const int nv = T.nv();
#pragma unroll
      for (int c = 0; c < nv; c++) tauin[c] = ldv(args.tau, e, c);
    }
  };

  if constexpr (!kTeam) {
    constexpr bool kInlineLinks = kFK && Tab::kStatic && (OPS & ~OP_FK) != 0;
    if constexpr (kInlineLinks) links_of(0);
#pragma unroll
    for (int i = 1; i < nj; i++) {
      pass1(i);
      if constexpr (kInlineLinks) links_of(i);
    }
    if constexpr (kFK && !kInlineLinks) link_poses();
    load_tau();
    if constexpr (kCRBA || kRNEA || kABA) {
#pragma unroll
      for (int i = nj - 1; i >= 1; i--) pass2(i);
    }
    if constexpr (kFdM) mass_matrix_dynamics();
    if constexpr (kArt) {
#pragma unroll
      for (int i = 1; i < nj; i++) pass3(i);
    }
  } else {
    // (loops unrolled: with compile-time team tables every joint index is a constant)
    const int nt = tm.ntrunk(), sm = tm.smax(), na = tm.nattach();
#pragma unroll
    for (int k = 0; k < nt; k++) pass1(tm.trunk(k));
#pragma unroll
    for (int k = 0; k < sm; k++) {
      const int j = tm.sched(k);
      if (j > 0) pass1(j);
    }
    if constexpr (kFK) link_poses();
    load_tau();
    if constexpr (kCRBA || kRNEA || kABA) {
      // trunk slots start at zero; attach joints keep their own force / bias aside so that
      // the branch contributions alone are summed across the team
      Mot fbase[kRNEA ? MAXJ : 1], pbase[kArt ? MAXJ : 1];
#pragma unroll
      for (int k = 0; k < nt; k++) {
        const int t = tm.trunk(k);
        if constexpr (kCRBA) CC[t] = RBI{0.0, mk(0, 0, 0), {0, 0, 0, 0, 0, 0}};
        if constexpr (kArt) AC[t] = Sym6{{0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0}};
      }
      const Mot zero{mk(0, 0, 0), mk(0, 0, 0)};
#pragma unroll
      for (int k = 0; k < na; k++) {
        const int t = tm.attach(k);
        if constexpr (kRNEA) {
          fbase[t] = frc[t];
          frc[t] = zero;
        }
        if constexpr (kArt) {
          pbase[t] = pA[t];
          pA[t] = zero;
        }
      }
#pragma unroll
      for (int k = sm - 1; k >= 0; k--) {
        const int j = tm.sched(k);
        if (j > 0) pass2(j);
      }
      // each attach joint's branch contributions (forces, composite and articulated
      // inertias, bias forces), summed over the team in one exchange
      constexpr int kSums = (kRNEA ? 6 : 0) + (kCRBA ? 10 : 0) + (kArt ? 27 : 0);
#pragma unroll
      for (int k = 0; k < na; k++) {
        const int t = tm.attach(k);
        double v[kSums];
        int c = 0;
        auto put6 = [&](const Mot& m) {
          v[c++] = m.v.x; v[c++] = m.v.y; v[c++] = m.v.z; v[c++] = m.w.x; v[c++] = m.w.y; v[c++] = m.w.z;
        };
        auto get6 = [&](Mot& m) {
          m.v.x = v[c++]; m.v.y = v[c++]; m.v.z = v[c++]; m.w.x = v[c++]; m.w.y = v[c++]; m.w.z = v[c++];
        };
        if constexpr (kRNEA) put6(frc[t]);
        if constexpr (kCRBA) {
          const RBI& r = CC[t];
          v[c++] = r.m; v[c++] = r.h.x; v[c++] = r.h.y; v[c++] = r.h.z;
#pragma unroll
          for (int q = 0; q < 6; q++) v[c++] = r.I[q];
        }
        if constexpr (kArt) {
          const Sym6& a6 = AC[t];
#pragma unroll
          for (int q = 0; q < 6; q++) v[c++] = a6.A[q];
#pragma unroll
          for (int q = 0; q < 6; q++) v[c++] = a6.C[q];
#pragma unroll
          for (int q = 0; q < 9; q++) v[c++] = a6.B[q];
          put6(pA[t]);
        }
        tm.sum_many(v, kSums);
        c = 0;
        if constexpr (kRNEA) {
          get6(frc[t]);
          frc[t] = add6(fbase[t], frc[t]);
        }
        if constexpr (kCRBA) {
          RBI& r = CC[t];
          r.m = v[c++]; r.h.x = v[c++]; r.h.y = v[c++]; r.h.z = v[c++];
#pragma unroll
          for (int q = 0; q < 6; q++) r.I[q] = v[c++];
        }
        if constexpr (kArt) {
          Sym6& a6 = AC[t];
#pragma unroll
          for (int q = 0; q < 6; q++) a6.A[q] = v[c++];
#pragma unroll
          for (int q = 0; q < 6; q++) a6.C[q] = v[c++];
#pragma unroll
          for (int q = 0; q < 9; q++) a6.B[q] = v[c++];
          get6(pA[t]);
          pA[t] = add6(pbase[t], pA[t]);
        }
      }
#pragma unroll
      for (int k = nt - 1; k >= 0; k--) pass2(tm.trunk(k));
    }
    if constexpr (kArt) {
#pragma unroll
      for (int k = 0; k < nt; k++) pass3(tm.trunk(k));
#pragma unroll
      for (int k = 0; k < sm; k++) {
        const int j = tm.sched(k);
        if (j > 0) pass3(j);
      }
    }
  }
}

template <int MAXJ, int OPS>
SG_HD void step_env(const DModel* __restrict__ model, const StepArgs& args, const int64_t e) {
  step_env_t<MAXJ, OPS>(RuntimeTab{model}, args, e);
}

template <int MAXJ, int OPS>
__global__ void __launch_bounds__(32) step_kernel(const DModel* __restrict__ model, const StepArgs args) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= args.n) return;
  step_env<MAXJ, OPS>(model, args, e);
}

// L lanes per environment: one warp holds 32 / L environments. Every lane takes part in the
// team sums; lanes past the end repeat the last environment and store nothing.
template <int MAXJ, int OPS>
__global__ void __launch_bounds__(32) step_team_kernel(const DModel* __restrict__ model, const int* __restrict__ team,
                                                       const StepArgs args) {
  const int L = team[0], lane = threadIdx.x & 31;
  const int64_t e = int64_t(blockIdx.x) * (32 / L) + lane / L;
  const bool valid = e < args.n;
  const TeamLanes tm{team, lane % L, valid};
  step_env_t<MAXJ, OPS>(RuntimeTab{model}, args, valid ? e : args.n - 1, tm);
}

}  // namespace sgdyn
