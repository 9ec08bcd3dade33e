// Launcher interface between the C-ABI layer and the CUDA kernels.
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>

#include <cstdint>
#endif

#include "device_model.h"

namespace sgdyn {

// A batched 2-D array: element (env, col) lives at p[env * es + col * cs].
// Row-major [N][cols] is es = cols, cs = 1; column-major / SoA [cols][N] is es = 1, cs = N.
struct Arr {
  double* p;
  int64_t es, cs;
};

enum Ops : int { OP_FK = 1, OP_JAC = 2, OP_CRBA = 4, OP_RNEA = 8, OP_ABA = 16, OP_ALL = 31 };
// Sweep variant bit (not an op): forward dynamics by the composite-rigid-body method, M from
// CRBA factored as L^T D L with the tree's sparsity and qdd = M^-1 (tau - b), b the bias
// forces (RNEA at zero acceleration); inverse dynamics then reads tau = b + M qdd.
constexpr int OP_FD_CRBA = 32;
// The five-op step split in two concurrent launches over the same environments: CRBA + RNEA +
// ABA, and FK + Jacobian, whose short warps fill FP64 schedulers the long ones leave idle.
enum SplitOps : int { OP_SPLIT_A = OP_FK | OP_JAC, OP_SPLIT_B = OP_CRBA | OP_RNEA | OP_ABA };

struct StepArgs {
  int64_t n;
  Arr q, qd, qdd, tau;                  // inputs
  Arr poses, J, M, tau_out, qdd_out;    // outputs (p == nullptr when not requested)
};

struct LinkJacArgs {
  int64_t n;
  int link, local;
  Arr q, J;
};

struct CoriolisArgs {
  int64_t n;
  Arr q, qd, C;
};

struct IkArgs {
  int64_t n;
  int link, max_iter, has_q0, has_mask;
  double eps, dt, damp;
  Arr target, q0, q_out, err;
  const int* mask;
  int* success;
};

// Adjoint (vector-Jacobian product) of RNEA or ABA.
//   RNEA: x = qdd, bar = taubar -> o1 = qbar, o2 = qdbar, o3 = qddbar
//   ABA:  x = tau, bar = qddbar -> o1 = qbar, o2 = qdbar, o3 = taubar
struct VjpArgs {
  int64_t n;
  Arr q, qd, x, bar, o1, o2, o3;
};

// Adjoint of link positions (pbar, n x nlinks*3) and rotations (Rbar, nlinks*9, optional).
struct FkVjpArgs {
  int64_t n;
  Arr q, pbar, Rbar, qbar;
};

// Dense derivative matrices, rows = outputs, columns = tangent inputs.
//   RNEA: x = qdd -> d_q = dtau/dq, d_qd = dtau/dqd, d_x = dtau/dqdd (= M)
//   ABA:  x = tau -> d_q = dqdd/dq, d_qd = dqdd/dqd, d_x = dqdd/dtau (= M^-1)
// Two launches: a preparation kernel (one thread per environment: forward sweep, subtree
// composites and, for ABA, the L^T D L factor of M and qdd) writes its results to
// `scratch` as structure of arrays ([field][env], `lay.total` doubles per environment);
// the column kernel (one thread per environment and tree column) reads them.
struct DerivLayout {
  int S, v, a, F, H, Ib, Db, P, Q, L, Dinv, total;  // first field of each block
};
struct DerivArgs {
  int64_t n;
  Arr q, qd, x, d_q, d_qd, d_x;
  double* scratch;
  DerivLayout lay;
};

// Semi-implicit Euler rollout qd += dt ABA(q, qd, tau_t); q += dt qd, with q / qd
// checkpoints every K steps (segment s starts at step s K). Contiguous env-major arrays:
// q0 [n][nq], qd0 [n][nv], tau [T][n][nv], q_ckpt [C][n][nq], qd_ckpt [C][n][nv].
// The backward runs in groups of segments [s_lo, s_lo + s_cnt), latest group first.
struct RolloutArgs {
  int64_t n;
  int T, K;
  int s_lo, s_cnt;
  double dt;
  const double *q0, *qd0, *tau;
  double *qT, *qdT, *q_ckpt, *qd_ckpt;
  // backward
  const double *qT_bar, *qdT_bar;
  double *q0_bar, *qd0_bar, *tau_bar, *scratch;
};

#ifndef __CUDACC_RTC__
// Device, managed, or mapped pinned host memory (usable by a kernel at this address).
bool device_accessible(const void* p);

// Joint-count bucket for the per-thread stash (16, 32 or 64 joints incl. universe).
int stash_bucket(int nj);

// Fused world-frame sweep: any subset of {FK poses, full WORLD Jacobian, CRBA, RNEA, ABA}.
cudaError_t launch_step(const DModel* dm, int nj, int ops, const StepArgs& a, cudaStream_t s);
// Forward dynamics alone with three lanes per environment (team3.cuh; one-DoF joints and a
// free-flyer root).
cudaError_t launch_aba3(const DModel* dm, int nj, const StepArgs& a, cudaStream_t s);
// The same sweep with `lanes` lanes per environment (team table `team` on the device).
cudaError_t launch_step_team(const DModel* dm, int nj, const int* team, int lanes, int ops, const StepArgs& a,
                             cudaStream_t s);
cudaError_t launch_link_jacobian(const DModel* dm, int nj, const LinkJacArgs& a, cudaStream_t s);
cudaError_t launch_coriolis(const DModel* dm, int nj, const CoriolisArgs& a, cudaStream_t s);
cudaError_t launch_ik(const DModel* dm, int nj, const IkArgs& a, cudaStream_t s);
cudaError_t launch_rnea_vjp(const DModel* dm, int nj, const VjpArgs& a, cudaStream_t s);
cudaError_t launch_aba_vjp(const DModel* dm, int nj, const VjpArgs& a, cudaStream_t s);
cudaError_t launch_fk_vjp(const DModel* dm, int nj, const FkVjpArgs& a, cudaStream_t s);
cudaError_t launch_rnea_derivatives(const DModel* dm, int nj, const DerivArgs& a, cudaStream_t s);
cudaError_t launch_aba_derivatives(const DModel* dm, int nj, const DerivArgs& a, cudaStream_t s);
cudaError_t launch_rollout_forward(const DModel* dm, int nj, const RolloutArgs& a, cudaStream_t s);
// The forward rollout with three lanes per environment (team3.cuh; one-DoF joints and a
// free-flyer root).
cudaError_t launch_rollout_forward3(const DModel* dm, int nj, const RolloutArgs& a, cudaStream_t s);
cudaError_t launch_rollout_recompute(const DModel* dm, int nj, const RolloutArgs& a, cudaStream_t s);
cudaError_t launch_rollout_reverse(const DModel* dm, int nj, const RolloutArgs& a, cudaStream_t s);
// The reverse rollout with three lanes per environment (team3.cuh; one-DoF joints and a
// free-flyer root).
cudaError_t launch_rollout_reverse3(const DModel* dm, int nj, const RolloutArgs& a, cudaStream_t s);
// Fields: S, P, Q: 6 per tree column; v, a, F, H: 6 per joint; Ib, Db: 10 per joint
// (m, h, I xx xy xz yy yz zz); L: the packed factor (nv (nv + 1) / 2), Dinv: nv (ABA only).
inline DerivLayout deriv_layout(int nj, int nv, bool aba) {
  DerivLayout l;
  l.S = 0;
  l.v = l.S + 6 * nv;
  l.a = l.v + 6 * nj;
  l.F = l.a + 6 * nj;
  l.H = l.F + 6 * nj;
  l.Ib = l.H + 6 * nj;
  l.Db = l.Ib + 10 * nj;
  l.P = l.Db + 10 * nj;
  l.Q = l.P + 6 * nv;
  l.L = l.Q + 6 * nv;
  l.Dinv = l.L + (aba ? nv * (nv + 1) / 2 : 0);
  l.total = l.Dinv + (aba ? nv : 0);
  return l;
}
// doubles of rollout-backward scratch per environment and segment (the minimum scratch is
// one segment for all environments; k segments' worth lets k segments recompute at once)
int64_t rollout_scratch_doubles_per_env(int nj, int nq, int nv, int K);
// Bytes of rollout-backward scratch for n environments (one segment each), or -1 when the
// product does not fit in an int64_t.
inline int64_t rollout_scratch_bytes_for(int nj, int nq, int nv, int K, int64_t n) {
  const int64_t per = 8 * rollout_scratch_doubles_per_env(nj, nq, nv, K);
  if (n < 0 || (per > 0 && n > INT64_MAX / per)) return -1;
  return per * n;
}

// Whole rollout backward: groups of as many segments as the scratch holds, latest first;
// per group one recompute launch over (segment, env) and one reverse launch over envs.
// `recompute` / `reverse` launch one group (RolloutArgs with s_lo / s_cnt set).
template <class Recompute, class Reverse>
cudaError_t rollout_backward_grouped(RolloutArgs a, int64_t seg_doubles, int64_t scratch_doubles,
                                     Recompute recompute, Reverse reverse) {
  const int nseg = (a.T + a.K - 1) / a.K;
  const int64_t fit = seg_doubles > 0 ? scratch_doubles / seg_doubles : 0;
  const int G = int(fit < nseg ? fit : nseg);
  if (nseg == 0) {  // no steps: the adjoint passes through
    a.s_lo = 0;
    a.s_cnt = 0;
    return reverse(a);
  }
  if (G <= 0) return cudaErrorInvalidValue;
  for (int hi = nseg; hi > 0; hi -= G) {
    a.s_lo = hi - G > 0 ? hi - G : 0;
    a.s_cnt = hi - a.s_lo;
    if (cudaError_t e = recompute(a)) return e;
    if (cudaError_t e = reverse(a)) return e;
  }
  return cudaSuccess;
}
#endif  // __CUDACC_RTC__

}  // namespace sgdyn
