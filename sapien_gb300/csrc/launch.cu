// Bucket dispatch for the fused sweep.
#include "kernels.h"

namespace sgdyn {

cudaError_t launch_step_j16(const DModel*, int, const StepArgs&, cudaStream_t);
cudaError_t launch_step_j32(const DModel*, int, const StepArgs&, cudaStream_t);
cudaError_t launch_step_j64(const DModel*, int, const StepArgs&, cudaStream_t);
cudaError_t launch_step_team_j16(const DModel*, const int*, int, int, const StepArgs&, cudaStream_t);
cudaError_t launch_step_team_j32(const DModel*, const int*, int, int, const StepArgs&, cudaStream_t);
cudaError_t launch_step_team_j64(const DModel*, const int*, int, int, const StepArgs&, cudaStream_t);

cudaError_t launch_step_team(const DModel* dm, int nj, const int* team, int lanes, int ops, const StepArgs& a,
                             cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  switch (stash_bucket(nj)) {
    case 16: return launch_step_team_j16(dm, team, lanes, ops, a, s);
    case 32: return launch_step_team_j32(dm, team, lanes, ops, a, s);
    case 64: return launch_step_team_j64(dm, team, lanes, ops, a, s);
    default: return cudaErrorInvalidValue;
  }
}

int stash_bucket(int nj) { return nj <= 16 ? 16 : nj <= 32 ? 32 : nj <= 64 ? 64 : 0; }

cudaError_t launch_step(const DModel* dm, int nj, int ops, const StepArgs& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  switch (stash_bucket(nj)) {
    case 16: return launch_step_j16(dm, ops, a, s);
    case 32: return launch_step_j32(dm, ops, a, s);
    case 64: return launch_step_j64(dm, ops, a, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sgdyn

#include "aux_kernels.cuh"

namespace sgdyn {

#define SG_DECL(J)                                                                    \
  cudaError_t launch_link_jacobian_j##J(const DModel*, const LinkJacArgs&, cudaStream_t); \
  cudaError_t launch_coriolis_j##J(const DModel*, const CoriolisArgs&, cudaStream_t);    \
  cudaError_t launch_ik_j##J(const DModel*, const IkArgs&, cudaStream_t);
SG_DECL(16)
SG_DECL(32)
SG_DECL(64)
#undef SG_DECL

cudaError_t launch_link_jacobian(const DModel* dm, int nj, const LinkJacArgs& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  switch (stash_bucket(nj)) {
    case 16: return launch_link_jacobian_j16(dm, a, s);
    case 32: return launch_link_jacobian_j32(dm, a, s);
    case 64: return launch_link_jacobian_j64(dm, a, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_coriolis(const DModel* dm, int nj, const CoriolisArgs& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  switch (stash_bucket(nj)) {
    case 16: return launch_coriolis_j16(dm, a, s);
    case 32: return launch_coriolis_j32(dm, a, s);
    case 64: return launch_coriolis_j64(dm, a, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_ik(const DModel* dm, int nj, const IkArgs& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  switch (stash_bucket(nj)) {
    case 16: return launch_ik_j16(dm, a, s);
    case 32: return launch_ik_j32(dm, a, s);
    case 64: return launch_ik_j64(dm, a, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sgdyn

#include "diff_kernels.cuh"

namespace sgdyn {

#define SG_DISPATCH(kernel, Args)                                                        \
  cudaError_t launch_##kernel##_j16(const DModel*, const Args&, cudaStream_t);            \
  cudaError_t launch_##kernel##_j32(const DModel*, const Args&, cudaStream_t);            \
  cudaError_t launch_##kernel##_j64(const DModel*, const Args&, cudaStream_t);            \
  cudaError_t launch_##kernel(const DModel* dm, int nj, const Args& a, cudaStream_t s) {  \
    if (a.n <= 0) return cudaSuccess;                                                    \
    switch (stash_bucket(nj)) {                                                          \
      case 16: return launch_##kernel##_j16(dm, a, s);                                   \
      case 32: return launch_##kernel##_j32(dm, a, s);                                   \
      case 64: return launch_##kernel##_j64(dm, a, s);                                   \
      default: return cudaErrorInvalidValue;                                             \
    }                                                                                    \
  }
SG_DISPATCH(rnea_vjp, VjpArgs)
SG_DISPATCH(aba_vjp, VjpArgs)
SG_DISPATCH(fk_vjp, FkVjpArgs)
SG_DISPATCH(rnea_derivatives, DerivArgs)
SG_DISPATCH(aba_derivatives, DerivArgs)
SG_DISPATCH(rollout_forward, RolloutArgs)
SG_DISPATCH(rollout_forward3, RolloutArgs)
SG_DISPATCH(rollout_recompute, RolloutArgs)
SG_DISPATCH(rollout_reverse, RolloutArgs)
SG_DISPATCH(rollout_reverse3, RolloutArgs)
SG_DISPATCH(aba3, StepArgs)
#undef SG_DISPATCH

int64_t rollout_scratch_doubles_per_env(int nj, int nq, int nv, int K) {
  return int64_t(K) * stash_doubles_per_step(nj, nq, nv);
}

}  // namespace sgdyn
