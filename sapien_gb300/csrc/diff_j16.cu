// Instantiations of the differentiation kernels for trees of up to 16 joints.
#include "diff_kernels.cuh"
#include "team3.cuh"

namespace sgdyn {

#define SG_LAUNCH(kernel, Args)                                                      \
  cudaError_t launch_##kernel##_j16(const DModel* dm, const Args& a, cudaStream_t s) { \
    kernel##_kernel<16><<<unsigned((a.n + 31) / 32), 32, 0, s>>>(dm, a);             \
    return cudaGetLastError();                                                      \
  }
SG_LAUNCH(rnea_vjp, VjpArgs)
SG_LAUNCH(aba_vjp, VjpArgs)
SG_LAUNCH(fk_vjp, FkVjpArgs)
SG_LAUNCH(rollout_forward, RolloutArgs)
SG_LAUNCH(rollout_reverse, RolloutArgs)
#undef SG_LAUNCH

cudaError_t launch_rnea_derivatives_j16(const DModel* dm, const DerivArgs& a, cudaStream_t s) {
  deriv_prepare_kernel<16, false><<<unsigned((a.n + 31) / 32), 32, 0, s>>>(dm, a);
  if (cudaError_t e = cudaGetLastError()) return e;
  const int64_t nv = (a.lay.Q - a.lay.P) / 6;
  rnea_deriv_columns_kernel<16><<<unsigned((a.n * nv + 127) / 128), 128, 0, s>>>(dm, a);
  return cudaGetLastError();
}
cudaError_t launch_aba_derivatives_j16(const DModel* dm, const DerivArgs& a, cudaStream_t s) {
  deriv_prepare_kernel<16, true><<<unsigned((a.n + 31) / 32), 32, 0, s>>>(dm, a);
  if (cudaError_t e = cudaGetLastError()) return e;
  const int64_t nv = (a.lay.Q - a.lay.P) / 6;
  aba_deriv_columns_kernel<16><<<unsigned((a.n * nv + 127) / 128), 128, 0, s>>>(dm, a);
  return cudaGetLastError();
}
cudaError_t launch_rollout_forward3_j16(const DModel* dm, const RolloutArgs& a, cudaStream_t s) {
  rollout_forward3_kernel<16><<<unsigned((a.n + 9) / 10), 32, 0, s>>>(dm, a);
  return cudaGetLastError();
}
cudaError_t launch_rollout_reverse3_j16(const DModel* dm, const RolloutArgs& a, cudaStream_t s) {
  rollout_reverse3_kernel<16><<<unsigned((a.n + 9) / 10), 32, 0, s>>>(dm, a);
  return cudaGetLastError();
}
cudaError_t launch_aba3_j16(const DModel* dm, const StepArgs& a, cudaStream_t s) {
  aba3_kernel<16><<<unsigned((a.n + 9) / 10), 32, 0, s>>>(dm, a);
  return cudaGetLastError();
}
cudaError_t launch_rollout_recompute_j16(const DModel* dm, const RolloutArgs& a, cudaStream_t s) {
  rollout_recompute_kernel<16><<<unsigned((a.n * a.s_cnt + 31) / 32), 32, 0, s>>>(dm, a);
  return cudaGetLastError();
}

}  // namespace sgdyn
