// Bucket dispatch for the fused sweep.
#include "kernels.h"

namespace sgdyn {

cudaError_t launch_step_j16(const DModel*, int, const StepArgs&, cudaStream_t);
cudaError_t launch_step_j32(const DModel*, int, const StepArgs&, cudaStream_t);
cudaError_t launch_step_j64(const DModel*, int, const StepArgs&, cudaStream_t);

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
