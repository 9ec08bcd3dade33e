// Instantiations of the fused sweep for trees of up to 32 joints (incl. universe).
#include "step_kernel.cuh"

namespace sgdyn {

cudaError_t launch_step_j32(const DModel* dm, int ops, const StepArgs& a, cudaStream_t s) {
  const unsigned blocks = unsigned((a.n + 31) / 32);
  switch (ops) {
#define SG_CASE(O) \
  case O: step_kernel<32, O><<<blocks, 32, 0, s>>>(dm, a); break;
    SG_CASE(OP_FK)
    SG_CASE(OP_JAC)
    SG_CASE(OP_FK | OP_JAC)
    SG_CASE(OP_CRBA)
    SG_CASE(OP_RNEA)
    SG_CASE(OP_ABA)
    SG_CASE(OP_RNEA | OP_ABA)
    SG_CASE(OP_CRBA | OP_RNEA | OP_ABA)
    SG_CASE(OP_ALL)
#undef SG_CASE
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_step_team_j32(const DModel* dm, const int* team, int lanes, int ops, const StepArgs& a,
                                  cudaStream_t s) {
  const int per = 32 / lanes;
  const unsigned blocks = unsigned((a.n + per - 1) / per);
  switch (ops) {
#define SG_CASE(O) \
  case O: step_team_kernel<32, O><<<blocks, 32, 0, s>>>(dm, team, a); break;
    SG_CASE(OP_FK)
    SG_CASE(OP_JAC)
    SG_CASE(OP_FK | OP_JAC)
    SG_CASE(OP_CRBA)
    SG_CASE(OP_RNEA)
    SG_CASE(OP_ABA)
    SG_CASE(OP_RNEA | OP_ABA)
    SG_CASE(OP_CRBA | OP_RNEA | OP_ABA)
    SG_CASE(OP_ALL)
#undef SG_CASE
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace sgdyn
