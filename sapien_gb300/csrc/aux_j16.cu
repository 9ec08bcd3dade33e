// Instantiations of the link-Jacobian, Coriolis and IK kernels for trees of up to 16 joints.
#include "aux_kernels.cuh"

namespace sgdyn {

cudaError_t launch_link_jacobian_j16(const DModel* dm, const LinkJacArgs& a, cudaStream_t s) {
  link_jacobian_kernel<16><<<unsigned((a.n + 31) / 32), 32, 0, s>>>(dm, a);
  return cudaGetLastError();
}
cudaError_t launch_coriolis_j16(const DModel* dm, const CoriolisArgs& a, cudaStream_t s) {
  coriolis_kernel<16><<<unsigned((a.n + 31) / 32), 32, 0, s>>>(dm, a);
  return cudaGetLastError();
}
cudaError_t launch_ik_j16(const DModel* dm, const IkArgs& a, cudaStream_t s) {
  static int occ = 0;
  if (occ == 0 && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ik_kernel<16>, 32, 0) != cudaSuccess) occ = 1;
  ik_kernel<16><<<balanced_grid(a.n, occ), 32, 0, s>>>(dm, a);
  return cudaGetLastError();
}

}  // namespace sgdyn
