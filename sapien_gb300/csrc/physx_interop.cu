// Interop with SAPIEN's batched GPU articulation state.
//
// SAPIEN's GPU physics keeps qpos / qvel / qf of all articulations in float32 buffers of
// shape [nArt, maxDof] with a row stride of maxDof elements (src/physx/physx_system.cpp:
// 1074-1081), exported to users as CUDA array handles / DLPack / torch tensors. This file
// computes PhysxArticulation::computePassiveForce(gravity, coriolisAndCentrifugal)
// (src/physx/articulation.cpp:400-418) for every articulation straight from those buffers:
// float32 state promoted to FP64, RNEA(q, qd, 0) with gravity and/or velocity terms, the
// result rounded to float32 into a qf-shaped buffer (e.g. PhysX's own qf buffer, for
// gravity compensation). The model's joint order must be SAPIEN's active-joint order, as
// create_pinocchio_model sets it.
#include <cuda_runtime.h>

#include <string>

#include "../../include/sgdyn.h"
#include "trace.h"
#include "model.h"
#include "step_kernel.cuh"

struct sgdyn_model {
  sgdyn::Model* impl;
};

namespace sgdyn {

int set_last_error(int code, const std::string& msg);

namespace {

// Runtime table with gravity replaced (zero when gravity terms are not wanted).
struct GravityTab {
  static constexpr bool kStatic = false;
  const DModel* m;
  double g[3];
  __device__ __forceinline__ int nj() const { return m->nj; }
  __device__ __forceinline__ int nv() const { return m->nv; }
  __device__ __forceinline__ int nq_ext() const { return m->nq_ext; }
  __device__ __forceinline__ int nlinks() const { return m->nlinks; }
  __device__ __forceinline__ double gravity(int k) const { return g[k]; }
  __device__ __forceinline__ const DJoint& joint(int i) const { return model_joints(m)[i]; }
  __device__ __forceinline__ const DLink& link(int l) const { return model_links(m)[l]; }
};

struct PassiveArgs {
  int64_t n;
  const float* qpos;
  const float* qvel;
  int64_t in_stride;
  float* qf;
  int64_t out_stride;
  int gravity, coriolis;
};

template <int MAXJ>
__global__ void __launch_bounds__(32) passive_force_kernel(const DModel* __restrict__ model, const PassiveArgs a) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  constexpr int MAXV = MAXJ + 5;
  const int nv = model->nv, nq = model->nq_ext;
  double q[MAXV + 1], qd[MAXV], zero[MAXV], tau[MAXV];
  for (int c = 0; c < nq; c++) q[c] = double(a.qpos[e * a.in_stride + c]);
  for (int c = 0; c < nv; c++) {
    qd[c] = a.coriolis ? double(a.qvel[e * a.in_stride + c]) : 0.0;
    zero[c] = 0.0;
  }
  GravityTab T{model, {a.gravity ? model->gravity[0] : 0.0, a.gravity ? model->gravity[1] : 0.0,
                       a.gravity ? model->gravity[2] : 0.0}};
  StepArgs io{};
  io.n = 1;
  io.q = Arr{q, 0, 1};
  io.qd = Arr{qd, 0, 1};
  io.qdd = Arr{zero, 0, 1};
  io.tau_out = Arr{tau, 0, 1};
  step_env_t<MAXJ, OP_RNEA>(T, io, 0);
  for (int c = 0; c < nv; c++) a.qf[e * a.out_stride + c] = float(tau[c]);
}

}  // namespace
}  // namespace sgdyn

using namespace sgdyn;

extern "C" int sgdyn_compute_passive_force_f32(const sgdyn_model* m, int64_t n, const float* qpos, const float* qvel,
                                               int64_t in_stride, int gravity, int coriolis_and_centrifugal,
                                               float* qf, int64_t out_stride, void* stream) {
  SG_TRACE("sgdyn_compute_passive_force_f32");
  if (!m || !m->impl) return set_last_error(SGDYN_ERR_NULL, "null model");
  Model& Mo = *m->impl;
  if (Mo.has_free_flyer()) return set_last_error(SGDYN_ERR_UNSUPPORTED, "passive force needs a fixed-base model");
  if (stash_bucket(Mo.njoints()) == 0) return set_last_error(SGDYN_ERR_UNSUPPORTED, "model has too many joints");
  if (n < 0) return set_last_error(SGDYN_ERR_RUNTIME, "negative batch size");
  if (in_stride < Mo.nq_ext() || out_stride < Mo.nv())
    return set_last_error(SGDYN_ERR_RUNTIME, "row stride smaller than the model's dof");
  if (n == 0) return SGDYN_OK;
  if (!device_accessible(qpos) || !device_accessible(qf) || (coriolis_and_centrifugal && !device_accessible(qvel)))
    return set_last_error(SGDYN_ERR_NULL, "qpos / qvel / qf is null or not device memory");
  int err = 0;
  const DModel* dm = Mo.device_table(&err);
  if (!dm) return set_last_error(SGDYN_ERR_CUDA, "model upload failed");
  PassiveArgs a{n, qpos, qvel, in_stride, qf, out_stride, gravity ? 1 : 0, coriolis_and_centrifugal ? 1 : 0};
  const unsigned blocks = unsigned((n + 31) / 32);
  auto s = static_cast<cudaStream_t>(stream);
  switch (stash_bucket(Mo.njoints())) {
    case 16: passive_force_kernel<16><<<blocks, 32, 0, s>>>(dm, a); break;
    case 32: passive_force_kernel<32><<<blocks, 32, 0, s>>>(dm, a); break;
    default: passive_force_kernel<64><<<blocks, 32, 0, s>>>(dm, a); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_last_error(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return SGDYN_OK;
}
