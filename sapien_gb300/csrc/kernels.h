// Launcher interface between the C-ABI layer and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "device_model.h"

namespace sgdyn {

// A batched 2-D array: element (env, col) lives at p[env * es + col * cs].
// Row-major [N][cols] is es = cols, cs = 1; column-major / SoA [cols][N] is es = 1, cs = N.
struct Arr {
  double* p;
  int64_t es, cs;
};

enum Ops : int { OP_FK = 1, OP_JAC = 2, OP_CRBA = 4, OP_RNEA = 8, OP_ABA = 16, OP_ALL = 31 };

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

// Joint-count bucket for the per-thread stash (16, 32 or 64 joints incl. universe).
int stash_bucket(int nj);

// Fused world-frame sweep: any subset of {FK poses, full WORLD Jacobian, CRBA, RNEA, ABA}.
cudaError_t launch_step(const DModel* dm, int nj, int ops, const StepArgs& a, cudaStream_t s);
cudaError_t launch_link_jacobian(const DModel* dm, int nj, const LinkJacArgs& a, cudaStream_t s);
cudaError_t launch_coriolis(const DModel* dm, int nj, const CoriolisArgs& a, cudaStream_t s);
cudaError_t launch_ik(const DModel* dm, int nj, const IkArgs& a, cudaStream_t s);

}  // namespace sgdyn
