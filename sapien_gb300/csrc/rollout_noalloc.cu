// Allocation-free reverse rollout: sgdyn_rollout_backward_noalloc.
//
// sgdyn_rollout_backward needs a caller-provided device scratch buffer that holds one
// checkpoint segment's recomputed intermediates. Some callers cannot allocate device
// memory at the point where they need gradients: a real-time control or planning loop
// that reserves all of its memory at start-up and must not enter the CUDA allocator
// while it runs (allocation latency is unbounded, and a failed allocation mid-loop has
// no recovery), or a plug-in invoked by a host application that owns the device memory
// budget and gives plug-ins none. For them this file keeps the scratch in a fixed
// file-scope device array that exists for as long as the library is loaded.
//
// Properties a caller must know:
//  * The array holds SGDYN_NOALLOC_SCRATCH_BYTES (64 MiB) on every GPU that loads the
//    library, until the process exits. A call that needs more (8 * n * checkpoint_every *
//    per-step doubles, see sgdyn_rollout_scratch_bytes) is rejected with
//    SGDYN_ERR_RUNTIME before any work is enqueued.
//  * Nothing here calls cudaMalloc, cudaFree or an allocating library routine. The model
//    tables must already be on the device (sgdyn_model_upload, or any earlier compute
//    call on that device); otherwise the call fails instead of uploading them.
//  * Every call looks up the array's device address on the current device with
//    cudaGetSymbolAddress. The first lookup on a device may load the library's device code
//    there, so make one call on each device before any stream capture begins and outside
//    any time-critical loop: a call with n = 0 does the lookup and nothing else. The address
//    is not cached, so a call after a device reset finds the array in the new context.
//  * All calls on a device share the one array, and it keeps whatever the last call left
//    in it. Every scratch value a call reads is first written by that same call, so no
//    clearing is needed, but two calls whose kernels overlap on the GPU (different
//    streams, or different host threads) race on the array: serialise them.
#include <cuda_runtime.h>

#include <functional>
#include <string>

#include "../../include/sgdyn.h"
#include "kernels.h"
#include "model.h"

struct sgdyn_model {
  sgdyn::Model* impl;
};

namespace sgdyn {

int set_last_error(int code, const std::string& msg);
int call_guarded(const std::function<int()>& body);
int rollout_lanes_for(const Model& M, int64_t n);

namespace {

constexpr int64_t kNoAllocScratchBytes = SGDYN_NOALLOC_SCRATCH_BYTES;
static_assert(kNoAllocScratchBytes % 256 == 0, "scratch size");

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchBytes / sizeof(double)];

// Device address of g_noalloc_scratch in the current device's context.
double* scratch_on_current_device(std::string* why) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    *why = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
    return nullptr;
  }
  return static_cast<double*>(p);
}

}  // namespace
}  // namespace sgdyn

using namespace sgdyn;

extern "C" int sgdyn_rollout_backward_noalloc(const sgdyn_model* m, int64_t n, int T, double dt,
                                              int checkpoint_every, const double* q_ckpt, const double* qd_ckpt,
                                              const double* tau, const double* qT_bar, const double* qdT_bar,
                                              double* q0_bar, double* qd0_bar, double* tau_bar, void* stream) {
  return call_guarded([&]() -> int {
    if (!m || !m->impl) return set_last_error(SGDYN_ERR_NULL, "null model");
    Model& Mo = *m->impl;
    if (stash_bucket(Mo.njoints()) == 0) return set_last_error(SGDYN_ERR_UNSUPPORTED, "model has too many joints");
    for (auto& J : Mo.joints)
      if (J.kind == JK_FREEFLYER && J.parent != 0)
        return set_last_error(SGDYN_ERR_UNSUPPORTED, "rollouts need the free-flyer joint at the root");
    if (n < 0 || T < 0) return set_last_error(SGDYN_ERR_RUNTIME, "negative size");
    if (checkpoint_every <= 0) return set_last_error(SGDYN_ERR_RUNTIME, "checkpoint_every must be positive");
    const int64_t need = rollout_scratch_bytes_for(Mo.njoints(), Mo.nq_ext(), Mo.nv(), checkpoint_every, n);
    if (need < 0 || need > kNoAllocScratchBytes)
      return set_last_error(SGDYN_ERR_RUNTIME, "allocation-free rollout backward needs " +
                                                   (need < 0 ? std::string("more than INT64_MAX") : std::to_string(need)) +
                                                   " bytes of scratch but holds " +
                                                   std::to_string(kNoAllocScratchBytes) +
                                                   "; use fewer environments, a shorter checkpoint interval, or "
                                                   "sgdyn_rollout_backward with your own buffer");
    std::string why;
    double* scratch = scratch_on_current_device(&why);  // also the warm-up an n = 0 call does
    if (!scratch) return set_last_error(SGDYN_ERR_CUDA, why);
    if (n == 0) return SGDYN_OK;
    if (!device_accessible(q0_bar) || !device_accessible(qd0_bar))
      return set_last_error(SGDYN_ERR_NULL, "q0_bar / qd0_bar is null or not device memory");
    if (T > 0 && (!device_accessible(q_ckpt) || !device_accessible(qd_ckpt) || !device_accessible(tau) || !device_accessible(tau_bar)))
      return set_last_error(SGDYN_ERR_NULL, "checkpoint, tau or tau_bar is null or not device memory");
    if ((qT_bar && !device_accessible(qT_bar)) || (qdT_bar && !device_accessible(qdT_bar)))
      return set_last_error(SGDYN_ERR_NULL, "adjoint input is not device memory");
    const DModel* dm = Mo.find_device_table();
    if (!dm)
      return set_last_error(SGDYN_ERR_RUNTIME,
                            "model tables are not on this device; call sgdyn_model_upload first (this entry point "
                            "does not allocate)");
    RolloutArgs a{};
    a.n = n;
    a.T = T;
    a.K = checkpoint_every;
    a.dt = dt;
    a.tau = tau;
    a.q_ckpt = const_cast<double*>(q_ckpt);
    a.qd_ckpt = const_cast<double*>(qd_ckpt);
    a.qT_bar = qT_bar;
    a.qdT_bar = qdT_bar;
    a.q0_bar = q0_bar;
    a.qd0_bar = qd0_bar;
    a.tau_bar = tau_bar;
    a.scratch = scratch;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nj = Mo.njoints();
    const int lanes = rollout_lanes_for(Mo, n);
    cudaError_t e = rollout_backward_grouped(
        a, need / 8, kNoAllocScratchBytes / 8,
        [&](const RolloutArgs& g) { return launch_rollout_recompute(dm, nj, g, st); },
        [&](const RolloutArgs& g) {
          return lanes == 3 ? launch_rollout_reverse3(dm, nj, g, st) : launch_rollout_reverse(dm, nj, g, st);
        });
    if (e != cudaSuccess) return set_last_error(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
    return SGDYN_OK;
  });
}
