// C-ABI entry points (declared in include/sgdyn.h): argument validation, error
// translation and kernel dispatch. Errors follow the reference's exception split
// (pinocchio/pinocchio_model.cpp:33-36, 105, 121, 136): std::invalid_argument for bad
// names -> SGDYN_ERR_INVALID_ARGUMENT, std::runtime_error -> SGDYN_ERR_RUNTIME.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sgdyn.h"
#include "trace.h"
#include "jit.h"
#include "kernels.h"
#include "model.h"

struct sgdyn_model {
  sgdyn::Model* impl;
};

namespace sgdyn {

// Rejects pageable host pointers before they reach a kernel.
bool device_accessible(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return true;
  // pinned host memory mapped at the same address in the device's space: kernels read and
  // write it directly over the host link (no staging copy)
  return at.type == cudaMemoryTypeHost && at.devicePointer == p;
}

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const std::invalid_argument& e) {
    return fail(SGDYN_ERR_INVALID_ARGUMENT, e.what());
  } catch (const std::exception& e) {
    return fail(SGDYN_ERR_RUNTIME, e.what());
  } catch (...) {
    return fail(SGDYN_ERR_RUNTIME, "unknown error");
  }
}


Arr make_arr(const void* p, int64_t n, int64_t cols, int layout) {
  Arr a;
  a.p = static_cast<double*>(const_cast<void*>(p));
  if (layout == SGDYN_ENV_MAJOR) {
    a.es = cols;
    a.cs = 1;
  } else {
    a.es = 1;
    a.cs = n;
  }
  return a;
}

int check_model(const sgdyn_model* m) {
  if (!m || !m->impl) return fail(SGDYN_ERR_NULL, "null model");
  const Model& M = *m->impl;
  if (stash_bucket(M.njoints()) == 0)
    return fail(SGDYN_ERR_UNSUPPORTED, "model has more than 63 moving joints");
  int nff = 0;
  for (auto& J : M.joints) nff += J.kind == JK_FREEFLYER;
  if (nff > 1) return fail(SGDYN_ERR_UNSUPPORTED, "model has more than one free-flyer joint");
  return SGDYN_OK;
}

struct Req {
  const void* p;
  const char* name;
};
int check_ptrs(std::initializer_list<Req> reqs) {
  for (auto& r : reqs)
    if (!device_accessible(r.p)) return fail(SGDYN_ERR_NULL, std::string(r.name) + " is null or not device memory");
  return SGDYN_OK;
}

// A second stream per device (created once, kept for the process) for work that runs beside
// the caller's stream: the rollout backward's recompute launches and the FK + Jacobian half
// of a split five-op step; null if it cannot be created.
cudaStream_t side_stream() {
  static std::mutex mu;
  static std::map<int, cudaStream_t> streams;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  auto it = streams.find(dev);
  if (it != streams.end()) return it->second;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) s = nullptr;
  streams[dev] = s;
  return s;
}

// Whether the five-op step runs as two concurrent launches (CRBA + RNEA + ABA on the caller's
// stream, FK + Jacobian on the side stream, joined by events): 0 never, 1 always, 2
// automatic (the default: when one warp per 32 environments gives fewer than two warps per
// FP64 scheduler, so the FK + Jacobian warps land on idle or lightly loaded schedulers).
// Never while the caller's stream is being captured.
std::atomic<int> g_split_mode{2};

int device_schedulers() {
  static int schedulers = 0;
  if (schedulers == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    schedulers = 4 * (sms > 0 ? sms : 1);
  }
  return schedulers;
}

// Lanes per environment of the forward rollout, of the backward's reverse sweep (the
// recompute keeps one lane: all its segments run at once and fill the GPU) and of forward
// dynamics requested alone: 1, or 3 (team3.cuh: one lane per axis; one-DoF joints and a
// free-flyer root). The setting: 0 automatic (the default: three lanes while one warp per ten
// environments leaves no FP64 scheduler with two warps), 1 or 3.
std::atomic<int> g_rollout_lanes{0};

int rollout_lanes(const Model& M, int64_t n) {
  for (auto& J : M.joints)
    if (J.kind == JK_FREEFLYER && J.parent != 0) return 1;  // a free flyer only as the root
  const int mode = g_rollout_lanes.load();
  if (mode != 0) return mode;
  return (n + 9) / 10 <= int64_t(device_schedulers()) ? 3 : 1;
}

}  // namespace

// Lanes per environment of the rollout kernels for this model and batch (1 or 3).
int rollout_lanes_for(const Model& M, int64_t n) { return rollout_lanes(M, n); }

namespace {

bool use_split(int64_t n) {
  const int mode = g_split_mode.load();
  if (mode != 2) return mode == 1;
  return (n + 31) / 32 < 2 * int64_t(device_schedulers());
}

// Lanes per environment for a single-model sweep: the model's setting, or (0 = automatic)
// the count with the shortest estimated time when the batch leaves FP64 schedulers idle. A
// small batch is bound by one warp's sequential sweep, so the estimate is the team plan's
// critical path (trunk + heaviest lane) times the number of warp rounds the lanes need.
int choose_lanes(Model& M, int64_t n) {
  if (M.lanes > 0) return M.lanes;
  const int schedulers = device_schedulers();
  if ((n + 31) / 32 * 2 > schedulers) return 1;  // the batch alone fills the GPU
  int best = 1;
  double best_est = 0;
  for (int L : {1, 2, 4, 8}) {
    const int cp = M.team_critical_path(L);
    const double rounds = std::max(1.0, double((n * L + 31) / 32) / schedulers);
    const double est = cp * rounds;
    if (L == 1) best_est = est;
    else if (est < 0.8 * best_est) {
      best = L;
      best_est = est;
    }
  }
  return best;
}

int run_step(const sgdyn_model* m, int64_t n, int ops, const double* q, const double* qd, const double* qdd,
             const double* tau, double* poses, double* J, double* M, double* tau_out, double* qdd_out, int layout,
             void* stream) {
  if (int rc = check_model(m)) return rc;
  if (n < 0) return fail(SGDYN_ERR_RUNTIME, "negative batch size");
  if (layout != SGDYN_ENV_MAJOR && layout != SGDYN_COL_MAJOR) return fail(SGDYN_ERR_RUNTIME, "bad layout");
  if (ops <= 0 || ops > OP_ALL) return fail(SGDYN_ERR_RUNTIME, "bad op mask");
  if (n == 0) return SGDYN_OK;
  Model& Mo = *m->impl;
  if (int rc = check_ptrs({{q, "q"}})) return rc;
  if (ops & (OP_RNEA | OP_ABA))
    if (int rc = check_ptrs({{qd, "qd"}})) return rc;
  if (ops & OP_RNEA)
    if (int rc = check_ptrs({{qdd, "qdd"}, {tau_out, "tau_out"}})) return rc;
  if (ops & OP_ABA)
    if (int rc = check_ptrs({{tau, "tau"}, {qdd_out, "qdd_out"}})) return rc;
  if (ops & OP_FK)
    if (int rc = check_ptrs({{poses, "link_poses"}})) return rc;
  if (ops & OP_JAC)
    if (int rc = check_ptrs({{J, "J"}})) return rc;
  if (ops & OP_CRBA)
    if (int rc = check_ptrs({{M, "M"}})) return rc;
  int err = 0;
  const DModel* dm = Mo.device_table(&err);
  if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
  const int64_t nv = Mo.nv();
  StepArgs a;
  a.n = n;
  a.q = make_arr(q, n, Mo.nq_ext(), layout);
  a.qd = make_arr(qd, n, nv, layout);
  a.qdd = make_arr(qdd, n, nv, layout);
  a.tau = make_arr(tau, n, nv, layout);
  a.poses = make_arr(poses, n, int64_t(Mo.nlinks()) * 7, layout);
  a.J = make_arr(J, n, 6 * nv, layout);
  a.M = make_arr(M, n, nv * nv, layout);
  a.tau_out = make_arr(tau_out, n, nv, layout);
  a.qdd_out = make_arr(qdd_out, n, nv, layout);
  auto s = static_cast<cudaStream_t>(stream);
  static const int fused[] = {OP_ALL, OP_CRBA | OP_RNEA | OP_ABA, OP_RNEA | OP_ABA, OP_FK | OP_JAC};
  int rest = ops;
  std::vector<int> launches;
  for (int f : fused)
    if ((rest & f) == f && f != 0 && __builtin_popcount(f) > 1) {
      launches.push_back(f);
      rest &= ~f;
    }
  for (int b = 1; b <= OP_ABA; b <<= 1)
    if (rest & b) launches.push_back(b);
  const int lanes = choose_lanes(Mo, n);
  const int* team = nullptr;
  if (lanes > 1) {
    team = Mo.device_team(lanes, &err);
    if (!team) return fail(SGDYN_ERR_CUDA, "team table upload failed");
  } else if (ops == OP_ABA && rollout_lanes(Mo, n) == 3) {  // forward dynamics alone on three lanes
    std::string why;
    if (launch_aba3_jit(Mo, a, s, &why)) return SGDYN_OK;
    cudaError_t e = launch_aba3(dm, Mo.njoints(), a, s);
    if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
    return SGDYN_OK;
  } else if (ops == OP_ALL && use_split(n)) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) cs = cudaStreamCaptureStatusActive;
    cudaStream_t s2 = cs == cudaStreamCaptureStatusNone ? side_stream() : nullptr;
    if (s2) {
      auto one = [&](int o, cudaStream_t st) -> cudaError_t {
        std::string why;
        if (launch_step_jit(Mo, o, a, st, &why)) return cudaSuccess;
        return launch_step(dm, Mo.njoints(), o, a, st);
      };
      cudaEvent_t fork = nullptr, join = nullptr;
      cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(fork, s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, fork, 0);
      if (e == cudaSuccess) e = one(OP_SPLIT_B, s);
      if (e == cudaSuccess) e = one(OP_SPLIT_A, s2);
      if (e == cudaSuccess) e = cudaEventRecord(join, s2);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
      if (fork) cudaEventDestroy(fork);  // released once the recorded work completes
      if (join) cudaEventDestroy(join);
      if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
      return SGDYN_OK;
    }
  }
  for (int o : launches) {
    if (team) {  // several lanes per environment
      std::string why;
      if (launch_step_roles_jit(Mo, lanes, o, a, s, &why)) continue;  // one warp per role, specialised
      cudaError_t e = launch_step_team(dm, Mo.njoints(), team, lanes, o, a, s);
      if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
      continue;
    }
    std::string why;
    if (launch_step_jit(Mo, o, a, s, &why)) continue;  // model-specialised kernel
    cudaError_t e = launch_step(dm, Mo.njoints(), o, a, s);
    if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  }
  return SGDYN_OK;
}


// Differentiation kernels support a free flyer only as the root joint.
int check_diff_model(const sgdyn_model* m) {
  if (int rc = check_model(m)) return rc;
  for (auto& J : m->impl->joints)
    if (J.kind == JK_FREEFLYER && J.parent != 0)
      return fail(SGDYN_ERR_UNSUPPORTED, "derivatives need the free-flyer joint at the root");
  return SGDYN_OK;
}

int common_checks(int64_t n, int layout) {
  if (n < 0) return fail(SGDYN_ERR_RUNTIME, "negative batch size");
  if (layout != SGDYN_ENV_MAJOR && layout != SGDYN_COL_MAJOR) return fail(SGDYN_ERR_RUNTIME, "bad layout");
  return SGDYN_OK;
}

int launch_status(cudaError_t e) {
  if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return SGDYN_OK;
}

}  // namespace
}  // namespace sgdyn

namespace sgdyn {
// Records a message for sgdyn_last_error() from entry points defined in other files.
int set_last_error(int code, const std::string& msg) { return fail(code, msg); }
// Runs an entry point's body with C++ exceptions turned into status codes, for entry
// points defined in other files.
int call_guarded(const std::function<int()>& body) { return guarded(body); }
}  // namespace sgdyn

using namespace sgdyn;

extern "C" {

const char* sgdyn_last_error(void) { return g_err.c_str(); }

int sgdyn_model_from_urdf(const char* urdf_xml, const double gravity[3], sgdyn_model** out) {
  if (!urdf_xml || !gravity || !out) return fail(SGDYN_ERR_NULL, "null argument");
  return guarded([&] {
    *out = nullptr;
    Model* M = Model::from_urdf(urdf_xml, gravity);
    *out = new sgdyn_model{M};
    return SGDYN_OK;
  });
}

int sgdyn_model_from_articulation(const sgdyn_link_desc* links, int nlinks, const sgdyn_joint_desc* joints,
                                  int njoints, const double gravity[3], int force_fix_root, sgdyn_model** out) {
  if (!links || (!joints && njoints > 0) || !gravity || !out) return fail(SGDYN_ERR_NULL, "null argument");
  static_assert(sizeof(sgdyn_link_desc) == sizeof(ArtLink), "link layout");
  static_assert(sizeof(sgdyn_joint_desc) == sizeof(ArtJoint), "joint layout");
  return guarded([&] {
    *out = nullptr;
    Model* M = Model::from_articulation(reinterpret_cast<const ArtLink*>(links), nlinks,
                                        reinterpret_cast<const ArtJoint*>(joints), njoints, gravity,
                                        force_fix_root != 0);
    *out = new sgdyn_model{M};
    return SGDYN_OK;
  });
}

void sgdyn_model_free(sgdyn_model* m) {
  if (!m) return;
  delete m->impl;
  delete m;
}

int sgdyn_model_set_joint_order(sgdyn_model* m, const char* const* names, int n) {
  if (!m || (!names && n > 0) || n < 0) return fail(SGDYN_ERR_NULL, "null argument");
  return guarded([&] {
    std::vector<std::string> v(names, names + n);
    m->impl->set_joint_order(v);
    return SGDYN_OK;
  });
}

int sgdyn_model_set_link_order(sgdyn_model* m, const char* const* names, int n) {
  if (!m || (!names && n > 0) || n < 0) return fail(SGDYN_ERR_NULL, "null argument");
  return guarded([&] {
    std::vector<std::string> v(names, names + n);
    m->impl->set_link_order(v);
    return SGDYN_OK;
  });
}

int sgdyn_model_info(const sgdyn_model* m, int* nq_ext, int* nv, int* nlinks, int* njoints) {
  if (!m) return fail(SGDYN_ERR_NULL, "null model");
  if (nq_ext) *nq_ext = m->impl->nq_ext();
  if (nv) *nv = m->impl->nv();
  if (nlinks) *nlinks = m->impl->nlinks();
  if (njoints) *njoints = m->impl->njoints();
  return SGDYN_OK;
}

int sgdyn_model_random_configuration(const sgdyn_model* m, int64_t n, uint64_t seed, double* qpos) {
  if (!m || !m->impl || (n > 0 && !qpos)) return fail(SGDYN_ERR_NULL, "null argument");
  if (n < 0) return fail(SGDYN_ERR_RUNTIME, "negative batch size");
  return guarded([&] {
    m->impl->random_configuration(n, seed, qpos);
    return SGDYN_OK;
  });
}

int sgdyn_model_joint_kind(const sgdyn_model* m, int k, int* kind) {
  if (!m || !kind) return fail(SGDYN_ERR_NULL, "null argument");
  const Model& M = *m->impl;
  // external order = increasing q column
  for (int j = 1; j < M.njoints(); j++) {
    int rank = 0;
    for (int i = 1; i < M.njoints(); i++)
      if (M.ext_qcol_of_joint(i) < M.ext_qcol_of_joint(j)) rank++;
    if (rank == k) {
      *kind = M.joints[j].kind;
      return SGDYN_OK;
    }
  }
  return fail(SGDYN_ERR_RUNTIME, "joint index out of bound");
}

int sgdyn_model_joint_name(const sgdyn_model* m, int j, const char** name) {
  if (!m || !name) return fail(SGDYN_ERR_NULL, "null argument");
  if (j < 1 || j >= m->impl->njoints()) return fail(SGDYN_ERR_RUNTIME, "joint index out of bound");
  *name = m->impl->joints[j].name.c_str();
  return SGDYN_OK;
}

int sgdyn_model_body_count(const sgdyn_model* m, int* nbodies) {
  if (!m || !nbodies) return fail(SGDYN_ERR_NULL, "null argument");
  *nbodies = int(m->impl->bodies.size());
  return SGDYN_OK;
}

int sgdyn_model_body_name(const sgdyn_model* m, int b, const char** name) {
  if (!m || !name) return fail(SGDYN_ERR_NULL, "null argument");
  if (b < 0 || b >= int(m->impl->bodies.size())) return fail(SGDYN_ERR_RUNTIME, "body index out of bound");
  *name = m->impl->bodies[b].name.c_str();
  return SGDYN_OK;
}

int sgdyn_model_upload(sgdyn_model* m) {
  if (!m) return fail(SGDYN_ERR_NULL, "null model");
  int err = 0;
  if (!m->impl->device_table(&err)) return fail(SGDYN_ERR_CUDA, "model upload failed");
  return SGDYN_OK;
}

int sgdyn_model_table(const sgdyn_model* m, const void** data, int64_t* bytes) {
  if (!m || !data || !bytes) return fail(SGDYN_ERR_NULL, "null argument");
  *data = m->impl->host_table().data();
  *bytes = int64_t(m->impl->host_table().size());
  return SGDYN_OK;
}

int sgdyn_model_team_table(const sgdyn_model* m, int lanes, const int** data, int* count) {
  if (int rc = check_model(m)) return rc;
  if (!data || !count) return fail(SGDYN_ERR_NULL, "null argument");
  if (lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8) return fail(SGDYN_ERR_RUNTIME, "lanes must be 1, 2, 4 or 8");
  thread_local std::vector<int> buf;
  buf = m->impl->team_table(lanes);
  *data = buf.data();
  *count = int(buf.size());
  return SGDYN_OK;
}

int sgdyn_jit_max_joints(int max_joints, int* max_joints_out) {
  jit_max_joints(max_joints, max_joints_out);
  return SGDYN_OK;
}

int sgdyn_fd_method(int mode, int* mode_out) {
  if (mode != -1 && (mode < 0 || mode > 2)) return fail(SGDYN_ERR_RUNTIME, "forward-dynamics method must be -1, 0, 1 or 2");
  fd_method(mode, mode_out);
  return SGDYN_OK;
}

int sgdyn_fd_by_mass_matrix(const sgdyn_model* m, int ops, int* yes) {
  if (int rc = check_model(m)) return rc;
  if (!yes) return fail(SGDYN_ERR_NULL, "null argument");
  *yes = fd_by_mass_matrix(*m->impl, ops) ? 1 : 0;
  return SGDYN_OK;
}

int sgdyn_model_set_lanes(sgdyn_model* m, int lanes) {
  if (int rc = check_model(m)) return rc;
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8)
    return fail(SGDYN_ERR_RUNTIME, "lanes must be 0 (automatic), 1, 2, 4 or 8");
  m->impl->lanes = lanes;
  return SGDYN_OK;
}

int sgdyn_jit_config(int enable, int64_t min_n, int* enabled_out, int64_t* min_n_out) {
  set_jit_config(enable, min_n);
  get_jit_config(enabled_out, min_n_out);
  return SGDYN_OK;
}

// ops > 0: the fused sweep with that op set; -1: the forward rollout kernel; -2 / -3: the
// RNEA / ABA vector-Jacobian product kernels; -4: the forward rollout with three lanes per
// environment; -5: the backward's reverse sweep with three lanes per environment; -6:
// forward dynamics alone with three lanes per environment
static bool jit_kind_ok(int ops) { return (ops > 0 && ops <= OP_ALL) || (ops >= -7 && ops <= -1); }

int sgdyn_rollout_lanes(int lanes, int* lanes_out) {
  if (lanes != -1 && lanes != 0 && lanes != 1 && lanes != 3)
    return fail(SGDYN_ERR_RUNTIME, "rollout lanes must be -1, 0 (automatic), 1 or 3");
  if (lanes >= 0) g_rollout_lanes.store(lanes);
  if (lanes_out) *lanes_out = g_rollout_lanes.load();
  return SGDYN_OK;
}

int sgdyn_step_split(int mode, int* mode_out) {
  if (mode != -1 && (mode < 0 || mode > 2)) return fail(SGDYN_ERR_RUNTIME, "split mode must be -1, 0, 1 or 2");
  if (mode >= 0) g_split_mode.store(mode);
  if (mode_out) *mode_out = g_split_mode.load();
  return SGDYN_OK;
}

int sgdyn_jit_prepare(const sgdyn_model* m, int ops) {
  if (!m) return fail(SGDYN_ERR_NULL, "null model");
  if (!jit_kind_ok(ops)) return fail(SGDYN_ERR_RUNTIME, "bad op mask");
  if (ops == -7 && m->impl->lanes <= 1) return fail(SGDYN_ERR_RUNTIME, "the model runs with one lane per environment");
  std::string why;
  const bool ok = ops > 0     ? prepare_step_jit(*m->impl, ops, &why)
                  : ops == -7 ? prepare_step_roles_jit(*m->impl, m->impl->lanes, OP_CRBA | OP_RNEA | OP_ABA, &why)
                  : ops == -1 ? prepare_rollout_jit(*m->impl, &why)
                  : ops == -6 ? prepare_aba3_jit(*m->impl, &why)
                  : ops <= -4 ? prepare_rollout3_jit(*m->impl, ops == -5, &why)
                              : prepare_vjp_jit(*m->impl, ops == -3, &why);
  if (!ok) return fail(SGDYN_ERR_UNSUPPORTED, "run-time compilation unavailable: " + why);
  return SGDYN_OK;
}

int sgdyn_jit_source(const sgdyn_model* m, int ops, const char** source) {
  if (!m || !source) return fail(SGDYN_ERR_NULL, "null argument");
  if (!jit_kind_ok(ops)) return fail(SGDYN_ERR_RUNTIME, "bad op mask");
  if (ops == -7 && m->impl->lanes <= 1) return fail(SGDYN_ERR_RUNTIME, "the model runs with one lane per environment");
  thread_local std::string buf;
  buf = ops > 0     ? step_jit_source(*m->impl, ops)
        : ops == -7 ? step_roles_jit_source(*m->impl, m->impl->lanes, OP_CRBA | OP_RNEA | OP_ABA)
        : ops == -1 ? rollout_jit_source(*m->impl)
        : ops == -6 ? aba3_jit_source(*m->impl)
        : ops <= -4 ? rollout3_jit_source(*m->impl, ops == -5)
                    : vjp_jit_source(*m->impl, ops == -3);
  *source = buf.c_str();
  return SGDYN_OK;
}

int sgdyn_compute_forward_kinematics(const sgdyn_model* m, int64_t n, const double* q, double* link_poses,
                                     int layout, void* stream) {
  SG_TRACE("sgdyn_compute_forward_kinematics");
  return guarded([&] {
    return run_step(m, n, OP_FK, q, nullptr, nullptr, nullptr, link_poses, nullptr, nullptr, nullptr, nullptr, layout,
                    stream);
  });
}

int sgdyn_compute_full_jacobian(const sgdyn_model* m, int64_t n, const double* q, double* J, int layout,
                                void* stream) {
  SG_TRACE("sgdyn_compute_full_jacobian");
  return guarded([&] {
    return run_step(m, n, OP_JAC, q, nullptr, nullptr, nullptr, nullptr, J, nullptr, nullptr, nullptr, layout, stream);
  });
}

int sgdyn_compute_generalized_mass_matrix(const sgdyn_model* m, int64_t n, const double* q, double* M, int layout,
                                          void* stream) {
  SG_TRACE("sgdyn_compute_generalized_mass_matrix");
  return guarded([&] {
    return run_step(m, n, OP_CRBA, q, nullptr, nullptr, nullptr, nullptr, nullptr, M, nullptr, nullptr, layout,
                    stream);
  });
}

int sgdyn_compute_inverse_dynamics(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                   const double* qdd, double* tau, int layout, void* stream) {
  SG_TRACE("sgdyn_compute_inverse_dynamics");
  return guarded([&] {
    return run_step(m, n, OP_RNEA, q, qd, qdd, nullptr, nullptr, nullptr, nullptr, tau, nullptr, layout, stream);
  });
}

int sgdyn_compute_forward_dynamics(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                   const double* tau, double* qdd, int layout, void* stream) {
  SG_TRACE("sgdyn_compute_forward_dynamics");
  return guarded([&] {
    return run_step(m, n, OP_ABA, q, qd, nullptr, tau, nullptr, nullptr, nullptr, nullptr, qdd, layout, stream);
  });
}

int sgdyn_step(const sgdyn_model* m, int64_t n, int ops, const double* q, const double* qd, const double* qdd,
               const double* tau, double* link_poses, double* J, double* M, double* tau_out, double* qdd_out,
               int layout, void* stream) {
  SG_TRACE("sgdyn_step");
  return guarded([&] {
    return run_step(m, n, ops, q, qd, qdd, tau, link_poses, J, M, tau_out, qdd_out, layout, stream);
  });
}

int sgdyn_compute_link_jacobian(const sgdyn_model* m, int64_t n, int link, int local, const double* q, double* J,
                                int layout, void* stream) {
  SG_TRACE("sgdyn_compute_link_jacobian");
  return guarded([&] {
    if (int rc = check_model(m)) return rc;
    Model& Mo = *m->impl;
    if (link < 0 || link >= Mo.nlinks()) return fail(SGDYN_ERR_RUNTIME, "link index out of bound");
    if (n < 0) return fail(SGDYN_ERR_RUNTIME, "negative batch size");
    if (layout != SGDYN_ENV_MAJOR && layout != SGDYN_COL_MAJOR) return fail(SGDYN_ERR_RUNTIME, "bad layout");
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q, "q"}, {J, "J"}})) return rc;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    LinkJacArgs a;
    a.n = n;
    a.link = link;
    a.local = local ? 1 : 0;
    a.q = make_arr(q, n, Mo.nq_ext(), layout);
    a.J = make_arr(J, n, 6 * int64_t(Mo.nv()), layout);
    cudaError_t e = launch_link_jacobian(dm, Mo.njoints(), a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
    return SGDYN_OK;
  });
}

int sgdyn_compute_single_link_local_jacobian(const sgdyn_model* m, int64_t n, int link, const double* q, double* J,
                                             int layout, void* stream) {
  SG_TRACE("sgdyn_compute_single_link_local_jacobian");
  return sgdyn_compute_link_jacobian(m, n, link, 1, q, J, layout, stream);
}

int sgdyn_compute_coriolis_matrix(const sgdyn_model* m, int64_t n, const double* q, const double* qd, double* C,
                                  int layout, void* stream) {
  SG_TRACE("sgdyn_compute_coriolis_matrix");
  return guarded([&] {
    if (int rc = check_model(m)) return rc;
    Model& Mo = *m->impl;
    if (n < 0) return fail(SGDYN_ERR_RUNTIME, "negative batch size");
    if (layout != SGDYN_ENV_MAJOR && layout != SGDYN_COL_MAJOR) return fail(SGDYN_ERR_RUNTIME, "bad layout");
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q, "q"}, {qd, "qd"}, {C, "C"}})) return rc;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    CoriolisArgs a;
    a.n = n;
    a.q = make_arr(q, n, Mo.nq_ext(), layout);
    a.qd = make_arr(qd, n, Mo.nv(), layout);
    a.C = make_arr(C, n, int64_t(Mo.nv()) * Mo.nv(), layout);
    cudaError_t e = launch_coriolis(dm, Mo.njoints(), a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
    return SGDYN_OK;
  });
}

int sgdyn_compute_inverse_kinematics(const sgdyn_model* m, int64_t n, int link, const double* target,
                                     const double* q0, const int* mask, double eps, int max_iterations, double dt,
                                     double damp, double* q_out, int* success, double* err_out, int layout,
                                     void* stream) {
  SG_TRACE("sgdyn_compute_inverse_kinematics");
  return guarded([&] {
    if (int rc = check_model(m)) return rc;
    Model& Mo = *m->impl;
    if (link < 0 || link >= Mo.nlinks()) return fail(SGDYN_ERR_RUNTIME, "link index out of bound");
    if (n < 0) return fail(SGDYN_ERR_RUNTIME, "negative batch size");
    if (max_iterations < 0) return fail(SGDYN_ERR_RUNTIME, "negative max_iterations");
    if (layout != SGDYN_ENV_MAJOR && layout != SGDYN_COL_MAJOR) return fail(SGDYN_ERR_RUNTIME, "bad layout");
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{target, "target"}, {q_out, "q_out"}, {success, "success"}, {err_out, "err"}}))
      return rc;
    if (q0)
      if (int rc = check_ptrs({{q0, "q0"}})) return rc;
    if (mask)
      if (int rc = check_ptrs({{mask, "mask"}})) return rc;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    IkArgs a;
    a.n = n;
    a.link = link;
    a.max_iter = max_iterations;
    a.has_q0 = q0 != nullptr;
    a.has_mask = mask != nullptr;
    a.eps = eps;
    a.dt = dt;
    a.damp = damp;
    a.target = make_arr(target, n, 7, layout);
    a.q0 = make_arr(q0, n, Mo.nq_ext(), layout);
    a.q_out = make_arr(q_out, n, Mo.nq_ext(), layout);
    a.err = make_arr(err_out, n, 6, layout);
    a.mask = mask;
    a.success = success;
    cudaError_t e = launch_ik(dm, Mo.njoints(), a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
    return SGDYN_OK;
  });
}

int sgdyn_compute_inverse_dynamics_vjp(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                       const double* qdd, const double* tau_bar, double* q_bar, double* qd_bar,
                                       double* qdd_bar, int layout, void* stream) {
  SG_TRACE("sgdyn_compute_inverse_dynamics_vjp");
  return guarded([&] {
    if (int rc = check_diff_model(m)) return rc;
    if (int rc = common_checks(n, layout)) return rc;
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q, "q"}, {qd, "qd"}, {qdd, "qdd"}, {tau_bar, "tau_bar"}})) return rc;
    for (const void* o : {(const void*)q_bar, (const void*)qd_bar, (const void*)qdd_bar})
      if (o && !device_accessible(o)) return fail(SGDYN_ERR_NULL, "output is not device memory");
    Model& Mo = *m->impl;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    const int64_t nv = Mo.nv();
    VjpArgs a;
    a.n = n;
    a.q = make_arr(q, n, Mo.nq_ext(), layout);
    a.qd = make_arr(qd, n, nv, layout);
    a.x = make_arr(qdd, n, nv, layout);
    a.bar = make_arr(tau_bar, n, nv, layout);
    a.o1 = make_arr(q_bar, n, nv, layout);
    a.o2 = make_arr(qd_bar, n, nv, layout);
    a.o3 = make_arr(qdd_bar, n, nv, layout);
    std::string why;
    if (launch_vjp_jit(Mo, false, a, static_cast<cudaStream_t>(stream), &why)) return SGDYN_OK;
    return launch_status(launch_rnea_vjp(dm, Mo.njoints(), a, static_cast<cudaStream_t>(stream)));
  });
}

int sgdyn_compute_forward_dynamics_vjp(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                       const double* tau, const double* qdd_bar, double* q_bar, double* qd_bar,
                                       double* tau_bar, int layout, void* stream) {
  SG_TRACE("sgdyn_compute_forward_dynamics_vjp");
  return guarded([&] {
    if (int rc = check_diff_model(m)) return rc;
    if (int rc = common_checks(n, layout)) return rc;
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q, "q"}, {qd, "qd"}, {tau, "tau"}, {qdd_bar, "qdd_bar"}})) return rc;
    for (const void* o : {(const void*)q_bar, (const void*)qd_bar, (const void*)tau_bar})
      if (o && !device_accessible(o)) return fail(SGDYN_ERR_NULL, "output is not device memory");
    Model& Mo = *m->impl;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    const int64_t nv = Mo.nv();
    VjpArgs a;
    a.n = n;
    a.q = make_arr(q, n, Mo.nq_ext(), layout);
    a.qd = make_arr(qd, n, nv, layout);
    a.x = make_arr(tau, n, nv, layout);
    a.bar = make_arr(qdd_bar, n, nv, layout);
    a.o1 = make_arr(q_bar, n, nv, layout);
    a.o2 = make_arr(qd_bar, n, nv, layout);
    a.o3 = make_arr(tau_bar, n, nv, layout);
    std::string why;
    if (launch_vjp_jit(Mo, true, a, static_cast<cudaStream_t>(stream), &why)) return SGDYN_OK;
    return launch_status(launch_aba_vjp(dm, Mo.njoints(), a, static_cast<cudaStream_t>(stream)));
  });
}

int sgdyn_compute_forward_kinematics_vjp(const sgdyn_model* m, int64_t n, const double* q, const double* pos_bar,
                                         const double* rot_bar, double* q_bar, int layout, void* stream) {
  SG_TRACE("sgdyn_compute_forward_kinematics_vjp");
  return guarded([&] {
    if (int rc = check_diff_model(m)) return rc;
    if (int rc = common_checks(n, layout)) return rc;
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q, "q"}, {pos_bar, "pos_bar"}, {q_bar, "q_bar"}})) return rc;
    if (rot_bar && !device_accessible(rot_bar)) return fail(SGDYN_ERR_NULL, "rot_bar is not device memory");
    Model& Mo = *m->impl;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    FkVjpArgs a;
    a.n = n;
    a.q = make_arr(q, n, Mo.nq_ext(), layout);
    a.pbar = make_arr(pos_bar, n, 3 * int64_t(Mo.nlinks()), layout);
    a.Rbar = make_arr(rot_bar, n, 9 * int64_t(Mo.nlinks()), layout);
    a.qbar = make_arr(q_bar, n, Mo.nv(), layout);
    return launch_status(launch_fk_vjp(dm, Mo.njoints(), a, static_cast<cudaStream_t>(stream)));
  });
}

static int derivatives(bool aba, const sgdyn_model* m, int64_t n, const double* q, const double* qd, const double* x,
                       double* d_q, double* d_qd, double* d_x, int layout, void* stream) {
  return guarded([&] {
    if (int rc = check_diff_model(m)) return rc;
    if (int rc = common_checks(n, layout)) return rc;
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q, "q"}, {qd, "qd"}, {x, aba ? "tau" : "qdd"}, {d_q, "d_q"}, {d_qd, "d_qd"}}))
      return rc;
    if (d_x && !device_accessible(d_x)) return fail(SGDYN_ERR_NULL, "output is not device memory");
    Model& Mo = *m->impl;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    const int64_t nv = Mo.nv();
    DerivArgs a;
    a.n = n;
    a.q = make_arr(q, n, Mo.nq_ext(), layout);
    a.qd = make_arr(qd, n, nv, layout);
    a.x = make_arr(x, n, nv, layout);
    a.d_q = make_arr(d_q, n, nv * nv, layout);
    a.d_qd = make_arr(d_qd, n, nv * nv, layout);
    a.d_x = make_arr(d_x, n, nv * nv, layout);
    a.lay = deriv_layout(Mo.njoints(), int(nv), aba);
    auto s = static_cast<cudaStream_t>(stream);
    // stream-ordered scratch for the preparation kernel's per-environment results
    void* scratch = nullptr;
    cudaError_t me = cudaMallocAsync(&scratch, size_t(a.lay.total) * size_t(n) * sizeof(double), s);
    if (me != cudaSuccess) return fail(SGDYN_ERR_CUDA, std::string("scratch allocation failed: ") + cudaGetErrorString(me));
    a.scratch = static_cast<double*>(scratch);
    const int rc = launch_status(aba ? launch_aba_derivatives(dm, Mo.njoints(), a, s)
                                     : launch_rnea_derivatives(dm, Mo.njoints(), a, s));
    cudaFreeAsync(scratch, s);
    return rc;
  });
}

int sgdyn_compute_rnea_derivatives(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                   const double* qdd, double* dtau_dq, double* dtau_dqd, double* dtau_dqdd,
                                   int layout, void* stream) {
  SG_TRACE("sgdyn_compute_rnea_derivatives");
  return derivatives(false, m, n, q, qd, qdd, dtau_dq, dtau_dqd, dtau_dqdd, layout, stream);
}

int sgdyn_compute_aba_derivatives(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                  const double* tau, double* dqdd_dq, double* dqdd_dqd, double* dqdd_dtau,
                                  int layout, void* stream) {
  SG_TRACE("sgdyn_compute_aba_derivatives");
  return derivatives(true, m, n, q, qd, tau, dqdd_dq, dqdd_dqd, dqdd_dtau, layout, stream);
}

static int rollout_checks(const sgdyn_model* m, int64_t n, int T, int K) {
  if (int rc = check_diff_model(m)) return rc;
  if (n < 0 || T < 0) return fail(SGDYN_ERR_RUNTIME, "negative size");
  if (K <= 0) return fail(SGDYN_ERR_RUNTIME, "checkpoint_every must be positive");
  return SGDYN_OK;
}

int sgdyn_rollout_forward(const sgdyn_model* m, int64_t n, int T, double dt, const double* q0, const double* qd0,
                          const double* tau, int checkpoint_every, double* q_ckpt, double* qd_ckpt, double* qT,
                          double* qdT, void* stream) {
  SG_TRACE("sgdyn_rollout_forward");
  return guarded([&] {
    if (int rc = rollout_checks(m, n, T, checkpoint_every)) return rc;
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q0, "q0"}, {qd0, "qd0"}, {qT, "qT"}, {qdT, "qdT"}})) return rc;
    if (T > 0)
      if (int rc = check_ptrs({{tau, "tau"}})) return rc;
    if ((q_ckpt == nullptr) != (qd_ckpt == nullptr)) return fail(SGDYN_ERR_NULL, "give both checkpoint arrays or none");
    if (q_ckpt)
      if (int rc = check_ptrs({{q_ckpt, "q_ckpt"}, {qd_ckpt, "qd_ckpt"}})) return rc;
    Model& Mo = *m->impl;
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    RolloutArgs a{};
    a.n = n;
    a.T = T;
    a.K = checkpoint_every;
    a.dt = dt;
    a.q0 = q0; a.qd0 = qd0; a.tau = tau;
    a.qT = qT; a.qdT = qdT; a.q_ckpt = q_ckpt; a.qd_ckpt = qd_ckpt;
    std::string why;
    const auto st = static_cast<cudaStream_t>(stream);
    if (rollout_lanes(Mo, n) == 3) {
      if (launch_rollout3_jit(Mo, a, st, &why)) return SGDYN_OK;
      return launch_status(launch_rollout_forward3(dm, Mo.njoints(), a, st));
    }
    if (launch_rollout_jit(Mo, a, st, &why)) return SGDYN_OK;
    return launch_status(launch_rollout_forward(dm, Mo.njoints(), a, st));
  });
}

int sgdyn_rollout_scratch_bytes(const sgdyn_model* m, int64_t n, int checkpoint_every, int64_t* bytes) {
  if (!m || !bytes) return fail(SGDYN_ERR_NULL, "null argument");
  if (checkpoint_every <= 0 || n < 0) return fail(SGDYN_ERR_RUNTIME, "bad sizes");
  const Model& Mo = *m->impl;
  const int64_t b = rollout_scratch_bytes_for(Mo.njoints(), Mo.nq_ext(), Mo.nv(), checkpoint_every, n);
  if (b < 0) return fail(SGDYN_ERR_RUNTIME, "scratch size overflows int64");
  *bytes = b;
  return SGDYN_OK;
}

}  // extern "C"

namespace {

// Rollout backward with the recompute of the next (earlier) group of segments running on a
// second stream while the current group's reverse sweep runs on the caller's stream. The
// reverse sweep at small batches keeps one warp per SM busy and leaves the other FP64
// schedulers idle; the recompute fills them. Groups alternate between two halves of the
// scratch; a recompute waits for the reverse that last used its half.
// The backward's reverse sweep with three lanes per environment: the model-specialised
// kernel if run-time compilation serves it, else the generic one.
cudaError_t reverse3(Model& M, const DModel* dm, int nj, const RolloutArgs& g, cudaStream_t s) {
  std::string why;
  if (launch_rollout_reverse3_jit(M, g, s, &why)) return cudaSuccess;
  return launch_rollout_reverse3(dm, nj, g, s);
}

cudaError_t rollout_backward_overlapped(Model& M, const DModel* dm, int nj, int lanes, RolloutArgs a,
                                        int64_t seg_doubles, int G, cudaStream_t s1, cudaStream_t s2) {
  const int nseg = (a.T + a.K - 1) / a.K;
  std::vector<RolloutArgs> groups;
  for (int hi = nseg; hi > 0; hi -= G) {
    RolloutArgs g = a;
    g.s_lo = hi - G > 0 ? hi - G : 0;
    g.s_cnt = hi - g.s_lo;
    g.scratch = a.scratch + int64_t(groups.size() % 2) * G * seg_doubles;
    groups.push_back(g);
  }
  const int m = int(groups.size());
  std::vector<cudaEvent_t> ev(2 * m + 1, nullptr);
  cudaError_t e = cudaSuccess;
  for (auto& x : ev)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
  cudaEvent_t start = ev[2 * m];
  auto rec = [&](int k) { return ev[k]; };
  auto rev = [&](int k) { return ev[m + k]; };
  if (e == cudaSuccess) e = cudaEventRecord(start, s1);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, start, 0);
  if (e == cudaSuccess) e = launch_rollout_recompute(dm, nj, groups[0], s2);
  if (e == cudaSuccess) e = cudaEventRecord(rec(0), s2);
  for (int k = 0; k < m && e == cudaSuccess; k++) {
    e = cudaStreamWaitEvent(s1, rec(k), 0);
    if (e == cudaSuccess)
      e = lanes == 3 ? reverse3(M, dm, nj, groups[k], s1) : launch_rollout_reverse(dm, nj, groups[k], s1);
    if (e == cudaSuccess) e = cudaEventRecord(rev(k), s1);
    if (e == cudaSuccess && k + 1 < m) {
      if (k >= 1) e = cudaStreamWaitEvent(s2, rev(k - 1), 0);
      if (e == cudaSuccess) e = launch_rollout_recompute(dm, nj, groups[k + 1], s2);
      if (e == cudaSuccess) e = cudaEventRecord(rec(k + 1), s2);
    }
  }
  for (auto& x : ev)
    if (x) cudaEventDestroy(x);  // released once the recorded work completes
  return e;
}

}  // namespace

extern "C" {

int sgdyn_rollout_backward(const sgdyn_model* m, int64_t n, int T, double dt, int checkpoint_every,
                           const double* q_ckpt, const double* qd_ckpt, const double* tau, const double* qT_bar,
                           const double* qdT_bar, double* q0_bar, double* qd0_bar, double* tau_bar, double* scratch,
                           int64_t scratch_bytes, void* stream) {
  SG_TRACE("sgdyn_rollout_backward");
  return guarded([&] {
    if (int rc = rollout_checks(m, n, T, checkpoint_every)) return rc;
    if (n == 0) return SGDYN_OK;
    if (int rc = check_ptrs({{q0_bar, "q0_bar"}, {qd0_bar, "qd0_bar"}})) return rc;
    if (T > 0)
      if (int rc = check_ptrs({{q_ckpt, "q_ckpt"}, {qd_ckpt, "qd_ckpt"}, {tau, "tau"}, {tau_bar, "tau_bar"},
                               {scratch, "scratch"}}))
        return rc;
    for (const void* o : {(const void*)qT_bar, (const void*)qdT_bar})
      if (o && !device_accessible(o)) return fail(SGDYN_ERR_NULL, "adjoint input is not device memory");
    Model& Mo = *m->impl;
    const int64_t need = rollout_scratch_bytes_for(Mo.njoints(), Mo.nq_ext(), Mo.nv(), checkpoint_every, n);
    if (need < 0) return fail(SGDYN_ERR_RUNTIME, "scratch size overflows int64");
    if (T > 0 && scratch_bytes < need)
      return fail(SGDYN_ERR_RUNTIME, "scratch too small: need " + std::to_string(need) + " bytes");
    int err = 0;
    const DModel* dm = Mo.device_table(&err);
    if (!dm) return fail(SGDYN_ERR_CUDA, "model upload failed");
    RolloutArgs a{};
    a.n = n;
    a.T = T;
    a.K = checkpoint_every;
    a.dt = dt;
    a.tau = tau;
    a.q_ckpt = const_cast<double*>(q_ckpt);
    a.qd_ckpt = const_cast<double*>(qd_ckpt);
    a.qT_bar = qT_bar; a.qdT_bar = qdT_bar;
    a.q0_bar = q0_bar; a.qd0_bar = qd0_bar; a.tau_bar = tau_bar; a.scratch = scratch;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nj = Mo.njoints();
    const int lanes = rollout_lanes(Mo, n);
    // two scratch halves of G segments each and at least two groups: overlap recompute and
    // reverse on two streams (not while the caller's stream is being captured)
    const int nseg = T > 0 ? (T + checkpoint_every - 1) / checkpoint_every : 0;
    const int64_t fit = need > 0 ? scratch_bytes / need : 0;
    // about as long a recompute of the next group as a reverse sweep of the current one:
    // fifths of the segments for the one-lane reverse, halves for the three-lane one
    const int G = int(std::min<int64_t>(fit / 2, std::max(1, lanes == 3 ? (nseg + 1) / 2 : nseg / 5)));
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) cs = cudaStreamCaptureStatusActive;
    if (nseg >= 2 && G >= 1 && (nseg + G - 1) / G >= 2 && cs == cudaStreamCaptureStatusNone)
      if (cudaStream_t s2 = side_stream())
        return launch_status(rollout_backward_overlapped(Mo, dm, nj, lanes, a, need / 8, G, st, s2));
    return launch_status(rollout_backward_grouped(
        a, need / 8, scratch_bytes / 8, [&](const RolloutArgs& g) { return launch_rollout_recompute(dm, nj, g, st); },
        [&](const RolloutArgs& g) {
          return lanes == 3 ? reverse3(Mo, dm, nj, g, st) : launch_rollout_reverse(dm, nj, g, st);
        }));
  });
}

}  // extern "C"
