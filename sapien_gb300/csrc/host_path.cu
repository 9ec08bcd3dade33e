// Single-instance (and small-batch) calls answered on the host by the same sweep code the
// kernels run: step_env_t, link_jacobian_env, coriolis_env and ik_env are host-device
// templates, instantiated here for the CPU and reading the model's host copy of the table.
//
// Why: the reference's callers use PinocchioModel one configuration at a time
// (pinocchio/pinocchio_model.cpp:146-300; the viewer's IK gizmo runs 100 CLIK iterations per
// frame, python/py_package/utils/viewer/transform_window.py:125-131). On the GPU one
// environment is one thread's sequential sweep, so such a call costs tens of microseconds of
// kernel time plus a launch and a synchronisation; on a host core it costs microseconds.
// Batches belong on the GPU (sgdyn_step and friends); nothing here is a fallback for them.
//
// Arguments follow the device entry points, with HOST pointers and a thread count instead of
// a stream: environments are split into contiguous ranges over `nthreads` threads
// (<= 1: the calling thread only).
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sgdyn.h"
#include "aux_kernels.cuh"
#include "jit.h"
#include "model.h"

struct sgdyn_model {
  sgdyn::Model* impl;
};

namespace sgdyn {

int set_last_error(int code, const std::string& msg);
int call_guarded(const std::function<int()>& body);

namespace {

Arr host_arr(const void* p, int64_t n, int64_t cols, int layout) {
  Arr a;
  a.p = static_cast<double*>(const_cast<void*>(p));
  a.es = layout == SGDYN_ENV_MAJOR ? cols : 1;
  a.cs = layout == SGDYN_ENV_MAJOR ? 1 : n;
  return a;
}

// Contiguous ranges of [0, n) over up to nthreads threads (the caller's thread takes the
// first range).
template <class Body>
void parallel_envs(int64_t n, int nthreads, const Body& body) {
  const int64_t t = nthreads <= 1 ? 1 : std::min<int64_t>(nthreads, n);
  if (t <= 1) {
    body(0, n);
    return;
  }
  std::vector<std::thread> pool;
  const int64_t base = n / t, extra = n % t;
  int64_t start = base + (extra > 0 ? 1 : 0);
  for (int64_t k = 1; k < t; k++) {
    const int64_t len = base + (k < extra ? 1 : 0);
    pool.emplace_back(body, start, start + len);
    start += len;
  }
  body(0, base + (extra > 0 ? 1 : 0));
  for (auto& th : pool) th.join();
}

int check(const sgdyn_model* m, int64_t n, int layout) {
  if (!m || !m->impl) return set_last_error(SGDYN_ERR_NULL, "null model");
  if (stash_bucket(m->impl->njoints()) == 0)
    return set_last_error(SGDYN_ERR_UNSUPPORTED, "model has more than 63 moving joints");
  int nff = 0;
  for (auto& J : m->impl->joints) nff += J.kind == JK_FREEFLYER;
  if (nff > 1) return set_last_error(SGDYN_ERR_UNSUPPORTED, "model has more than one free-flyer joint");
  if (n < 0) return set_last_error(SGDYN_ERR_RUNTIME, "negative batch size");
  if (layout != SGDYN_ENV_MAJOR && layout != SGDYN_COL_MAJOR) return set_last_error(SGDYN_ERR_RUNTIME, "bad layout");
  return SGDYN_OK;
}

const DModel* table(const sgdyn_model* m) { return reinterpret_cast<const DModel*>(m->impl->host_table().data()); }

template <int MAXJ, int OPS>
void step_range(const DModel* dm, const StepArgs& a, int64_t lo, int64_t hi) {
  for (int64_t e = lo; e < hi; e++) step_env_t<MAXJ, OPS>(RuntimeTab{dm}, a, e);
}

template <int MAXJ>
bool step_bucket(int ops, const DModel* dm, const StepArgs& a, int64_t lo, int64_t hi) {
  switch (ops) {
#define SG_CASE(O) \
  case O: step_range<MAXJ, O>(dm, a, lo, hi); return true;
    SG_CASE(OP_FK)
    SG_CASE(OP_JAC)
    SG_CASE(OP_FK | OP_JAC)
    SG_CASE(OP_CRBA)
    SG_CASE(OP_RNEA)
    SG_CASE(OP_ABA)
    SG_CASE(OP_RNEA | OP_ABA)
    SG_CASE(OP_CRBA | OP_RNEA | OP_ABA)
    SG_CASE(OP_ALL)
    // forward dynamics from the mass matrix
    SG_CASE(OP_ABA | OP_FD_CRBA)
    SG_CASE(OP_RNEA | OP_ABA | OP_FD_CRBA)
    SG_CASE(OP_CRBA | OP_RNEA | OP_ABA | OP_FD_CRBA)
    SG_CASE(OP_ALL | OP_FD_CRBA)
#undef SG_CASE
    default: return false;
  }
}

bool run_ops(int bucket, int ops, const DModel* dm, const StepArgs& a, int64_t lo, int64_t hi) {
  switch (bucket) {
    case 16: return step_bucket<16>(ops, dm, a, lo, hi);
    case 32: return step_bucket<32>(ops, dm, a, lo, hi);
    case 64: return step_bucket<64>(ops, dm, a, lo, hi);
    default: return false;
  }
}

// The per-environment body of a bucketed template, for every environment of [lo, hi).
#define SG_BUCKETED(fn, bucket, ...)                                        \
  do {                                                                      \
    switch (bucket) {                                                       \
      case 16: for (int64_t e = lo; e < hi; e++) fn<16>(__VA_ARGS__, e); break; \
      case 32: for (int64_t e = lo; e < hi; e++) fn<32>(__VA_ARGS__, e); break; \
      case 64: for (int64_t e = lo; e < hi; e++) fn<64>(__VA_ARGS__, e); break; \
    }                                                                       \
  } while (0)

}  // namespace
}  // namespace sgdyn

using namespace sgdyn;

extern "C" {

int sgdyn_host_step(const sgdyn_model* m, int64_t n, int ops, const double* q, const double* qd, const double* qdd,
                    const double* tau, double* link_poses, double* J, double* M, double* tau_out, double* qdd_out,
                    int layout, int nthreads) {
  return call_guarded([&]() -> int {
    if (int rc = check(m, n, layout)) return rc;
    if (ops <= 0 || ops > OP_ALL) return set_last_error(SGDYN_ERR_RUNTIME, "bad op mask");
    if (n == 0) return SGDYN_OK;
    const Model& Mo = *m->impl;
    struct Need {
      bool on;
      const void* p;
      const char* name;
    };
    for (const Need& r : {Need{true, q, "q"}, Need{(ops & (OP_RNEA | OP_ABA)) != 0, qd, "qd"},
                          Need{(ops & OP_RNEA) != 0, qdd, "qdd"}, Need{(ops & OP_RNEA) != 0, tau_out, "tau_out"},
                          Need{(ops & OP_ABA) != 0, tau, "tau"}, Need{(ops & OP_ABA) != 0, qdd_out, "qdd_out"},
                          Need{(ops & OP_FK) != 0, link_poses, "link_poses"}, Need{(ops & OP_JAC) != 0, J, "J"},
                          Need{(ops & OP_CRBA) != 0, M, "M"}})
      if (r.on && !r.p) return set_last_error(SGDYN_ERR_NULL, std::string(r.name) + " is null");
    const int64_t nv = Mo.nv();
    StepArgs a;
    a.n = n;
    a.q = host_arr(q, n, Mo.nq_ext(), layout);
    a.qd = host_arr(qd, n, nv, layout);
    a.qdd = host_arr(qdd, n, nv, layout);
    a.tau = host_arr(tau, n, nv, layout);
    a.poses = host_arr(link_poses, n, int64_t(Mo.nlinks()) * 7, layout);
    a.J = host_arr(J, n, 6 * nv, layout);
    a.M = host_arr(M, n, nv * nv, layout);
    a.tau_out = host_arr(tau_out, n, nv, layout);
    a.qdd_out = host_arr(qdd_out, n, nv, layout);
    // the op set as the fused sweeps the device side also uses, then single ops
    int parts[8], np = 0;
    int rest = ops;
    for (int f : {int(OP_ALL), OP_CRBA | OP_RNEA | OP_ABA, OP_RNEA | OP_ABA, OP_FK | OP_JAC})
      if ((rest & f) == f) {
        parts[np++] = f;
        rest &= ~f;
      }
    for (int b = 1; b <= OP_ABA; b <<= 1)
      if (rest & b) parts[np++] = b;
    // forward dynamics from the mass matrix only when sgdyn_fd_method forces it: on the host
    // its loops over run-time tables measured no faster than the articulated-body passes
    int fd_mode = 0;
    fd_method(-1, &fd_mode);
    for (int k = 0; k < np; k++)
      if (fd_mode == 2 && fd_by_mass_matrix(Mo, parts[k])) parts[k] |= OP_FD_CRBA;
    const DModel* dm = table(m);
    const int bucket = stash_bucket(Mo.njoints());
    parallel_envs(n, nthreads, [&](int64_t lo, int64_t hi) {
      for (int k = 0; k < np; k++) run_ops(bucket, parts[k], dm, a, lo, hi);
    });
    return SGDYN_OK;
  });
}

int sgdyn_host_compute_link_jacobian(const sgdyn_model* m, int64_t n, int link, int local, const double* q,
                                     double* J, int layout, int nthreads) {
  return call_guarded([&]() -> int {
    if (int rc = check(m, n, layout)) return rc;
    const Model& Mo = *m->impl;
    if (link < 0 || link >= Mo.nlinks()) return set_last_error(SGDYN_ERR_RUNTIME, "link index out of bound");
    if (n == 0) return SGDYN_OK;
    if (!q || !J) return set_last_error(SGDYN_ERR_NULL, "q or J is null");
    LinkJacArgs a;
    a.n = n;
    a.link = link;
    a.local = local ? 1 : 0;
    a.q = host_arr(q, n, Mo.nq_ext(), layout);
    a.J = host_arr(J, n, 6 * int64_t(Mo.nv()), layout);
    const DModel* dm = table(m);
    const int bucket = stash_bucket(Mo.njoints());
    parallel_envs(n, nthreads, [&](int64_t lo, int64_t hi) { SG_BUCKETED(link_jacobian_env, bucket, dm, a); });
    return SGDYN_OK;
  });
}

int sgdyn_host_compute_coriolis_matrix(const sgdyn_model* m, int64_t n, const double* q, const double* qd, double* C,
                                       int layout, int nthreads) {
  return call_guarded([&]() -> int {
    if (int rc = check(m, n, layout)) return rc;
    if (n == 0) return SGDYN_OK;
    if (!q || !qd || !C) return set_last_error(SGDYN_ERR_NULL, "q, qd or C is null");
    const Model& Mo = *m->impl;
    CoriolisArgs a;
    a.n = n;
    a.q = host_arr(q, n, Mo.nq_ext(), layout);
    a.qd = host_arr(qd, n, Mo.nv(), layout);
    a.C = host_arr(C, n, int64_t(Mo.nv()) * Mo.nv(), layout);
    const DModel* dm = table(m);
    const int bucket = stash_bucket(Mo.njoints());
    parallel_envs(n, nthreads, [&](int64_t lo, int64_t hi) { SG_BUCKETED(coriolis_env, bucket, dm, a); });
    return SGDYN_OK;
  });
}

int sgdyn_host_compute_inverse_kinematics(const sgdyn_model* m, int64_t n, int link, const double* target,
                                          const double* q0, const int* mask, double eps, int max_iterations,
                                          double dt, double damp, double* q_out, int* success, double* err_out,
                                          int layout, int nthreads) {
  return call_guarded([&]() -> int {
    if (int rc = check(m, n, layout)) return rc;
    const Model& Mo = *m->impl;
    if (link < 0 || link >= Mo.nlinks()) return set_last_error(SGDYN_ERR_RUNTIME, "link index out of bound");
    if (max_iterations < 0) return set_last_error(SGDYN_ERR_RUNTIME, "negative max_iterations");
    if (n == 0) return SGDYN_OK;
    if (!target || !q_out || !success || !err_out)
      return set_last_error(SGDYN_ERR_NULL, "target, q_out, success or err is null");
    IkArgs a;
    a.n = n;
    a.link = link;
    a.max_iter = max_iterations;
    a.has_q0 = q0 != nullptr;
    a.has_mask = mask != nullptr;
    a.eps = eps;
    a.dt = dt;
    a.damp = damp;
    a.target = host_arr(target, n, 7, layout);
    a.q0 = host_arr(q0, n, Mo.nq_ext(), layout);
    a.q_out = host_arr(q_out, n, Mo.nq_ext(), layout);
    a.err = host_arr(err_out, n, 6, layout);
    a.mask = mask;
    a.success = success;
    const DModel* dm = table(m);
    const int bucket = stash_bucket(Mo.njoints());
    parallel_envs(n, nthreads, [&](int64_t lo, int64_t hi) { SG_BUCKETED(ik_env, bucket, dm, a); });
    return SGDYN_OK;
  });
}

}  // extern "C"
