// Run-time specialisation of the fused sweep per model (NVRTC).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "kernels.h"

namespace sgdyn {

class Model;

// Launches the model-specialised sweep if run-time compilation is enabled, available and
// the batch is large enough; returns false (with the reason) when the caller should use the
// generic kernel. Compiles and caches on first use of (model tables, ops, device).
bool launch_step_jit(Model& M, int ops, const StepArgs& a, cudaStream_t s, std::string* why);
// The fused sweep with L lanes per environment as one warp per role of the team (a block of
// L warps holds 32 environments; team table and roles compiled in), for models run with
// teams; false (with the reason) when the caller should use the generic team kernel.
bool launch_step_roles_jit(Model& M, int lanes, int ops, const StepArgs& a, cudaStream_t s, std::string* why);
std::string step_roles_jit_source(const Model& M, int lanes, int ops);
// For a heterogeneous batch of n environments: whether the role-warp sweep of (M, lanes, ops)
// is available (compiling it if needed), and its launch over `count` environments whose
// rows of the call's arrays are rows[0 .. count - 1] (device memory), with integrate: then
// a semi-implicit Euler step of those rows of a.q, a.qd (in place) by dt from a.qdd_out.
bool step_roles_jit_ready(Model& M, int lanes, int ops, int64_t n, std::string* why);
bool launch_step_roles_rows_jit(Model& M, int lanes, int ops, const StepArgs& a, const int* rows, int64_t count,
                                double dt, bool integrate, cudaStream_t s, std::string* why);
bool prepare_step_roles_jit(Model& M, int lanes, int ops, std::string* why);
// Same for the RNEA / ABA vector-Jacobian product kernels.
bool launch_vjp_jit(Model& M, bool aba, const VjpArgs& a, cudaStream_t s, std::string* why);
std::string vjp_jit_source(const Model& M, bool aba);
bool prepare_vjp_jit(Model& M, bool aba, std::string* why);
// Same for the forward rollout kernel.
bool launch_rollout_jit(Model& M, const RolloutArgs& a, cudaStream_t s, std::string* why);
std::string rollout_jit_source(const Model& M);
bool prepare_rollout_jit(Model& M, std::string* why);
// The forward rollout and the backward's reverse sweep with three lanes per environment
// (team3.cuh).
bool launch_rollout3_jit(Model& M, const RolloutArgs& a, cudaStream_t s, std::string* why);
bool launch_rollout_reverse3_jit(Model& M, const RolloutArgs& a, cudaStream_t s, std::string* why);
std::string rollout3_jit_source(const Model& M, bool reverse);
bool prepare_rollout3_jit(Model& M, bool reverse, std::string* why);
// Forward dynamics alone with three lanes per environment (team3.cuh).
bool launch_aba3_jit(Model& M, const StepArgs& a, cudaStream_t s, std::string* why);
std::string aba3_jit_source(const Model& M);
bool prepare_aba3_jit(Model& M, std::string* why);
// Compiles (or loads from the cache) now; false with the reason if not possible.
bool prepare_step_jit(Model& M, int ops, std::string* why);
void set_jit_config(int enable, int64_t min_n);
// The generated translation unit (for inspection and tests).
std::string step_jit_source(const Model& M, int ops);
void get_jit_config(int* enable, int64_t* min_n);
// Forward dynamics in the specialised sweep: 0 automatic, 1 articulated-body passes, 2 from
// the mass matrix (L^T D L); < 0 leaves the setting. out receives the setting.
void fd_method(int mode, int* out);
// Whether the specialised sweep for `ops` computes forward dynamics from the mass matrix.
bool fd_by_mass_matrix(const Model& M, int ops);
// Size limit (joints incl. the universe) for run-time specialisation; < 0 leaves it.
void jit_max_joints(int max_joints, int* out);

}  // namespace sgdyn
