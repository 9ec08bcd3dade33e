"""ctypes binding of libsgdyn.so (the C ABI declared in include/sgdyn.h).

The library is built in-tree by ``sapien_gb300.build_native.build()``. Loading fails
loudly when it is missing: there is no CPU fallback for any compute entry point.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsgdyn.so")

OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_RUNTIME = -2
ERR_CUDA = -3
ERR_UNSUPPORTED = -4
ERR_NULL = -5

ENV_MAJOR = 0
COL_MAJOR = 1

OP_FK = 1
OP_JACOBIAN = 2
OP_MASS_MATRIX = 4
OP_INVERSE_DYNAMICS = 8
OP_FORWARD_DYNAMICS = 16
OP_ALL = 31

# Every symbol include/sgdyn.h declares (checked by the CPU test-suite).
EXPORTED = (
    "sgdyn_last_error",
    "sgdyn_model_from_urdf",
    "sgdyn_model_free",
    "sgdyn_model_set_joint_order",
    "sgdyn_model_set_link_order",
    "sgdyn_model_info",
    "sgdyn_model_joint_kind",
    "sgdyn_model_random_configuration",
    "sgdyn_model_joint_name",
    "sgdyn_model_body_count",
    "sgdyn_model_body_name",
    "sgdyn_model_upload",
    "sgdyn_model_table",
    "sgdyn_compute_forward_kinematics",
    "sgdyn_compute_full_jacobian",
    "sgdyn_compute_link_jacobian",
    "sgdyn_compute_single_link_local_jacobian",
    "sgdyn_compute_generalized_mass_matrix",
    "sgdyn_compute_coriolis_matrix",
    "sgdyn_compute_inverse_dynamics",
    "sgdyn_compute_forward_dynamics",
    "sgdyn_step",
    "sgdyn_compute_inverse_kinematics",
    "sgdyn_compute_inverse_dynamics_vjp",
    "sgdyn_compute_forward_dynamics_vjp",
    "sgdyn_compute_forward_kinematics_vjp",
    "sgdyn_compute_rnea_derivatives",
    "sgdyn_compute_aba_derivatives",
    "sgdyn_rollout_forward",
    "sgdyn_rollout_scratch_bytes",
    "sgdyn_rollout_backward",
    "sgdyn_rollout_backward_noalloc",
    "sgdyn_batch_create",
    "sgdyn_batch_free",
    "sgdyn_batch_info",
    "sgdyn_batch_set_launch",
    "sgdyn_batch_set_lanes",
    "sgdyn_batch_step",
    "sgdyn_batch_integrate",
    "sgdyn_batch_step_integrate",
    "sgdyn_model_set_lanes",
    "sgdyn_model_team_table",
    "sgdyn_jit_max_joints",
    "sgdyn_fd_method",
    "sgdyn_fd_by_mass_matrix",
    "sgdyn_jit_config",
    "sgdyn_jit_prepare",
    "sgdyn_jit_source",
    "sgdyn_model_from_articulation",
    "sgdyn_compute_passive_force_f32",
    "sgdyn_step_split",
    "sgdyn_rollout_lanes",
    "sgdyn_host_step",
    "sgdyn_host_compute_link_jacobian",
    "sgdyn_host_compute_coriolis_matrix",
    "sgdyn_host_compute_inverse_kinematics",
)

_lib = None


class SgdynError(RuntimeError):
    pass


def load():
    """Load libsgdyn.so (raises ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"sapien_gb300 native library not found at {LIB_PATH}; build it with "
            "`python -c 'import sapien_gb300.build_native as b; b.build()'`"
        )
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    P = ctypes.POINTER
    L.sgdyn_last_error.restype = ctypes.c_char_p
    L.sgdyn_last_error.argtypes = []
    L.sgdyn_model_from_urdf.argtypes = [ctypes.c_char_p, P(dbl), P(vp)]
    L.sgdyn_model_free.argtypes = [vp]
    L.sgdyn_model_free.restype = None
    L.sgdyn_model_set_joint_order.argtypes = [vp, P(ctypes.c_char_p), i32]
    L.sgdyn_model_set_link_order.argtypes = [vp, P(ctypes.c_char_p), i32]
    L.sgdyn_model_info.argtypes = [vp, P(i32), P(i32), P(i32), P(i32)]
    L.sgdyn_model_joint_kind.argtypes = [vp, i32, P(i32)]
    L.sgdyn_model_random_configuration.argtypes = [vp, i64, ctypes.c_uint64, vp]
    L.sgdyn_model_joint_name.argtypes = [vp, i32, P(ctypes.c_char_p)]
    L.sgdyn_model_body_count.argtypes = [vp, P(i32)]
    L.sgdyn_model_body_name.argtypes = [vp, i32, P(ctypes.c_char_p)]
    L.sgdyn_model_upload.argtypes = [vp]
    L.sgdyn_model_table.argtypes = [vp, P(vp), P(i64)]
    L.sgdyn_compute_forward_kinematics.argtypes = [vp, i64, vp, vp, i32, vp]
    L.sgdyn_compute_full_jacobian.argtypes = [vp, i64, vp, vp, i32, vp]
    L.sgdyn_compute_link_jacobian.argtypes = [vp, i64, i32, i32, vp, vp, i32, vp]
    L.sgdyn_compute_single_link_local_jacobian.argtypes = [vp, i64, i32, vp, vp, i32, vp]
    L.sgdyn_compute_generalized_mass_matrix.argtypes = [vp, i64, vp, vp, i32, vp]
    L.sgdyn_compute_coriolis_matrix.argtypes = [vp, i64, vp, vp, vp, i32, vp]
    L.sgdyn_compute_inverse_dynamics.argtypes = [vp, i64, vp, vp, vp, vp, i32, vp]
    L.sgdyn_compute_forward_dynamics.argtypes = [vp, i64, vp, vp, vp, vp, i32, vp]
    L.sgdyn_step.argtypes = [vp, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32, vp]
    L.sgdyn_compute_inverse_kinematics.argtypes = [vp, i64, i32, vp, vp, vp, dbl, i32, dbl, dbl, vp, vp, vp, i32, vp]
    L.sgdyn_step_split.argtypes = [i32, P(i32)]
    L.sgdyn_rollout_lanes.argtypes = [i32, P(i32)]
    L.sgdyn_host_step.argtypes = [vp, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32, i32]
    L.sgdyn_host_compute_link_jacobian.argtypes = [vp, i64, i32, i32, vp, vp, i32, i32]
    L.sgdyn_host_compute_coriolis_matrix.argtypes = [vp, i64, vp, vp, vp, i32, i32]
    L.sgdyn_host_compute_inverse_kinematics.argtypes = [vp, i64, i32, vp, vp, vp, dbl, i32, dbl, dbl, vp, vp, vp, i32,
                                                        i32]
    L.sgdyn_compute_inverse_dynamics_vjp.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, i32, vp]
    L.sgdyn_compute_forward_dynamics_vjp.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, i32, vp]
    L.sgdyn_compute_forward_kinematics_vjp.argtypes = [vp, i64, vp, vp, vp, vp, i32, vp]
    L.sgdyn_compute_rnea_derivatives.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, i32, vp]
    L.sgdyn_compute_aba_derivatives.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, i32, vp]
    L.sgdyn_rollout_forward.argtypes = [vp, i64, i32, dbl, vp, vp, vp, i32, vp, vp, vp, vp, vp]
    L.sgdyn_rollout_scratch_bytes.argtypes = [vp, i64, i32, P(i64)]
    L.sgdyn_rollout_backward.argtypes = [vp, i64, i32, dbl, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, i64, vp]
    L.sgdyn_batch_create.argtypes = [P(vp), i32, P(i32), i64, P(vp)]
    L.sgdyn_batch_free.argtypes = [vp]
    L.sgdyn_batch_free.restype = None
    L.sgdyn_batch_info.argtypes = [vp, P(i64), P(i32), P(i32), P(i32)]
    L.sgdyn_batch_set_launch.argtypes = [vp, i32, i32, i32]
    L.sgdyn_batch_set_lanes.argtypes = [vp, P(i32)]
    L.sgdyn_batch_step.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.sgdyn_batch_integrate.argtypes = [vp, dbl, vp, vp, vp, vp]
    L.sgdyn_batch_step_integrate.argtypes = [vp, dbl, vp, vp, vp, vp, vp]
    L.sgdyn_model_from_articulation.argtypes = [vp, i32, vp, i32, P(dbl), i32, P(vp)]
    L.sgdyn_compute_passive_force_f32.argtypes = [vp, i64, vp, vp, i64, i32, i32, vp, i64, vp]
    L.sgdyn_jit_config.argtypes = [i32, i64, P(i32), P(i64)]
    L.sgdyn_model_set_lanes.argtypes = [vp, i32]
    L.sgdyn_model_team_table.argtypes = [vp, i32, P(P(i32)), P(i32)]
    L.sgdyn_jit_max_joints.argtypes = [i32, P(i32)]
    L.sgdyn_fd_method.argtypes = [i32, P(i32)]
    L.sgdyn_fd_by_mass_matrix.argtypes = [vp, i32, P(i32)]
    L.sgdyn_jit_prepare.argtypes = [vp, i32]
    L.sgdyn_jit_source.argtypes = [vp, i32, P(ctypes.c_char_p)]
    L.sgdyn_rollout_backward_noalloc.argtypes = [vp, i64, i32, dbl, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    _lib = L
    return L


def last_error():
    return load().sgdyn_last_error().decode()


def check(rc):
    """Translate a status code into the reference's Python exception types."""
    if rc == OK:
        return
    msg = last_error()
    if rc == ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise SgdynError(msg)
