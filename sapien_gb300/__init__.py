"""sapien_gb300: GB300-native batched articulated-body dynamics.

A from-scratch rebuild of SAPIEN's ``PinocchioModel`` path (forward kinematics, link
poses, Jacobians, CRBA mass matrix, RNEA, ABA, CLIK inverse kinematics) as FP64 CUDA
kernels for sm_103a behind a C ABI (include/sgdyn.h), with the reference's Python
surface kept as a drop-in and batched tensor overloads added beside it.
"""
from .pinocchio_model import PinocchioModel, Pose  # noqa: F401
from . import synthetic  # noqa: F401

__all__ = ["PinocchioModel", "Pose", "synthetic"]
