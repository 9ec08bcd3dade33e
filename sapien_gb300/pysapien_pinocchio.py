"""The reference's module name for its pybind PinocchioModel (pinocchio/pinocchio_model.cpp:306-367).

SAPIEN's Python wrapper imports ``PinocchioModel`` from ``pysapien_pinocchio`` when pip
``pinocchio`` is absent (python/py_package/wrapper/pinocchio_model.py:295-314); pointing that
import at ``sapien_gb300.pysapien_pinocchio`` gives the same class name and surface backed by
this library.
"""
from .pinocchio_model import PinocchioModel, Pose

__all__ = ["PinocchioModel", "Pose"]
