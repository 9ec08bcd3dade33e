"""Model construction from a SAPIEN-style articulation, without writing URDF text.

``create_pinocchio_model(articulation, gravity)`` mirrors SAPIEN's
``PhysxArticulation.create_pinocchio_model`` (python/py_package/wrapper/pinocchio_model.py:
317-326): the kinematic tree SAPIEN's URDF exporter would write
(python/py_package/wrapper/urdf_exporter.py:21-152, root forced fixed) is built natively
through ``sgdyn_model_from_articulation``, the joint order is set to the active joints and
the link order to the articulation's links. It accepts either the dataclasses below or any
object with SAPIEN's attribute names (``links[i].mass / cmass_local_pose / inertia``,
``joints[j].type / parent_link / child_link / pose_in_parent / pose_in_child / limit``).

``export_kinematic_chain_urdf`` restates the exporter itself, for the URDF path.
"""
from __future__ import annotations

import ctypes
import math
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .pinocchio_model import PinocchioModel, Pose


@dataclass
class LinkDesc:
    index: int
    mass: float
    cmass_local_pose: Pose = field(default_factory=Pose)
    inertia: tuple = (0.0, 0.0, 0.0)


@dataclass
class JointDesc:
    type: str  # "fixed", "revolute", "revolute_unwrapped", "prismatic", "free"
    parent_link: LinkDesc | None
    child_link: LinkDesc
    pose_in_parent: Pose = field(default_factory=Pose)
    pose_in_child: Pose = field(default_factory=Pose)
    limit: tuple = ((-math.pi, math.pi),)


@dataclass
class ArticulationDesc:
    links: list
    joints: list

    @property
    def active_joints(self):
        return [j for j in self.joints if j.type != "fixed" and not (j.parent_link is None)]


def _pose7(pose):
    p = np.asarray(pose.p, dtype=np.float64).reshape(3)
    q = np.asarray(pose.q, dtype=np.float64).reshape(4)
    return list(p) + list(q)


class _Link(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("cmass_pose", ctypes.c_double * 7), ("inertia", ctypes.c_double * 3)]


class _Joint(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("parent", ctypes.c_int), ("child", ctypes.c_int),
                ("pose_in_parent", ctypes.c_double * 7), ("pose_in_child", ctypes.c_double * 7),
                ("lower", ctypes.c_double), ("upper", ctypes.c_double)]


def _joint_code(t, is_root):
    if t == "fixed":
        return 0
    if is_root:
        return 3
    if t.startswith("revolute"):
        return 1
    if t == "prismatic":
        return 2
    raise ValueError(f"invalid joint type {t}")


def create_pinocchio_model(articulation, gravity=(0.0, 0.0, -9.81)):
    """PinocchioModel for a SAPIEN-style articulation (root forced fixed), built natively."""
    links = list(articulation.links)
    joints = list(articulation.joints)
    la = (_Link * len(links))()
    for i, l in enumerate(links):
        la[i].mass = float(l.mass)
        la[i].cmass_pose[:] = _pose7(l.cmass_local_pose)
        la[i].inertia[:] = [float(x) for x in np.asarray(l.inertia).reshape(3)]
    ja = (_Joint * max(len(joints), 1))()
    for k, j in enumerate(joints):
        root = j.parent_link is None
        ja[k].type = _joint_code(j.type, root)
        ja[k].parent = -1 if root else int(j.parent_link.index)
        ja[k].child = int(j.child_link.index)
        ja[k].pose_in_parent[:] = _pose7(j.pose_in_parent)
        ja[k].pose_in_child[:] = _pose7(j.pose_in_child)
        lim = np.asarray(j.limit, dtype=np.float64).reshape(-1)
        ja[k].lower, ja[k].upper = (float(lim[0]), float(lim[1])) if lim.size >= 2 else (-np.inf, np.inf)
    g = (ctypes.c_double * 3)(*[float(x) for x in gravity])
    h = ctypes.c_void_p()
    N.check(N.load().sgdyn_model_from_articulation(ctypes.cast(la, ctypes.c_void_p), len(links),
                                                   ctypes.cast(ja, ctypes.c_void_p), len(joints), g, 1,
                                                   ctypes.byref(h)))
    return PinocchioModel._from_handle(h, joint_order_set=True, link_order_set=True)


# ---- the exporter, restated (URDF path) ---------------------------------------------
def _rpy(pose):
    w, x, y, z = (float(v) for v in np.asarray(pose.q, dtype=np.float64))
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    # R = Rz(yaw) Ry(pitch) Rx(roll); every angle from atan2, so a pitch near +-pi/2 (an
    # axis frame turning x onto z) keeps full precision, as the reference's Eigen-based
    # conversion does (include/sapien/math/conversion.h:53-57)
    yaw = math.atan2(R[1, 0], R[0, 0])
    pitch = math.atan2(-R[2, 0], math.hypot(R[0, 0], R[1, 0]))
    s, c = math.sin(yaw), math.cos(yaw)
    roll = math.atan2(s * R[0, 2] - c * R[1, 2], c * R[1, 1] - s * R[0, 1])
    return roll, pitch, yaw


def _inv(pose):
    w, x, y, z = (float(v) for v in np.asarray(pose.q, dtype=np.float64))
    qi = np.array([w, -x, -y, -z])
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    p = -R.T @ np.asarray(pose.p, dtype=np.float64)
    out = Pose()
    out.p, out.q = p, qi  # keep float64 (Pose stores float32 by default)
    return out


def _f(v):
    return " ".join(repr(float(x)) for x in v)


def export_kinematic_chain_urdf(articulation, force_fix_root=False):
    """URDF text in the form SAPIEN's exporter writes (link_i / joint_i names, dummy links)."""
    robot = ET.Element("robot", {"name": ""})
    ET.SubElement(robot, "link", {"name": "world"})
    for l in articulation.links:
        el = ET.SubElement(robot, "link", {"name": f"link_{l.index}"})
        ine = ET.SubElement(el, "inertial")
        ET.SubElement(ine, "origin", {"xyz": _f(np.asarray(l.cmass_local_pose.p, dtype=np.float64)),
                                      "rpy": _f(_rpy(l.cmass_local_pose))})
        ET.SubElement(ine, "mass", {"value": repr(float(l.mass))})
        i3 = np.asarray(l.inertia, dtype=np.float64).reshape(3)
        ET.SubElement(ine, "inertia", {"ixx": repr(float(i3[0])), "iyy": repr(float(i3[1])),
                                       "izz": repr(float(i3[2])), "ixy": "0", "ixz": "0", "iyz": "0"})
    for j in articulation.joints:
        name = f"joint_{j.child_link.index}"
        if j.parent_link is None:
            t = "fixed" if (j.type == "fixed" or force_fix_root) else "floating"
            ej = ET.SubElement(robot, "joint", {"name": name, "type": t})
            ET.SubElement(ej, "parent", {"link": "world"})
            ET.SubElement(ej, "child", {"link": f"link_{j.child_link.index}"})
            continue
        lim = np.asarray(j.limit, dtype=np.float64).reshape(-1)
        if j.type == "fixed":
            t = "fixed"
        elif j.type == "prismatic":
            t = "prismatic"
        elif j.type.startswith("revolute"):
            t = "continuous" if (lim[0] < -1e5 and lim[1] > 1e5) else "revolute"
        else:
            raise ValueError(f"invalid joint type {j.type}")
        ej = ET.SubElement(robot, "joint", {"name": name, "type": t})
        ET.SubElement(ej, "origin", {"xyz": _f(np.asarray(j.pose_in_parent.p, dtype=np.float64)),
                                     "rpy": _f(_rpy(j.pose_in_parent))})
        ET.SubElement(ej, "axis", {"xyz": "1 0 0"})
        ET.SubElement(ej, "parent", {"link": f"link_{j.parent_link.index}"})
        ET.SubElement(ej, "child", {"link": f"link_dummy_{j.child_link.index}"})
        if t in ("prismatic", "revolute"):
            ET.SubElement(ej, "limit", {"effort": "0", "velocity": "0", "lower": repr(max(float(lim[0]), -1e5)),
                                        "upper": repr(min(float(lim[1]), 1e5))})
        ET.SubElement(robot, "link", {"name": f"link_dummy_{j.child_link.index}"})
        c2j = _inv(j.pose_in_child)
        ed = ET.SubElement(robot, "joint", {"name": f"joint_dummy_{j.child_link.index}", "type": "fixed"})
        ET.SubElement(ed, "origin", {"xyz": _f(c2j.p), "rpy": _f(_rpy(c2j))})
        ET.SubElement(ed, "axis", {"xyz": "0 0 0"})
        ET.SubElement(ed, "parent", {"link": f"link_dummy_{j.child_link.index}"})
        ET.SubElement(ed, "child", {"link": f"link_{j.child_link.index}"})
    return ET.tostring(robot, encoding="utf8").decode()


def random_articulation(n_moving=6, seed=0):
    """Seeded articulation: fixed root, a chain of revolute / prismatic / unbounded revolute
    joints with one fixed joint in the middle; random poses, masses and inertias."""
    rng = np.random.default_rng(seed)

    def rpose():
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        p = Pose()
        p.p, p.q = rng.uniform(-0.3, 0.3, 3), q
        return p

    nl = n_moving + 2
    links = [LinkDesc(i, float(rng.uniform(0.5, 3.0)), rpose(), tuple(rng.uniform(1e-3, 5e-2, 3)))
             for i in range(nl)]
    joints = [JointDesc("fixed", None, links[0])]
    kinds = ["revolute", "prismatic", "revolute_unwrapped"]
    for i in range(1, nl):
        t = "fixed" if i == nl // 2 else kinds[i % 3]
        lim = ((-1e6, 1e6),) if t == "revolute_unwrapped" else ((-2.5, 2.5),)
        joints.append(JointDesc(t, links[i - 1], links[i], rpose(), rpose(), lim))
    return ArticulationDesc(links, joints)
