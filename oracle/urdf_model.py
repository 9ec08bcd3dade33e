"""URDF -> kinematic-tree tables for the CPU oracle (test infrastructure only).

This is the oracle's own model builder. It shares no code with the product's C++
URDF reader, so a parity test that feeds the same URDF text to both exercises the
product's model construction as well as its kinematics/dynamics kernels.

It restates the model-construction semantics that the reference reaches through
``pinocchio::urdf::buildModelFromXML`` (called at pinocchio/pinocchio_model.cpp:42,
Pinocchio v2.6.18, fetched at pinocchio/cmake/pinocchio.cmake:46-53 and absent from
the reference tree):

* The URDF root link is welded to the universe joint 0 (no root joint is passed by
  ``fromURDFXML``), so its inertia never moves.
* Links are visited depth first; the children of a link are visited in the
  byte-wise lexicographic order of their joint names (urdfdom keeps joints in a
  ``std::map`` keyed by name and builds ``child_links`` in that order).
* A moving joint (revolute / continuous / prismatic / floating) gets the placement
  ``parent_body_frame.placement * joint.origin`` relative to the moving joint that
  carries the parent link; the child link's inertia is attached to it at identity.
* A fixed joint adds no degree of freedom: the child link's inertia is transported
  by ``parent_body_frame.placement * joint.origin`` and added to the carrying joint,
  and the child link's BODY frame inherits that placement.
* revolute -> 1 DoF rotation (nq=1), continuous -> unbounded rotation stored as
  (cos, sin) (nq=2, nv=1), prismatic -> translation (nq=1), floating -> free flyer
  (nq=7: x y z qx qy qz qw, nv=6).
* Link inertials: com = origin.xyz, rotational inertia = R(origin.rpy) I R^T.
* RPY -> rotation goes through the urdfdom half-angle quaternion formula and the
  unit-quaternion -> matrix formula.
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

# Joint kinds used by the oracle tables (oracle-local numbering).
JT_UNIVERSE = 0
JT_REVOLUTE = 1
JT_PRISMATIC = 2
JT_CONTINUOUS = 3
JT_FREEFLYER = 4

_NQ = {JT_REVOLUTE: 1, JT_PRISMATIC: 1, JT_CONTINUOUS: 2, JT_FREEFLYER: 7}
_NV = {JT_REVOLUTE: 1, JT_PRISMATIC: 1, JT_CONTINUOUS: 1, JT_FREEFLYER: 6}


def quat_to_matrix(w, x, y, z):
    """Unit quaternion (w, x, y, z) -> rotation matrix (no renormalisation)."""
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
        ]
    )


def rpy_to_matrix(roll, pitch, yaw):
    """URDF fixed-axis roll/pitch/yaw -> rotation, via the half-angle quaternion."""
    phi, the, psi = roll / 2.0, pitch / 2.0, yaw / 2.0
    x = math.sin(phi) * math.cos(the) * math.cos(psi) - math.cos(phi) * math.sin(the) * math.sin(psi)
    y = math.cos(phi) * math.sin(the) * math.cos(psi) + math.sin(phi) * math.cos(the) * math.sin(psi)
    z = math.cos(phi) * math.cos(the) * math.sin(psi) - math.sin(phi) * math.sin(the) * math.cos(psi)
    w = math.cos(phi) * math.cos(the) * math.cos(psi) + math.sin(phi) * math.sin(the) * math.sin(psi)
    n = math.sqrt(x * x + y * y + z * z + w * w)
    return quat_to_matrix(w / n, x / n, y / n, z / n)


def _floats(s, n, default):
    if s is None:
        return list(default)
    vals = [float(t) for t in s.split()]
    if len(vals) != n:
        raise ValueError(f"expected {n} numbers, got {s!r}")
    return vals


def _origin(elem):
    """(R, p) of an <origin> child (identity when absent)."""
    o = elem.find("origin") if elem is not None else None
    if o is None:
        return np.eye(3), np.zeros(3)
    xyz = _floats(o.get("xyz"), 3, (0, 0, 0))
    rpy = _floats(o.get("rpy"), 3, (0, 0, 0))
    return rpy_to_matrix(*rpy), np.array(xyz, dtype=float)


def spatial_inertia(m, c, Ic):
    """6x6 spatial inertia in [linear; angular] ordering about the frame origin."""
    cx = np.array([[0, -c[2], c[1]], [c[2], 0, -c[0]], [-c[1], c[0], 0]])
    I6 = np.zeros((6, 6))
    I6[:3, :3] = m * np.eye(3)
    I6[:3, 3:] = -m * cx
    I6[3:, :3] = m * cx
    I6[3:, 3:] = Ic - m * cx @ cx
    return I6


@dataclass
class OracleModel:
    """Flat kinematic tree in depth-first joint order (joint 0 = universe)."""

    gravity: np.ndarray
    parent: list = field(default_factory=lambda: [0])
    jtype: list = field(default_factory=lambda: [JT_UNIVERSE])
    axis: list = field(default_factory=lambda: [np.zeros(3)])
    placement: list = field(default_factory=lambda: [(np.eye(3), np.zeros(3))])
    inertia6: list = field(default_factory=lambda: [np.zeros((6, 6))])
    joint_names: list = field(default_factory=lambda: ["universe"])
    # BODY frames: link name -> (carrying joint, placement in that joint frame)
    body_frames: dict = field(default_factory=dict)
    link_names_in_order: list = field(default_factory=list)
    link_order: list = field(default_factory=list)  # set by set_link_order
    joint_order: list = field(default_factory=list)  # set by set_joint_order

    @property
    def njoints(self):
        return len(self.parent)

    @property
    def nqs(self):
        return [0] + [_NQ[t] for t in self.jtype[1:]]

    @property
    def nvs(self):
        return [0] + [_NV[t] for t in self.jtype[1:]]

    @property
    def nv(self):
        return sum(self.nvs)

    @property
    def nq(self):
        return sum(self.nqs)

    def set_joint_order(self, names):
        ids = []
        for n in names:
            if n not in self.joint_names or n == "universe":
                raise ValueError(f"invalid joint name {n}")
            ids.append(self.joint_names.index(n))
        if sum(self.nvs[i] for i in ids) != self.nv:
            raise RuntimeError("setJointOrder failed")
        self.joint_order = ids

    def set_link_order(self, names):
        for n in names:
            if n not in self.body_frames:
                raise ValueError(f"invalid link name {n}")
        self.link_order = list(names)


def _rotate_inertia6(I6, R, p):
    """Express a 6x6 spatial inertia given in frame B in frame A, where
    x_A = R x_B + p (force transform X* I X^-1)."""
    px = np.array([[0, -p[2], p[1]], [p[2], 0, -p[0]], [-p[1], p[0], 0]])
    Xf = np.zeros((6, 6))  # force transform B -> A: [R 0; p^R R]
    Xf[:3, :3] = R
    Xf[3:, 3:] = R
    Xf[3:, :3] = px @ R
    return Xf @ I6 @ Xf.T


def build_model(urdf: str, gravity=(0.0, 0.0, -9.81)) -> OracleModel:
    root = ET.fromstring(urdf)
    links = {}
    for le in root.findall("link"):
        name = le.get("name")
        inertial = le.find("inertial")
        if inertial is None:
            links[name] = np.zeros((6, 6))
            continue
        R, c = _origin(inertial)
        me = inertial.find("mass")
        m = float(me.get("value")) if me is not None else 0.0
        ie = inertial.find("inertia")
        vals = {k: float(ie.get(k, 0.0)) if ie is not None else 0.0 for k in ("ixx", "ixy", "ixz", "iyy", "iyz", "izz")}
        I = np.array(
            [
                [vals["ixx"], vals["ixy"], vals["ixz"]],
                [vals["ixy"], vals["iyy"], vals["iyz"]],
                [vals["ixz"], vals["iyz"], vals["izz"]],
            ]
        )
        links[name] = spatial_inertia(m, c, R @ I @ R.T)
    joints = {}
    child_of = {}
    for je in root.findall("joint"):
        name = je.get("name")
        jt = je.get("type")
        parent = je.find("parent").get("link")
        child = je.find("child").get("link")
        R, p = _origin(je)
        ax = je.find("axis")
        axis = np.array(_floats(ax.get("xyz") if ax is not None else None, 3, (1, 0, 0)))
        joints[name] = dict(type=jt, parent=parent, child=child, R=R, p=p, axis=axis)
        if child in child_of:
            raise ValueError(f"link {child} has two parents")
        child_of[child] = name
    roots = [l for l in links if l not in child_of]
    if len(roots) != 1:
        raise ValueError(f"URDF must have exactly one root link, found {roots}")
    children = {l: [] for l in links}
    for jn in sorted(joints.keys(), key=lambda s: s.encode()):
        children[joints[jn]["parent"]].append(jn)

    model = OracleModel(gravity=np.array(gravity, dtype=float))
    rootname = roots[0]
    model.inertia6[0] = model.inertia6[0] + links[rootname]
    model.body_frames[rootname] = (0, (np.eye(3), np.zeros(3)))
    model.link_names_in_order.append(rootname)

    def visit(link):
        pj, (pR, pp) = model.body_frames[link]
        for jn in children[link]:
            j = joints[jn]
            R = pR @ j["R"]
            p = pR @ j["p"] + pp
            child = j["child"]
            if j["type"] == "fixed":
                model.inertia6[pj] = model.inertia6[pj] + _rotate_inertia6(links[child], R, p)
                model.body_frames[child] = (pj, (R, p))
            else:
                kind = {
                    "revolute": JT_REVOLUTE,
                    "continuous": JT_CONTINUOUS,
                    "prismatic": JT_PRISMATIC,
                    "floating": JT_FREEFLYER,
                }.get(j["type"])
                if kind is None:
                    raise ValueError(f"unsupported joint type {j['type']}")
                ax = j["axis"]
                ax = ax / np.linalg.norm(ax) if kind != JT_FREEFLYER else np.zeros(3)
                model.parent.append(pj)
                model.jtype.append(kind)
                model.axis.append(ax)
                model.placement.append((R, p))
                model.inertia6.append(links[child].copy())
                model.joint_names.append(jn)
                jid = len(model.parent) - 1
                model.body_frames[child] = (jid, (np.eye(3), np.zeros(3)))
            model.link_names_in_order.append(child)
            visit(child)

    visit(rootname)
    return model
