"""The reference's own robots as test inputs: tests/golden/{panda,movo_simple,sawyer,fetch}.urdf
(written from the reference project's assets by tests/golden/make_robot_fixtures.py).

Joint and link orders are the ones SAPIEN's URDF loader gives an articulation
(python/py_package/wrapper/urdf_loader.py:469-588, :629-648): links in depth-first
pre-order from the root link, the children of a link in the order their joints appear in
the file; the active joints are the non-fixed parent joints of those links, in the same
order. ``robot.create_pinocchio_model()`` passes exactly these orders to
``set_joint_order`` / ``set_link_order`` (python/py_package/wrapper/pinocchio_model.py:317-329),
so the q vectors of the reference's own tests index joints this way.
"""
import math
import os
import xml.etree.ElementTree as ET

import numpy as np

from sapien_gb300 import synthetic as syn

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# unittest/test_physx/test_articulation.py:75-97: movo_simple at this q, FK link poses and
# compute_inverse_dynamics(q, 0, 0)
MOVO_REFERENCE_Q = [0.1, 0.1, 0.1, 0.2, 0.2, 0.2, 0.2, 0.2, 0.2, 0.2, 0.3, 0.4, 0.5]

# end-effector links used for the IK cases
EE_LINK = {"panda": "panda_hand", "movo_simple": "right_ee_link", "sawyer": "right_hand", "fetch": "gripper_link"}

# robots whose URDF carries inertias for every moving subtree (panda.urdf has no <inertial>)
DYNAMICS = ("movo_simple", "sawyer", "fetch")

_KIND = {"revolute": syn.REVOLUTE, "continuous": syn.CONTINUOUS, "prismatic": syn.PRISMATIC}


def sapien_loader_order(urdf):
    """(link names, active joints as (name, type, (lower, upper))) in SAPIEN's loader order."""
    root = ET.fromstring(urdf)
    links = [l.get("name") for l in root.findall("link")]
    joints = root.findall("joint")
    children = {name: [] for name in links}
    parent_joint = {}
    for j in joints:
        p, c = j.find("parent").get("link"), j.find("child").get("link")
        children[p].append(j)
        parent_joint[c] = j
    roots = [l for l in links if l not in parent_joint]
    assert len(roots) == 1, roots
    order, active, stack = [], [], [roots[0]]
    while stack:
        name = stack.pop()
        order.append(name)
        j = parent_joint.get(name)
        if j is not None and j.get("type") != "fixed":
            lim = j.find("limit")
            lo = float(lim.get("lower", "0")) if lim is not None else 0.0
            hi = float(lim.get("upper", "0")) if lim is not None else 0.0
            if j.get("type") == "continuous":
                lo, hi = -math.pi, math.pi
            active.append((j.get("name"), j.get("type"), (lo, hi)))
        for cj in reversed(children[name]):
            stack.append(cj.find("child").get("link"))
    return order, active


def load(name):
    """A SyntheticRobot-compatible description of a reference robot fixture."""
    with open(os.path.join(GOLDEN, name + ".urdf")) as f:
        urdf = f.read()
    link_names, active = sapien_loader_order(urdf)
    kinds = [_KIND[t] for _, t, _ in active]
    limits = [lim for _, _, lim in active]
    return syn.SyntheticRobot(name=name, urdf=urdf, joint_names=[a[0] for a in active], joint_kinds=kinds,
                              joint_limits=limits, link_names=link_names,
                              ee_link=link_names.index(EE_LINK[name]), nv=len(active), nq_ext=len(active))


NAMES = ("panda", "movo_simple", "sawyer", "fetch")


def movo_reference_inputs():
    q = np.array(MOVO_REFERENCE_Q, dtype=np.float64)
    return q, np.zeros_like(q), np.zeros_like(q)


# ---- the articulation SAPIEN's URDF loader would build, for create_pinocchio_model ----
class _Pose64:
    """A pose with float64 p and q (w, x, y, z); sapien.Pose's attribute names."""

    def __init__(self, T):
        self.p = np.array(T[:3, 3], dtype=np.float64)
        self.q = _quat_wxyz(T[:3, :3])


def _quat_wxyz(R):
    t = np.trace(R)
    if t > 0:
        r = math.sqrt(t + 1.0)
        k = 0.5 / r
        return np.array([0.5 * r, (R[2, 1] - R[1, 2]) * k, (R[0, 2] - R[2, 0]) * k, (R[1, 0] - R[0, 1]) * k])
    i = int(np.argmax([R[0, 0], R[1, 1], R[2, 2]]))
    j, k_ = (i + 1) % 3, (i + 2) % 3
    r = math.sqrt(R[i, i] - R[j, j] - R[k_, k_] + 1.0)
    q = np.zeros(4)
    q[1 + i] = 0.5 * r
    k = 0.5 / r
    q[0] = (R[k_, j] - R[j, k_]) * k
    q[1 + j] = (R[j, i] + R[i, j]) * k
    q[1 + k_] = (R[k_, i] + R[i, k_]) * k
    return q


def _origin(e):
    """4x4 transform of a URDF <origin> element (xyz, fixed-axis rpy: Rz(y) Ry(p) Rx(r))."""
    T = np.eye(4)
    if e is None:
        return T
    xyz = [float(v) for v in e.get("xyz", "0 0 0").split()]
    r, p, y = [float(v) for v in e.get("rpy", "0 0 0").split()]
    cr, sr, cp, sp, cy, sy = math.cos(r), math.sin(r), math.cos(p), math.sin(p), math.cos(y), math.sin(y)
    T[:3, :3] = [[cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr],
                 [sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr],
                 [-sp, cp * sr, cp * cr]]
    T[:3, 3] = xyz
    return T


def sapien_articulation(robot):
    """ArticulationDesc of the articulation SAPIEN's URDF loader builds from the robot's
    URDF (root fixed): link inertias as principal moments in a rotated inertial frame
    (urdf_loader.py:259-293), joint frames with the motion axis as x
    (pose_in_parent = origin * axis frame, pose_in_child = axis frame, urdf_loader.py:504-569).
    Links without inertial data get zero mass (SAPIEN would derive one from collision
    shapes, which the fixtures do not keep; such links here are all fixed-joint frames)."""
    from sapien_gb300.articulation import ArticulationDesc, JointDesc, LinkDesc

    root = ET.fromstring(robot.urdf)
    by_name = {l.get("name"): l for l in root.findall("link")}
    parent_joint = {j.find("child").get("link"): j for j in root.findall("joint")}
    links = []
    for i, name in enumerate(robot.link_names):
        inertial = by_name[name].find("inertial")
        mass, cm, eig = 0.0, np.eye(4), np.zeros(3)
        if inertial is not None:
            m = float(inertial.find("mass").get("value"))
            a = inertial.find("inertia").attrib
            I = np.array([[float(a.get("ixx", 0)), float(a.get("ixy", 0)), float(a.get("ixz", 0))],
                          [float(a.get("ixy", 0)), float(a.get("iyy", 0)), float(a.get("iyz", 0))],
                          [float(a.get("ixz", 0)), float(a.get("iyz", 0)), float(a.get("izz", 0))]])
            if m != 0 and np.any(I != 0):
                if np.array_equal(np.diag(np.diag(I)), I):
                    eig, vecs = np.diag(I).copy(), np.eye(3)
                else:
                    eig, vecs = np.linalg.eigh(I)
                    if np.linalg.det(vecs) < 0:
                        vecs[:, 2] = -vecs[:, 2]
                rot = np.eye(4)
                rot[:3, :3] = vecs
                mass, cm = m, _origin(inertial.find("origin")) @ rot
        links.append(LinkDesc(index=i, mass=mass, cmass_local_pose=_Pose64(cm), inertia=tuple(eig)))
    joints = []
    for i, name in enumerate(robot.link_names):
        j = parent_joint.get(name)
        if j is None:
            joints.append(JointDesc(type="fixed", parent_link=None, child_link=links[i]))
            continue
        ax = j.find("axis")
        axis = np.array([float(v) for v in (ax.get("xyz") if ax is not None else "1 0 0").split()])
        axis = axis / np.linalg.norm(axis) if np.linalg.norm(axis) >= 1e-3 else np.array([1.0, 0.0, 0.0])
        other = [0.0, 0.0, 1.0] if abs(axis @ [1.0, 0.0, 0.0]) > 0.9 else [1.0, 0.0, 0.0]
        a1 = np.cross(axis, other)
        a1 /= np.linalg.norm(a1)
        t_axis = np.eye(4)
        t_axis[:3, 0], t_axis[:3, 1], t_axis[:3, 2] = axis, a1, np.cross(axis, a1)
        kind = j.get("type")
        lim = j.find("limit")
        lo = float(lim.get("lower", "0")) if lim is not None else 0.0
        hi = float(lim.get("upper", "0")) if lim is not None else 0.0
        jtype, limit = {"revolute": ("revolute_unwrapped", ((lo, hi),)),
                        "continuous": ("revolute", ((-np.inf, np.inf),)),
                        "prismatic": ("prismatic", ((lo, hi),)),
                        "fixed": ("fixed", ())}[kind]
        parent = links[robot.link_names.index(j.find("parent").get("link"))]
        joints.append(JointDesc(type=jtype, parent_link=parent, child_link=links[i],
                                pose_in_parent=_Pose64(_origin(j.find("origin")) @ t_axis),
                                pose_in_child=_Pose64(t_axis), limit=limit))
    return ArticulationDesc(links=links, joints=joints)
