"""Seeded synthetic kinematic trees and input batches.

The reference publishes no benchmark data for this path, so workloads are seeded
synthetic robots written as URDF text (the same input the reference's
``PinocchioModel(urdf, gravity)`` constructor takes, pinocchio/pinocchio_model.cpp:39-47):

* ``serial_chain(7)``  - fixed-base serial revolute chain (7 DoF);
* ``arm_with_fingers()`` - 7 revolute arm + 2 prismatic fingers on the last link
  (9 DoF, finger range [0, 0.04] m);
* ``quadruped()``  - floating base + 4 legs x 3 revolute (18 DoF);
* ``humanoid()``   - floating base, spine of 3, two arms of 7, two legs of 6 (30 DoF);
* ``serial_chain(6)`` - 6-DoF revolute arm.

Link offsets are U[0.05, 0.4] m along random unit directions, joint axes random unit
vectors, masses U[0.5, 3] kg (floating bases U[5, 15] kg), rotational inertias
R diag(U[1e-3, 5e-2]) R^T with a random rotation R, centres of mass U[-0.05, 0.05]^3.

``sapien_style=True`` writes the same robot the way SAPIEN's URDF exporter does
(python/py_package/wrapper/urdf_exporter.py:21-152): every moving joint has axis
``1 0 0`` and an ``rpy`` origin that turns x onto the wanted axis, is followed by a
dummy link and a fixed ``joint_dummy_*`` joint, and inertias are principal moments
with an ``rpy`` inertial frame. That variant exercises fixed-joint merging and rotated
placements in the model builder.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

REVOLUTE, PRISMATIC, CONTINUOUS, FLOATING = "revolute", "prismatic", "continuous", "floating"


def _unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def _rand_rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
        ]
    )


def _rpy_of(R):
    """Fixed-axis roll, pitch, yaw of a rotation (R = Rz(y) Ry(p) Rx(r))."""
    yaw = math.atan2(R[1, 0], R[0, 0])
    pitch = math.atan2(-R[2, 0], math.hypot(R[0, 0], R[1, 0]))
    s, c = math.sin(yaw), math.cos(yaw)
    roll = math.atan2(s * R[0, 2] - c * R[1, 2], c * R[1, 1] - s * R[0, 1])
    return roll, pitch, yaw


def _rot_x_to(a):
    """A rotation whose first column is the unit vector a."""
    a = a / np.linalg.norm(a)
    t = np.array([0.0, 0.0, 1.0]) if abs(a[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    b = np.cross(a, t)
    b /= np.linalg.norm(b)
    c = np.cross(a, b)
    return np.stack([a, b, c], axis=1)


def _num(x):
    return repr(float(x))


def _fmt(v):
    return " ".join(_num(x) for x in v)


@dataclass
class JointSpec:
    name: str
    kind: str
    parent: int  # parent link index
    child: int  # child link index
    offset: np.ndarray
    axis: np.ndarray
    lower: float = -math.pi
    upper: float = math.pi


@dataclass
class SyntheticRobot:
    """A generated robot: URDF text plus the orders a caller passes to the model."""

    name: str
    urdf: str
    joint_names: list  # active joints, external order
    joint_kinds: list
    joint_limits: list
    link_names: list
    ee_link: int
    nv: int
    nq_ext: int
    specs: list = field(default_factory=list)

    def sample(self, n, seed=0, tau_std=10.0):
        """Seeded inputs: q ~ U[limits] (free flyer: U[-1,1]^3 + random unit
        quaternion x y z w), qd, qdd ~ N(0, 1), tau ~ N(0, tau_std^2)."""
        rng = np.random.default_rng(seed)
        cols = []
        for kind, (lo, hi) in zip(self.joint_kinds, self.joint_limits):
            if kind == FLOATING:
                p = rng.uniform(-1, 1, size=(n, 3))
                quat = rng.normal(size=(n, 4))
                quat /= np.linalg.norm(quat, axis=1, keepdims=True)
                cols.append(np.concatenate([p, quat], axis=1))
            else:
                cols.append(rng.uniform(lo, hi, size=(n, 1)))
        q = np.concatenate(cols, axis=1)
        qd = rng.normal(size=(n, self.nv))
        qdd = rng.normal(size=(n, self.nv))
        tau = rng.normal(scale=tau_std, size=(n, self.nv))
        return q, qd, qdd, tau


def _make(name, specs, nlinks, rng, sapien_style, base_mass=None):
    masses = [rng.uniform(0.5, 3.0) for _ in range(nlinks)]
    if base_mass is not None:
        masses[1] = base_mass
    inertias = []
    for _ in range(nlinks):
        R = _rand_rot(rng)
        d = rng.uniform(1e-3, 5e-2, size=3)
        com = rng.uniform(-0.05, 0.05, size=3)
        inertias.append((R, d, com))
    lines = [f'<robot name="{name}">']
    has_world = any(s.kind == FLOATING for s in specs)
    if has_world:
        lines.append('  <link name="world"/>')
    for li in range(nlinks):
        if has_world and li == 0:
            continue
        R, d, com = inertias[li]
        lines.append(f'  <link name="link_{li}">')
        lines.append("    <inertial>")
        if sapien_style:
            lines.append(f'      <origin xyz="{_fmt(com)}" rpy="{_fmt(_rpy_of(R))}"/>')
            lines.append(f'      <mass value="{_num(masses[li])}"/>')
            lines.append(f'      <inertia ixx="{_num(d[0])}" iyy="{_num(d[1])}" izz="{_num(d[2])}" ixy="0" ixz="0" iyz="0"/>')
        else:
            I = R @ np.diag(d) @ R.T
            lines.append(f'      <origin xyz="{_fmt(com)}" rpy="0 0 0"/>')
            lines.append(f'      <mass value="{_num(masses[li])}"/>')
            lines.append(
                f'      <inertia ixx="{_num(I[0, 0])}" ixy="{_num(I[0, 1])}" ixz="{_num(I[0, 2])}" '
                f'iyy="{_num(I[1, 1])}" iyz="{_num(I[1, 2])}" izz="{_num(I[2, 2])}"/>'
            )
        lines.append("    </inertial>")
        lines.append("  </link>")
    for s in specs:
        parent = "world" if s.kind == FLOATING else f"link_{s.parent}"
        child = f"link_{s.child}"
        if s.kind == FLOATING:
            lines.append(f'  <joint name="{s.name}" type="floating">')
            lines.append(f'    <parent link="{parent}"/>')
            lines.append(f'    <child link="{child}"/>')
            lines.append("  </joint>")
            continue
        if sapien_style:
            Rj = _rot_x_to(s.axis)
            lines.append(f'  <joint name="{s.name}" type="{s.kind}">')
            lines.append(f'    <origin xyz="{_fmt(s.offset)}" rpy="{_fmt(_rpy_of(Rj))}"/>')
            lines.append('    <axis xyz="1 0 0"/>')
            lines.append(f'    <parent link="{parent}"/>')
            lines.append(f'    <child link="link_dummy_{s.child}"/>')
            if s.kind != CONTINUOUS:
                lines.append(f'    <limit effort="0" velocity="0" lower="{_num(s.lower)}" upper="{_num(s.upper)}"/>')
            lines.append("  </joint>")
            lines.append(f'  <link name="link_dummy_{s.child}"/>')
            # child frame rotated back so the link keeps its un-rotated orientation
            c2j = Rj.T
            lines.append(f'  <joint name="joint_dummy_{s.child}" type="fixed">')
            lines.append(f'    <origin xyz="0 0 0" rpy="{_fmt(_rpy_of(c2j))}"/>')
            lines.append('    <axis xyz="0 0 0"/>')
            lines.append(f'    <parent link="link_dummy_{s.child}"/>')
            lines.append(f'    <child link="{child}"/>')
            lines.append("  </joint>")
        else:
            lines.append(f'  <joint name="{s.name}" type="{s.kind}">')
            lines.append(f'    <origin xyz="{_fmt(s.offset)}" rpy="0 0 0"/>')
            lines.append(f'    <axis xyz="{_fmt(s.axis)}"/>')
            lines.append(f'    <parent link="{parent}"/>')
            lines.append(f'    <child link="{child}"/>')
            if s.kind != CONTINUOUS:
                lines.append(f'    <limit effort="0" velocity="0" lower="{_num(s.lower)}" upper="{_num(s.upper)}"/>')
            lines.append("  </joint>")
    lines.append("</robot>")
    urdf = "\n".join(lines)
    joint_names = [s.name for s in specs]
    kinds = [s.kind for s in specs]
    limits = [(s.lower, s.upper) for s in specs]
    link_names = [f"link_{i}" for i in range(nlinks) if not (has_world and i == 0)]
    nv = sum(6 if k == FLOATING else 1 for k in kinds)
    nq_ext = sum(7 if k == FLOATING else 1 for k in kinds)
    ee = link_names.index(f"link_{specs[-1].child}") if specs else 0
    return SyntheticRobot(name, urdf, joint_names, kinds, limits, link_names, ee, nv, nq_ext, specs)


def _offset(rng):
    return rng.uniform(0.05, 0.4) * _unit(rng)


def serial_chain(ndof=7, seed=0, sapien_style=False, kinds=None):
    """Fixed-base chain link_0 -> ... -> link_ndof of revolute joints (or `kinds`)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(1, ndof + 1):
        kind = kinds[i - 1] if kinds else REVOLUTE
        lo, hi = (-0.5, 0.5) if kind == PRISMATIC else (-math.pi, math.pi)
        specs.append(JointSpec(f"joint_{i}", kind, i - 1, i, _offset(rng), _unit(rng), lo, hi))
    return _make(f"chain{ndof}", specs, ndof + 1, rng, sapien_style)


def arm_with_fingers(seed=1, sapien_style=False):
    """7 revolute joints in series, then 2 prismatic fingers on the last arm link."""
    rng = np.random.default_rng(seed)
    specs = [JointSpec(f"joint_{i}", REVOLUTE, i - 1, i, _offset(rng), _unit(rng)) for i in range(1, 8)]
    for k in (8, 9):
        specs.append(JointSpec(f"joint_{k}", PRISMATIC, 7, k, _offset(rng), _unit(rng), 0.0, 0.04))
    return _make("arm9", specs, 10, rng, sapien_style)


def quadruped(seed=2, sapien_style=False):
    """Floating base (link_1) with 4 legs of 3 revolute joints."""
    rng = np.random.default_rng(seed)
    specs = [JointSpec("joint_1", FLOATING, 0, 1, np.zeros(3), np.zeros(3), 0, 0)]
    li = 2
    for leg in range(4):
        parent = 1
        for k in range(3):
            specs.append(JointSpec(f"joint_{li}", REVOLUTE, parent, li, _offset(rng), _unit(rng)))
            parent = li
            li += 1
    return _make("quadruped18", specs, li, rng, sapien_style, base_mass=rng.uniform(5, 15))


def humanoid(seed=3, sapien_style=False):
    """Floating pelvis; spine of 3; two arms of 7 on the spine top; two legs of 6."""
    rng = np.random.default_rng(seed)
    specs = [JointSpec("joint_1", FLOATING, 0, 1, np.zeros(3), np.zeros(3), 0, 0)]
    li = 2

    def chain(parent, n):
        nonlocal li
        for _ in range(n):
            specs.append(JointSpec(f"joint_{li}", REVOLUTE, parent, li, _offset(rng), _unit(rng)))
            parent = li
            li += 1
        return parent

    top = chain(1, 3)
    chain(top, 7)
    chain(top, 7)
    chain(1, 6)
    chain(1, 6)
    return _make("humanoid30", specs, li, rng, sapien_style, base_mass=rng.uniform(5, 15))


def by_name(name, **kw):
    return {
        "chain7": lambda: serial_chain(7, **kw),
        "arm6": lambda: serial_chain(6, seed=kw.pop("seed", 4), **kw),
        "arm9": lambda: arm_with_fingers(**kw),
        "quadruped18": lambda: quadruped(**kw),
        "humanoid30": lambda: humanoid(**kw),
    }[name]()


def hetero_mix(n, seed=0, fractions=(0.5, 0.3, 0.2)):
    """Seeded mix of 6-DoF arms, floating-base quadrupeds and floating-base humanoids:
    returns (robots, model_of_env) with robots = [arm6, quadruped18, humanoid]."""
    robots = [serial_chain(6, seed=4), quadruped(), humanoid()]
    rng = np.random.default_rng(seed)
    counts = [int(round(f * n)) for f in fractions[:-1]]
    counts.append(n - sum(counts))
    model_of_env = np.concatenate([np.full(c, k, dtype=np.int32) for k, c in enumerate(counts)])
    rng.shuffle(model_of_env)
    return robots, model_of_env
