"""Writes the robot fixtures tests/golden/{panda,movo_simple}.urdf from the reference's own
robot descriptions, keeping only what the dynamics path reads.

Sources (inside the reference project):
  assets/robot/panda/panda.urdf       7 revolute arm joints + 2 prismatic fingers (one with a
                                      <mimic> tag, which Pinocchio's URDF parser ignores)
  unittest/assets/movo_simple.urdf    the robot of unittest/test_physx/test_articulation.py:75-97:
                                      13 DoF (a prismatic lift, 2 revolute head joints, 7
                                      continuous arm joints, 3 revolute gripper fingers) and 16
                                      fixed joints
  assets/robot/sawyer/sawyer.urdf     7 revolute + 2 prismatic fingers with inertias (panda.urdf
                                      has none, so it serves kinematics only)
  assets/robot/fetch/fetch.urdf       15 DoF, branched: continuous wheels, a prismatic torso
                                      lift, head, 7-DoF arm with continuous rolls, 2 fingers

Kept: the robot name; every link with its <inertial> (origin, mass, inertia); every joint
with its type, <origin>, <parent>, <child>, <axis>, <limit>, <dynamics> and <mimic>.
Dropped: <visual>, <collision>, <material>, <transmission>, <gazebo> and comments, none of
which the kinematic tree or the inertias depend on. Attribute values are copied as written,
so a URDF reader gives bit-identical tables on the fixture and on the original.

Usage: python tests/golden/make_robot_fixtures.py [REFERENCE_ROOT] [--check]
(REFERENCE_ROOT defaults to /root/reference; --check compares instead of writing.)
"""
import os
import sys
import xml.etree.ElementTree as ET

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = {
    "panda.urdf": os.path.join("assets", "robot", "panda", "panda.urdf"),
    "movo_simple.urdf": os.path.join("unittest", "assets", "movo_simple.urdf"),
    "sawyer.urdf": os.path.join("assets", "robot", "sawyer", "sawyer.urdf"),
    "fetch.urdf": os.path.join("assets", "robot", "fetch", "fetch.urdf"),
}
JOINT_CHILDREN = ("origin", "parent", "child", "axis", "limit", "dynamics", "mimic")


def _elem(tag, attrib, indent):
    attrs = "".join(f' {k}="{v}"' for k, v in attrib.items())
    return f"{indent}<{tag}{attrs}/>"


def strip(urdf_text, source_name):
    root = ET.fromstring(urdf_text)
    out = ['<?xml version="1.0"?>',
           f"<!-- derived from the reference project's {source_name} by make_robot_fixtures.py: "
           "links with their inertial data and joints only -->",
           f'<robot name="{root.get("name")}">']
    for child in root:
        if child.tag == "link":
            inertial = child.find("inertial")
            if inertial is None:
                out.append(f'  <link name="{child.get("name")}"/>')
                continue
            out.append(f'  <link name="{child.get("name")}">')
            out.append("    <inertial>")
            for tag in ("origin", "mass", "inertia"):
                e = inertial.find(tag)
                if e is not None:
                    out.append(_elem(tag, e.attrib, "      "))
            out.append("    </inertial>")
            out.append("  </link>")
        elif child.tag == "joint":
            out.append(f'  <joint name="{child.get("name")}" type="{child.get("type")}">')
            for tag in JOINT_CHILDREN:
                e = child.find(tag)
                if e is not None:
                    out.append(_elem(tag, e.attrib, "    "))
            out.append("  </joint>")
    out.append("</robot>")
    return "\n".join(out) + "\n"


def main(argv):
    check = "--check" in argv
    args = [a for a in argv if not a.startswith("--")]
    ref = args[0] if args else "/root/reference"
    bad = 0
    for name, rel in SOURCES.items():
        with open(os.path.join(ref, rel)) as f:
            text = strip(f.read(), rel)
        dst = os.path.join(HERE, name)
        if check:
            same = os.path.exists(dst) and open(dst).read() == text
            print(f"{name}: {'up to date' if same else 'DIFFERS'}")
            bad += not same
        else:
            with open(dst, "w") as f:
                f.write(text)
            print(f"wrote {dst}")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
