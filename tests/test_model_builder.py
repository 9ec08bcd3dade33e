"""Host-side checks that need no GPU: the product's C++ URDF model builder against the
oracle's independent Python builder, the C-ABI exports, and the reference's error
behaviour for orders and names."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import urdf_model as um
from sapien_gb300 import PinocchioModel, synthetic as syn
from sapien_gb300 import _native as N

import reference_robots as rr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DJOINT = np.dtype([("R", "<f8", 9), ("p", "<f8", 3), ("axis", "<f8", 3), ("m", "<f8"), ("h", "<f8", 3),
                   ("I", "<f8", 6), ("parent", "<i4"), ("kind", "<i4"), ("axis_kind", "<i4"), ("flags", "<i4"),
                   ("qcol", "<i4"), ("vcol", "<i4"), ("nv", "<i4"), ("depth", "<i4"), ("ivx", "<i4"),
                   ("subtree_end", "<i4"), ("pad", "<i4", 4)])
DLINK = np.dtype([("R", "<f8", 9), ("p", "<f8", 3), ("joint", "<i4"), ("flags", "<i4"), ("pad", "<i4", 2)])
DFRAME = np.dtype([("C", "<f8", 9), ("pad", "<f8")])
assert DJOINT.itemsize == 256 and DLINK.itemsize == 112 and DFRAME.itemsize == 80


def parse_table(raw):
    hdr = np.frombuffer(raw, dtype="<i4", count=8)
    nj, nv, nqe, nl = (int(x) for x in hdr[:4])
    grav = np.frombuffer(raw, dtype="<f8", count=3, offset=32)
    joints = np.frombuffer(raw, dtype=DJOINT, count=nj, offset=64)
    links = np.frombuffer(raw, dtype=DLINK, count=nl, offset=64 + 256 * nj)
    frames = np.frombuffer(raw, dtype=DFRAME, count=nj, offset=64 + 256 * nj + 112 * nl)
    assert len(raw) == 64 + 256 * nj + 112 * nl + 80 * nj
    return dict(nj=nj, nv=nv, nq_ext=nqe, nlinks=nl, gravity=grav, joints=joints, links=links, frames=frames)


def model_frame_quantities(t):
    """Undo the table's canonical joint frames (F' = F C, axis +z): per joint the placement
    (R, p), axis, first moment and rotational inertia in the model's joint frames, and per
    link its (R, p) in its joint's model frame."""
    C = [f["C"].reshape(3, 3) for f in t["frames"]]
    out = []
    for j in range(t["nj"]):
        J = t["joints"][j]
        Cj, Cp = C[j], C[J["parent"]] if j > 0 else np.eye(3)
        I = J["I"]
        Im = np.array([[I[0], I[1], I[2]], [I[1], I[3], I[4]], [I[2], I[4], I[5]]])
        out.append(dict(R=Cp @ J["R"].reshape(3, 3) @ Cj.T, p=Cp @ J["p"], axis=Cj @ J["axis"], h=Cj @ J["h"],
                        I=Cj @ Im @ Cj.T))
    links = [dict(R=C[L["joint"]] @ L["R"].reshape(3, 3), p=C[L["joint"]] @ L["p"]) for L in t["links"]]
    return out, links


def spatial6(m, h, I):
    hx = np.array([[0, -h[2], h[1]], [h[2], 0, -h[0]], [-h[1], h[0], 0]])
    Iw = np.array([[I[0], I[1], I[2]], [I[1], I[3], I[4]], [I[2], I[4], I[5]]])
    S = np.zeros((6, 6))
    S[:3, :3] = m * np.eye(3)
    S[:3, 3:] = -hx
    S[3:, :3] = hx
    S[3:, 3:] = Iw
    return S


ROBOTS = {
    "chain7": lambda: syn.serial_chain(7),
    "arm9": lambda: syn.arm_with_fingers(),
    "arm9_sapien": lambda: syn.arm_with_fingers(sapien_style=True),
    "quadruped18": lambda: syn.quadruped(),
    "humanoid": lambda: syn.humanoid(),
    "humanoid_sapien": lambda: syn.humanoid(sapien_style=True),
    "mixed_chain": lambda: syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                "continuous", "prismatic"]),
}


def compare_with_oracle_builder(urdf, joint_order, link_order):
    pm = PinocchioModel(urdf, [0, 0, -9.81])
    pm.set_joint_order(joint_order)
    pm.set_link_order(link_order)
    t = parse_table(pm.table_bytes())
    om = um.build_model(urdf, (0, 0, -9.81))
    assert t["nj"] == om.njoints
    assert t["nv"] == om.nv
    assert pm.joint_names == om.joint_names[1:]
    mj, ml = model_frame_quantities(t)
    for j in range(1, om.njoints):
        J, G = t["joints"][j], mj[j]
        assert J["parent"] == om.parent[j]
        assert J["kind"] == om.jtype[j]
        C = t["frames"][j]["C"].reshape(3, 3)
        assert np.abs(C @ C.T - np.eye(3)).max() < 1e-15 and abs(np.linalg.det(C) - 1) < 1e-15
        R, p = om.placement[j]
        assert np.abs(G["R"] - R).max() < 1e-15
        assert np.abs(G["p"] - p).max() < 1e-15
        if om.jtype[j] != um.JT_FREEFLYER:
            if J["axis_kind"] == 2:  # canonical frame: axis +z
                assert np.array_equal(J["axis"], [0.0, 0.0, 1.0])
            else:  # own frame kept
                assert np.array_equal(C, np.eye(3))
            assert np.abs(G["axis"] - om.axis[j]).max() < 1e-15
        else:
            assert np.array_equal(C, np.eye(3))
        Ig = G["I"]
        S = spatial6(J["m"], G["h"], [Ig[0, 0], Ig[0, 1], Ig[0, 2], Ig[1, 1], Ig[1, 2], Ig[2, 2]])
        assert np.abs(S - om.inertia6[j]).max() < 1e-13 * max(1, np.abs(S).max())
        # subtree = the contiguous depth-first range [j, subtree_end)
        def is_desc(k):
            while k > 0 and k != j:
                k = om.parent[k]
            return k == j
        assert all(is_desc(k) for k in range(j, J["subtree_end"]))
        assert not any(is_desc(k) for k in range(J["subtree_end"], om.njoints))
    # external columns follow the joint order
    qc, vc = 0, 0
    for name in joint_order:
        j = om.joint_names.index(name)
        J = t["joints"][j]
        assert J["qcol"] == qc and J["vcol"] == vc
        qc += 7 if om.jtype[j] == um.JT_FREEFLYER else 1
        vc += 6 if om.jtype[j] == um.JT_FREEFLYER else 1
    assert t["nq_ext"] == qc
    # link frames
    for li, name in enumerate(link_order):
        jid, (R, p) = om.body_frames[name]
        L = t["links"][li]
        assert L["joint"] == jid
        assert np.abs(ml[li]["R"] - R).max() < 1e-15
        assert np.abs(ml[li]["p"] - p).max() < 1e-15


@pytest.mark.parametrize("name", list(ROBOTS))
def test_builder_matches_oracle_builder(name):
    r = ROBOTS[name]()
    compare_with_oracle_builder(r.urdf, r.joint_names, r.link_names)


@pytest.mark.parametrize("name", rr.NAMES)
def test_builder_on_reference_robots(name):
    """The reference's panda (7R + 2P, a <mimic> finger) and movo_simple (continuous joints,
    16 fixed joints merged into bodies) fixtures: the product's tables equal the oracle
    builder's, in SAPIEN's loader order and in a reversed joint order."""
    r = rr.load(name)
    compare_with_oracle_builder(r.urdf, r.joint_names, r.link_names)
    compare_with_oracle_builder(r.urdf, r.joint_names[::-1], r.link_names[::-1])
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    pm.set_joint_order(r.joint_names)
    pm.set_link_order(r.link_names)
    assert pm.nv == r.nv and pm.nq_ext == r.nq_ext


def test_reference_robot_orders_follow_sapien_loader():
    """Depth-first pre-order, children in file order (urdf_loader.py:469-588)."""
    movo = rr.load("movo_simple")
    assert movo.nv == len(rr.MOVO_REFERENCE_Q) == 13
    assert movo.link_names[:4] == ["base_link", "base_chassis_link", "linear_actuator_fixed_link",
                                   "linear_actuator_link"]
    assert movo.joint_names[0] == "linear_joint"
    assert [k for k in movo.joint_kinds].count(syn.CONTINUOUS) == 7
    panda = rr.load("panda")
    assert panda.joint_names == [f"panda_joint{i}" for i in range(1, 8)] + ["panda_finger_joint1",
                                                                           "panda_finger_joint2"]
    assert len(panda.link_names) == 12


def test_library_exports_every_declared_symbol():
    header = open(os.path.join(ROOT, "include", "sgdyn.h")).read()
    declared = set(re.findall(r"^\s*(?:int|void|const char\*)\s+(sgdyn_\w+)\s*\(", header, re.M))
    assert declared == set(N.EXPORTED)
    L = N.load()
    for s in declared:
        assert hasattr(L, s), s


def test_reference_error_behaviour():
    r = syn.arm_with_fingers()
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    with pytest.raises(RuntimeError, match="posS2P failed"):
        pm.compute_inverse_dynamics(np.zeros(9), np.zeros(9), np.zeros(9))
    with pytest.raises(ValueError):
        pm.set_joint_order(r.joint_names[:-1] + ["no_such_joint"])
    with pytest.raises(RuntimeError):
        pm.set_joint_order(r.joint_names[:-1])  # missing DoF
    with pytest.raises(ValueError):
        pm.set_link_order(["no_such_link"])
    pm.set_joint_order(r.joint_names)
    pm.set_link_order(r.link_names)
    with pytest.raises(RuntimeError, match="link index out of bound"):
        pm.get_link_pose(len(r.link_names))
    with pytest.raises(RuntimeError, match="posS2P failed"):
        pm.compute_forward_kinematics(np.zeros(8))


def test_bad_urdf_is_rejected():
    with pytest.raises(RuntimeError):
        PinocchioModel("<robot><link name='a'/>", [0, 0, -9.81])
    planar = """<robot name="x"><link name="a"/><link name="b"/>
      <joint name="j" type="planar"><parent link="a"/><child link="b"/></joint></robot>"""
    with pytest.raises(RuntimeError, match="unsupported joint type"):
        PinocchioModel(planar, [0, 0, -9.81])
    two_roots = """<robot name="x"><link name="a"/><link name="b"/></robot>"""
    with pytest.raises(RuntimeError, match="root"):
        PinocchioModel(two_roots, [0, 0, -9.81])


def test_xml_reader_tolerates_comments_and_entities():
    urdf = """<?xml version="1.0"?>
<!-- comment with <joint name="fake"> inside -->
<robot name="a&amp;b">
  <link name="base"><!-- c --></link>
  <link name="l1"><inertial><mass value="1.5"/><inertia ixx="1" iyy="1" izz="1"/></inertial></link>
  <joint name="j1" type="continuous"><parent link="base"/><child link="l1"/><axis xyz="0 0 1"/>
    <![CDATA[ ignored <text> ]]>
  </joint>
  <transmission name="t"><joint name="j1"/></transmission>
</robot>"""
    pm = PinocchioModel(urdf, [0, 0, -9.81])
    assert pm.joint_names == ["j1"]
    assert pm.nq_ext == 1 and pm.nv == 1


def test_lanes_and_run_time_compilation_settings_are_validated():
    r = syn.arm_with_fingers()
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    for bad in (3, 16, -1):
        with pytest.raises(RuntimeError, match="lanes"):
            pm.set_lanes(bad)
    for ok in (0, 1, 2, 4, 8):
        pm.set_lanes(ok)
    L = N.load()
    old = ctypes.c_int()
    assert L.sgdyn_jit_max_joints(-1, ctypes.byref(old)) == N.OK and old.value > 0
    assert L.sgdyn_jit_max_joints(32, None) == N.OK
    cur = ctypes.c_int()
    assert L.sgdyn_jit_max_joints(-1, ctypes.byref(cur)) == N.OK and cur.value == 32
    assert L.sgdyn_jit_max_joints(old.value, None) == N.OK
    src = ctypes.c_char_p()
    pm.set_lanes(1)
    assert L.sgdyn_jit_source(pm._h, -7, ctypes.byref(src)) != N.OK  # the model runs with one lane
    assert L.sgdyn_jit_source(pm._h, -8, ctypes.byref(src)) != N.OK  # no such kernel kind
    assert L.sgdyn_rollout_lanes(2, None) != N.OK and "rollout lanes" in N.last_error()


@pytest.mark.parametrize("name", ["arm9", "arm9_sapien", "mixed_chain"])
def test_random_configuration_within_limits_and_reproducible(name):
    """getRandomConfiguration: each revolute / prismatic coordinate uniform within its URDF
    limits, each continuous angle uniform in [-pi, pi), reproducible for a seed."""
    r = ROBOTS[name]()
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    pm.set_joint_order(r.joint_names)
    n = 4000
    q = pm.get_random_configuration_batched(n, seed=7)
    assert q.shape == (n, r.nq_ext) and q.dtype == np.float64
    assert np.array_equal(q, pm.get_random_configuration_batched(n, seed=7))
    assert not np.array_equal(q, pm.get_random_configuration_batched(n, seed=8))
    for c, (kind, (lo, hi)) in enumerate(zip(r.joint_kinds, r.joint_limits)):
        if kind == syn.CONTINUOUS:
            lo, hi = -np.pi, np.pi
        assert lo <= q[:, c].min() and q[:, c].max() < hi, (c, kind)
        assert abs(q[:, c].mean() - 0.5 * (lo + hi)) < 5 * (hi - lo) / np.sqrt(12 * n), (c, kind)
    one = pm.get_random_configuration(seed=3)
    assert one.shape == (r.nq_ext,)
    assert np.array_equal(one, pm.get_random_configuration_batched(1, seed=3)[0])


def test_random_configuration_refuses_free_flyer():
    r = syn.quadruped()
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    pm.set_joint_order(r.joint_names)
    with pytest.raises(RuntimeError, match="free-flyer"):
        pm.get_random_configuration()


def test_reference_module_name_is_kept():
    from sapien_gb300 import pysapien_pinocchio

    assert pysapien_pinocchio.PinocchioModel is PinocchioModel


def test_forward_dynamics_route_choice():
    """sgdyn_fd_by_mass_matrix reports the route the specialised sweep (and the host path)
    takes: from the mass matrix where it costs fewer FP64 operations than the
    articulated-body passes. Small trees take it for every op set holding ABA, the 35-DoF
    humanoid only when CRBA is computed anyway, the 40-joint chain (sum of depth^2 ~ nv^3 / 6)
    never; op sets without ABA never; sgdyn_fd_method forces either route."""
    robots = {"arm9": syn.arm_with_fingers(), "quadruped": syn.quadruped(), "humanoid": syn.humanoid(),
              "chain40": syn.serial_chain(40, seed=23)}
    L = N.load()
    old = ctypes.c_int()
    assert L.sgdyn_fd_method(-1, ctypes.byref(old)) == N.OK and old.value == 0
    for bad in (3, -2):
        assert L.sgdyn_fd_method(bad, None) != N.OK
    want = {"arm9": (1, 1, 1, 1), "quadruped": (1, 1, 1, 1), "humanoid": (0, 0, 1, 1), "chain40": (0, 0, 0, 0)}
    for name, r in robots.items():
        pm = PinocchioModel(r.urdf, [0, 0, -9.81])
        pm.set_joint_order(r.joint_names)
        got = []
        for ops in (16, 24, 28, 31):
            y = ctypes.c_int()
            assert L.sgdyn_fd_by_mass_matrix(pm._h, ops, ctypes.byref(y)) == N.OK
            got.append(y.value)
        assert tuple(got) == want[name], name
        y = ctypes.c_int()
        assert L.sgdyn_fd_by_mass_matrix(pm._h, 8 | 4 | 1 | 2, ctypes.byref(y)) == N.OK and y.value == 0
        try:
            for mode, forced in ((1, 0), (2, 1)):
                assert L.sgdyn_fd_method(mode, None) == N.OK
                assert L.sgdyn_fd_by_mass_matrix(pm._h, 16, ctypes.byref(y)) == N.OK and y.value == forced
        finally:
            L.sgdyn_fd_method(old.value, None)
