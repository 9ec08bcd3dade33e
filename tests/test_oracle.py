"""Pins the CPU oracle (no GPU): closed forms, dynamics identities, finite differences.

The reference holds no golden vectors for this path (its only test,
unittest/test_physx/test_articulation.py:75-97, compares against PhysX at run time), so
the oracle is pinned here by analytic known answers and by identities every correct
rigid-body dynamics implementation satisfies.
"""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle, se3_exp6, se3_jlog6, se3_log6
from sapien_gb300 import synthetic as syn


def _model(robot):
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    return o


ROBOTS = {
    "chain7": lambda: syn.serial_chain(7),
    "arm9": lambda: syn.arm_with_fingers(),
    "arm9_sapien": lambda: syn.arm_with_fingers(sapien_style=True),
    "quadruped18": lambda: syn.quadruped(),
    "humanoid30": lambda: syn.humanoid(),
    "mixed_chain": lambda: syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                "continuous", "prismatic"]),
}


def pendulum_urdf(m, l, Iyy, axis="0 1 0", kind="revolute"):
    return f"""<robot name="p">
  <link name="base"/>
  <link name="bob"><inertial><origin xyz="0 0 {-l}" rpy="0 0 0"/><mass value="{m}"/>
    <inertia ixx="0.01" ixy="0" ixz="0" iyy="{Iyy}" iyz="0" izz="0.01"/></inertial></link>
  <joint name="j" type="{kind}"><origin xyz="0 0 0" rpy="0 0 0"/><axis xyz="{axis}"/>
    <parent link="base"/><child link="bob"/><limit lower="-3" upper="3" effort="0" velocity="0"/></joint>
</robot>"""


def two_link_urdf(m1, m2, l1, lc1, lc2, I1, I2):
    return f"""<robot name="two">
  <link name="base"/>
  <link name="l1"><inertial><origin xyz="{lc1} 0 0"/><mass value="{m1}"/>
    <inertia ixx="0.01" ixy="0" ixz="0" iyy="0.01" iyz="0" izz="{I1}"/></inertial></link>
  <link name="l2"><inertial><origin xyz="{lc2} 0 0"/><mass value="{m2}"/>
    <inertia ixx="0.01" ixy="0" ixz="0" iyy="0.01" iyz="0" izz="{I2}"/></inertial></link>
  <joint name="j1" type="revolute"><axis xyz="0 0 1"/><parent link="base"/><child link="l1"/></joint>
  <joint name="j2" type="revolute"><origin xyz="{l1} 0 0"/><axis xyz="0 0 1"/><parent link="l1"/><child link="l2"/></joint>
</robot>"""


@pytest.mark.parametrize("kind", ["revolute", "continuous"])
def test_pendulum_closed_form(kind):
    """Continuous joints are stored as (cos, sin) inside but take the angle at the API."""
    m, l, Iyy, g = 1.7, 0.6, 0.03, 9.81
    o = Oracle(pendulum_urdf(m, l, Iyy, kind=kind), (0, 0, -g))
    o.set_joint_order(["j"])
    o.set_link_order(["base", "bob"])
    rng = np.random.default_rng(0)
    for _ in range(10):
        th, thd, thdd = rng.uniform(-3, 3), rng.normal(), rng.normal()
        tau = o.compute_inverse_dynamics([th], [thd], [thdd])[0]
        expect = (Iyy + m * l * l) * thdd + m * g * l * math.sin(th)
        assert abs(tau - expect) < 1e-12 * max(1, abs(expect))
        M = o.compute_generalized_mass_matrix([th])
        assert abs(M[0, 0] - (Iyy + m * l * l)) < 1e-14
        a = o.compute_forward_dynamics([th], [thd], [tau])[0]
        assert abs(a - thdd) < 1e-12
        # link frame of the bob is the joint frame: rotation about y by th
        T = o.link_poses([th])[1]
        Ry = np.array([[math.cos(th), 0, math.sin(th)], [0, 1, 0], [-math.sin(th), 0, math.cos(th)]])
        assert np.abs(T[:3, :3] - Ry).max() < 1e-15


def test_two_link_closed_form():
    m1, m2, l1, lc1, lc2, I1, I2, g = 1.3, 0.9, 0.5, 0.22, 0.31, 0.021, 0.013, 9.81
    o = Oracle(two_link_urdf(m1, m2, l1, lc1, lc2, I1, I2), (0, -g, 0))
    o.set_joint_order(["j1", "j2"])
    o.set_link_order(["base", "l1", "l2"])
    rng = np.random.default_rng(1)
    for _ in range(10):
        q = rng.uniform(-3, 3, 2)
        qd = rng.normal(size=2)
        c2, s2 = math.cos(q[1]), math.sin(q[1])
        M11 = I1 + I2 + m1 * lc1 ** 2 + m2 * (l1 ** 2 + lc2 ** 2 + 2 * l1 * lc2 * c2)
        M12 = I2 + m2 * (lc2 ** 2 + l1 * lc2 * c2)
        M22 = I2 + m2 * lc2 ** 2
        M = np.array([[M11, M12], [M12, M22]])
        h = -m2 * l1 * lc2 * s2
        C = np.array([[h * qd[1], h * (qd[0] + qd[1])], [-h * qd[0], 0.0]])
        gv = np.array([(m1 * lc1 + m2 * l1) * g * math.cos(q[0]) + m2 * lc2 * g * math.cos(q[0] + q[1]),
                       m2 * lc2 * g * math.cos(q[0] + q[1])])
        assert np.abs(o.compute_generalized_mass_matrix(q) - M).max() < 1e-14
        assert np.abs(o.compute_coriolis_matrix(q, qd) - C).max() < 1e-13
        assert np.abs(o.compute_inverse_dynamics(q, [0, 0], [0, 0]) - gv).max() < 1e-13
        qdd = rng.normal(size=2)
        assert np.abs(o.compute_inverse_dynamics(q, qd, qdd) - (M @ qdd + C @ qd + gv)).max() < 1e-12
        # Jacobians of link l2 (frame at joint 2, at (l1 c1, l1 s1, 0), rotated by q1 + q2 about
        # z): WORLD = spatial velocity at the world origin, columns (p_i x z, z); LOCAL = the
        # link frame's own velocity in its axes
        c1, s1, c12, s12 = math.cos(q[0]), math.sin(q[0]), math.cos(q.sum()), math.sin(q.sum())
        Jw = np.zeros((6, 2))
        Jw[5, :] = 1
        Jw[0, 1], Jw[1, 1] = l1 * s1, -l1 * c1
        R12 = np.array([[c12, -s12, 0], [s12, c12, 0], [0, 0, 1]])
        Jl = np.zeros((6, 2))
        Jl[:3, 0] = R12.T @ np.array([-l1 * s1, l1 * c1, 0])
        Jl[5, :] = 1
        o.compute_full_jacobian(q)
        assert np.abs(o.get_link_jacobian(2) - Jw).max() < 1e-15
        assert np.abs(o.get_link_jacobian(2, local=True) - Jl).max() < 1e-15
        assert np.abs(o.compute_single_link_local_jacobian(q, 2) - Jl).max() < 1e-15


def cart_pole_urdf(mc, mp, l, Iyy):
    return f"""<robot name="cp">
  <link name="rail"/>
  <link name="cart"><inertial><mass value="{mc}"/>
    <inertia ixx="0.02" ixy="0" ixz="0" iyy="0.03" iyz="0" izz="0.04"/></inertial></link>
  <link name="pole"><inertial><origin xyz="0 0 {l}"/><mass value="{mp}"/>
    <inertia ixx="0.01" ixy="0" ixz="0" iyy="{Iyy}" iyz="0" izz="0.01"/></inertial></link>
  <joint name="slide" type="prismatic"><axis xyz="1 0 0"/><parent link="rail"/><child link="cart"/>
    <limit lower="-5" upper="5" effort="0" velocity="0"/></joint>
  <joint name="hinge" type="revolute"><axis xyz="0 1 0"/><parent link="cart"/><child link="pole"/>
    <limit lower="-3.2" upper="3.2" effort="0" velocity="0"/></joint>
</robot>"""


def test_cart_pole_closed_form():
    """Prismatic cart (x) carrying a pole hinged about y (angle th, centre of mass l up the
    pole): from the Lagrangian T = (mc + mp) xd^2 / 2 + mp l cos(th) xd thd + (mp l^2 + Iyy)
    thd^2 / 2, V = mp g l cos(th): M = [[mc + mp, mp l c], [mp l c, mp l^2 + Iyy]],
    C = [[0, -mp l s thd], [0, 0]], gravity torques (0, -mp g l s)."""
    mc, mp, l, Iyy, g = 1.9, 0.7, 0.45, 0.012, 9.81
    o = Oracle(cart_pole_urdf(mc, mp, l, Iyy), (0, 0, -g))
    o.set_joint_order(["slide", "hinge"])
    o.set_link_order(["rail", "cart", "pole"])
    rng = np.random.default_rng(2)
    for _ in range(10):
        q, qd, qdd = rng.uniform(-3, 3, 2), rng.normal(size=2), rng.normal(size=2)
        c, s_ = math.cos(q[1]), math.sin(q[1])
        M = np.array([[mc + mp, mp * l * c], [mp * l * c, mp * l * l + Iyy]])
        C = np.array([[0.0, -mp * l * s_ * qd[1]], [0.0, 0.0]])
        gv = np.array([0.0, -mp * g * l * s_])
        assert np.abs(o.compute_generalized_mass_matrix(q) - M).max() < 1e-14
        assert np.abs(o.compute_coriolis_matrix(q, qd) - C).max() < 1e-13
        tau = o.compute_inverse_dynamics(q, qd, qdd)
        assert np.abs(tau - (M @ qdd + C @ qd + gv)).max() < 1e-12
        assert np.abs(o.compute_forward_dynamics(q, qd, tau) - qdd).max() < 1e-12


def floating_body_urdf(m, c, rpy, I):
    return f"""<robot name="fb">
  <link name="world"/>
  <link name="body"><inertial><origin xyz="{c[0]} {c[1]} {c[2]}" rpy="{rpy[0]} {rpy[1]} {rpy[2]}"/>
    <mass value="{m}"/><inertia ixx="{I[0]}" ixy="{I[1]}" ixz="{I[2]}" iyy="{I[3]}" iyz="{I[4]}" izz="{I[5]}"/>
  </inertial></link>
  <joint name="ff" type="floating"><parent link="world"/><child link="body"/></joint>
</robot>"""


def test_floating_body_newton_euler():
    """One free-floating rigid body: RNEA against the Newton-Euler equations written with
    3-vectors in the body frame. q = (x y z qx qy qz qw) with R(q) body -> world; qd, qdd =
    body twist (v, w) and its derivative; the classical acceleration of the centre of mass c
    is a_v + w x v + a_w x c + w x (w x c); gravity enters as R^T g. tau = (F, c x F + Ic a_w
    + w x Ic w) with F = m (that acceleration - R^T g). Also M = the body's 6x6 inertia about
    its origin and ABA = RNEA^-1."""
    rng = np.random.default_rng(4)
    m, c, rpy = 2.3, np.array([0.11, -0.07, 0.19]), (0.3, -0.5, 1.1)
    Ip = np.array([0.03, 0.004, -0.002, 0.05, 0.006, 0.04])  # principal frame at rpy, SPD
    g = np.array([0.0, 0.0, -9.81])
    o = Oracle(floating_body_urdf(m, c, rpy, Ip), tuple(g))
    o.set_joint_order(["ff"])
    o.set_link_order(["world", "body"])
    # inertia about the centre of mass in the body frame: R_rpy I R_rpy^T
    cr, sr, cp, sp, cy, sy = (math.cos(rpy[0]), math.sin(rpy[0]), math.cos(rpy[1]), math.sin(rpy[1]),
                              math.cos(rpy[2]), math.sin(rpy[2]))
    Rrpy = np.array([[cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr],
                     [sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr],
                     [-sp, cp * sr, cp * cr]])
    Il = np.array([[Ip[0], Ip[1], Ip[2]], [Ip[1], Ip[3], Ip[4]], [Ip[2], Ip[4], Ip[5]]])
    Ic = Rrpy @ Il @ Rrpy.T
    cx = np.array([[0, -c[2], c[1]], [c[2], 0, -c[0]], [-c[1], c[0], 0]])
    M6 = np.zeros((6, 6))
    M6[:3, :3], M6[:3, 3:], M6[3:, :3], M6[3:, 3:] = m * np.eye(3), -m * cx, m * cx, Ic + m * cx.T @ cx
    for _ in range(10):
        quat = rng.normal(size=4)
        quat /= np.linalg.norm(quat)
        q = np.concatenate([rng.normal(size=3), quat])
        qd, qdd = rng.normal(size=6), rng.normal(size=6)
        x, y, z, w = quat
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        v, om, av, aw = qd[:3], qd[3:], qdd[:3], qdd[3:]
        acc_c = av + np.cross(om, v) + np.cross(aw, c) + np.cross(om, np.cross(om, c))
        F = m * (acc_c - R.T @ g)
        N = np.cross(c, F) + Ic @ aw + np.cross(om, Ic @ om)
        expect = np.concatenate([F, N])
        tau = o.compute_inverse_dynamics(q, qd, qdd)
        assert np.abs(tau - expect).max() <= 1e-12 * np.abs(expect).max()
        assert np.abs(o.compute_generalized_mass_matrix(q) - M6).max() <= 1e-14
        assert np.abs(o.compute_forward_dynamics(q, qd, tau) - qdd).max() <= 1e-11 * np.abs(qdd).max()


@pytest.mark.parametrize("name", list(ROBOTS))
def test_dynamics_identities(name):
    robot = ROBOTS[name]()
    o = _model(robot)
    q, qd, qdd, tau = robot.sample(6, seed=3)
    nv = robot.nv
    z = np.zeros(nv)
    for e in range(len(q)):
        M = o.compute_generalized_mass_matrix(q[e])
        assert np.array_equal(M, M.T)
        assert np.linalg.eigvalsh(M).min() > 0
        t = o.compute_inverse_dynamics(q[e], qd[e], qdd[e])
        h = o.compute_inverse_dynamics(q[e], qd[e], z)
        g = o.compute_inverse_dynamics(q[e], z, z)
        scale = max(1.0, np.abs(t).max())
        assert np.abs(M @ qdd[e] + h - t).max() < 1e-12 * scale
        a = o.compute_forward_dynamics(q[e], qd[e], tau[e])
        assert np.abs(o.compute_inverse_dynamics(q[e], qd[e], a) - tau[e]).max() < 1e-11 * max(1, np.abs(tau[e]).max())
        assert np.abs(a - np.linalg.solve(M, tau[e] - h)).max() < 1e-9 * max(1, np.abs(a).max())
        C = o.compute_coriolis_matrix(q[e], qd[e])
        assert np.abs(C @ qd[e] - (h - g)).max() < 1e-11 * max(1, np.abs(h - g).max())


@pytest.mark.parametrize("name", ["chain7", "arm9", "quadruped18", "humanoid30"])
def test_kinetic_energy_matches_body_sum(name):
    """1/2 qd^T M qd = sum over bodies of 1/2 v_b^T I_b v_b, with v_b the body's spatial
    velocity in its own frame from the single-link local Jacobian and I_b its spatial
    inertia from the URDF (an independent path through the oracle's builder)."""
    from oracle import urdf_model as um

    robot = ROBOTS[name]()
    o = _model(robot)
    om = um.build_model(robot.urdf)
    q, qd, _, _ = robot.sample(5, seed=12)
    # the link whose frame is its joint's frame, one per moving joint
    link_of = {}
    for li, lname in enumerate(robot.link_names):
        jid, (R, p) = om.body_frames[lname]
        if jid > 0 and np.allclose(R, np.eye(3)) and np.allclose(p, 0) and jid not in link_of:
            link_of[jid] = li
    assert sorted(link_of) == list(range(1, om.njoints))
    for e in range(len(q)):
        M = o.compute_generalized_mass_matrix(q[e])
        t_m = 0.5 * qd[e] @ M @ qd[e]
        t_b = 0.0
        for jid, li in link_of.items():
            v = o.compute_single_link_local_jacobian(q[e], li) @ qd[e]
            t_b += 0.5 * v @ om.inertia6[jid] @ v
        assert abs(t_m - t_b) <= 1e-12 * max(1.0, abs(t_m))


@pytest.mark.parametrize("name", ["arm9", "humanoid30", "mixed_chain"])
def test_coriolis_is_christoffel(name):
    """Mdot = C + C^T (finite differences along qd) and C(q, x) y = C(q, y) x."""
    robot = ROBOTS[name]()
    o = _model(robot)
    q, qd, _, _ = robot.sample(3, seed=5)
    eps = 1e-6
    for e in range(len(q)):
        C = o.compute_coriolis_matrix(q[e], qd[e])
        Mp = o.compute_generalized_mass_matrix(o.integrate(q[e], eps * qd[e]))
        Mm = o.compute_generalized_mass_matrix(o.integrate(q[e], -eps * qd[e]))
        Mdot = (Mp - Mm) / (2 * eps)
        assert np.abs(Mdot - (C + C.T)).max() < 1e-6 * max(1, np.abs(Mdot).max())
        if syn.FLOATING in robot.joint_kinds:
            continue  # a free flyer's velocity is a body twist: no coordinate symmetry
        x = np.random.default_rng(e).normal(size=robot.nv)
        Cx = o.compute_coriolis_matrix(q[e], x)
        assert np.abs(C @ x - Cx @ qd[e]).max() < 1e-10 * max(1, np.abs(C @ x).max())


@pytest.mark.parametrize("name", ["arm9", "quadruped18", "mixed_chain"])
def test_jacobian_matches_fk_differences(name):
    robot = ROBOTS[name]()
    o = _model(robot)
    q, qd, _, _ = robot.sample(3, seed=9)
    eps = 1e-6
    for e in range(len(q)):
        o.compute_full_jacobian(q[e])
        Tp = o.link_poses(o.integrate(q[e], eps * qd[e]))
        Tm = o.link_poses(o.integrate(q[e], -eps * qd[e]))
        T0 = o.link_poses(q[e])
        for li in range(o.nlinks):
            J = o.get_link_jacobian(li, local=False)
            v = J @ qd[e]  # spatial velocity at the world origin
            pdot = (Tp[li, :3, 3] - Tm[li, :3, 3]) / (2 * eps)
            Rdot = (Tp[li, :3, :3] - Tm[li, :3, :3]) / (2 * eps)
            W = Rdot @ T0[li, :3, :3].T
            w = np.array([W[2, 1], W[0, 2], W[1, 0]])
            assert np.abs(w - v[3:]).max() < 1e-7
            assert np.abs(pdot - (v[:3] + np.cross(v[3:], T0[li, :3, 3]))).max() < 1e-7
            # local Jacobian = actInv(link pose) applied to the world one
            Jl = o.get_link_jacobian(li, local=True)
            R, p = T0[li, :3, :3], T0[li, :3, 3]
            vl = np.concatenate([R.T @ (v[:3] - np.cross(p, v[3:])), R.T @ v[3:]])
            assert np.abs(Jl @ qd[e] - vl).max() < 1e-12 * max(1, np.abs(vl).max())
            Js = o.compute_single_link_local_jacobian(q[e], li)
            assert np.abs(Js - Jl).max() < 1e-12 * max(1, np.abs(Jl).max())


@pytest.mark.parametrize("name", ["arm9", "humanoid30"])
def test_long_double_agrees(name):
    robot = ROBOTS[name]()
    o = _model(robot)
    q, qd, qdd, tau = robot.sample(4, seed=13)
    d = [o.compute_inverse_dynamics(q[e], qd[e], qdd[e]) for e in range(4)]
    a = [o.compute_forward_dynamics(q[e], qd[e], tau[e]) for e in range(4)]
    o.set_long_double(True)
    for e in range(4):
        dl = o.compute_inverse_dynamics(q[e], qd[e], qdd[e])
        al = o.compute_forward_dynamics(q[e], qd[e], tau[e])
        assert np.abs(d[e] - dl).max() < 1e-12 * np.abs(dl).max()
        assert np.abs(a[e] - al).max() < 1e-10 * np.abs(al).max()


def test_sapien_style_export_matches_plain():
    """Fixed-joint merging and rotated joint frames leave the dynamics unchanged."""
    plain, sap = syn.arm_with_fingers(), syn.arm_with_fingers(sapien_style=True)
    o1, o2 = _model(plain), _model(sap)
    q, qd, qdd, tau = plain.sample(5, seed=21)
    r1 = o1.batch_step(q, qd, qdd, tau)
    r2 = o2.batch_step(q, qd, qdd, tau)
    for k in r1:
        assert np.abs(r1[k] - r2[k]).max() < 1e-11 * max(1, np.abs(r1[k]).max()), k


def test_se3_log_exp_and_jlog6():
    rng = np.random.default_rng(2)
    for scale in (1e-9, 1e-4, 0.3, 1.0, 3.0):
        nu = rng.normal(size=6)
        nu[3:] *= scale / np.linalg.norm(nu[3:])
        T = se3_exp6(nu)
        assert np.abs(se3_log6(T) - nu).max() < 1e-12
        J = se3_jlog6(T)
        h = 1e-6
        Jfd = np.zeros((6, 6))
        for k in range(6):
            d = np.zeros(6)
            d[k] = h
            Jfd[:, k] = (se3_log6(T @ se3_exp6(d)) - se3_log6(T @ se3_exp6(-d))) / (2 * h)
        assert np.abs(J - Jfd).max() < 1e-7


def test_ik_reaches_fk_targets():
    robot = syn.serial_chain(7)
    o = _model(robot)
    q, _, _, _ = robot.sample(8, seed=4)
    ee = robot.ee_link
    q0 = q + np.random.default_rng(0).normal(scale=0.2, size=q.shape)
    ok_count = 0
    for e in range(len(q)):
        T = o.link_poses(q[e])[ee]
        qs, ok, err = o.compute_inverse_kinematics(ee, T, initial_qpos=q0[e], eps=1e-10, max_iterations=200, damp=1e-8,
                                                   dt=1.0)
        if ok:
            ok_count += 1
            assert np.linalg.norm(err) < 1e-10
            Ts = o.link_poses(qs)[ee]
            assert np.abs(Ts - T).max() < 1e-9
    assert ok_count >= 6
