"""GPU parity of the link-Jacobian, Coriolis and CLIK kernels against the CPU oracle.

Tolerances (normwise relative per environment): Jacobians and Coriolis 1e-10; IK (a
100-iteration nonlinear iteration) 1e-8 on q and on the log6 error.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel, Pose, synthetic as syn

pytestmark = pytest.mark.gpu

ROBOTS = {
    "arm9": lambda: syn.arm_with_fingers(),
    "arm9_sapien": lambda: syn.arm_with_fingers(sapien_style=True),
    "quadruped18": lambda: syn.quadruped(),
    "humanoid": lambda: syn.humanoid(),
    "mixed_chain": lambda: syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                "continuous", "prismatic"]),
}


def T():
    import torch

    return torch


def pair(robot):
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    return pm, o


def rel(g, o):
    return np.abs(g - o).max() / max(np.abs(o).max(), 1e-300)


def quat_wxyz_from_R(R):
    t = np.trace(R)
    if t > 0:
        r = np.sqrt(t + 1)
        k = 0.5 / r
        return np.array([0.5 * r, (R[2, 1] - R[1, 2]) * k, (R[0, 2] - R[2, 0]) * k, (R[1, 0] - R[0, 1]) * k])
    i = int(np.argmax([R[0, 0], R[1, 1], R[2, 2]]))
    j, k_ = (i + 1) % 3, (i + 2) % 3
    r = np.sqrt(R[i, i] - R[j, j] - R[k_, k_] + 1)
    q = np.zeros(4)
    q[1 + i] = 0.5 * r
    k = 0.5 / r
    q[0] = (R[k_, j] - R[j, k_]) * k
    q[1 + j] = (R[j, i] + R[i, j]) * k
    q[1 + k_] = (R[k_, i] + R[i, k_]) * k
    return q


def R_from_quat_wxyz(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


@pytest.mark.parametrize("name", list(ROBOTS))
def test_link_jacobians_match_oracle(name):
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    n = 20
    q, _, _, _ = robot.sample(n, seed=31)
    qt = T().from_numpy(q).cuda()
    for li in range(len(robot.link_names)):
        Jw = pm.compute_link_jacobian_batched(qt, li, local=False).cpu().numpy()
        Jl = pm.compute_link_jacobian_batched(qt, li, local=True).cpu().numpy()
        Js = pm.compute_single_link_local_jacobian_batched(qt, li).cpu().numpy()
        for e in range(n):
            o.compute_full_jacobian(q[e])
            rw = o.get_link_jacobian(li, local=False)
            rl = o.get_link_jacobian(li, local=True)
            rs = o.compute_single_link_local_jacobian(q[e], li)
            assert rel(Jw[e], rw) <= 1e-10
            assert rel(Jl[e], rl) <= 1e-10
            assert rel(Js[e], rs) <= 1e-10


def test_drop_in_link_jacobian_calls():
    robot = syn.arm_with_fingers(sapien_style=True)
    pm, o = pair(robot)
    q, _, _, _ = robot.sample(2, seed=3)
    for e in range(2):
        pm.compute_full_jacobian(q[e])
        o.compute_full_jacobian(q[e])
        for li in range(len(robot.link_names)):
            for local in (False, True):
                assert rel(pm.get_link_jacobian(li, local), o.get_link_jacobian(li, local)) <= 1e-10
            assert rel(pm.compute_single_link_local_jacobian(q[e], li),
                       o.compute_single_link_local_jacobian(q[e], li)) <= 1e-10
    with pytest.raises(RuntimeError, match="link index out of bound"):
        pm.get_link_jacobian(99)


@pytest.mark.parametrize("name", list(ROBOTS))
def test_coriolis_matches_oracle(name):
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    n = 40
    q, qd, _, _ = robot.sample(n, seed=41)
    C = pm.compute_coriolis_matrix_batched(T().from_numpy(q).cuda(), T().from_numpy(qd).cuda()).cpu().numpy()
    for e in range(n):
        assert rel(C[e], o.compute_coriolis_matrix(q[e], qd[e])) <= 1e-10
    # single-instance drop-in
    assert rel(pm.compute_coriolis_matrix(q[0], qd[0]), o.compute_coriolis_matrix(q[0], qd[0])) <= 1e-10


def _ik_case(robot, n, seed, link=None):
    pm, o = pair(robot)
    q, _, _, _ = robot.sample(n, seed=seed)
    link = robot.ee_link if link is None else link
    targets7 = np.zeros((n, 7))
    targets44 = np.zeros((n, 4, 4))
    for e in range(n):
        Tm = o.link_poses(q[e])[link]
        qq = quat_wxyz_from_R(Tm[:3, :3])
        targets7[e, :3] = Tm[:3, 3]
        targets7[e, 3:] = qq
        targets44[e] = np.eye(4)
        targets44[e, :3, :3] = R_from_quat_wxyz(qq)
        targets44[e, :3, 3] = Tm[:3, 3]
    q0 = q + np.random.default_rng(seed).normal(scale=0.3, size=q.shape)
    if syn.FLOATING in robot.joint_kinds:  # keep free-flyer quaternions unit
        off = 0
        for kind in robot.joint_kinds:
            if kind == syn.FLOATING:
                q0[:, off + 3:off + 7] /= np.linalg.norm(q0[:, off + 3:off + 7], axis=1, keepdims=True)
                off += 7
            else:
                off += 1
    return pm, o, q0, targets7, targets44, link


@pytest.mark.parametrize("name", ["arm9", "arm9_sapien", "mixed_chain", "quadruped18"])
def test_ik_fixed_iterations_match_oracle(name):
    robot = ROBOTS[name]()
    n = 48
    pm, o, q0, t7, t44, link = _ik_case(robot, n, seed=51)
    kw = dict(eps=0.0, max_iterations=60, dt=0.3, damp=1e-3)
    qg, okg, errg = pm.compute_inverse_kinematics_batched(link, T().from_numpy(t7).cuda(), T().from_numpy(q0).cuda(),
                                                          None, **kw)
    qr, okr, errr = o.batch_ik(link, t44, q0, **kw)
    qg, errg = qg.cpu().numpy(), errg.cpu().numpy()
    assert not okg.cpu().numpy().any() and not okr.any()
    for e in range(n):
        assert rel(qg[e], qr[e]) <= 1e-8, e
        assert np.abs(errg[e] - errr[e]).max() <= 1e-8 * max(1e-3, np.abs(errr[e]).max()), e


def test_ik_converges_and_success_flags_agree():
    robot = syn.arm_with_fingers()
    n = 64
    pm, o, q0, t7, t44, link = _ik_case(robot, n, seed=61)
    kw = dict(eps=1e-6, max_iterations=500, dt=0.5, damp=1e-6)
    qg, okg, errg = pm.compute_inverse_kinematics_batched(link, T().from_numpy(t7).cuda(), T().from_numpy(q0).cuda(),
                                                          None, **kw)
    qr, okr, errr = o.batch_ik(link, t44, q0, **kw)
    okg = okg.cpu().numpy()
    assert okg.mean() > 0.8
    assert (okg == okr).mean() > 0.95
    errg = errg.cpu().numpy()
    assert np.all(np.linalg.norm(errg[okg], axis=1) < 1e-6)


def test_ik_mask_freezes_joints_and_drop_in_call():
    robot = syn.arm_with_fingers()
    pm, o, q0, t7, t44, link = _ik_case(robot, 4, seed=71)
    mask = [1, 1, 1, 0, 1, 1, 1, 1, 1]
    qg, _, _ = pm.compute_inverse_kinematics_batched(link, T().from_numpy(t7).cuda(), T().from_numpy(q0).cuda(),
                                                     mask, eps=0.0, max_iterations=20)
    assert np.array_equal(qg.cpu().numpy()[:, 3], q0[:, 3])
    # single-instance: float32 Pose target, reference defaults except iterations
    pose = Pose(t7[0, :3], t7[0, 3:])
    q, ok, err = pm.compute_inverse_kinematics(link, pose, initial_qpos=q0[0], max_iterations=50)
    T44 = np.eye(4)
    T44[:3, :3] = R_from_quat_wxyz(pose.q.astype(np.float64))
    T44[:3, 3] = pose.p.astype(np.float64)
    qr, okr, errr = o.compute_inverse_kinematics(link, T44, initial_qpos=q0[0], max_iterations=50)
    assert ok == okr
    assert rel(q, qr) <= 1e-8
    assert err.shape == (6,)
