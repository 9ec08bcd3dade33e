"""GPU parity on the reference's own robots (tests/golden/*.urdf, orders as SAPIEN's URDF
loader gives them): every kernel against the CPU oracle, plus the one reference test on
this path, unittest/test_physx/test_articulation.py:75-97 (movo_simple at a fixed q: link
poses after compute_forward_kinematics, and compute_inverse_dynamics(q, 0, 0)).

Tolerances (normwise relative per environment): FK / Jacobians / CRBA / Coriolis / RNEA
1e-10, ABA and fixed-iteration IK 1e-8. panda.urdf carries no inertias, so it is checked
on the kinematic kernels only.
"""
import numpy as np
import pytest

import reference_robots as rr
from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel
from sapien_gb300.articulation import create_pinocchio_model
from test_aux_gpu import R_from_quat_wxyz, quat_wxyz_from_R
from test_parity_gpu import oracle_pose7, quat_from_R, rel_per_env

pytestmark = pytest.mark.gpu

TOL = {"poses": 1e-10, "J": 1e-10, "M": 1e-10, "tau": 1e-10, "C": 1e-10, "qdd": 1e-8, "ik": 1e-8}


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


def cu(a):
    return T().from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", rr.NAMES)
def test_sweep_kernels_on_reference_robot(name):
    """FK (all link poses), full WORLD Jacobian and, for robots with inertias, CRBA, RNEA
    and ABA from the fused sweep and from the per-op entry points."""
    robot = rr.load(name)
    pm, o = pair(robot)
    n = 96
    q, qd, qdd, tau = robot.sample(n, seed=2024)
    dyn = name in rr.DYNAMICS
    r = o.batch_step(q, qd, qdd, tau, ops=31 if dyn else 3, nthreads=8)
    got = {"poses": pm.compute_forward_kinematics_batched(cu(q)).cpu().numpy(),
           "J": pm.compute_full_jacobian_batched(cu(q)).cpu().numpy()}
    want = {"poses": oracle_pose7(r["poses"]), "J": r["J"]}
    if dyn:
        fused = pm.step_batched(cu(q), cu(qd), cu(qdd), cu(tau))
        got.update(M=pm.compute_generalized_mass_matrix_batched(cu(q)).cpu().numpy(),
                   tau=pm.compute_inverse_dynamics_batched(cu(q), cu(qd), cu(qdd)).cpu().numpy(),
                   qdd=pm.compute_forward_dynamics_batched(cu(q), cu(qd), cu(tau)).cpu().numpy())
        want.update(M=r["M"], tau=r["tau"], qdd=r["qdd"])
        for k, f in (("poses", "link_poses"), ("J", "jacobian"), ("M", "mass_matrix"), ("tau", "qf"),
                     ("qdd", "qacc")):
            e = rel_per_env(fused[f].cpu().numpy(), want[k])
            assert e <= TOL[k], f"{name} fused {k}: {e:.3e}"
    for k in got:
        e = rel_per_env(got[k], want[k])
        assert e <= TOL[k], f"{name} {k}: {e:.3e}"


@pytest.mark.parametrize("name", rr.NAMES)
def test_link_jacobians_on_reference_robot(name):
    robot = rr.load(name)
    pm, o = pair(robot)
    n = 6
    q, _, _, _ = robot.sample(n, seed=7)
    qt = cu(q)
    for li in range(len(robot.link_names)):
        Jw = pm.compute_link_jacobian_batched(qt, li, local=False).cpu().numpy()
        Jl = pm.compute_link_jacobian_batched(qt, li, local=True).cpu().numpy()
        Js = pm.compute_single_link_local_jacobian_batched(qt, li).cpu().numpy()
        for e in range(n):
            o.compute_full_jacobian(q[e])
            for g, w in ((Jw[e], o.get_link_jacobian(li, local=False)), (Jl[e], o.get_link_jacobian(li, local=True)),
                         (Js[e], o.compute_single_link_local_jacobian(q[e], li))):
                assert np.abs(g - w).max() <= TOL["J"] * max(np.abs(w).max(), 1e-300), (name, li, e)


@pytest.mark.parametrize("name", rr.DYNAMICS)
def test_coriolis_on_reference_robot(name):
    robot = rr.load(name)
    pm, o = pair(robot)
    n = 24
    q, qd, _, _ = robot.sample(n, seed=8)
    C = pm.compute_coriolis_matrix_batched(cu(q), cu(qd)).cpu().numpy()
    R = np.stack([o.compute_coriolis_matrix(q[e], qd[e]) for e in range(n)])
    assert rel_per_env(C, R) <= TOL["C"]


@pytest.mark.parametrize("name", rr.NAMES)
def test_ik_on_reference_robot(name):
    """Damped-least-squares CLIK on the end-effector link for a fixed number of
    iterations from perturbed starts, against the oracle's CLIK loop."""
    robot = rr.load(name)
    pm, o = pair(robot)
    n = 32
    q, _, _, _ = robot.sample(n, seed=9)
    link = robot.ee_link
    t7, t44 = np.zeros((n, 7)), np.zeros((n, 4, 4))
    for e in range(n):
        Tm = o.link_poses(q[e])[link]
        qq = quat_wxyz_from_R(Tm[:3, :3])
        t7[e, :3], t7[e, 3:] = Tm[:3, 3], qq
        t44[e] = np.eye(4)
        t44[e, :3, :3] = R_from_quat_wxyz(qq)
        t44[e, :3, 3] = Tm[:3, 3]
    q0 = q + np.random.default_rng(10).normal(scale=0.2, size=q.shape)
    kw = dict(eps=0.0, max_iterations=40, dt=0.3, damp=1e-3)
    qg, _, errg = pm.compute_inverse_kinematics_batched(link, cu(t7), cu(q0), None, **kw)
    qr, _, errr = o.batch_ik(link, t44, q0, **kw)
    qg, errg = qg.cpu().numpy(), errg.cpu().numpy()
    for e in range(n):
        assert np.abs(qg[e] - qr[e]).max() <= TOL["ik"] * np.abs(qr[e]).max(), (name, e)
        assert np.abs(errg[e] - errr[e]).max() <= TOL["ik"] * max(1e-3, np.abs(errr[e]).max()), (name, e)


def test_movo_reference_case_single_instance():
    """test_articulation.py:75-97 through the drop-in calls: compute_forward_kinematics(q),
    get_link_pose(i) for every link (float32 Pose, as the reference returns), and
    compute_inverse_dynamics(q, 0, 0) (the gravity torque the reference compares with
    PhysX's passive force) against the oracle."""
    robot = rr.load("movo_simple")
    pm, o = pair(robot)
    q, qd, qdd = rr.movo_reference_inputs()
    pm.compute_forward_kinematics(q)
    o.compute_forward_kinematics(q)
    for li in range(len(robot.link_names)):
        pose = pm.get_link_pose(li)
        T4 = o.get_link_pose_matrix(li)
        assert pose.p.dtype == np.float32
        assert np.abs(pose.p.astype(np.float64) - T4[:3, 3]).max() <= 1e-6, li
        qr = quat_from_R(T4[:3, :3])
        assert min(np.abs(pose.q - qr).max(), np.abs(pose.q + qr).max()) <= 1e-6, li
    tau = pm.compute_inverse_dynamics(q, qd, qdd)
    ref = o.compute_inverse_dynamics(q, qd, qdd)
    assert np.abs(tau - ref).max() <= TOL["tau"] * np.abs(ref).max()
    # float64 poses of the same configuration through the batched entry point
    P = pm.compute_forward_kinematics_batched(cu(q[None])).cpu().numpy()
    assert rel_per_env(P, oracle_pose7(o.batch_step(q[None], ops=1)["poses"])) <= TOL["poses"]


@pytest.mark.parametrize("name", rr.DYNAMICS)
def test_create_pinocchio_model_path_on_reference_robot(name):
    """The articulation SAPIEN's loader builds from the robot, through the native
    create_pinocchio_model (python/py_package/wrapper/pinocchio_model.py:317-329), gives
    the URDF path's link poses, gravity torque and mass matrix."""
    robot = rr.load(name)
    art = rr.sapien_articulation(robot)
    pa = create_pinocchio_model(art)
    pm, _ = pair(robot)
    q, qd, _, _ = robot.sample(16, seed=11)
    z = np.zeros_like(qd)
    for f in ("compute_forward_kinematics_batched", "compute_generalized_mass_matrix_batched"):
        a, b = getattr(pa, f)(cu(q)).cpu().numpy(), getattr(pm, f)(cu(q)).cpu().numpy()
        assert rel_per_env(a, b) <= 1e-10, f
    a = pa.compute_inverse_dynamics_batched(cu(q), cu(z), cu(z)).cpu().numpy()
    b = pm.compute_inverse_dynamics_batched(cu(q), cu(z), cu(z)).cpu().numpy()
    assert rel_per_env(a, b) <= 1e-10
    if name == "movo_simple":
        q0, _, _ = rr.movo_reference_inputs()
        pa.compute_forward_kinematics(q0)
        pm.compute_forward_kinematics(q0)
        for li in range(len(robot.link_names)):
            assert np.abs(pa.get_link_pose(li).p - pm.get_link_pose(li).p).max() <= 1e-6
