"""The host instantiation of the sweeps (sgdyn_host_* entry points, which answer the
reference's one-configuration calls) against the CPU oracle, on the CPU.

Same tolerances as the GPU parity tests (normwise relative per environment): FK /
Jacobians / CRBA / Coriolis / RNEA 1e-10, ABA and fixed-iteration IK 1e-8.
"""
import ctypes

import numpy as np
import pytest

import reference_robots as rr
from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel, Pose, synthetic as syn
from sapien_gb300 import _native as N

ROBOTS = {
    "chain7": lambda: syn.serial_chain(7),
    "arm9": lambda: syn.arm_with_fingers(),
    "arm9_sapien": lambda: syn.arm_with_fingers(sapien_style=True),
    "quadruped18": lambda: syn.quadruped(),
    "humanoid": lambda: syn.humanoid(),
    "mixed_chain": lambda: syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                "continuous", "prismatic"]),
    "chain40": lambda: syn.serial_chain(40, seed=23),
    "movo_simple": lambda: rr.load("movo_simple"),
    "sawyer": lambda: rr.load("sawyer"),
    "fetch": lambda: rr.load("fetch"),
}


def pair(robot):
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    return pm, o


def rel(g, r):
    return np.abs(g - r).max() / max(np.abs(r).max(), 1e-300)


def quat_from_R(R):
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


@pytest.mark.parametrize("name", list(ROBOTS))
def test_host_batch_step_matches_oracle(name):
    """sgdyn_host_step over a batch on 4 threads: FK poses, WORLD Jacobian, CRBA, RNEA, ABA."""
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    n, nv, nl = 48, robot.nv, len(robot.link_names)
    q, qd, qdd, tau = robot.sample(n, seed=77)
    out = {"poses": np.empty((n, nl, 7)), "J": np.empty((n, 6, nv)), "M": np.empty((n, nv, nv)),
           "tau": np.empty((n, nv)), "qdd": np.empty((n, nv))}
    a = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    N.check(N.load().sgdyn_host_step(pm._h, n, N.OP_ALL, a(q), a(qd), a(qdd), a(tau), a(out["poses"]), a(out["J"]),
                                     a(out["M"]), a(out["tau"]), a(out["qdd"]), N.ENV_MAJOR, 4))
    r = o.batch_step(q, qd, qdd, tau, nthreads=4)
    for e in range(n):
        for li in range(nl):
            assert np.abs(out["poses"][e, li, :3] - r["poses"][e, li, 9:]).max() <= 1e-10 * max(
                1.0, np.abs(r["poses"][e, :, 9:]).max())
            qr = quat_from_R(r["poses"][e, li, :9].reshape(3, 3))
            assert min(np.abs(out["poses"][e, li, 3:] - qr).max(), np.abs(out["poses"][e, li, 3:] + qr).max()) <= 1e-10
        assert rel(out["J"][e], r["J"][e]) <= 1e-10
        assert rel(out["M"][e], r["M"][e]) <= 1e-10
        assert rel(out["tau"][e], r["tau"][e]) <= 1e-10
        assert rel(out["qdd"][e], r["qdd"][e]) <= 1e-8


@pytest.mark.parametrize("name", ["arm9", "quadruped18", "humanoid", "chain40", "fetch"])
def test_host_forward_dynamics_routes_match_oracle(name):
    """Forward dynamics by the articulated-body passes (sgdyn_fd_method 1) and from the mass
    matrix (method 2: L^T D L with the tree's sparsity, the loop form of the steps the
    run-time compiler emits per model; inverse dynamics in the same sweep as b + M qdd), for
    every op set holding ABA, against the oracle and each other."""
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    n, nv, nl = 24, robot.nv, len(robot.link_names)
    q, qd, qdd, tau = robot.sample(n, seed=5)
    r = o.batch_step(q, qd, qdd, tau, nthreads=4)
    L = N.load()
    a = lambda x: x.ctypes.data_as(ctypes.c_void_p) if x is not None else None  # noqa: E731
    old = ctypes.c_int()
    assert L.sgdyn_fd_method(-1, ctypes.byref(old)) == N.OK
    outs = {}
    try:
        for mode in (1, 2):
            assert L.sgdyn_fd_method(mode, None) == N.OK
            for ops in (16, 24, 28, 31):
                o_ = {"M": np.full((n, nv, nv), np.nan) if ops & 4 else None,
                      "tau": np.full((n, nv), np.nan) if ops & 8 else None, "qdd": np.full((n, nv), np.nan)}
                poses = np.empty((n, nl, 7)) if ops & 1 else None
                J = np.empty((n, 6, nv)) if ops & 2 else None
                N.check(L.sgdyn_host_step(pm._h, n, ops, a(q), a(qd), a(qdd), a(tau), a(poses), a(J), a(o_["M"]),
                                          a(o_["tau"]), a(o_["qdd"]), N.ENV_MAJOR, 4))
                outs[(mode, ops)] = {k: v for k, v in o_.items() if v is not None}
    finally:
        L.sgdyn_fd_method(old.value, None)
    want = {"M": r["M"], "tau": r["tau"], "qdd": r["qdd"]}
    for (mode, ops), g in outs.items():
        for k, v in g.items():
            tol = 1e-8 if k == "qdd" else 1e-10
            for e in range(n):
                assert rel(v[e], want[k][e]) <= tol, (mode, ops, k, e)
                assert rel(v[e], outs[(3 - mode, ops)][k][e]) <= (1e-10 if k == "qdd" else 1e-12), (mode, ops, k)


def test_chain7_single_instance_1000_samples_on_host():
    """The CPU-runnable reference configuration (seeded 7-DoF revolute chain, 1000 samples)
    through the single-instance drop-in methods, answered on the host."""
    robot = syn.serial_chain(7)
    pm, o = pair(robot)
    assert pm.single_instance == "host"
    n = 1000
    q, qd, qdd, tau = robot.sample(n, seed=0)
    nl = len(robot.link_names)
    worst = dict.fromkeys(("poses", "J", "M", "tau", "qdd"), 0.0)

    def upd(k, g, r):
        worst[k] = max(worst[k], rel(g, r))

    for e in range(n):
        pm.compute_forward_kinematics(q[e])
        o.compute_forward_kinematics(q[e])
        for li in range(nl):
            upd("poses", pm.get_link_pose(li).p.astype(np.float64), o.get_link_pose_matrix(li)[:3, 3])
        pm.compute_full_jacobian(q[e])
        o.compute_full_jacobian(q[e])
        for li in range(nl):
            upd("J", pm.get_link_jacobian(li), o.get_link_jacobian(li))
        upd("M", pm.compute_generalized_mass_matrix(q[e]), o.compute_generalized_mass_matrix(q[e]))
        upd("tau", pm.compute_inverse_dynamics(q[e], qd[e], qdd[e]), o.compute_inverse_dynamics(q[e], qd[e], qdd[e]))
        upd("qdd", pm.compute_forward_dynamics(q[e], qd[e], tau[e]), o.compute_forward_dynamics(q[e], qd[e], tau[e]))
    assert worst["poses"] <= 2e-7, worst  # float32 positions
    assert worst["J"] <= 1e-10 and worst["M"] <= 1e-10 and worst["tau"] <= 1e-10, worst
    assert worst["qdd"] <= 1e-8, worst


@pytest.mark.parametrize("name", ["arm9_sapien", "humanoid", "movo_simple", "fetch"])
def test_host_link_jacobians_and_coriolis_match_oracle(name):
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    q, qd, _, _ = robot.sample(3, seed=5)
    for e in range(3):
        pm.compute_full_jacobian(q[e])
        o.compute_full_jacobian(q[e])
        for li in range(len(robot.link_names)):
            for local in (False, True):
                assert rel(pm.get_link_jacobian(li, local), o.get_link_jacobian(li, local)) <= 1e-10
            assert rel(pm.compute_single_link_local_jacobian(q[e], li),
                       o.compute_single_link_local_jacobian(q[e], li)) <= 1e-10
        assert rel(pm.compute_coriolis_matrix(q[e], qd[e]), o.compute_coriolis_matrix(q[e], qd[e])) <= 1e-10


@pytest.mark.parametrize("name", ["arm9", "mixed_chain", "quadruped18", "movo_simple"])
def test_host_ik_matches_oracle(name):
    """Single-instance CLIK with the reference's defaults except the iteration count, from a
    perturbed start, against the oracle's CLIK loop: same iterate, success flag and error."""
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    q, _, _, _ = robot.sample(4, seed=9)
    rng = np.random.default_rng(10)
    link = robot.ee_link
    for e in range(4):
        Tm = o.link_poses(q[e])[link]
        pose = Pose(Tm[:3, 3], quat_from_R(Tm[:3, :3]))
        T44 = pose.to_transformation_matrix()
        q0 = q[e] + rng.normal(scale=0.2, size=q[e].shape)
        if syn.FLOATING in robot.joint_kinds:
            q0[3:7] /= np.linalg.norm(q0[3:7])
        for kw in (dict(max_iterations=60, eps=0.0, dt=0.3, damp=1e-3), dict(max_iterations=200)):
            qg, okg, errg = pm.compute_inverse_kinematics(link, pose, initial_qpos=q0, **kw)
            qr, okr, errr = o.compute_inverse_kinematics(link, T44, initial_qpos=q0, **kw)
            assert okg == okr
            assert rel(qg, qr) <= 1e-8, (name, e, kw)
            assert np.abs(errg - errr).max() <= 1e-8 * max(1e-3, np.abs(errr).max())


def test_host_entry_points_validate_arguments():
    r = syn.arm_with_fingers()
    pm, _ = pair(r)
    L = N.load()
    q = np.zeros(r.nq_ext)
    a = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    assert L.sgdyn_host_step(pm._h, 1, N.OP_INVERSE_DYNAMICS, a(q), None, None, None, None, None, None, None, None,
                             N.ENV_MAJOR, 1) == N.ERR_NULL
    assert L.sgdyn_host_step(pm._h, 1, 64, a(q), None, None, None, None, None, None, None, None, N.ENV_MAJOR,
                             1) == N.ERR_RUNTIME
    J = np.empty(6 * r.nv)
    assert L.sgdyn_host_compute_link_jacobian(pm._h, 1, 99, 0, a(q), a(J), N.ENV_MAJOR, 1) == N.ERR_RUNTIME
    assert "link index out of bound" in N.last_error()
    with pytest.raises(ValueError):
        pm.single_instance = "gpu"
