"""GPU parity: the CUDA kernels (through the C ABI) against the CPU oracle.

Tolerances (normwise relative, per environment: max|gpu - oracle| / max|oracle|):
FK / Jacobian / CRBA / RNEA 1e-10, ABA 1e-8.
"""
import ctypes

import numpy as np
import pytest

from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel, synthetic as syn
from sapien_gb300 import _native as N

pytestmark = pytest.mark.gpu

TOL = {"poses": 1e-10, "J": 1e-10, "M": 1e-10, "tau": 1e-10, "qdd": 1e-8}

ROBOTS = {
    "chain7": lambda: syn.serial_chain(7),
    "arm9": lambda: syn.arm_with_fingers(),
    "arm9_sapien": lambda: syn.arm_with_fingers(sapien_style=True),
    "quadruped18": lambda: syn.quadruped(),
    "humanoid": lambda: syn.humanoid(),
    "humanoid_sapien": lambda: syn.humanoid(sapien_style=True),
    "arm6": lambda: syn.serial_chain(6, seed=4),
    "mixed_chain": lambda: syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                "continuous", "prismatic"]),
    # joint-count bucket edges (16 / 32 / 64 joints incl. the universe)
    "chain15": lambda: syn.serial_chain(15, seed=21),
    "chain16": lambda: syn.serial_chain(16, seed=22),
    "chain40": lambda: syn.serial_chain(40, seed=23),
}


def torch():
    import torch as t

    return t


def pair(robot):
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    return pm, o


def quat_from_R(R):
    """(w, x, y, z), Shepperd's method: same branch rule as the kernels and the oracle."""
    t = np.trace(R)
    q = np.zeros(4)
    if t > 0:
        r = np.sqrt(t + 1)
        q[0] = 0.5 * r
        k = 0.5 / r
        q[1:] = [(R[2, 1] - R[1, 2]) * k, (R[0, 2] - R[2, 0]) * k, (R[1, 0] - R[0, 1]) * k]
    else:
        i = 0
        if R[1, 1] > R[0, 0]:
            i = 1
        if R[2, 2] > R[i, i]:
            i = 2
        j, k_ = (i + 1) % 3, (i + 2) % 3
        r = np.sqrt(R[i, i] - R[j, j] - R[k_, k_] + 1)
        q[1 + i] = 0.5 * r
        k = 0.5 / r
        q[0] = (R[k_, j] - R[j, k_]) * k
        q[1 + j] = (R[j, i] + R[i, j]) * k
        q[1 + k_] = (R[k_, i] + R[i, k_]) * k
    return q


def oracle_pose7(poses12):
    n, nl, _ = poses12.shape
    out = np.zeros((n, nl, 7))
    for e in range(n):
        for li in range(nl):
            out[e, li, :3] = poses12[e, li, 9:]
            out[e, li, 3:] = quat_from_R(poses12[e, li, :9].reshape(3, 3))
    return out


def rel_per_env(g, o):
    g = g.reshape(g.shape[0], -1)
    o = o.reshape(o.shape[0], -1)
    return (np.abs(g - o).max(axis=1) / np.maximum(np.abs(o).max(axis=1), 1e-300)).max()


def run_step(pm, q, qd, qdd, tau):
    T = torch()
    dev = T.device("cuda", 0)
    t = lambda a: T.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    out = pm.step_batched(t(q), t(qd), t(qdd), t(tau))
    T.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("name", list(ROBOTS))
def test_fused_step_matches_oracle(name):
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    q, qd, qdd, tau = robot.sample(77, seed=101)
    g = run_step(pm, q, qd, qdd, tau)
    r = o.batch_step(q, qd, qdd, tau, nthreads=8)
    errs = {
        "poses": rel_per_env(g["link_poses"], oracle_pose7(r["poses"])),
        "J": rel_per_env(g["jacobian"], r["J"]),
        "M": rel_per_env(g["mass_matrix"], r["M"]),
        "tau": rel_per_env(g["qf"], r["tau"]),
        "qdd": rel_per_env(g["qacc"], r["qdd"]),
    }
    for k, v in errs.items():
        assert v <= TOL[k], f"{name}: {k} relative error {v:.3e} > {TOL[k]:g}"
    assert np.array_equal(g["mass_matrix"], np.swapaxes(g["mass_matrix"], 1, 2))


@pytest.mark.parametrize("name", ["arm9", "humanoid"])
def test_single_op_entry_points_match_fused(name):
    robot = ROBOTS[name]()
    pm, _ = pair(robot)
    T = torch()
    q, qd, qdd, tau = robot.sample(50, seed=5)
    t = lambda a: T.from_numpy(a).cuda()  # noqa: E731
    fused = pm.step_batched(t(q), t(qd), t(qdd), t(tau))
    sep = {
        "link_poses": pm.compute_forward_kinematics_batched(t(q)),
        "jacobian": pm.compute_full_jacobian_batched(t(q)),
        "mass_matrix": pm.compute_generalized_mass_matrix_batched(t(q)),
        "qf": pm.compute_inverse_dynamics_batched(t(q), t(qd), t(qdd)),
        "qacc": pm.compute_forward_dynamics_batched(t(q), t(qd), t(tau)),
    }
    # Same sweep compiled per op set: the compiler may contract a different set of
    # multiply-adds per instantiation, so results agree to rounding, amplified for ABA by
    # the conditioning of the 35-DoF floating-base humanoid.
    for k, v in sep.items():
        a, b = v.cpu().numpy(), fused[k].cpu().numpy()
        assert rel_per_env(a, b) < (1e-11 if k == "qacc" else 1e-13), k


@pytest.mark.parametrize("where", ["cuda", "host"])
def test_drop_in_single_instance_api(where):
    robot = syn.arm_with_fingers(sapien_style=True)
    pm, o = pair(robot)
    pm.single_instance = where
    q, qd, qdd, tau = robot.sample(3, seed=17)
    for e in range(3):
        pm.compute_forward_kinematics(q[e])
        Tref = o.link_poses(q[e])
        for li in range(len(robot.link_names)):
            pose = pm.get_link_pose(li)
            assert pose.p.dtype == np.float32 and pose.q.dtype == np.float32
            assert np.abs(pose.p - Tref[li, :3, 3]).max() < 1e-6
            qr = quat_from_R(Tref[li, :3, :3])
            assert min(np.abs(pose.q - qr).max(), np.abs(pose.q + qr).max()) < 1e-6
        tt = pm.compute_inverse_dynamics(q[e], qd[e], qdd[e])
        assert np.abs(tt - o.compute_inverse_dynamics(q[e], qd[e], qdd[e])).max() <= 1e-10 * np.abs(tt).max()
        a = pm.compute_forward_dynamics(q[e], qd[e], tau[e])
        assert np.abs(a - o.compute_forward_dynamics(q[e], qd[e], tau[e])).max() <= 1e-8 * np.abs(a).max()
        M = pm.compute_generalized_mass_matrix(q[e])
        assert np.abs(M - o.compute_generalized_mass_matrix(q[e])).max() <= 1e-10 * np.abs(M).max()


@pytest.mark.parametrize("where", ["cuda", "host"])
def test_chain7_single_instance_1000_samples(where):
    """The CPU-runnable reference configuration: a seeded 7-DoF revolute chain (offsets
    U[0.05, 0.4] m along random unit axes, random unit joint axes, masses U[0.5, 3] kg,
    inertias R diag(U[1e-3, 5e-2]) R^T) and 1000 samples q ~ U[-pi, pi], qd, qdd ~ N(0, 1),
    tau ~ N(0, 10), through the single-instance drop-in methods: FK + get_link_pose (float32
    poses, as the reference returns them), full Jacobian + get_link_jacobian, mass matrix,
    RNEA and ABA against the oracle."""
    robot = syn.serial_chain(7)
    pm, o = pair(robot)
    pm.single_instance = where
    n = 1000
    q, qd, qdd, tau = robot.sample(n, seed=0)
    nl = len(robot.link_names)
    worst = dict.fromkeys(("poses", "J", "M", "tau", "qdd"), 0.0)

    def upd(k, g, r):
        worst[k] = max(worst[k], np.abs(g - r).max() / max(np.abs(r).max(), 1e-300))

    for e in range(n):
        pm.compute_forward_kinematics(q[e])
        o.compute_forward_kinematics(q[e])
        for li in range(nl):
            pose = pm.get_link_pose(li)
            T4 = o.get_link_pose_matrix(li)
            upd("poses", pose.p.astype(np.float64), T4[:3, 3])
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


def test_col_major_layout_through_c_abi():
    robot = syn.arm_with_fingers()
    pm, o = pair(robot)
    T = torch()
    n = 45
    q, qd, qdd, tau = robot.sample(n, seed=8)
    # structure-of-arrays buffers: [cols][n]
    qT = T.from_numpy(np.ascontiguousarray(q.T)).cuda()
    qdT = T.from_numpy(np.ascontiguousarray(qd.T)).cuda()
    qddT = T.from_numpy(np.ascontiguousarray(qdd.T)).cuda()
    tauT = T.from_numpy(np.ascontiguousarray(tau.T)).cuda()
    nv = robot.nv
    tau_o = T.empty(nv, n, dtype=T.float64, device="cuda")
    qdd_o = T.empty(nv, n, dtype=T.float64, device="cuda")
    M_o = T.empty(nv * nv, n, dtype=T.float64, device="cuda")
    L = N.load()
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    pm._prepare(qT.device)
    rc = L.sgdyn_step(pm._h, n, N.OP_INVERSE_DYNAMICS | N.OP_FORWARD_DYNAMICS | N.OP_MASS_MATRIX, p(qT), p(qdT),
                      p(qddT), p(tauT), None, None, p(M_o), p(tau_o), p(qdd_o), N.COL_MAJOR, None)
    assert rc == 0, N.last_error()
    T.cuda.synchronize()
    r = o.batch_step(q, qd, qdd, tau, ops=4 | 8 | 16)
    assert rel_per_env(tau_o.cpu().numpy().T, r["tau"]) <= 1e-10
    assert rel_per_env(qdd_o.cpu().numpy().T, r["qdd"]) <= 1e-8
    assert rel_per_env(M_o.cpu().numpy().T.reshape(n, nv, nv), r["M"]) <= 1e-10


@pytest.mark.parametrize("layout", ["env_major", "col_major"])
def test_pinned_host_buffers_read_and_written_in_place(layout):
    """Mapped pinned host memory is accepted at the C ABI: the kernel reads the inputs and
    writes every output straight in host memory, bitwise equal to the device-buffer run."""
    robot = syn.arm_with_fingers()
    pm, _ = pair(robot)
    T = torch()
    n, nv, nl = 77, robot.nv, len(robot.link_names)
    q, qd, qdd, tau = robot.sample(n, seed=12)
    lay = N.ENV_MAJOR if layout == "env_major" else N.COL_MAJOR
    arr = (lambda a: a) if layout == "env_major" else (lambda a: a.reshape(n, -1).T)  # noqa: E731
    ins = [np.ascontiguousarray(arr(x)) for x in (q, qd, qdd, tau)]
    shapes = [(n, nl * 7), (n, 6 * nv), (n, nv * nv), (n, nv), (n, nv)]
    shapes = shapes if layout == "env_major" else [(c, r) for r, c in shapes]
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    L = N.load()
    res = {}
    for where in ("device", "host"):
        if where == "device":
            tin = [T.from_numpy(x).cuda() for x in ins]
            tout = [T.full(sh, float("nan"), dtype=T.float64, device="cuda") for sh in shapes]
        else:
            tin = [T.from_numpy(x).pin_memory() for x in ins]
            tout = [T.full(sh, float("nan"), dtype=T.float64).pin_memory() for sh in shapes]
        pm._prepare(T.device("cuda", 0))
        rc = L.sgdyn_step(pm._h, n, N.OP_ALL, *[p(x) for x in tin], *[p(x) for x in tout], lay, None)
        assert rc == 0, N.last_error()
        T.cuda.synchronize()
        res[where] = [x.cpu() for x in tout]
    for a, b in zip(res["device"], res["host"]):
        assert not T.isnan(b).any()
        assert T.equal(a, b)


@pytest.mark.parametrize("name", ["humanoid", "quadruped", "arm9"])
def test_lanes_per_environment_single_model(name):
    """Teams of 2, 4 or 8 lanes per environment (and the automatic choice) reproduce the
    one-lane sweep to rounding and write every output entry (buffers start as NaN)."""
    robot = {"humanoid": syn.humanoid(), "quadruped": syn.quadruped(), "arm9": syn.arm_with_fingers()}[name]
    pm, o = pair(robot)
    T = torch()
    n = 77
    q, qd, qdd, tau = (T.from_numpy(a).cuda() for a in robot.sample(n, seed=31))

    nv, nl = robot.nv, len(robot.link_names)
    shapes = {"link_poses": (n, nl * 7), "jacobian": (n, 6 * nv), "mass_matrix": (n, nv * nv), "qf": (n, nv),
              "qacc": (n, nv)}
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731

    def run(lanes):
        pm.set_lanes(lanes)
        out = {k: T.full(sh, float("nan"), dtype=T.float64, device="cuda") for k, sh in shapes.items()}
        pm._prepare(q.device)
        rc = N.load().sgdyn_step(pm._h, n, N.OP_ALL, p(q), p(qd), p(qdd), p(tau), *[p(out[k]) for k in shapes],
                                 N.ENV_MAJOR, None)
        assert rc == 0, N.last_error()
        T.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in out.items()}

    ref = run(1)
    for lanes in (2, 4, 8, 0):
        got = run(lanes)
        for k in ref:
            assert not np.isnan(got[k]).any(), (lanes, k)
            assert rel_per_env(got[k], ref[k]) <= 1e-11, (lanes, k)
    r = o.batch_step(*(x.cpu().numpy() for x in (q, qd, qdd, tau)), ops=4 | 8 | 16)
    assert rel_per_env(got["qf"], r["tau"]) <= 1e-10
    assert rel_per_env(got["qacc"], r["qdd"]) <= 1e-8
    assert rel_per_env(got["mass_matrix"], r["M"].reshape(n, -1)) <= 1e-10
    pm.set_lanes(0)


def test_edge_cases_and_pointer_checks():
    robot = syn.serial_chain(7)
    pm, o = pair(robot)
    T = torch()
    L = N.load()
    empty = T.empty(0, robot.nq_ext, dtype=T.float64, device="cuda")
    assert pm.compute_inverse_dynamics_batched(empty, empty[:, :7], empty[:, :7]).shape == (0, 7)
    # a host pointer must be rejected with an error status, never reach a kernel
    qh = T.zeros(4, robot.nq_ext, dtype=T.float64)
    out = T.empty(4, robot.nv, dtype=T.float64, device="cuda")
    rc = L.sgdyn_compute_inverse_dynamics(pm._h, 4, ctypes.c_void_p(qh.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                          N.ENV_MAJOR, None)
    assert rc == N.ERR_NULL
    assert "not device memory" in N.last_error()
    with pytest.raises(TypeError):
        pm.compute_inverse_dynamics_batched(qh, qh, qh)
    # single environment
    q, qd, qdd, _ = robot.sample(1, seed=2)
    t = pm.compute_inverse_dynamics(q[0], qd[0], qdd[0])
    assert np.abs(t - o.compute_inverse_dynamics(q[0], qd[0], qdd[0])).max() <= 1e-10 * np.abs(t).max()


def test_full_size_batch_properties_and_parity():
    """16384 environments of the 9-DoF arm: parity on every environment plus
    size-independent identities computed on the GPU alone."""
    robot = syn.arm_with_fingers()
    pm, o = pair(robot)
    T = torch()
    n = 16384
    q, qd, qdd, tau = robot.sample(n, seed=1)
    g = run_step(pm, q, qd, qdd, tau)
    r = o.batch_step(q, qd, qdd, tau, nthreads=8)
    assert rel_per_env(g["qf"], r["tau"]) <= 1e-10
    assert rel_per_env(g["qacc"], r["qdd"]) <= 1e-8
    assert rel_per_env(g["mass_matrix"], r["M"]) <= 1e-10
    # RNEA(q, qd, ABA(q, qd, tau)) == tau, all on the GPU
    t = lambda a: T.from_numpy(a).cuda()  # noqa: E731
    back = pm.compute_inverse_dynamics_batched(t(q), t(qd), T.from_numpy(g["qacc"]).cuda()).cpu().numpy()
    assert rel_per_env(back, tau) <= 1e-9


def test_floating_body_newton_euler_on_gpu():
    """The CUDA RNEA / CRBA / ABA of one free-floating rigid body against the Newton-Euler
    closed form of tests/test_oracle.py (body-frame twist, gravity as R^T g), batched."""
    import math

    from test_oracle import floating_body_urdf

    m, c, rpy = 2.3, np.array([0.11, -0.07, 0.19]), (0.3, -0.5, 1.1)
    Ip = np.array([0.03, 0.004, -0.002, 0.05, 0.006, 0.04])
    g = np.array([0.0, 0.0, -9.81])
    pm = PinocchioModel(floating_body_urdf(m, c, rpy, Ip), list(g))
    pm.set_joint_order(["ff"])
    pm.set_link_order(["world", "body"])
    cr, sr, cp, sp, cy, sy = (math.cos(rpy[0]), math.sin(rpy[0]), math.cos(rpy[1]), math.sin(rpy[1]),
                              math.cos(rpy[2]), math.sin(rpy[2]))
    Rrpy = np.array([[cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr],
                     [sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr],
                     [-sp, cp * sr, cp * cr]])
    Il = np.array([[Ip[0], Ip[1], Ip[2]], [Ip[1], Ip[3], Ip[4]], [Ip[2], Ip[4], Ip[5]]])
    Ic = Rrpy @ Il @ Rrpy.T
    rng = np.random.default_rng(6)
    n = 100
    quat = rng.normal(size=(n, 4))
    quat /= np.linalg.norm(quat, axis=1, keepdims=True)
    q = np.concatenate([rng.normal(size=(n, 3)), quat], axis=1)
    qd, qdd = rng.normal(size=(n, 6)), rng.normal(size=(n, 6))
    T = torch()
    tau = pm.compute_inverse_dynamics_batched(T.from_numpy(q).cuda(), T.from_numpy(qd).cuda(),
                                              T.from_numpy(qdd).cuda()).cpu().numpy()
    back = pm.compute_forward_dynamics_batched(T.from_numpy(q).cuda(), T.from_numpy(qd).cuda(),
                                               T.from_numpy(tau).cuda()).cpu().numpy()
    for e in range(n):
        x, y, z, w = quat[e]
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        v, om, av, aw = qd[e, :3], qd[e, 3:], qdd[e, :3], qdd[e, 3:]
        F = m * (av + np.cross(om, v) + np.cross(aw, c) + np.cross(om, np.cross(om, c)) - R.T @ g)
        expect = np.concatenate([F, np.cross(c, F) + Ic @ aw + np.cross(om, Ic @ om)])
        assert np.abs(tau[e] - expect).max() <= 1e-12 * np.abs(expect).max(), e
        assert np.abs(back[e] - qdd[e]).max() <= 1e-10 * np.abs(qdd[e]).max(), e


def test_cart_pole_closed_form_on_gpu():
    """The CUDA sweeps on a prismatic cart with a hinged pole against the Lagrangian closed
    form of tests/test_oracle.py: M, the Coriolis matrix, RNEA and ABA, batched."""
    import math

    from test_oracle import cart_pole_urdf

    mc, mp, l, Iyy, g = 1.9, 0.7, 0.45, 0.012, 9.81
    pm = PinocchioModel(cart_pole_urdf(mc, mp, l, Iyy), [0, 0, -g])
    pm.set_joint_order(["slide", "hinge"])
    pm.set_link_order(["rail", "cart", "pole"])
    rng = np.random.default_rng(3)
    n = 64
    q, qd, qdd = rng.uniform(-3, 3, (n, 2)), rng.normal(size=(n, 2)), rng.normal(size=(n, 2))
    T = torch()
    cq, cqd, cqdd = (T.from_numpy(x).cuda() for x in (q, qd, qdd))
    Mg = pm.compute_generalized_mass_matrix_batched(cq).cpu().numpy().reshape(n, 2, 2)
    Cg = pm.compute_coriolis_matrix_batched(cq, cqd).cpu().numpy().reshape(n, 2, 2)
    tau = pm.compute_inverse_dynamics_batched(cq, cqd, cqdd)
    back = pm.compute_forward_dynamics_batched(cq, cqd, tau).cpu().numpy()
    tau = tau.cpu().numpy()
    for e in range(n):
        c, s = math.cos(q[e, 1]), math.sin(q[e, 1])
        M = np.array([[mc + mp, mp * l * c], [mp * l * c, mp * l * l + Iyy]])
        C = np.array([[0.0, -mp * l * s * qd[e, 1]], [0.0, 0.0]])
        gv = np.array([0.0, -mp * g * l * s])
        assert np.abs(Mg[e] - M).max() < 1e-14
        assert np.abs(Cg[e] - C).max() < 1e-13
        assert np.abs(tau[e] - (M @ qdd[e] + C @ qd[e] + gv)).max() < 1e-12
        assert np.abs(back[e] - qdd[e]).max() < 1e-12


@pytest.mark.parametrize("name", ["arm9", "humanoid", "quadruped18", "chain40"])
def test_host_path_matches_device_kernels(name):
    """The host instantiation of the sweep (sgdyn_host_step, several threads) and the CUDA
    kernels agree to rounding on the same batch."""
    import ctypes

    robot = ROBOTS[name]()
    pm, _ = pair(robot)
    q, qd, qdd, tau = robot.sample(64, seed=3)
    g = run_step(pm, q, qd, qdd, tau)
    n, nv, nl = 64, robot.nv, len(robot.link_names)
    out = {"link_poses": np.empty((n, nl, 7)), "jacobian": np.empty((n, 6, nv)), "mass_matrix": np.empty((n, nv, nv)),
           "qf": np.empty((n, nv)), "qacc": np.empty((n, nv))}
    a = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    N.check(N.load().sgdyn_host_step(pm._h, n, N.OP_ALL, a(q), a(qd), a(qdd), a(tau), a(out["link_poses"]),
                                     a(out["jacobian"]), a(out["mass_matrix"]), a(out["qf"]), a(out["qacc"]),
                                     N.ENV_MAJOR, 4))
    for k in out:
        assert rel_per_env(out[k], g[k]) <= (1e-10 if k == "qacc" else 1e-12), k


@pytest.mark.parametrize("name", ["arm9", "humanoid", "chain40"])
def test_step_as_two_kinds_of_warps_matches_single_kind(name):
    """sgdyn_step for all five ops as one kind of warp (split mode 0) and as CRBA + RNEA +
    ABA warps beside FK + Jacobian warps (mode 1), generic and run-time-compiled kernels:
    equal to rounding, and both equal to the oracle."""
    import ctypes

    robot = ROBOTS[name]()
    pm, o = pair(robot)
    L = N.load()
    old = ctypes.c_int()
    assert L.sgdyn_step_split(-1, ctypes.byref(old)) == N.OK and old.value == 2
    q, qd, qdd, tau = robot.sample(200, seed=12)
    r = o.batch_step(q, qd, qdd, tau, nthreads=8)
    want = {"link_poses": oracle_pose7(r["poses"]), "jacobian": r["J"], "mass_matrix": r["M"], "qf": r["tau"],
            "qacc": r["qdd"]}
    outs = {}
    old_jit, old_min = ctypes.c_int(), ctypes.c_int64()
    L.sgdyn_jit_config(-1, -1, ctypes.byref(old_jit), ctypes.byref(old_min))
    try:
        for jit in (0, 1):
            L.sgdyn_jit_config(jit, 0, None, None)
            for mode in (0, 1):
                assert L.sgdyn_step_split(mode, None) == N.OK
                outs[(jit, mode)] = run_step(pm, q, qd, qdd, tau)
    finally:
        L.sgdyn_step_split(2, None)
        L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)
    for key, g in outs.items():
        for k, w in want.items():
            tol = 1e-8 if k == "qacc" else 1e-10
            assert rel_per_env(g[k], w) <= tol, (key, k)
            assert rel_per_env(g[k], outs[(0, 0)][k]) <= (1e-11 if k == "qacc" else 1e-13), (key, k)


@pytest.mark.parametrize("name", ["arm9", "arm9_sapien", "mixed_chain", "chain40", "quadruped18", "humanoid",
                                  "humanoid_sapien"])
def test_three_lane_forward_dynamics_matches_oracle(name):
    """compute_forward_dynamics_batched on a small batch runs one team of three lanes per
    environment (sgdyn_rollout_lanes automatic); forced one lane and three lanes, generic and
    run-time compiled, against the oracle, env-major and structure-of-arrays."""
    import ctypes

    T = torch()
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    n = 57
    q, qd, _, tau = robot.sample(n, seed=19)
    ref = o.batch_step(q, qd, None, tau, ops=16, nthreads=8)["qdd"]
    L = N.load()
    old_jit, old_min = ctypes.c_int(), ctypes.c_int64()
    L.sgdyn_jit_config(-1, -1, ctypes.byref(old_jit), ctypes.byref(old_min))
    try:
        for jit in (0, 1):
            L.sgdyn_jit_config(jit, 0, None, None)
            for lanes in (0, 1, 3):
                assert L.sgdyn_rollout_lanes(lanes, None) == N.OK
                t = lambda a: T.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
                g = pm.compute_forward_dynamics_batched(t(q), t(qd), t(tau)).cpu().numpy()
                assert rel_per_env(g, ref) <= 1e-8, (jit, lanes)
                # structure of arrays through the C ABI
                qs, qds, taus = (t(a.T) for a in (q, qd, tau))
                out = T.empty(robot.nv, n, dtype=T.float64, device="cuda")
                P = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
                assert L.sgdyn_compute_forward_dynamics(pm._h, n, P(qs), P(qds), P(taus), P(out), N.COL_MAJOR,
                                                        ctypes.c_void_p(T.cuda.current_stream().cuda_stream)) == N.OK
                assert rel_per_env(out.cpu().numpy().T, ref) <= 1e-8, (jit, lanes, "soa")
    finally:
        L.sgdyn_rollout_lanes(0, None)
        L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)


def step_ops(pm, ops, q, qd, qdd, tau):
    """sgdyn_step with an op mask through the C ABI (env-major device buffers)."""
    T = torch()
    dev = T.device("cuda", 0)
    t = lambda a: T.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    n, nv, nl = q.shape[0], pm.nv, pm.nlinks
    outs = {"link_poses": (N.OP_FK, (n, nl, 7)), "jacobian": (N.OP_JACOBIAN, (n, 6, nv)),
            "mass_matrix": (N.OP_MASS_MATRIX, (n, nv, nv)), "qf": (N.OP_INVERSE_DYNAMICS, (n, nv)),
            "qacc": (N.OP_FORWARD_DYNAMICS, (n, nv))}
    bufs = {k: T.full(shape, np.nan, dtype=T.float64, device=dev) if ops & bit else None
            for k, (bit, shape) in outs.items()}
    P = lambda x: ctypes.c_void_p(x.data_ptr() if x is not None else 0)  # noqa: E731
    ins = [t(q), t(qd), t(qdd), t(tau)]
    rc = N.load().sgdyn_step(pm._h, n, ops, *[P(x) for x in ins], *[P(bufs[k]) for k in outs], N.ENV_MAJOR,
                             ctypes.c_void_p(T.cuda.current_stream().cuda_stream))
    assert rc == N.OK, N.last_error()
    T.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in bufs.items() if v is not None}


@pytest.mark.parametrize("name", ["arm9", "arm9_sapien", "chain7", "mixed_chain", "quadruped18", "humanoid",
                                  "humanoid_sapien", "chain40"])
def test_forward_dynamics_routes_match_oracle(name):
    """The run-time-specialised sweep computes forward dynamics by the articulated-body passes
    (sgdyn_fd_method 1) or from the mass matrix (method 2: CRBA, bias forces at zero
    acceleration, M = L^T D L with the tree's sparsity; inverse dynamics in the same sweep as
    b + M qdd). The op sets holding ABA (two of them on the large trees, whose unrolled sweeps
    take long to compile), both methods, against the oracle and each other."""
    robot = ROBOTS[name]()
    pm, o = pair(robot)
    op_sets = (16, 24, 28, 31) if robot.nv <= 18 else (16, 28)
    n = 96
    q, qd, qdd, tau = robot.sample(n, seed=23)
    r = o.batch_step(q, qd, qdd, tau, nthreads=8)
    want = {"link_poses": oracle_pose7(r["poses"]), "jacobian": r["J"], "mass_matrix": r["M"], "qf": r["tau"],
            "qacc": r["qdd"]}
    tol = {"link_poses": TOL["poses"], "jacobian": TOL["J"], "mass_matrix": TOL["M"], "qf": TOL["tau"],
           "qacc": TOL["qdd"]}
    L = N.load()
    old_jit, old_min, old_max, old_fd = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_int()
    L.sgdyn_jit_config(-1, -1, ctypes.byref(old_jit), ctypes.byref(old_min))
    L.sgdyn_jit_max_joints(-1, ctypes.byref(old_max))
    assert L.sgdyn_fd_method(-1, ctypes.byref(old_fd)) == N.OK and old_fd.value == 0
    outs = {}
    try:
        L.sgdyn_jit_config(1, 0, None, None)
        L.sgdyn_jit_max_joints(64, None)
        for mode in (1, 2):
            assert L.sgdyn_fd_method(mode, None) == N.OK
            for ops in op_sets:
                route = ctypes.c_int()
                assert L.sgdyn_fd_by_mass_matrix(pm._h, ops, ctypes.byref(route)) == N.OK
                assert route.value == (mode == 2)
                outs[(mode, ops)] = step_ops(pm, ops, q, qd, qdd, tau)
    finally:
        L.sgdyn_fd_method(old_fd.value, None)
        L.sgdyn_jit_max_joints(old_max.value, None)
        L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)
    for key, g in outs.items():
        for k, v in g.items():
            assert not np.isnan(v).any(), (key, k)
            assert rel_per_env(v, want[k]) <= tol[k], (key, k, rel_per_env(v, want[k]))
            other = outs[(3 - key[0], key[1])][k]
            assert rel_per_env(v, other) <= (1e-10 if k == "qacc" else 1e-12), (key, k)
