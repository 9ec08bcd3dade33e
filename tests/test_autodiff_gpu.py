"""GPU adjoint kernels against FP64 central finite differences of the CPU oracle.

Gradient tolerance: 1e-6 relative (normwise per environment) for FD with h = 1e-6;
exact identities (dtau/dqdd = M, dqdd/dtau = M^-1, VJP = row combination of the dense
derivatives, checkpoint-interval invariance) at 1e-10 or tighter.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel, autodiff as ad, synthetic as syn

pytestmark = pytest.mark.gpu
H = 1e-6


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


def rel(g, r):
    return np.abs(g - r).max() / max(np.abs(r).max(), 1e-300)


FIXED = {
    "arm9": lambda: syn.arm_with_fingers(),
    "arm9_sapien": lambda: syn.arm_with_fingers(sapien_style=True),
    "mixed_chain": lambda: syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                "continuous", "prismatic"]),
}


def fd_grad(f, x, w):
    """w . d f / d x by central differences (x, w 1-D)."""
    g = np.zeros(x.size)
    for k in range(x.size):
        e = np.zeros(x.size)
        e[k] = H
        g[k] = (w @ f(x + e) - w @ f(x - e)) / (2 * H)
    return g


@pytest.mark.parametrize("name", list(FIXED))
def test_rnea_and_aba_vjp_match_finite_differences(name):
    robot = FIXED[name]()
    pm, o = pair(robot)
    n = 6
    q, qd, qdd, tau = robot.sample(n, seed=81)
    w = np.random.default_rng(2).normal(size=(n, robot.nv))
    qb, qdb, qddb = (x.cpu().numpy() for x in ad.inverse_dynamics_vjp(pm, cu(q), cu(qd), cu(qdd), cu(w)))
    ab = [x.cpu().numpy() for x in ad.forward_dynamics_vjp(pm, cu(q), cu(qd), cu(tau), cu(w))]
    for e in range(n):
        assert rel(qb[e], fd_grad(lambda x: o.compute_inverse_dynamics(x, qd[e], qdd[e]), q[e], w[e])) < 1e-6
        assert rel(qdb[e], fd_grad(lambda x: o.compute_inverse_dynamics(q[e], x, qdd[e]), qd[e], w[e])) < 1e-6
        assert rel(qddb[e], fd_grad(lambda x: o.compute_inverse_dynamics(q[e], qd[e], x), qdd[e], w[e])) < 1e-6
        assert rel(ab[0][e], fd_grad(lambda x: o.compute_forward_dynamics(x, qd[e], tau[e]), q[e], w[e])) < 1e-6
        assert rel(ab[1][e], fd_grad(lambda x: o.compute_forward_dynamics(q[e], x, tau[e]), qd[e], w[e])) < 1e-6
        assert rel(ab[2][e], fd_grad(lambda x: o.compute_forward_dynamics(q[e], qd[e], x), tau[e], w[e])) < 1e-6


def test_fk_vjp_matches_finite_differences():
    robot = syn.arm_with_fingers(sapien_style=True)
    pm, o = pair(robot)
    n, L = 4, len(robot.link_names)
    q, _, _, _ = robot.sample(n, seed=91)
    rng = np.random.default_rng(3)
    pb = rng.normal(size=(n, L, 3))
    rb = rng.normal(size=(n, L, 3, 3))
    qb = ad.forward_kinematics_vjp(pm, cu(q), cu(pb), cu(rb)).cpu().numpy()
    for e in range(n):
        def f(x):
            Tm = o.link_poses(x)
            return np.concatenate([Tm[:, :3, 3].ravel(), Tm[:, :3, :3].ravel()])
        wv = np.concatenate([pb[e].ravel(), rb[e].ravel()])
        assert rel(qb[e], fd_grad(f, q[e], wv)) < 1e-6


@pytest.mark.parametrize("name", ["humanoid", "quadruped18", "arm9"])
def test_dense_derivatives_match_finite_differences(name):
    robot = {"humanoid": syn.humanoid, "quadruped18": syn.quadruped, "arm9": syn.arm_with_fingers}[name]()
    pm, o = pair(robot)
    n, nv = 3, robot.nv
    q, qd, qdd, tau = robot.sample(n, seed=97)
    dq, dqd, M = (x.cpu().numpy() for x in ad.rnea_derivatives(pm, cu(q), cu(qd), cu(qdd)))
    aq, aqd, Minv = (x.cpu().numpy() for x in ad.aba_derivatives(pm, cu(q), cu(qd), cu(tau)))
    for e in range(n):
        # q derivatives in the tangent space: perturb with integrate(q, +-h e_k)
        fdq_t = np.zeros((nv, nv))
        fdq_a = np.zeros((nv, nv))
        for k in range(nv):
            d = np.zeros(nv)
            d[k] = H
            qp, qm = o.integrate(q[e], d), o.integrate(q[e], -d)
            fdq_t[:, k] = (o.compute_inverse_dynamics(qp, qd[e], qdd[e]) - o.compute_inverse_dynamics(qm, qd[e], qdd[e])) / (2 * H)
            fdq_a[:, k] = (o.compute_forward_dynamics(qp, qd[e], tau[e]) - o.compute_forward_dynamics(qm, qd[e], tau[e])) / (2 * H)
        fdqd_t = np.stack([(o.compute_inverse_dynamics(q[e], qd[e] + H * np.eye(nv)[k], qdd[e])
                            - o.compute_inverse_dynamics(q[e], qd[e] - H * np.eye(nv)[k], qdd[e])) / (2 * H)
                           for k in range(nv)], axis=1)
        fdqd_a = np.stack([(o.compute_forward_dynamics(q[e], qd[e] + H * np.eye(nv)[k], tau[e])
                            - o.compute_forward_dynamics(q[e], qd[e] - H * np.eye(nv)[k], tau[e])) / (2 * H)
                           for k in range(nv)], axis=1)
        assert rel(dq[e], fdq_t) < 1e-6
        assert rel(dqd[e], fdqd_t) < 1e-6
        assert rel(aq[e], fdq_a) < 1e-6
        assert rel(aqd[e], fdqd_a) < 1e-6
        Mref = o.compute_generalized_mass_matrix(q[e])
        assert rel(M[e], Mref) < 1e-10
        assert rel(Minv[e], np.linalg.inv(Mref)) < 1e-8


def test_dense_derivatives_do_not_depend_on_the_column_split():
    """Every column is computed the same way whatever the batch size (one thread per
    environment and column, reading the prepared per-environment data), so a small batch and
    the same environments inside batches of 4096 and 8192 agree bit for bit."""
    robot = syn.humanoid()
    pm, _ = pair(robot)
    q, qd, qdd, tau = robot.sample(8192, seed=17)
    half = [x.cpu() for x in ad.aba_derivatives(pm, cu(q[:4096]), cu(qd[:4096]), cu(tau[:4096]))]
    big_r = [x[:5].cpu() for x in ad.rnea_derivatives(pm, cu(q), cu(qd), cu(qdd))]
    big_a = [x[:5].cpu() for x in ad.aba_derivatives(pm, cu(q), cu(qd), cu(tau))]
    small_r = [x.cpu() for x in ad.rnea_derivatives(pm, cu(q[:5]), cu(qd[:5]), cu(qdd[:5]))]
    small_a = [x.cpu() for x in ad.aba_derivatives(pm, cu(q[:5]), cu(qd[:5]), cu(tau[:5]))]
    for x, y in zip(big_r + big_a, small_r + small_a):
        assert T().equal(x, y)
    for x, y in zip(half, small_a):
        assert T().equal(x[:5], y)


def test_dense_derivatives_of_a_40_joint_chain():
    """The 64-joint kernels (largest per-thread frames): dtau/dqdd = M, dqdd/dtau = M^-1 and
    rows equal to the reverse-mode VJP."""
    robot = syn.serial_chain(40, seed=2)
    pm, o = pair(robot)
    q, qd, qdd, tau = robot.sample(6, seed=9)
    dq, dqd, M = (x.cpu().numpy() for x in ad.rnea_derivatives(pm, cu(q), cu(qd), cu(qdd)))
    aq, aqd, Minv = (x.cpu().numpy() for x in ad.aba_derivatives(pm, cu(q), cu(qd), cu(tau)))
    w = np.random.default_rng(3).normal(size=(6, robot.nv))
    qb, qdb, _ = (x.cpu().numpy() for x in ad.inverse_dynamics_vjp(pm, cu(q), cu(qd), cu(qdd), cu(w)))
    assert rel(qb, np.einsum("er,erc->ec", w, dq)) < 1e-11
    assert rel(qdb, np.einsum("er,erc->ec", w, dqd)) < 1e-11
    for e in range(6):
        Mref = o.compute_generalized_mass_matrix(q[e])
        assert rel(M[e], Mref) < 1e-10
        assert rel(Minv[e] @ Mref, np.eye(robot.nv)) < 1e-8
    # dqdd/d(q, qd) = -M^-1 dtau/d(q, qd) at qdd = ABA(q, qd, tau)
    qdd_a = np.stack([o.compute_forward_dynamics(q[e], qd[e], tau[e]) for e in range(6)])
    dq_a, dqd_a, _ = (x.cpu().numpy() for x in ad.rnea_derivatives(pm, cu(q), cu(qd), cu(qdd_a)))
    for e in range(6):
        assert rel(aq[e], -Minv[e] @ dq_a[e]) < 1e-8
        assert rel(aqd[e], -Minv[e] @ dqd_a[e]) < 1e-8


def test_vjp_equals_dense_rows():
    robot = syn.arm_with_fingers()
    pm, _ = pair(robot)
    q, qd, qdd, tau = robot.sample(16, seed=7)
    w = np.random.default_rng(5).normal(size=(16, robot.nv))
    dq, dqd, M = (x.cpu().numpy() for x in ad.rnea_derivatives(pm, cu(q), cu(qd), cu(qdd)))
    qb, qdb, qddb = (x.cpu().numpy() for x in ad.inverse_dynamics_vjp(pm, cu(q), cu(qd), cu(qdd), cu(w)))
    assert rel(qb, np.einsum("er,erc->ec", w, dq)) < 1e-12
    assert rel(qdb, np.einsum("er,erc->ec", w, dqd)) < 1e-12
    assert rel(qddb, np.einsum("er,erc->ec", w, M)) < 1e-12


def test_autograd_functions():
    torch = T()
    robot = syn.arm_with_fingers()
    pm, o = pair(robot)
    q, qd, qdd, tau = robot.sample(5, seed=11)
    qt, qdt, qddt = (cu(x).requires_grad_() for x in (q, qd, qdd))
    out = ad.inverse_dynamics(pm, qt, qdt, qddt)
    out.pow(2).sum().backward()
    tb = 2 * out.detach()
    ref = ad.inverse_dynamics_vjp(pm, cu(q), cu(qd), cu(qdd), tb)
    for g, r in zip((qt.grad, qdt.grad, qddt.grad), ref):
        assert torch.equal(g, r)
    qt2 = cu(q).requires_grad_()
    pos = ad.link_positions(pm, qt2)
    pos[:, robot.ee_link].sum().backward()
    pb = np.zeros((5, len(robot.link_names), 3))
    pb[:, robot.ee_link] = 1
    assert rel(qt2.grad.cpu().numpy(), ad.forward_kinematics_vjp(pm, cu(q), cu(pb)).cpu().numpy()) < 1e-14


def _rollout_setup(n=16, T=200, seed=123):
    robot = syn.arm_with_fingers()
    pm, o = pair(robot)
    q0, qd0, _, _ = robot.sample(n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    tau = rng.normal(scale=5.0, size=(T, n, robot.nv))
    targets = rng.uniform(-0.5, 0.5, size=(n, 3))
    return robot, pm, o, q0, qd0, tau, targets


def test_rollout_forward_matches_oracle():
    robot, pm, o, q0, qd0, tau, targets = _rollout_setup()
    qT, qdT, _, _ = ad.rollout_forward(pm, cu(q0), cu(qd0), cu(tau), 1.0 / 500)
    rq, rqd, _ = o.rollout(q0, qd0, tau, 1.0 / 500, robot.ee_link, targets)
    assert rel(qT.cpu().numpy(), rq) < 1e-9
    assert rel(qdT.cpu().numpy(), rqd) < 1e-9


def test_rollout_gradient_matches_finite_differences():
    """Config: 9-DoF arm, T = 200 steps at dt = 1/500, tau ~ N(0, 5) per step, q/qd
    checkpoints every 20 steps, loss = sum |p_ee(q_T) - target|^2, 16 environments."""
    torch = T()
    robot, pm, o, q0, qd0, tau, targets = _rollout_setup()
    dt, ee = 1.0 / 500, robot.ee_link
    q0t, qd0t, taut = cu(q0).requires_grad_(), cu(qd0).requires_grad_(), cu(tau).requires_grad_()
    qT, _ = ad.rollout(pm, q0t, qd0t, taut, dt, checkpoint_every=20)
    pos = ad.link_positions(pm, qT)[:, ee]
    loss = ((pos - cu(targets)) ** 2).sum()
    loss.backward()
    g_q0, g_qd0, g_tau = q0t.grad.cpu().numpy(), qd0t.grad.cpu().numpy(), taut.grad.cpu().numpy()

    def L(q0_, qd0_, tau_):
        return o.rollout(q0_, qd0_, tau_, dt, ee, targets)[2]  # per-env losses

    n, nv = q0.shape
    fq, fqd = np.zeros_like(q0), np.zeros_like(qd0)
    for k in range(nv):
        e = np.zeros(nv)
        e[k] = H
        fq[:, k] = (L(q0 + e, qd0, tau) - L(q0 - e, qd0, tau)) / (2 * H)
        fqd[:, k] = (L(q0, qd0 + e, tau) - L(q0, qd0 - e, tau)) / (2 * H)
    for env in range(n):
        assert rel(g_q0[env], fq[env]) < 1e-6
        assert rel(g_qd0[env], fqd[env]) < 1e-6
    # tau: each entry moves the loss by O(dt^2), below central-difference noise, so compare
    # directional derivatives along random directions of the whole [T, nv] control sequence
    rng = np.random.default_rng(9)
    for _ in range(4):
        D = rng.normal(size=tau.shape)
        fd = (L(q0, qd0, tau + H * D) - L(q0, qd0, tau - H * D)) / (2 * H)
        dd = np.einsum("tek,tek->e", g_tau, D)
        assert np.abs(dd - fd).max() <= 1e-6 * np.abs(fd).max()
    # checkpoint interval does not change the result
    q0b1, qd0b1, tb1 = ad.rollout_backward(pm, *ad.rollout_forward(pm, cu(q0), cu(qd0), cu(tau), dt, 1)[2:], cu(tau),
                                           dt, 1, qT_bar=torch.ones_like(qT))
    q0b2, qd0b2, tb2 = ad.rollout_backward(pm, *ad.rollout_forward(pm, cu(q0), cu(qd0), cu(tau), dt, 200)[2:],
                                           cu(tau), dt, 200, qT_bar=torch.ones_like(qT))
    assert rel(q0b1.cpu().numpy(), q0b2.cpu().numpy()) < 1e-12
    assert rel(tb1.cpu().numpy(), tb2.cpu().numpy()) < 1e-12


@pytest.mark.parametrize("T,K", [(50, 7), (20, 20), (0, 5)])
def test_rollout_backward_segment_groups_agree(T, K):
    """The backward recomputes as many checkpoint segments at once as the scratch holds; one
    segment at a time, three at a time and all at once give bitwise-equal gradients (every
    environment runs the same operations in the same order)."""
    import ctypes

    import torch

    from sapien_gb300 import _native as N

    r = syn.arm_with_fingers()
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    pm.set_joint_order(r.joint_names)
    pm.set_link_order(r.link_names)
    n, dt = 40, 2e-3
    q0, qd0, _, tau1 = (torch.from_numpy(a).cuda() for a in r.sample(n, seed=8))
    tau = (0.3 * tau1).unsqueeze(0).repeat(T, 1, 1).contiguous()
    _, _, qc, qdc = ad.rollout_forward(pm, q0, qd0, tau, dt, K)
    if qc is None or qc.numel() == 0:
        qc = torch.empty(0, n, pm.nq_ext, dtype=torch.float64, device="cuda")
        qdc = torch.empty(0, n, pm.nv, dtype=torch.float64, device="cuda")
    g = torch.Generator(device="cpu").manual_seed(1)
    qTb = torch.randn(n, pm.nq_ext, generator=g, dtype=torch.float64).cuda()
    qdTb = torch.randn(n, pm.nv, generator=g, dtype=torch.float64).cuda()
    nb = ctypes.c_int64()
    assert N.load().sgdyn_rollout_scratch_bytes(pm._h, n, K, ctypes.byref(nb)) == 0
    outs = [ad.rollout_backward(pm, qc, qdc, tau, dt, K, qTb, qdTb, max_scratch_bytes=k * nb.value)
            for k in (1, 3, 1000)]
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert torch.equal(a, b)
    if T == 0:
        assert torch.equal(outs[0][0], qTb) and torch.equal(outs[0][1], qdTb)


FLOATING = {"quadruped18": lambda: syn.quadruped(), "humanoid": lambda: syn.humanoid()}


def _ff_rollout_setup(robot, n, T, seed):
    pm, o = pair(robot)
    q0, qd0, _, _ = robot.sample(n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    tau = rng.normal(scale=5.0, size=(T, n, robot.nv))
    targets = rng.uniform(-0.5, 0.5, size=(n, 3))
    return pm, o, q0, qd0, tau, targets


@pytest.mark.parametrize("name", list(FLOATING))
def test_floating_base_rollout_forward_matches_oracle(name):
    """Free-flyer root: the base moves on SE(3) by the body twist dt qd each step (the
    oracle's integrate), as in the heterogeneous rollout."""
    robot = FLOATING[name]()
    pm, o, q0, qd0, tau, targets = _ff_rollout_setup(robot, 24, 120, 31)
    qT, qdT, _, _ = ad.rollout_forward(pm, cu(q0), cu(qd0), cu(tau), 1.0 / 500)
    rq, rqd, _ = o.rollout(q0, qd0, tau, 1.0 / 500, robot.ee_link, targets)
    assert rel(qT.cpu().numpy(), rq) < 1e-9
    assert rel(qdT.cpu().numpy(), rqd) < 1e-9


def test_floating_base_rollout_gradient_matches_finite_differences():
    """The quadruped (free-flyer root + 4 legs of 3 joints), 16 environments, T = 200 at
    dt = 1/500, tau ~ N(0, 5) per step, checkpoints every 20 steps, loss = sum of squared
    distances of the end-effector link at q_T to seeded targets. The q0 gradient, mapped to
    the tangent space, against central differences of the oracle's rollout with q0
    perturbed on the manifold (integrate(q0, +-h e_k)); qd0 directly; tau along random
    directions."""
    torch = T()
    robot = syn.quadruped()
    n, steps, dt, ee = 16, 200, 1.0 / 500, robot.ee_link
    pm, o, q0, qd0, tau, targets = _ff_rollout_setup(robot, n, steps, 123)
    q0t, qd0t, taut = cu(q0).requires_grad_(), cu(qd0).requires_grad_(), cu(tau).requires_grad_()
    qT, _ = ad.rollout(pm, q0t, qd0t, taut, dt, checkpoint_every=20)
    loss = ((ad.link_positions(pm, qT)[:, ee] - cu(targets)) ** 2).sum()
    loss.backward()
    g_tan = ad.coordinate_to_tangent_grad(pm, cu(q0), q0t.grad).cpu().numpy()
    g_qd0, g_tau = qd0t.grad.cpu().numpy(), taut.grad.cpu().numpy()
    # the coordinate gradient is the tangent one pulled back through the chart
    back = ad.tangent_to_coordinate_grad(pm, cu(q0), cu(g_tan)).cpu().numpy()
    assert rel(back, q0t.grad.cpu().numpy()) < 1e-12

    def L(q0_, qd0_, tau_):
        return o.rollout(q0_, qd0_, tau_, dt, ee, targets)[2]

    nv = robot.nv
    fq, fqd = np.zeros((n, nv)), np.zeros((n, nv))
    for k in range(nv):
        d = np.zeros(nv)
        d[k] = H
        qp = np.stack([o.integrate(q0[e], d) for e in range(n)])
        qm = np.stack([o.integrate(q0[e], -d) for e in range(n)])
        fq[:, k] = (L(qp, qd0, tau) - L(qm, qd0, tau)) / (2 * H)
        fqd[:, k] = (L(q0, qd0 + d, tau) - L(q0, qd0 - d, tau)) / (2 * H)
    for env in range(n):
        assert rel(g_tan[env], fq[env]) < 1e-6, env
        assert rel(g_qd0[env], fqd[env]) < 1e-6, env
    rng = np.random.default_rng(9)
    for _ in range(3):
        D = rng.normal(size=tau.shape)
        fd = (L(q0, qd0, tau + H * D) - L(q0, qd0, tau - H * D)) / (2 * H)
        dd = np.einsum("tek,tek->e", g_tau, D)
        assert np.abs(dd - fd).max() <= 1e-6 * np.abs(fd).max()


def test_floating_base_rollout_backward_matches_single_step_vjps():
    """One step of the rollout backward equals the chain of the per-step pieces: the ABA
    adjoint (sgdyn_compute_forward_dynamics_vjp) and the SE(3) integrate adjoint, checked
    through checkpoint-interval invariance on the 35-DoF humanoid."""
    torch = T()
    robot = syn.humanoid()
    pm, _, q0, qd0, tau, _ = _ff_rollout_setup(robot, 40, 30, 7)
    dt = 1.0 / 500
    g = torch.Generator(device="cpu").manual_seed(3)
    qTb = torch.randn(40, pm.nq_ext, generator=g, dtype=torch.float64).cuda()
    qdTb = torch.randn(40, pm.nv, generator=g, dtype=torch.float64).cuda()
    outs = []
    for K in (1, 7, 30):
        _, _, qc, qdc = ad.rollout_forward(pm, cu(q0), cu(qd0), cu(tau), dt, K)
        outs.append(ad.rollout_backward(pm, qc, qdc, cu(tau), dt, K, qTb, qdTb))
    for o_ in outs[1:]:
        for a, b in zip(o_, outs[0]):
            assert rel(a.cpu().numpy(), b.cpu().numpy()) < 1e-12
    assert torch.all(outs[0][0][:, 6] == 0)  # the free flyer's seventh slot


ROLLOUT3 = {
    "arm9": lambda: syn.arm_with_fingers(),
    "arm9_sapien": lambda: syn.arm_with_fingers(sapien_style=True),
    "mixed_chain": lambda: syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                "continuous", "prismatic"]),
    "chain40": lambda: syn.serial_chain(40, seed=23),
    "quadruped18": lambda: syn.quadruped(),
    "humanoid": lambda: syn.humanoid(),
}


@pytest.mark.parametrize("name", list(ROLLOUT3))
def test_three_lane_rollout_forward_matches_one_lane_and_oracle(name):
    """The forward rollout with one lane per Cartesian axis (sgdyn_rollout_lanes(3)), generic
    and run-time-compiled, against one lane per environment and the oracle; 23 environments
    so that the last warp has teams past the end of the batch."""
    import ctypes

    from sapien_gb300 import _native as N

    robot = ROLLOUT3[name]()
    pm, o = pair(robot)
    n, steps, K, dt = 23, 60, 20, 1.0 / 500
    q0, qd0, _, _ = robot.sample(n, seed=4)
    tau = np.random.default_rng(5).normal(scale=5.0, size=(steps, n, robot.nv))
    L = N.load()
    old_jit, old_min = ctypes.c_int(), ctypes.c_int64()
    L.sgdyn_jit_config(-1, -1, ctypes.byref(old_jit), ctypes.byref(old_min))
    outs = {}
    try:
        for jit in (0, 1):
            L.sgdyn_jit_config(jit, 0, None, None)
            for lanes in (1, 3):
                assert L.sgdyn_rollout_lanes(lanes, None) == N.OK
                outs[(jit, lanes)] = [x.cpu().numpy() for x in ad.rollout_forward(pm, cu(q0), cu(qd0), cu(tau), dt, K)]
    finally:
        L.sgdyn_rollout_lanes(0, None)
        L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)
    rq, rqd, _ = o.rollout(q0, qd0, tau, dt, robot.ee_link, np.zeros((n, 3)))
    for key, (qT, qdT, qc, qdc) in outs.items():
        assert rel(qT, rq) < 1e-9 and rel(qdT, rqd) < 1e-9, key
        ref = outs[(0, 1)]
        assert rel(qc, ref[2]) < 1e-11 and rel(qdc, ref[3]) < 1e-11, key  # checkpoints


@pytest.mark.parametrize("name", ["arm9", "mixed_chain", "chain40", "quadruped18", "humanoid"])
def test_three_lane_rollout_backward_matches_one_lane(name):
    """The reverse sweep with one lane per Cartesian axis against one lane per environment,
    on the allocating and the allocation-free entry points: same adjoints to rounding (for
    a free-flyer root its tangent adjoint, the seventh slot zero)."""
    import ctypes

    import torch

    from sapien_gb300 import _native as N

    robot = ROLLOUT3[name]()
    pm, _ = pair(robot)
    n, steps, K, dt = 23, 40, 7, 1.0 / 500
    q0, qd0, _, _ = robot.sample(n, seed=14)
    tau = cu(np.random.default_rng(15).normal(scale=5.0, size=(steps, n, robot.nv)))
    g = torch.Generator(device="cpu").manual_seed(2)
    qTb = torch.randn(n, pm.nq_ext, generator=g, dtype=torch.float64).cuda()
    qdTb = torch.randn(n, pm.nv, generator=g, dtype=torch.float64).cuda()
    L = N.load()
    outs = {}
    old_jit, old_min = ctypes.c_int(), ctypes.c_int64()
    L.sgdyn_jit_config(-1, -1, ctypes.byref(old_jit), ctypes.byref(old_min))
    try:
        for lanes in (1, 3):
            assert L.sgdyn_rollout_lanes(lanes, None) == N.OK
            _, _, qc, qdc = ad.rollout_forward(pm, cu(q0), cu(qd0), tau, dt, K)
            outs[lanes] = [x.cpu().numpy() for x in ad.rollout_backward(pm, qc, qdc, tau, dt, K, qTb, qdTb)]
            if lanes == 3:  # the run-time-compiled reverse sweep
                L.sgdyn_jit_config(1, 0, None, None)
                outs["jit"] = [x.cpu().numpy() for x in ad.rollout_backward(pm, qc, qdc, tau, dt, K, qTb, qdTb)]
                L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)
            if lanes == 3:
                q0b = torch.empty(n, pm.nq_ext, dtype=torch.float64, device="cuda")
                qd0b = torch.empty(n, pm.nv, dtype=torch.float64, device="cuda")
                taub = torch.empty_like(tau)
                p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
                s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                assert L.sgdyn_rollout_backward_noalloc(pm._h, n, steps, dt, K, p(qc), p(qdc), p(tau), p(qTb),
                                                        p(qdTb), p(q0b), p(qd0b), p(taub), s) == N.OK, N.last_error()
                outs["noalloc"] = [x.cpu().numpy() for x in (q0b, qd0b, taub)]
    finally:
        L.sgdyn_rollout_lanes(0, None)
        L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)
    for key in (3, "jit", "noalloc"):
        for a, b in zip(outs[key], outs[1]):
            assert rel(a, b) < 1e-10, key
    if robot.nq_ext > robot.nv:
        assert all((outs[key][0][:, 6] == 0).all() for key in outs)
