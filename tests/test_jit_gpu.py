"""The model-specialised (run-time compiled) sweep against the generic kernel and the
oracle. Tolerances as in test_parity_gpu.py; specialised vs generic within 1e-13."""
import ctypes

import numpy as np
import pytest

from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel, synthetic as syn
from sapien_gb300 import _native as N

pytestmark = pytest.mark.gpu


def jit_config(enable, min_n):
    e, m = ctypes.c_int(), ctypes.c_int64()
    N.check(N.load().sgdyn_jit_config(enable, min_n, ctypes.byref(e), ctypes.byref(m)))
    return e.value, m.value


@pytest.fixture(autouse=True)
def any_tree_size():
    """Specialise trees of every size here (the default limit keeps large trees generic)."""
    old = ctypes.c_int()
    N.check(N.load().sgdyn_jit_max_joints(64, ctypes.byref(old)))
    yield
    N.check(N.load().sgdyn_jit_max_joints(old.value, None))


def rel_per_env(g, o):
    g = g.reshape(g.shape[0], -1)
    o = o.reshape(o.shape[0], -1)
    return (np.abs(g - o).max(axis=1) / np.maximum(np.abs(o).max(axis=1), 1e-300)).max()


@pytest.mark.parametrize("name", ["arm9", "arm9_sapien", "humanoid", "quadruped", "mixed"])
def test_specialised_sweep_matches_generic_and_oracle(name):
    import torch

    robot = {"arm9": syn.arm_with_fingers(), "arm9_sapien": syn.arm_with_fingers(sapien_style=True),
             "humanoid": syn.humanoid(), "quadruped": syn.quadruped(),
             "mixed": syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                          "continuous", "prismatic"])}[name]
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    pm.set_lanes(1)  # one lane per environment: the specialised kernel's domain
    q, qd, qdd, tau = (torch.from_numpy(a).cuda() for a in robot.sample(100, seed=23))
    old = jit_config(-1, -1)
    try:
        jit_config(0, -1)
        gen = {k: v.cpu().numpy() for k, v in pm.step_batched(q, qd, qdd, tau).items()}
        jit_config(1, 0)
        assert N.load().sgdyn_jit_prepare(pm._h, N.OP_ALL) == 0, N.last_error()
        spec = {k: v.cpu().numpy() for k, v in pm.step_batched(q, qd, qdd, tau).items()}
        single = pm.compute_forward_dynamics_batched(q, qd, tau).cpu().numpy()
    finally:
        jit_config(*old)
    for k in gen:
        assert rel_per_env(spec[k], gen[k]) <= 1e-13, k
    # forward dynamics alone may run on three lanes per environment (another summation order)
    assert rel_per_env(single, gen["qacc"]) <= 1e-12
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    r = o.batch_step(*(x.cpu().numpy() for x in (q, qd, qdd, tau)), ops=4 | 8 | 16)
    assert rel_per_env(spec["qf"], r["tau"]) <= 1e-10
    assert rel_per_env(spec["qacc"], r["qdd"]) <= 1e-8
    assert rel_per_env(spec["mass_matrix"], r["M"]) <= 1e-10


@pytest.mark.parametrize("name", ["arm9", "mixed"])
def test_specialised_rollout_matches_generic(name):
    """Checkpointed rollout: the model-specialised forward kernel reproduces the generic one
    (same operation order, tables folded to constants) to 1e-12 relative, and so do the
    gradients the (generic) backward computes from its checkpoints."""
    import torch

    from sapien_gb300 import autodiff as AD

    robot = {"arm9": syn.arm_with_fingers(),
             "mixed": syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                          "continuous", "prismatic"])}[name]
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    n, T, K, dt = 96, 30, 7, 2e-3
    q, qd, _, tau = (torch.from_numpy(a).cuda() for a in robot.sample(n, seed=5))
    taus = (0.2 * tau).unsqueeze(0).repeat(T, 1, 1).contiguous()
    g = torch.Generator(device="cpu").manual_seed(3)
    qTb = torch.randn(n, pm.nq_ext, generator=g, dtype=torch.float64).cuda()
    qdTb = torch.randn(n, pm.nv, generator=g, dtype=torch.float64).cuda()

    def run():
        qT, qdT, qc, qdc = AD.rollout_forward(pm, q, qd, taus, dt, K)
        q0b, qd0b, taub = AD.rollout_backward(pm, qc, qdc, taus, dt, K, qTb, qdTb)
        return [x.cpu().numpy() for x in (qT, qdT, qc, qdc, q0b, qd0b, taub)]

    old = jit_config(-1, -1)
    try:
        jit_config(0, -1)
        gen = run()
        jit_config(1, 0)
        spec = run()
    finally:
        jit_config(*old)
    for a, b in zip(spec, gen):
        a2, b2 = a.reshape(-1, a.shape[-1]), b.reshape(-1, b.shape[-1])
        assert rel_per_env(a2, b2) <= 1e-12


@pytest.mark.parametrize("name", ["arm9", "humanoid"])
def test_specialised_vjp_matches_generic(name):
    """RNEA / ABA vector-Jacobian products: the model-specialised kernels reproduce the
    generic ones (same operations, tables folded to constants)."""
    import torch

    from sapien_gb300 import autodiff as AD

    robot = {"arm9": syn.arm_with_fingers(), "humanoid": syn.humanoid()}[name]
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    q, qd, qdd, tau = (torch.from_numpy(a).cuda() for a in robot.sample(64, seed=7))

    def run():
        r = AD.inverse_dynamics_vjp(pm, q, qd, qdd, tau) + AD.forward_dynamics_vjp(pm, q, qd, tau, qdd)
        return [x.cpu().numpy() for x in r if x is not None]

    old = jit_config(-1, -1)
    try:
        jit_config(0, -1)
        gen = run()
        jit_config(1, 0)
        for kind in (-2, -3):
            assert N.load().sgdyn_jit_prepare(pm._h, kind) == 0, N.last_error()
        spec = run()
    finally:
        jit_config(*old)
    for a, b in zip(spec, gen):
        assert rel_per_env(a, b) <= 1e-13


@pytest.mark.parametrize("name,lanes", [("humanoid", 4), ("humanoid", 2), ("quadruped", 2), ("quadruped", 4)])
def test_role_warp_team_sweep_matches_generic_team_and_oracle(name, lanes):
    """A model run with teams of L lanes: the specialised sweep with one warp per role of the
    team (block of L warps, team sums through shared memory) against the generic team kernel
    (sums by warp shuffles) and the oracle, for the five ops and for CRBA + RNEA + ABA; 77
    environments, so the last block is partly empty."""
    import torch

    robot = {"humanoid": syn.humanoid(), "quadruped": syn.quadruped()}[name]
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    pm.set_lanes(lanes)
    q, qd, qdd, tau = (torch.from_numpy(a).cuda() for a in robot.sample(77, seed=29))
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    r = o.batch_step(*(x.cpu().numpy() for x in (q, qd, qdd, tau)), ops=4 | 8 | 16)
    for ops in (N.OP_ALL, N.OP_MASS_MATRIX | N.OP_INVERSE_DYNAMICS | N.OP_FORWARD_DYNAMICS):
        outs = {}
        old = jit_config(-1, -1)
        try:
            for jit in (0, 1):
                jit_config(jit, 0)
                outs[jit] = {k: v.cpu().numpy() for k, v in pm.step_batched(q, qd, qdd, tau, ops=ops).items()}
        finally:
            jit_config(*old)
        for k in outs[0]:
            assert rel_per_env(outs[1][k], outs[0][k]) <= (1e-11 if k == "qacc" else 1e-13), (ops, k)
        assert rel_per_env(outs[1]["mass_matrix"], r["M"]) <= 1e-10
        assert rel_per_env(outs[1]["qf"], r["tau"]) <= 1e-10
        assert rel_per_env(outs[1]["qacc"], r["qdd"]) <= 1e-8
