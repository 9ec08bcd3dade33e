"""Heterogeneous persistent-batch kernel: parity with the CPU oracle per model, CUDA-graph
replay, tile orders and autotuned launch shapes (all must leave results unchanged)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel, synthetic as syn
from sapien_gb300.hetero import OPS_DYNAMICS, HeteroBatch

pytestmark = pytest.mark.gpu


def rel_per_env(g, o):
    g = g.reshape(g.shape[0], -1)
    o = o.reshape(o.shape[0], -1)
    return (np.abs(g - o).max(axis=1) / np.maximum(np.abs(o).max(axis=1), 1e-300)).max()


def setup(n=300, seed=0):
    robots, moe = syn.hetero_mix(n, seed=seed)
    models, oracles, inputs = [], [], []
    for k, r in enumerate(robots):
        pm = PinocchioModel(r.urdf, [0, 0, -9.81])
        pm.set_joint_order(r.joint_names)
        pm.set_link_order(r.link_names)
        o = Oracle(r.urdf)
        o.set_joint_order(r.joint_names)
        o.set_link_order(r.link_names)
        models.append(pm)
        oracles.append(o)
        inputs.append(r.sample(int((moe == k).sum()), seed=10 + k))
    batch = HeteroBatch(models, moe)
    q = batch.pad_q([x[0] for x in inputs])
    qd = batch.pad_v([x[1] for x in inputs])
    qdd = batch.pad_v([x[2] for x in inputs])
    tau = batch.pad_v([x[3] for x in inputs])
    return batch, oracles, inputs, (q, qd, qdd, tau)


def check_against_oracle(batch, oracles, inputs, out):
    for k, (o, (q, qd, qdd, tau)) in enumerate(zip(oracles, inputs)):
        r = o.batch_step(q, qd, qdd, tau, ops=4 | 8 | 16, nthreads=8)
        assert rel_per_env(batch.unpad_v(out["qf"], k).cpu().numpy(), r["tau"]) <= 1e-10
        assert rel_per_env(batch.unpad_v(out["qacc"], k).cpu().numpy(), r["qdd"]) <= 1e-8
        assert rel_per_env(batch.unpad_M(out["mass_matrix"], k).cpu().numpy(), r["M"]) <= 1e-10


def test_hetero_step_matches_oracle():
    batch, oracles, inputs, (q, qd, qdd, tau) = setup()
    out = batch.step(q, qd, qdd, tau, OPS_DYNAMICS)
    check_against_oracle(batch, oracles, inputs, out)


def valid_blocks(batch, out):
    """Per-model valid parts of the padded outputs (the padding is unspecified)."""
    res = []
    for k in range(len(batch.models)):
        res += [batch.unpad_v(out["qf"], k), batch.unpad_v(out["qacc"], k), batch.unpad_M(out["mass_matrix"], k)]
    return res


def test_hetero_graph_replay_orders_and_launch_shapes_agree():
    import torch

    batch, oracles, inputs, (q, qd, qdd, tau) = setup(n=200, seed=3)
    ref = [v.clone() for v in valid_blocks(batch, batch.step(q, qd, qdd, tau))]
    g = batch.capture(q, qd, qdd, tau, steps=3)
    for v in g.outputs.values():
        v.fill_(float("nan"))
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(valid_blocks(batch, g.outputs), ref):
        assert torch.equal(a, b)
    for shape in ((1, 1, 1), (2, 4, 0), (8, 2, 1)):
        batch.set_launch(*shape)
        out = batch.step(q, qd, qdd, tau)
        for a, b in zip(valid_blocks(batch, out), ref):
            assert torch.equal(a, b), shape


def test_autotuner_picks_a_shape_and_keeps_results(tmp_path, monkeypatch):
    import torch

    from sapien_gb300 import autotune

    monkeypatch.setenv("SGDYN_AUTOTUNE_CACHE", str(tmp_path))
    batch, oracles, inputs, (q, qd, qdd, tau) = setup(n=160, seed=4)
    ref = [v.clone() for v in valid_blocks(batch, batch.step(q, qd, qdd, tau))]
    cands = [(1, 1, 0), (4, 1, 0), (2, 2, 1)]
    shape, table = autotune.tune_batch(batch, q, qd, qdd, tau, OPS_DYNAMICS, candidates=cands, lane_candidates=(1,))
    assert len(table) == 3 and tuple(shape) in set(cands)
    shape2, _ = autotune.tune_batch(batch, q, qd, qdd, tau, OPS_DYNAMICS, lane_candidates=(1,))  # from the cache
    assert tuple(shape2) == tuple(shape)
    out = batch.step(q, qd, qdd, tau)
    for a, b in zip(valid_blocks(batch, out), ref):
        assert torch.equal(a, b)
    # with lanes per environment in the search: a valid choice, results equal to rounding
    shape3, table3 = autotune.tune_batch(batch, q, qd, qdd, tau, OPS_DYNAMICS, candidates=cands)
    assert all(L in (1, 2, 4, 8) for L in batch.lanes) and len(table3) == 3 + 3 * 3 * len(batch.models)
    lanes = list(batch.lanes)
    batch.set_lanes([1] * len(batch.models))
    batch.set_lanes(lanes)
    out = batch.step(q, qd, qdd, tau)
    for a, b in zip(valid_blocks(batch, out), ref):
        assert rel_per_env(a.cpu().numpy(), b.cpu().numpy()) <= 1e-11


def test_lanes_per_environment_agree_with_one_lane():
    """Teams of 2, 4 or 8 lanes per environment (trunk on every lane, subtrees split among
    them, branch contributions summed with warp shuffles) give the one-lane results to
    rounding, write every output entry exactly where one lane does, and match the oracle."""
    import torch

    from sapien_gb300 import _native as N

    batch, oracles, inputs, (q, qd, qdd, tau) = setup(n=333, seed=5)

    def run(lanes):
        batch.set_lanes(lanes)
        out = batch.alloc_outputs(N.OP_ALL)
        for v in out.values():
            v.fill_(float("nan"))
        batch.step(q, qd, qdd, tau, N.OP_ALL, out)
        torch.cuda.synchronize()
        blocks = []
        for k, m in enumerate(batch.models):
            idx = torch.as_tensor(np.nonzero(batch.model_of_env == k)[0], device=q.device)
            blocks += [out["qf"][idx, : m.nv], out["qacc"][idx, : m.nv], out["mass_matrix"][idx, : m.nv * m.nv],
                       out["jacobian"][idx, : 6 * m.nv], out["link_poses"][idx, : 7 * m._nlinks]]
        return [b.cpu().numpy() for b in blocks], out

    ref, _ = run([1, 1, 1])
    for lanes in ([1, 4, 4], [2, 2, 2], [8, 8, 8], [4, 8, 2]):
        got, out = run(lanes)
        for a, b in zip(got, ref):
            assert not np.isnan(a).any(), lanes
            assert rel_per_env(a, b) <= 1e-11, lanes
    check_against_oracle(batch, oracles, inputs, out)


def test_hetero_rollout_graph_matches_oracle():
    """A whole heterogeneous rollout (ABA + semi-implicit Euler per step, free flyers on
    SE(3)) captured as one CUDA graph matches the oracle's step-by-step rollout."""
    import torch

    batch, oracles, inputs, (q, qd, qdd, tau) = setup(n=150, seed=7)
    batch.set_lanes([1, 2, 4])
    tau = 0.1 * tau
    steps, dt = 12, 2e-3
    ref = []
    for k, (o, (qk, qdk, _, tk)) in enumerate(zip(oracles, inputs)):
        qk, qdk, tk = qk.copy(), qdk.copy(), 0.1 * tk
        for _ in range(steps):
            for e in range(qk.shape[0]):
                a = o.compute_forward_dynamics(qk[e], qdk[e], tk[e])
                qdk[e] = qdk[e] + dt * a
                qk[e] = o.integrate(qk[e], dt * qdk[e])
        ref.append((qk, qdk))
    g = batch.capture_rollout(q, qd, tau, dt, steps)
    g.replay()
    torch.cuda.synchronize()
    for k, (qk, qdk) in enumerate(ref):
        m = batch.models[k]
        idx = torch.as_tensor(np.nonzero(batch.model_of_env == k)[0], device=q.device)
        gq = q[idx, : m.nq_ext].cpu().numpy()
        gqd = qd[idx, : m.nv].cpu().numpy()
        assert rel_per_env(gq, qk) <= 1e-9
        assert rel_per_env(gqd, qdk) <= 1e-8


def test_fused_rollout_step_equals_step_then_integrate():
    """sgdyn_batch_step_integrate (ABA and the Euler update in one launch) gives the same
    q, qd and qacc bit for bit as the two-launch sequence, one lane and teams alike."""
    import torch

    from sapien_gb300 import _native as N

    batch, oracles, inputs, (q, qd, qdd, tau) = setup(n=260, seed=9)
    tau = 0.1 * tau
    for lanes in ([1, 1, 1], [1, 2, 4]):
        batch.set_lanes(lanes)
        qa, qda, qb, qdb = q.clone(), qd.clone(), q.clone(), qd.clone()
        oa, ob = batch.alloc_outputs(N.OP_FORWARD_DYNAMICS), batch.alloc_outputs(N.OP_FORWARD_DYNAMICS)
        for _ in range(5):
            batch.rollout_step(qa, qda, tau, 2e-3, oa)
            batch.step(qb, qdb, None, tau, N.OP_FORWARD_DYNAMICS, ob)
            batch.integrate(qb, qdb, ob["qacc"], 2e-3)
        torch.cuda.synchronize()
        for k, m in enumerate(batch.models):
            idx = torch.as_tensor(np.nonzero(batch.model_of_env == k)[0], device=q.device)
            assert torch.equal(qa[idx, : m.nq_ext], qb[idx, : m.nq_ext]), lanes
            assert torch.equal(qda[idx, : m.nv], qdb[idx, : m.nv]), lanes
            assert torch.equal(oa["qacc"][idx, : m.nv], ob["qacc"][idx, : m.nv]), lanes


@pytest.mark.parametrize("lanes", [(1, 1, 1), (1, 2, 4), (2, 2, 4)])
def test_hetero_full_size_mix_matches_oracle(lanes):
    """The heterogeneous workload at its full size: 8192 robots (50 / 30 / 20 % 6-DoF arms,
    18-DoF quadrupeds, 35-DoF humanoids), RNEA + ABA + CRBA from a CUDA-graph replay with
    the lane counts the autotuner picks for this mix, every environment against the oracle."""
    import torch

    batch, oracles, inputs, (q, qd, qdd, tau) = setup(n=8192, seed=0)
    batch.set_lanes(list(lanes))
    g = batch.capture(q, qd, qdd, tau, steps=2)
    g.replay()
    torch.cuda.synchronize()
    check_against_oracle(batch, oracles, inputs, g.outputs)


def test_hetero_role_warp_sweeps_match_generic_and_graph():
    """With run-time compilation on, the models run with teams take the specialised
    one-warp-per-role sweep (a launch each, on side streams beside the persistent kernel,
    which keeps the one-lane models' tiles): results equal the generic team path to rounding
    and the oracle within tolerance, a CUDA-graph replay equals the direct step bit for bit,
    and three rollout steps (ABA with the Euler update fused into each launch) equal the
    generic path's to rounding."""
    import ctypes

    import torch

    from sapien_gb300 import _native as N

    batch, oracles, inputs, (q, qd, qdd, tau) = setup(n=600, seed=5)
    batch.set_lanes([1, 2, 4])
    L = N.load()
    old_jit, old_min = ctypes.c_int(), ctypes.c_int64()
    L.sgdyn_jit_config(-1, -1, ctypes.byref(old_jit), ctypes.byref(old_min))
    try:
        L.sgdyn_jit_config(0, 0, None, None)
        generic = batch.step(q, qd, qdd, tau, OPS_DYNAMICS)
        L.sgdyn_jit_config(1, 0, None, None)
        roles = batch.step(q, qd, qdd, tau, OPS_DYNAMICS)
        check_against_oracle(batch, oracles, inputs, roles)
        g = batch.capture(q, qd, qdd, tau, steps=2)
        g.replay()
        torch.cuda.synchronize()
    finally:
        L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)
    for a, b in zip(valid_blocks(batch, roles), valid_blocks(batch, generic)):
        assert rel_per_env(a.cpu().numpy(), b.cpu().numpy()) <= 1e-11
    for a, b in zip(valid_blocks(batch, g.outputs), valid_blocks(batch, roles)):
        assert torch.equal(a, b)
    # the rollout step (ABA, then the semi-implicit Euler update fused into each launch)
    states = {}
    try:
        for jit in (0, 1):
            L.sgdyn_jit_config(jit, 0, None, None)
            qs, qds = q.clone(), qd.clone()
            out = batch.alloc_outputs(N.OP_FORWARD_DYNAMICS)
            for _ in range(3):
                batch.rollout_step(qs, qds, tau, 1.0 / 500, out)
            torch.cuda.synchronize()
            states[jit] = (qs, qds)
    finally:
        L.sgdyn_jit_config(old_jit.value, old_min.value, None, None)
    for a, b in zip(states[1], states[0]):  # q, qd (padding untouched by both)
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.abs(a - b).max() <= 1e-11 * max(np.abs(b).max(), 1.0)
