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
    shape, table = autotune.tune_batch(batch, q, qd, qdd, tau, OPS_DYNAMICS, candidates=[(1, 1, 0), (4, 1, 0), (2, 2, 1)])
    assert len(table) == 3 and tuple(shape) in {(1, 1, 0), (4, 1, 0), (2, 2, 1)}
    shape2, _ = autotune.tune_batch(batch, q, qd, qdd, tau, OPS_DYNAMICS)  # served from the cache
    assert tuple(shape2) == tuple(shape)
    out = batch.step(q, qd, qdd, tau)
    for a, b in zip(valid_blocks(batch, out), ref):
        assert torch.equal(a, b)
