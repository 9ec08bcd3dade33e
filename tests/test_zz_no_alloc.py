"""The allocation-free rollout backward (sgdyn_rollout_backward_noalloc).

Callers that cannot enter the device allocator while they run (a real-time control or
planning loop that reserves all its memory at start-up, a plug-in whose host
application owns the GPU memory budget) use this entry point instead of
sgdyn_rollout_backward: it keeps its scratch in a fixed device array inside the library.
This file checks, through the C ABI, that two calls in a row give the same adjoints as
the allocating entry point, that a call needing more scratch than the array holds is
refused before any work, and that a model whose tables are not yet on the device is
refused instead of being uploaded. It sits last in collection order so that a failure
here cannot stop the rest of the suite from running first.
"""
import ctypes

import numpy as np
import pytest

from sapien_gb300 import PinocchioModel, autodiff as ad, synthetic as syn
from sapien_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _model(robot):
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    return pm


def test_noalloc_backward_matches_allocating_entry_point():
    import torch

    robot = syn.arm_with_fingers()
    pm = _model(robot)
    dev = torch.device("cuda", 0)
    pm._prepare(dev)  # model tables on the device before the allocation-free call
    n, T, K, dt = 64, 60, 20, 1.0 / 500
    q0, qd0, _, _ = robot.sample(n, seed=5)
    rng = np.random.default_rng(6)
    tau = torch.from_numpy(rng.normal(scale=5.0, size=(T, n, robot.nv))).to(dev)
    q0t, qd0t = torch.from_numpy(q0).to(dev), torch.from_numpy(qd0).to(dev)
    qT, qdT, qc, qdc = ad.rollout_forward(pm, q0t, qd0t, tau, dt, K)
    qT_bar = torch.from_numpy(rng.normal(size=(n, robot.nq_ext))).to(dev)
    qdT_bar = torch.from_numpy(rng.normal(size=(n, robot.nv))).to(dev)
    ref = ad.rollout_backward(pm, qc, qdc, tau, dt, K, qT_bar, qdT_bar)
    torch.cuda.synchronize()

    L = N.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    # an empty call only looks the array up on this device (the warm-up before a capture)
    rc = L.sgdyn_rollout_backward_noalloc(pm._h, 0, T, dt, K, None, None, None, None, None, None, None, None, stream)
    assert rc == N.OK, N.last_error()
    for call in range(2):  # the shared array keeps the previous call's contents
        q0b = torch.full((n, robot.nq_ext), float("nan"), dtype=torch.float64, device=dev)
        qd0b = torch.full((n, robot.nv), float("nan"), dtype=torch.float64, device=dev)
        taub = torch.full_like(tau, float("nan"))
        rc = L.sgdyn_rollout_backward_noalloc(pm._h, n, T, dt, K, _p(qc), _p(qdc), _p(tau), _p(qT_bar), _p(qdT_bar),
                                              _p(q0b), _p(qd0b), _p(taub), stream)
        assert rc == N.OK, N.last_error()
        torch.cuda.synchronize()
        for got, want in zip((q0b, qd0b, taub), ref):
            g, w = got.cpu().numpy(), want.cpu().numpy()
            assert np.isfinite(g).all()
            assert np.abs(g - w).max() <= 1e-12 * max(np.abs(w).max(), 1e-300), f"call {call}"


def test_noalloc_rejects_oversized_calls_and_unuploaded_models():
    import torch

    robot = syn.arm_with_fingers()
    pm = _model(robot)
    dev = torch.device("cuda", 0)
    L = N.load()
    nb = ctypes.c_int64()
    assert L.sgdyn_rollout_scratch_bytes(pm._h, 1, 20, ctypes.byref(nb)) == N.OK
    too_many = (64 << 20) // nb.value + 1
    dummy = torch.zeros(1, dtype=torch.float64, device=dev)
    rc = L.sgdyn_rollout_backward_noalloc(pm._h, too_many, 10, 0.002, 20, _p(dummy), _p(dummy), _p(dummy), None, None,
                                          _p(dummy), _p(dummy), _p(dummy), None)
    assert rc == N.ERR_RUNTIME
    assert "bytes of scratch" in N.last_error()
    # a batch size whose scratch size overflows int64 is refused, not wrapped around
    rc = L.sgdyn_rollout_backward_noalloc(pm._h, 1 << 61, 10, 0.002, 20, _p(dummy), _p(dummy), _p(dummy), None, None,
                                          _p(dummy), _p(dummy), _p(dummy), None)
    assert rc == N.ERR_RUNTIME
    assert "INT64_MAX" in N.last_error()
    assert L.sgdyn_rollout_scratch_bytes(pm._h, 1 << 61, 20, ctypes.byref(nb)) == N.ERR_RUNTIME
    # a model never uploaded to this device is refused, not uploaded
    fresh = _model(robot)
    rc = L.sgdyn_rollout_backward_noalloc(fresh._h, 4, 10, 0.002, 20, _p(dummy), _p(dummy), _p(dummy), None, None,
                                          _p(dummy), _p(dummy), _p(dummy), None)
    assert rc == N.ERR_RUNTIME
    assert "sgdyn_model_upload" in N.last_error()
