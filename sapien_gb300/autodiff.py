"""Differentiable dynamics on top of the adjoint kernels.

* ``inverse_dynamics(model, q, qd, qdd)`` / ``forward_dynamics(model, q, qd, tau)`` /
  ``link_positions(model, q)`` / ``link_poses_rt(model, q)``: ``torch.autograd.Function``
  wrappers whose backward passes call the hand-written adjoint kernels (RNEA adjoint,
  ABA adjoint = M^-1 solve + RNEA adjoint, link-pose adjoint).
* ``rollout(model, q0, qd0, tau, dt, checkpoint_every)``: a semi-implicit Euler rollout
  (qd += dt ABA(q, qd, tau_t); q += dt qd) run by one fused kernel that records only q / qd
  every ``checkpoint_every`` steps; its backward recomputes one segment at a time.
* ``rnea_derivatives`` / ``aba_derivatives``: dense tangent-space derivative matrices.

The reference has no derivative API (Pinocchio is built without autodiff,
pinocchio/cmake/pinocchio.cmake:4); these are additions. Gradients with respect to q are
tangent-space gradients; for models with a free-flyer joint q has 7 coordinates per free
flyer but its tangent has 6, so the autograd wrappers reject such models (use the dense
derivative functions, which return tangent-space matrices).
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _f64(t, cols, what):
    if t.dtype != torch.float64 or not t.is_cuda:
        raise TypeError(f"{what} must be a float64 CUDA tensor")
    if t.dim() != 2 or t.shape[1] != cols:
        raise RuntimeError(f"{what} must have shape [N, {cols}], got {tuple(t.shape)}")
    return t.contiguous()


def _require_no_free_flyer(model):
    if model.nq_ext != model.nv:
        raise NotImplementedError("autograd through q needs q and its tangent to coincide (no free-flyer joint); "
                                  "use rnea_derivatives / aba_derivatives for floating-base models")


# ---- raw adjoint calls -----------------------------------------------------------
def inverse_dynamics_vjp(model, q, qd, qdd, tau_bar):
    """(q_bar, qd_bar, qdd_bar) = tau_bar^T d RNEA / d(q, qd, qdd)."""
    model._require_order()
    q, qd, qdd, tb = (_f64(q, model.nq_ext, "q"), _f64(qd, model.nv, "qd"), _f64(qdd, model.nv, "qdd"),
                      _f64(tau_bar, model.nv, "tau_bar"))
    dev = q.device
    outs = [torch.empty_like(tb) for _ in range(3)]
    model._prepare(dev)
    with torch.cuda.device(dev):
        N.check(N.load().sgdyn_compute_inverse_dynamics_vjp(model._h, q.shape[0], _p(q), _p(qd), _p(qdd), _p(tb),
                                                             *[_p(o) for o in outs], N.ENV_MAJOR, _stream(dev)))
    return tuple(outs)


def forward_dynamics_vjp(model, q, qd, tau, qdd_bar):
    """(q_bar, qd_bar, tau_bar) = qdd_bar^T d ABA / d(q, qd, tau)."""
    model._require_order()
    q, qd, tau, qb = (_f64(q, model.nq_ext, "q"), _f64(qd, model.nv, "qd"), _f64(tau, model.nv, "tau"),
                      _f64(qdd_bar, model.nv, "qdd_bar"))
    dev = q.device
    outs = [torch.empty_like(qb) for _ in range(3)]
    model._prepare(dev)
    with torch.cuda.device(dev):
        N.check(N.load().sgdyn_compute_forward_dynamics_vjp(model._h, q.shape[0], _p(q), _p(qd), _p(tau), _p(qb),
                                                             *[_p(o) for o in outs], N.ENV_MAJOR, _stream(dev)))
    return tuple(outs)


def forward_kinematics_vjp(model, q, pos_bar, rot_bar=None):
    """q_bar from adjoints of link positions [N, L, 3] and (optionally) rotations [N, L, 3, 3]."""
    model._require_order()
    q = _f64(q, model.nq_ext, "q")
    n, L = q.shape[0], model.nlinks
    pb = _f64(pos_bar.reshape(n, 3 * L), 3 * L, "pos_bar")
    rb = _f64(rot_bar.reshape(n, 9 * L), 9 * L, "rot_bar") if rot_bar is not None else None
    dev = q.device
    out = torch.empty(n, model.nv, dtype=torch.float64, device=dev)
    model._prepare(dev)
    with torch.cuda.device(dev):
        N.check(N.load().sgdyn_compute_forward_kinematics_vjp(model._h, n, _p(q), _p(pb), _p(rb), _p(out),
                                                               N.ENV_MAJOR, _stream(dev)))
    return out


def _derivs(model, fn, q, qd, x):
    model._require_order()
    q, qd, x = _f64(q, model.nq_ext, "q"), _f64(qd, model.nv, "qd"), _f64(x, model.nv, "x")
    n, nv, dev = q.shape[0], model.nv, q.device
    outs = [torch.empty(n, nv, nv, dtype=torch.float64, device=dev) for _ in range(3)]
    model._prepare(dev)
    with torch.cuda.device(dev):
        N.check(fn(model._h, n, _p(q), _p(qd), _p(x), *[_p(o) for o in outs], N.ENV_MAJOR, _stream(dev)))
    return tuple(outs)


def rnea_derivatives(model, q, qd, qdd):
    """(dtau/dq, dtau/dqd, dtau/dqdd = M), each [N, nv, nv]; q-derivative in tangent space."""
    return _derivs(model, N.load().sgdyn_compute_rnea_derivatives, q, qd, qdd)


def aba_derivatives(model, q, qd, tau):
    """(dqdd/dq, dqdd/dqd, dqdd/dtau = M^-1), each [N, nv, nv]."""
    return _derivs(model, N.load().sgdyn_compute_aba_derivatives, q, qd, tau)


# ---- autograd functions ----------------------------------------------------------
class _InverseDynamics(torch.autograd.Function):
    @staticmethod
    def forward(ctx, model, q, qd, qdd):
        ctx.model = model
        ctx.save_for_backward(q, qd, qdd)
        return model.compute_inverse_dynamics_batched(q, qd, qdd)

    @staticmethod
    def backward(ctx, tau_bar):
        q, qd, qdd = ctx.saved_tensors
        qb, qdb, qddb = inverse_dynamics_vjp(ctx.model, q, qd, qdd, tau_bar.contiguous())
        return None, qb, qdb, qddb


class _ForwardDynamics(torch.autograd.Function):
    @staticmethod
    def forward(ctx, model, q, qd, tau):
        ctx.model = model
        ctx.save_for_backward(q, qd, tau)
        return model.compute_forward_dynamics_batched(q, qd, tau)

    @staticmethod
    def backward(ctx, qdd_bar):
        q, qd, tau = ctx.saved_tensors
        qb, qdb, tb = forward_dynamics_vjp(ctx.model, q, qd, tau, qdd_bar.contiguous())
        return None, qb, qdb, tb


def _quat_to_R(qwxyz):
    w, x, y, z = qwxyz.unbind(-1)
    return torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], dim=-1).reshape(*qwxyz.shape[:-1], 3, 3)


class _LinkPoses(torch.autograd.Function):
    @staticmethod
    def forward(ctx, model, q):
        ctx.model = model
        ctx.save_for_backward(q)
        poses = model.compute_forward_kinematics_batched(q)
        return poses[..., :3].contiguous(), _quat_to_R(poses[..., 3:7])

    @staticmethod
    def backward(ctx, pos_bar, rot_bar):
        (q,) = ctx.saved_tensors
        if pos_bar is None:
            pos_bar = torch.zeros(q.shape[0], ctx.model.nlinks, 3, dtype=q.dtype, device=q.device)
        qb = forward_kinematics_vjp(ctx.model, q, pos_bar.contiguous(),
                                    rot_bar.contiguous() if rot_bar is not None else None)
        return None, qb


def inverse_dynamics(model, q, qd, qdd):
    """Differentiable batched RNEA: [N, nv] tensors -> tau [N, nv]."""
    _require_no_free_flyer(model)
    return _InverseDynamics.apply(model, q, qd, qdd)


def forward_dynamics(model, q, qd, tau):
    """Differentiable batched ABA: [N, nv] tensors -> qdd [N, nv]."""
    _require_no_free_flyer(model)
    return _ForwardDynamics.apply(model, q, qd, tau)


def link_poses_rt(model, q):
    """Differentiable link poses: (positions [N, L, 3], rotations [N, L, 3, 3])."""
    _require_no_free_flyer(model)
    return _LinkPoses.apply(model, q)


def link_positions(model, q):
    return link_poses_rt(model, q)[0]


# ---- rollout -----------------------------------------------------------------------
def rollout_forward(model, q0, qd0, tau, dt, checkpoint_every=None):
    """Run the fused rollout kernel. tau: [T, N, nv]. Returns (qT, qdT, q_ckpt, qd_ckpt);
    the checkpoints are None when checkpoint_every is None (plain forward)."""
    model._require_order()
    q0, qd0 = _f64(q0, model.nq_ext, "q0"), _f64(qd0, model.nv, "qd0")
    n, dev = q0.shape[0], q0.device
    if tau.dim() != 3 or tau.shape[1] != n or tau.shape[2] != model.nv or tau.dtype != torch.float64:
        raise RuntimeError(f"tau must be float64 [T, {n}, {model.nv}]")
    tau = tau.contiguous()
    T = tau.shape[0]
    qT, qdT = torch.empty_like(q0), torch.empty_like(qd0)
    qc = qdc = None
    K = checkpoint_every or max(T, 1)
    if checkpoint_every:
        C = (T + K - 1) // K
        qc = torch.empty(C, n, model.nq_ext, dtype=torch.float64, device=dev)
        qdc = torch.empty(C, n, model.nv, dtype=torch.float64, device=dev)
    model._prepare(dev)
    with torch.cuda.device(dev):
        N.check(N.load().sgdyn_rollout_forward(model._h, n, T, float(dt), _p(q0), _p(qd0), _p(tau), int(K), _p(qc),
                                               _p(qdc), _p(qT), _p(qdT), _stream(dev)))
    return qT, qdT, qc, qdc


def rollout_backward(model, q_ckpt, qd_ckpt, tau, dt, checkpoint_every, qT_bar=None, qdT_bar=None,
                     max_scratch_bytes=4 << 30):
    """Reverse pass: returns (q0_bar, qd0_bar, tau_bar [T, N, nv]).

    The scratch holds as many checkpoint segments' intermediates as fit in
    ``max_scratch_bytes`` (at least one): that many segments are recomputed in parallel."""
    n, dev = q_ckpt.shape[1], q_ckpt.device
    T = tau.shape[0]
    nb = ctypes.c_int64()
    L = N.load()
    N.check(L.sgdyn_rollout_scratch_bytes(model._h, n, int(checkpoint_every), ctypes.byref(nb)))
    nseg = (T + int(checkpoint_every) - 1) // int(checkpoint_every)
    segs = max(1, min(nseg, int(max_scratch_bytes) // max(nb.value, 1)))
    scratch = torch.empty(max(segs * nb.value // 8, 1), dtype=torch.float64, device=dev)
    q0b = torch.empty(n, model.nq_ext, dtype=torch.float64, device=dev)
    qd0b = torch.empty(n, model.nv, dtype=torch.float64, device=dev)
    taub = torch.empty_like(tau)
    qTb = qT_bar.contiguous() if qT_bar is not None else None
    qdTb = qdT_bar.contiguous() if qdT_bar is not None else None
    model._prepare(dev)
    with torch.cuda.device(dev):
        N.check(L.sgdyn_rollout_backward(model._h, n, T, float(dt), int(checkpoint_every), _p(q_ckpt), _p(qd_ckpt),
                                         _p(tau.contiguous()), _p(qTb), _p(qdTb), _p(q0b), _p(qd0b), _p(taub),
                                         _p(scratch), scratch.numel() * 8, _stream(dev)))
    return q0b, qd0b, taub


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, model, q0, qd0, tau, dt, checkpoint_every):
        qT, qdT, qc, qdc = rollout_forward(model, q0, qd0, tau, dt, checkpoint_every)
        ctx.model, ctx.dt, ctx.K = model, dt, checkpoint_every
        ctx.save_for_backward(qc, qdc, tau)
        return qT, qdT

    @staticmethod
    def backward(ctx, qT_bar, qdT_bar):
        qc, qdc, tau = ctx.saved_tensors
        q0b, qd0b, taub = rollout_backward(ctx.model, qc, qdc, tau, ctx.dt, ctx.K, qT_bar, qdT_bar)
        return None, q0b, qd0b, taub, None, None


def rollout(model, q0, qd0, tau, dt, checkpoint_every=20):
    """Differentiable rollout: returns (qT, qdT). Gradients flow to q0, qd0 and tau."""
    _require_no_free_flyer(model)
    return _Rollout.apply(model, q0, qd0, tau, float(dt), int(checkpoint_every))
