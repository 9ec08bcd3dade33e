"""Differentiable dynamics on top of the adjoint kernels.

* ``inverse_dynamics(model, q, qd, qdd)`` / ``forward_dynamics(model, q, qd, tau)`` /
  ``link_positions(model, q)`` / ``link_poses_rt(model, q)``: ``torch.autograd.Function``
  wrappers whose backward passes call the hand-written adjoint kernels (RNEA adjoint,
  ABA adjoint = M^-1 solve + RNEA adjoint, link-pose adjoint).
* ``rollout(model, q0, qd0, tau, dt, checkpoint_every)``: a semi-implicit Euler rollout
  (qd += dt ABA(q, qd, tau_t); q <- q (+) dt qd, a free-flyer root on SE(3)) run by one fused kernel that records only q / qd
  every ``checkpoint_every`` steps; its backward recomputes one segment at a time.
* ``rnea_derivatives`` / ``aba_derivatives``: dense tangent-space derivative matrices.

The reference has no derivative API (Pinocchio is built without autodiff,
pinocchio/cmake/pinocchio.cmake:4); these are additions. The kernels return gradients with
respect to q in the tangent space. For a free-flyer joint (q block x y z qx qy qz qw,
tangent block = body twist, q exp6(eps)) the autograd wrappers turn them into coordinate
gradients through the chart eps = (R^T dp, 2 vec(quat^-1 * dquat)): the position gradient
is R g_lin and the quaternion gradient has no component along the quaternion itself, so it
gives the exact directional derivative along every perturbation that keeps the quaternion
unit. Gradients arriving for a free flyer's coordinates are mapped back the other way
(``coordinate_to_tangent_grad``). The raw ``*_vjp`` functions and the dense derivatives
stay in the tangent space.
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


# ---- free-flyer coordinates and tangents -------------------------------------------
def _joint_blocks(model):
    """(kind, q column, v column) of every joint in external order."""
    out, qc, vc = [], 0, 0
    for kind in model._kinds:
        out.append((kind, qc, vc))
        ff = kind == 4  # free flyer
        qc += 7 if ff else 1
        vc += 6 if ff else 1
    return out


def _ff_frame(q, qc):
    x, y, z, w = (q[:, qc + 3 + k] for k in range(4))
    R = _quat_to_R(torch.stack([w, x, y, z], dim=-1))
    return R, torch.stack([x, y, z], dim=-1), w


def tangent_to_coordinate_grad(model, q, g):
    """[N, nv] tangent-space gradient at q -> [N, nq_ext] coordinate gradient."""
    if model.nq_ext == model.nv:
        return g
    out = torch.zeros(q.shape[0], model.nq_ext, dtype=g.dtype, device=g.device)
    for kind, qc, vc in _joint_blocks(model):
        if kind != 4:
            out[:, qc] = g[:, vc]
            continue
        R, v, w = _ff_frame(q, qc)
        glin, gw = g[:, vc:vc + 3], g[:, vc + 3:vc + 6]
        out[:, qc:qc + 3] = (R @ glin.unsqueeze(-1)).squeeze(-1)
        out[:, qc + 3:qc + 6] = 2 * (w.unsqueeze(-1) * gw + torch.cross(v, gw, dim=-1))
        out[:, qc + 6] = -2 * (v * gw).sum(-1)
    return out


def coordinate_to_tangent_grad(model, q, gc):
    """[N, nq_ext] gradient with respect to q's coordinates -> [N, nv] tangent gradient (the
    transpose of the chart's derivative d q exp6(eps) / d eps at eps = 0)."""
    if model.nq_ext == model.nv:
        return gc
    out = torch.zeros(q.shape[0], model.nv, dtype=gc.dtype, device=gc.device)
    for kind, qc, vc in _joint_blocks(model):
        if kind != 4:
            out[:, vc] = gc[:, qc]
            continue
        R, v, w = _ff_frame(q, qc)
        gp, gv, gw = gc[:, qc:qc + 3], gc[:, qc + 3:qc + 6], gc[:, qc + 6]
        out[:, vc:vc + 3] = (R.transpose(-1, -2) @ gp.unsqueeze(-1)).squeeze(-1)
        out[:, vc + 3:vc + 6] = 0.5 * (w.unsqueeze(-1) * gv + torch.cross(gv, v, dim=-1) - v * gw.unsqueeze(-1))
    return out


def _tangent_in_q_layout(model, g):
    """[N, nv] tangent vector -> [N, nq_ext] array laid out as the rollout kernels take a
    configuration adjoint (a free flyer's six tangent entries in the first six slots of its
    seven)."""
    if model.nq_ext == model.nv:
        return g.contiguous()
    out = torch.zeros(g.shape[0], model.nq_ext, dtype=g.dtype, device=g.device)
    for kind, qc, vc in _joint_blocks(model):
        k = 6 if kind == 4 else 1
        out[:, qc:qc + k] = g[:, vc:vc + k]
    return out


def _tangent_from_q_layout(model, a):
    if model.nq_ext == model.nv:
        return a
    out = torch.empty(a.shape[0], model.nv, dtype=a.dtype, device=a.device)
    for kind, qc, vc in _joint_blocks(model):
        k = 6 if kind == 4 else 1
        out[:, vc:vc + k] = a[:, qc:qc + k]
    return out


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
        return None, tangent_to_coordinate_grad(ctx.model, q, qb), qdb, qddb


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
        return None, tangent_to_coordinate_grad(ctx.model, q, qb), qdb, tb


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
        return None, tangent_to_coordinate_grad(ctx.model, q, qb)


def inverse_dynamics(model, q, qd, qdd):
    """Differentiable batched RNEA: q [N, nq_ext], qd, qdd [N, nv] -> tau [N, nv]."""
    return _InverseDynamics.apply(model, q, qd, qdd)


def forward_dynamics(model, q, qd, tau):
    """Differentiable batched ABA: q [N, nq_ext], qd, tau [N, nv] -> qdd [N, nv]."""
    return _ForwardDynamics.apply(model, q, qd, tau)


def link_poses_rt(model, q):
    """Differentiable link poses: (positions [N, L, 3], rotations [N, L, 3, 3])."""
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
        ctx.save_for_backward(qc, qdc, tau, q0, qT)
        return qT, qdT

    @staticmethod
    def backward(ctx, qT_bar, qdT_bar):
        qc, qdc, tau, q0, qT = ctx.saved_tensors
        m = ctx.model
        if qT_bar is not None and m.nq_ext != m.nv:  # coordinates -> kernel layout of the tangent
            qT_bar = _tangent_in_q_layout(m, coordinate_to_tangent_grad(m, qT, qT_bar))
        q0b, qd0b, taub = rollout_backward(m, qc, qdc, tau, ctx.dt, ctx.K, qT_bar, qdT_bar)
        if m.nq_ext != m.nv:
            q0b = tangent_to_coordinate_grad(m, q0, _tangent_from_q_layout(m, q0b))
        return None, q0b, qd0b, taub, None, None


def rollout(model, q0, qd0, tau, dt, checkpoint_every=20):
    """Differentiable rollout: returns (qT, qdT). Gradients flow to q0, qd0 and tau; for a
    free-flyer root they are coordinate gradients (module docstring)."""
    return _Rollout.apply(model, q0, qd0, tau, float(dt), int(checkpoint_every))
