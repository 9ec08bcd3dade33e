"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import
this module. It mirrors the reference's ``PinocchioModel`` surface
(pinocchio/pinocchio_model.cpp:306-367): a model is built from URDF text and
gravity, ``set_joint_order`` / ``set_link_order`` fix the external ordering, and
the ``compute_*`` calls take external-order numpy vectors.

Parity status: parity unpinned (the reference ships no golden vectors for this
path; see oracle.cpp's header). Pinned instead by closed forms and identities.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from . import urdf_model as um

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lib = None


def build():
    """Compile the oracle library with make (g++)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        d, i = ctypes.c_double, ctypes.c_int
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [i, P(i), P(i), P(d), P(d), P(d), P(d), i, P(i), i, P(i), P(d)]
        L.orc_free.argtypes = [ctypes.c_void_p]
        for name in ("orc_rnea", "orc_aba"):
            getattr(L, name).argtypes = [ctypes.c_void_p, P(d), P(d), P(d), P(d)]
        L.orc_crba.argtypes = [ctypes.c_void_p, P(d), P(d)]
        L.orc_coriolis.argtypes = [ctypes.c_void_p, P(d), P(d), P(d)]
        L.orc_fk.argtypes = [ctypes.c_void_p, P(d), P(d)]
        L.orc_full_jacobian.argtypes = [ctypes.c_void_p, P(d), P(d)]
        L.orc_link_jacobian.argtypes = [ctypes.c_void_p, i, i, P(d)]
        L.orc_single_link_local_jacobian.argtypes = [ctypes.c_void_p, P(d), i, P(d)]
        L.orc_ik.argtypes = [ctypes.c_void_p, i, P(d), P(d), P(i), d, i, d, d, P(d), P(i), P(d)]
        L.orc_integrate.argtypes = [ctypes.c_void_p, P(d), P(d), P(d)]
        L.orc_neutral.argtypes = [ctypes.c_void_p, P(d)]
        L.orc_set_long_double.argtypes = [ctypes.c_void_p, i]
        L.orc_info.argtypes = [ctypes.c_void_p, P(i), P(i), P(i)]
        L.orc_log6.argtypes = [P(d), P(d)]
        L.orc_exp6.argtypes = [P(d), P(d)]
        L.orc_jlog6.argtypes = [P(d), P(d)]
        L.orc_count_ops.argtypes = [ctypes.c_void_p, P(d), P(d), P(d), P(d), P(ctypes.c_longlong)]
        L.orc_batch_step.argtypes = [ctypes.c_void_p, ctypes.c_long, i, P(d), P(d), P(d), P(d), P(d), P(d), P(d),
                                     P(d), P(d), i]
        L.orc_batch_ik.argtypes = [ctypes.c_void_p, ctypes.c_long, i, P(d), P(d), d, i, d, d, P(d), P(i), P(d), i]
        L.orc_rollout.argtypes = [ctypes.c_void_p, ctypes.c_long, i, d, P(d), P(d), P(d), i, P(d), P(d), P(d),
                                  P(d), i]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None else None


def _f64(x, n=None):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def se3_log6(M):
    """log6 of a 4x4 homogeneous transform -> (linear, angular)."""
    M = np.asarray(M, dtype=np.float64)
    m12 = _f64(np.concatenate([M[:3, :3].ravel(), M[:3, 3]]))
    out = np.zeros(6)
    lib().orc_log6(_dp(m12), _dp(out))
    return out


def se3_exp6(nu):
    out = np.zeros(12)
    lib().orc_exp6(_dp(_f64(nu, 6)), _dp(out))
    T = np.eye(4)
    T[:3, :3] = out[:9].reshape(3, 3)
    T[:3, 3] = out[9:]
    return T


def se3_jlog6(M):
    M = np.asarray(M, dtype=np.float64)
    m12 = _f64(np.concatenate([M[:3, :3].ravel(), M[:3, 3]]))
    out = np.zeros(36)
    lib().orc_jlog6(_dp(m12), _dp(out))
    return out.reshape(6, 6)


class Oracle:
    """CPU FP64 restatement of the reference PinocchioModel (one instance)."""

    def __init__(self, urdf: str, gravity=(0.0, 0.0, -9.81)):
        self.model = um.build_model(urdf, gravity)
        self._h = None
        self._long_double = False
        m = self.model
        # default orders: all moving joints in tree order, all links in tree order
        m.joint_order = list(range(1, m.njoints))
        m.link_order = list(m.link_names_in_order)
        self._rebuild()

    # -- construction -----------------------------------------------------
    def _rebuild(self):
        m = self.model
        if self._h:
            lib().orc_free(self._h)
        nj = m.njoints
        parent = np.array(m.parent, dtype=np.int32)
        jtype = np.array(m.jtype, dtype=np.int32)
        axis = _f64(np.array(m.axis).reshape(-1))
        placement = _f64(np.array([np.concatenate([R.ravel(), p]) for R, p in m.placement]).reshape(-1))
        inertia = _f64(np.array(m.inertia6).reshape(-1))
        grav = _f64(m.gravity)
        ext = np.array(m.joint_order, dtype=np.int32)
        lj = np.array([m.body_frames[n][0] for n in m.link_order], dtype=np.int32)
        lp = _f64(
            np.array([np.concatenate([m.body_frames[n][1][0].ravel(), m.body_frames[n][1][1]]) for n in m.link_order])
            .reshape(-1)
        ) if m.link_order else np.zeros(12)
        h = lib().orc_create(nj, _ip(parent), _ip(jtype), _dp(axis), _dp(placement), _dp(inertia), _dp(grav),
                             len(ext), _ip(ext), len(lj), _ip(lj), _dp(lp))
        if not h:
            raise RuntimeError("oracle model creation failed")
        self._h = h
        lib().orc_set_long_double(h, int(self._long_double))
        nq, nv, nqe = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib().orc_info(h, ctypes.byref(nq), ctypes.byref(nv), ctypes.byref(nqe))
        self.nq, self.nv, self.nq_ext = nq.value, nv.value, nqe.value
        self.nlinks = len(lj)

    def __del__(self):
        try:
            if self._h:
                lib().orc_free(self._h)
        except Exception:
            pass

    def set_long_double(self, on=True):
        self._long_double = bool(on)
        lib().orc_set_long_double(self._h, int(on))

    def set_joint_order(self, names):
        self.model.set_joint_order(names)
        self._rebuild()

    def set_link_order(self, names):
        self.model.set_link_order(names)
        self._rebuild()

    # -- single-instance API (external order) ------------------------------
    def compute_forward_kinematics(self, qpos):
        out = np.zeros(self.nlinks * 12)
        lib().orc_fk(self._h, _dp(_f64(qpos, self.nq_ext)), _dp(out))
        self._poses = out.reshape(self.nlinks, 12)

    def get_link_pose_matrix(self, link_index):
        """4x4 FP64 link pose from the last compute_forward_kinematics."""
        if not 0 <= link_index < self.nlinks:
            raise RuntimeError("link index out of bound")
        r = self._poses[link_index]
        T = np.eye(4)
        T[:3, :3] = r[:9].reshape(3, 3)
        T[:3, 3] = r[9:]
        return T

    def link_poses(self, qpos):
        self.compute_forward_kinematics(qpos)
        return np.array([self.get_link_pose_matrix(i) for i in range(self.nlinks)])

    def compute_full_jacobian(self, qpos):
        J = np.zeros(6 * self.nv)
        lib().orc_full_jacobian(self._h, _dp(_f64(qpos, self.nq_ext)), _dp(J))
        return J.reshape(6, self.nv)

    def get_link_jacobian(self, link_index, local=False):
        out = np.zeros(6 * self.nv)
        rc = lib().orc_link_jacobian(self._h, int(link_index), int(bool(local)), _dp(out))
        if rc != 0:
            raise RuntimeError("link index out of bound" if rc == -2 else "compute_full_jacobian not called")
        return out.reshape(6, self.nv)

    def compute_single_link_local_jacobian(self, qpos, link_index):
        out = np.zeros(6 * self.nv)
        rc = lib().orc_single_link_local_jacobian(self._h, _dp(_f64(qpos, self.nq_ext)), int(link_index), _dp(out))
        if rc != 0:
            raise RuntimeError("link index out of bound")
        return out.reshape(6, self.nv)

    def compute_generalized_mass_matrix(self, qpos):
        out = np.zeros(self.nv * self.nv)
        lib().orc_crba(self._h, _dp(_f64(qpos, self.nq_ext)), _dp(out))
        return out.reshape(self.nv, self.nv)

    def compute_coriolis_matrix(self, qpos, qvel):
        out = np.zeros(self.nv * self.nv)
        lib().orc_coriolis(self._h, _dp(_f64(qpos, self.nq_ext)), _dp(_f64(qvel, self.nv)), _dp(out))
        return out.reshape(self.nv, self.nv)

    def compute_inverse_dynamics(self, qpos, qvel, qacc):
        out = np.zeros(self.nv)
        lib().orc_rnea(self._h, _dp(_f64(qpos, self.nq_ext)), _dp(_f64(qvel, self.nv)), _dp(_f64(qacc, self.nv)),
                       _dp(out))
        return out

    def compute_forward_dynamics(self, qpos, qvel, qf):
        out = np.zeros(self.nv)
        rc = lib().orc_aba(self._h, _dp(_f64(qpos, self.nq_ext)), _dp(_f64(qvel, self.nv)), _dp(_f64(qf, self.nv)),
                           _dp(out))
        if rc != 0:
            raise RuntimeError("singular joint-space inertia")
        return out

    def compute_inverse_kinematics(self, link_index, target, initial_qpos=None, active_qmask=None, eps=1e-4,
                                   max_iterations=1000, dt=0.1, damp=1e-6):
        """target: 4x4 FP64 link pose. Returns (q, success, err6)."""
        T = np.asarray(target, dtype=np.float64)
        t12 = _f64(np.concatenate([T[:3, :3].ravel(), T[:3, 3]]))
        q0 = _f64(initial_qpos, self.nq_ext) if initial_qpos is not None and len(initial_qpos) else None
        mask = (np.ascontiguousarray(np.asarray(active_qmask, dtype=np.int32))
                if active_qmask is not None and len(active_qmask) else None)
        q = np.zeros(self.nq_ext)
        ok = ctypes.c_int()
        err = np.zeros(6)
        rc = lib().orc_ik(self._h, int(link_index), _dp(t12), _dp(q0), _ip(mask), float(eps), int(max_iterations),
                          float(dt), float(damp), _dp(q), ctypes.byref(ok), _dp(err))
        if rc == -2:
            raise RuntimeError("link index out of bound")
        if rc != 0:
            raise RuntimeError("IK solve failed")
        return q, bool(ok.value), err

    def integrate(self, q, v):
        out = np.zeros(self.nq_ext)
        lib().orc_integrate(self._h, _dp(_f64(q, self.nq_ext)), _dp(_f64(v, self.nv)), _dp(out))
        return out

    def neutral(self):
        out = np.zeros(self.nq_ext)
        lib().orc_neutral(self._h, _dp(out))
        return out

    # -- batched drivers (threads over environments) -----------------------
    def batch_step(self, q, qd=None, qdd=None, tau=None, ops=31, nthreads=1):
        """Run the selected ops for every environment; returns a dict of arrays."""
        q = _f64(q)
        n = q.shape[0]
        nv, nl = self.nv, self.nlinks
        out = {}
        poses = np.zeros((n, nl, 12)) if ops & 1 else None
        J = np.zeros((n, 6, nv)) if ops & 2 else None
        M = np.zeros((n, nv, nv)) if ops & 4 else None
        tau_o = np.zeros((n, nv)) if ops & 8 else None
        qdd_o = np.zeros((n, nv)) if ops & 16 else None
        z = np.zeros((n, nv))
        qd = _f64(qd) if qd is not None else z
        qdd = _f64(qdd) if qdd is not None else z
        tau = _f64(tau) if tau is not None else z
        lib().orc_batch_step(self._h, n, ops, _dp(q), _dp(qd), _dp(qdd), _dp(tau), _dp(poses), _dp(J), _dp(M),
                             _dp(tau_o), _dp(qdd_o), int(nthreads))
        for k, v in (("poses", poses), ("J", J), ("M", M), ("tau", tau_o), ("qdd", qdd_o)):
            if v is not None:
                out[k] = v
        return out

    OPS_COUNTED = ("fk", "jacobian", "crba", "rnea", "aba", "placements")

    def count_ops(self, q, qd, qdd, tau):
        """Floating-point operations of one evaluation of each op at this input (see
        orc_count_ops): {op: {"add", "mul", "div", "sqrt", "trig"}} for fk (link poses),
        jacobian, crba, rnea, aba and placements (the joint-placement pass all of them share)."""
        c = np.zeros(6 * 5, dtype=np.int64)
        rc = lib().orc_count_ops(self._h, _dp(_f64(q)), _dp(_f64(qd)), _dp(_f64(qdd)), _dp(_f64(tau)),
                                 c.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        if rc != 0:
            raise RuntimeError("orc_count_ops failed")
        keys = ("add", "mul", "div", "sqrt", "trig")
        return {op: dict(zip(keys, (int(x) for x in c[5 * i:5 * i + 5]))) for i, op in enumerate(self.OPS_COUNTED)}

    def batch_ik(self, link, targets, q0=None, eps=1e-4, max_iterations=1000, dt=0.1, damp=1e-6, nthreads=1):
        """targets: [n, 4, 4]. Returns (q [n, nq_ext], success [n], err [n, 6])."""
        targets = np.asarray(targets, dtype=np.float64)
        n = targets.shape[0]
        t12 = _f64(np.concatenate([targets[:, :3, :3].reshape(n, 9), targets[:, :3, 3]], axis=1))
        q = np.zeros((n, self.nq_ext))
        ok = np.zeros(n, dtype=np.int32)
        err = np.zeros((n, 6))
        q0a = _f64(q0) if q0 is not None else None
        lib().orc_batch_ik(self._h, n, int(link), _dp(t12), _dp(q0a), float(eps), int(max_iterations), float(dt),
                           float(damp), _dp(q), _ip(ok), _dp(err), int(nthreads))
        return q, ok.astype(bool), err

    def rollout(self, q0, qd0, tau, dt, link, targets, nthreads=1):
        """tau: [T, n, nv]. Returns (qT, qdT, loss_per_env)."""
        tau = _f64(tau)
        T, n = tau.shape[0], tau.shape[1]
        qT = np.zeros((n, self.nq_ext))
        qdT = np.zeros((n, self.nv))
        loss = np.zeros(n)
        lib().orc_rollout(self._h, n, T, float(dt), _dp(_f64(q0)), _dp(_f64(qd0)), _dp(tau), int(link),
                          _dp(_f64(targets)), _dp(qT), _dp(qdT), _dp(loss), int(nthreads))
        return qT, qdT, loss
