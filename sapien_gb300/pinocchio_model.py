"""Drop-in ``PinocchioModel`` backed by GB300 kernels, plus batched tensor overloads.

Mirrors the reference's pybind surface (pinocchio/pinocchio_model.cpp:306-367): method
names, argument names, defaults, return types and exception types. The ``*_batched``
methods are the additions: they take float64 CUDA tensors of shape [N, ...], run the CUDA
kernels of libsgdyn.so and return tensors on the same device, enqueued on the current
torch stream of that device. The reference's one-configuration methods run the same sweep
code compiled for the host (libsgdyn.so's sgdyn_host_* entry points) on the calling
thread, or, with ``single_instance="cuda"``, on the GPU as batches of one.

Behaviour kept from the reference:
* the joint order must be set (``set_joint_order``) before any compute call, else
  ``RuntimeError("posS2P failed")`` (pinocchio_model.cpp:49-72, 70);
* bad joint / link names raise ``ValueError`` (std::invalid_argument, :105, :121, :136);
* bad link indices raise ``RuntimeError("link index out of bound")`` (:151, :168, :189, :233);
* ``get_link_pose`` returns a float32 Pose (p, q = w x y z) from the last
  ``compute_forward_kinematics`` (:150-161);
* ``get_link_jacobian(local=True)`` is the link (body) frame Jacobian, as the code does,
  although the reference docstring states the opposite (:355-362 vs :181-183);
* ``compute_inverse_kinematics`` follows the C++ CLIK loop (:228-300): best iterate,
  ``eps`` early exit, ``max_iterations`` updates, returns (q, success, err6).
Differences: ``get_link_pose`` / ``get_link_jacobian`` before the matching compute call
raise ``RuntimeError`` instead of reading stale Pinocchio data; ``get_link_jacobian`` uses
the configuration of the last ``compute_full_jacobian`` even if other calls followed.
Floating (free-flyer) joints, which the reference rejects in posS2P, are accepted: their
q block is (x y z qx qy qz qw) and their velocity block the 6-D body twist.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _native as N

KIND_REVOLUTE, KIND_PRISMATIC, KIND_CONTINUOUS, KIND_FREEFLYER = 1, 2, 3, 4


class Pose:
    """Stand-in for ``sapien.Pose``: float32 position ``p`` and quaternion ``q`` (w, x, y, z)."""

    def __init__(self, p=(0.0, 0.0, 0.0), q=(1.0, 0.0, 0.0, 0.0)):
        self.p = np.asarray(p, dtype=np.float32).reshape(3)
        self.q = np.asarray(q, dtype=np.float32).reshape(4)

    def to_transformation_matrix(self):
        w, x, y, z = (float(v) for v in self.q)
        T = np.eye(4)
        T[:3, :3] = [
            [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
        ]
        T[:3, 3] = self.p
        return T

    def __repr__(self):
        return f"Pose([{', '.join(f'{v:g}' for v in self.p)}], [{', '.join(f'{v:g}' for v in self.q)}])"


def _torch():
    import torch

    return torch


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class _HostStage:
    """Pinned host memory mapped into the device address space, for the single-instance
    calls: the CPU writes the inputs in place, the kernel reads them and writes its results
    straight into host memory, and one stream synchronisation ends the call (no copy
    launches, no device allocations per call)."""

    def __init__(self, nq, nv, nl):
        torch = _torch()
        sizes = {"q": nq, "qd": nv, "qdd": nv, "tau": nv, "q0": nq, "target": 7, "poses": 7 * max(nl, 1),
                 "J": 6 * nv, "M": nv * nv, "out_v": nv, "out_q": nq, "err": 6}
        self.off, total = {}, 0
        for k, n in sizes.items():
            self.off[k] = (total, n)
            total += max(n, 1)
        self.buf = torch.empty(total, dtype=torch.float64).pin_memory()
        self.ibuf = torch.empty(nv + 1, dtype=torch.int32).pin_memory()
        self.np, self.inp = self.buf.numpy(), self.ibuf.numpy()
        self.key = (nq, nv, nl)

    def put(self, k, a):
        o, n = self.off[k]
        self.np[o:o + n] = a

    def get(self, k):
        o, n = self.off[k]
        return self.np[o:o + n].copy()

    def p(self, k):
        return ctypes.c_void_p(self.buf.data_ptr() + 8 * self.off[k][0])

    def ip(self, i):
        return ctypes.c_void_p(self.ibuf.data_ptr() + 4 * i)


SINGLE_INSTANCE_PATHS = ("host", "cuda")


class PinocchioModel:
    """Replacement of ``sapien.pysapien_pinocchio.PinocchioModel``.

    The ``*_batched`` methods run the CUDA kernels on batches of float64 CUDA tensors. The
    reference's one-configuration methods run, by default (``single_instance="host"``), the
    same sweep code compiled for the CPU on the calling thread: one environment is a
    sequential sweep, which a host core finishes in microseconds while a GPU call pays a
    launch and a synchronisation around one thread's work. ``single_instance="cuda"`` sends
    them to the GPU as batches of one instead."""

    def __init__(self, urdf, gravity=(0.0, 0.0, -9.81), single_instance="host"):
        L = N.load()
        g = (ctypes.c_double * 3)(*[float(x) for x in gravity])
        h = ctypes.c_void_p()
        N.check(L.sgdyn_model_from_urdf(urdf.encode(), g, ctypes.byref(h)))
        self._h = h
        self._init_state(False, False, single_instance)

    def _init_state(self, joint_order_set, link_order_set, single_instance):
        self._joint_order_set = joint_order_set
        self._link_order_set = link_order_set
        self._fk_cache = None
        self._jac_q = None
        self._device = None
        self.single_instance = single_instance
        self._refresh()

    @classmethod
    def _from_handle(cls, h, joint_order_set=False, link_order_set=False, single_instance="host"):
        """Wrap a model handle created through another C-ABI constructor."""
        self = cls.__new__(cls)
        self._h = h
        self._init_state(joint_order_set, link_order_set, single_instance)
        return self

    @property
    def single_instance(self):
        """Where the reference's one-configuration methods run: "host" or "cuda"."""
        return self._single_instance

    @single_instance.setter
    def single_instance(self, where):
        if where not in SINGLE_INSTANCE_PATHS:
            raise ValueError(f"single_instance must be one of {SINGLE_INSTANCE_PATHS}")
        self._single_instance = where

    def _on_host(self):
        return self._single_instance == "host"

    def _host_step(self, ops, q, qd=None, qdd=None, tau=None):
        """One environment through sgdyn_host_step; returns the requested outputs."""
        nv, nl = self.nv, self._nlinks
        out = {}
        if ops & N.OP_FK:
            out["poses"] = np.empty(7 * max(nl, 1))
        if ops & N.OP_JACOBIAN:
            out["J"] = np.empty(6 * nv)
        if ops & N.OP_MASS_MATRIX:
            out["M"] = np.empty(nv * nv)
        if ops & N.OP_INVERSE_DYNAMICS:
            out["tau"] = np.empty(nv)
        if ops & N.OP_FORWARD_DYNAMICS:
            out["qdd"] = np.empty(nv)
        a = lambda x: x.ctypes.data_as(ctypes.c_void_p) if x is not None else None  # noqa: E731
        N.check(N.load().sgdyn_host_step(self._h, 1, int(ops), a(q), a(qd), a(qdd), a(tau), a(out.get("poses")),
                                         a(out.get("J")), a(out.get("M")), a(out.get("tau")), a(out.get("qdd")),
                                         N.ENV_MAJOR, 1))
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                N.load().sgdyn_model_free(h)
            except Exception:
                pass
            self._h = None

    # ---- model information ---------------------------------------------
    def _refresh(self):
        L = N.load()
        nq, nv, nl, nj = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        N.check(L.sgdyn_model_info(self._h, ctypes.byref(nq), ctypes.byref(nv), ctypes.byref(nl), ctypes.byref(nj)))
        self.nq_ext, self.nv, self._nlinks, self.njoints = nq.value, nv.value, nl.value, nj.value
        kinds = []
        for k in range(self.njoints - 1):
            kk = ctypes.c_int()
            N.check(L.sgdyn_model_joint_kind(self._h, k, ctypes.byref(kk)))
            kinds.append(kk.value)
        self._kinds = kinds
        self._uploaded = set()

    @property
    def joint_names(self):
        """Moving joints in tree (depth-first) order."""
        L = N.load()
        out = []
        for j in range(1, self.njoints):
            s = ctypes.c_char_p()
            N.check(L.sgdyn_model_joint_name(self._h, j, ctypes.byref(s)))
            out.append(s.value.decode())
        return out

    @property
    def link_names(self):
        """All URDF links (BODY frames) in tree order."""
        L = N.load()
        nb = ctypes.c_int()
        N.check(L.sgdyn_model_body_count(self._h, ctypes.byref(nb)))
        out = []
        for b in range(nb.value):
            s = ctypes.c_char_p()
            N.check(L.sgdyn_model_body_name(self._h, b, ctypes.byref(s)))
            out.append(s.value.decode())
        return out

    @property
    def nlinks(self):
        return self._nlinks if self._link_order_set else 0

    def set_lanes(self, lanes=0):
        """Lanes per environment for the batched sweeps (0 = automatic, 1, 2, 4 or 8): several
        lanes share one environment of a wide tree, which pays off for small batches."""
        N.check(N.load().sgdyn_model_set_lanes(self._h, int(lanes)))

    def table_bytes(self):
        """Host copy of the packed kernel tables (see csrc/device_model.h)."""
        L = N.load()
        p, n = ctypes.c_void_p(), ctypes.c_int64()
        N.check(L.sgdyn_model_table(self._h, ctypes.byref(p), ctypes.byref(n)))
        return ctypes.string_at(p, n.value)

    # ---- orders ----------------------------------------------------------
    @staticmethod
    def _names(names):
        arr = (ctypes.c_char_p * len(names))(*[str(n).encode() for n in names])
        return arr, len(names)

    def set_joint_order(self, names):
        arr, n = self._names(list(names))
        N.check(N.load().sgdyn_model_set_joint_order(self._h, arr, n))
        self._joint_order_set = True
        self._refresh()

    def set_link_order(self, names):
        arr, n = self._names(list(names))
        N.check(N.load().sgdyn_model_set_link_order(self._h, arr, n))
        self._link_order_set = True
        self._fk_cache = None
        self._refresh()

    def get_random_configuration(self, seed=None):
        """getRandomConfiguration (pinocchio_model.cpp:142-144): one qpos in the joint order,
        each revolute or prismatic coordinate uniform within its URDF limits, each continuous
        angle uniform in [-pi, pi). `seed` (addition) makes the draw reproducible; without it
        the seed comes from the OS. Raises for a model with a free flyer (no limits)."""
        return self.get_random_configuration_batched(1, seed)[0]

    def get_random_configuration_batched(self, n, seed=None):
        """[n, nq] float64 host array of random configurations (see get_random_configuration);
        the same seed gives the same rows on every platform."""
        seed = int.from_bytes(os.urandom(8), "little") if seed is None else int(seed) & (2**64 - 1)
        out = np.empty((int(n), self.nq_ext), dtype=np.float64)
        N.check(N.load().sgdyn_model_random_configuration(self._h, int(n), seed,
                                                          out.ctypes.data_as(ctypes.c_void_p)))
        return out

    # ---- plumbing ----------------------------------------------------------
    def _require_order(self):
        if not self._joint_order_set and self.nv > 0:
            raise RuntimeError("posS2P failed")

    def _check_link(self, link_index):
        if not (0 <= int(link_index) < self.nlinks):
            raise RuntimeError("link index out of bound")

    def _dev(self):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("sapien_gb300 needs a CUDA device for compute calls")
        if self._device is None:
            self._device = torch.device("cuda", torch.cuda.current_device())
        return self._device

    def _prepare(self, device):
        torch = _torch()
        key = device.index
        if key not in self._uploaded:
            with torch.cuda.device(device):
                N.check(N.load().sgdyn_model_upload(self._h))
            self._uploaded.add(key)

    def _vec(self, x, n, what):
        a = np.asarray(x, dtype=np.float64).reshape(-1)
        if a.size != n:
            raise RuntimeError(f"{what} has size {a.size}, expected {n}" if what != "qpos" else "posS2P failed")
        return a

    def _single(self, *arrays):
        torch = _torch()
        dev = self._dev()
        return [torch.from_numpy(a.reshape(1, -1)).to(dev) for a in arrays]

    def _stage(self):
        self._dev()  # a clear error without a CUDA device
        key = (self.nq_ext, self.nv, self._nlinks)
        st = getattr(self, "_host_stage", None)
        if st is None or st.key != key:
            st = self._host_stage = _HostStage(*key)
        return st

    def _run1(self, fn, *args):
        """One single-instance C-ABI call on staged host buffers, then wait for it."""
        torch = _torch()
        dev = self._dev()
        self._prepare(dev)
        with torch.cuda.device(dev):
            stream = torch.cuda.current_stream(dev)
            N.check(fn(self._h, *args, ctypes.c_void_p(stream.cuda_stream)))
            stream.synchronize()

    def _check_batch(self, t, cols, what):
        torch = _torch()
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{what} must be a torch.Tensor")
        if t.dtype != torch.float64 or not t.is_cuda:
            raise TypeError(f"{what} must be a float64 CUDA tensor")
        if t.dim() != 2 or t.shape[1] != cols:
            raise RuntimeError(f"{what} must have shape [N, {cols}], got {tuple(t.shape)}")
        return t.contiguous()

    def _stream(self, device):
        return ctypes.c_void_p(_torch().cuda.current_stream(device).cuda_stream)

    # ---- batched overloads (additions) -------------------------------------
    def step_batched(self, qpos, qvel=None, qacc=None, qf=None, ops=N.OP_ALL):
        """Fused sweep: any subset of FK poses, WORLD Jacobian, mass matrix, inverse and forward
        dynamics on one batch. Returns a dict with keys among
        'link_poses' [N, nlinks, 7], 'jacobian' [N, 6, nv], 'mass_matrix' [N, nv, nv],
        'qf' (RNEA torques) [N, nv], 'qacc' (ABA accelerations) [N, nv]."""
        torch = _torch()
        self._require_order()
        q = self._check_batch(qpos, self.nq_ext, "qpos")
        n = q.shape[0]
        dev = q.device
        qd = self._check_batch(qvel, self.nv, "qvel") if ops & (N.OP_INVERSE_DYNAMICS | N.OP_FORWARD_DYNAMICS) else None
        qdd = self._check_batch(qacc, self.nv, "qacc") if ops & N.OP_INVERSE_DYNAMICS else None
        tau = self._check_batch(qf, self.nv, "qf") if ops & N.OP_FORWARD_DYNAMICS else None
        if ops & N.OP_FK and not self._link_order_set:
            raise RuntimeError("link index out of bound")
        out = {}
        e = lambda *s: torch.empty(*s, dtype=torch.float64, device=dev)  # noqa: E731
        poses = e(n, self._nlinks, 7) if ops & N.OP_FK else None
        J = e(n, 6, self.nv) if ops & N.OP_JACOBIAN else None
        M = e(n, self.nv, self.nv) if ops & N.OP_MASS_MATRIX else None
        tau_o = e(n, self.nv) if ops & N.OP_INVERSE_DYNAMICS else None
        qdd_o = e(n, self.nv) if ops & N.OP_FORWARD_DYNAMICS else None
        self._prepare(dev)
        with torch.cuda.device(dev):
            N.check(N.load().sgdyn_step(self._h, n, int(ops), _ptr(q), _ptr(qd), _ptr(qdd), _ptr(tau), _ptr(poses),
                                        _ptr(J), _ptr(M), _ptr(tau_o), _ptr(qdd_o), N.ENV_MAJOR, self._stream(dev)))
        for k, v in (("link_poses", poses), ("jacobian", J), ("mass_matrix", M), ("qf", tau_o), ("qacc", qdd_o)):
            if v is not None:
                out[k] = v
        return out

    def compute_forward_kinematics_batched(self, qpos):
        """[N, nq] -> FP64 link poses [N, nlinks, 7] = (x y z qw qx qy qz)."""
        return self.step_batched(qpos, ops=N.OP_FK)["link_poses"]

    def compute_full_jacobian_batched(self, qpos):
        """[N, nq] -> WORLD Jacobian [N, 6, nv] (rows vx vy vz wx wy wz)."""
        return self.step_batched(qpos, ops=N.OP_JACOBIAN)["jacobian"]

    def compute_generalized_mass_matrix_batched(self, qpos):
        return self.step_batched(qpos, ops=N.OP_MASS_MATRIX)["mass_matrix"]

    def compute_inverse_dynamics_batched(self, qpos, qvel, qacc):
        return self.step_batched(qpos, qvel, qacc, ops=N.OP_INVERSE_DYNAMICS)["qf"]

    def compute_forward_dynamics_batched(self, qpos, qvel, qf):
        return self.step_batched(qpos, qvel, qf=qf, ops=N.OP_FORWARD_DYNAMICS)["qacc"]

    def _batched_matrix_op(self, fn, qpos, extra, cols):
        torch = _torch()
        self._require_order()
        q = self._check_batch(qpos, self.nq_ext, "qpos")
        dev = q.device
        out = torch.empty(q.shape[0], cols, dtype=torch.float64, device=dev)
        self._prepare(dev)
        with torch.cuda.device(dev):
            N.check(fn(q, out, dev))
        return out

    def compute_link_jacobian_batched(self, qpos, link_index, local=False):
        """[N, nq] -> Jacobian of one link [N, 6, nv] (WORLD, or the link frame if local)."""
        self._check_link(link_index)
        L = N.load()
        out = self._batched_matrix_op(
            lambda q, o, d: L.sgdyn_compute_link_jacobian(self._h, q.shape[0], int(link_index), int(bool(local)),
                                                          _ptr(q), _ptr(o), N.ENV_MAJOR, self._stream(d)),
            qpos, None, 6 * self.nv)
        return out.view(-1, 6, self.nv)

    def compute_single_link_local_jacobian_batched(self, qpos, link_index):
        self._check_link(link_index)
        L = N.load()
        out = self._batched_matrix_op(
            lambda q, o, d: L.sgdyn_compute_single_link_local_jacobian(self._h, q.shape[0], int(link_index), _ptr(q),
                                                                       _ptr(o), N.ENV_MAJOR, self._stream(d)),
            qpos, None, 6 * self.nv)
        return out.view(-1, 6, self.nv)

    def compute_coriolis_matrix_batched(self, qpos, qvel):
        L = N.load()
        qd = self._check_batch(qvel, self.nv, "qvel")
        out = self._batched_matrix_op(
            lambda q, o, d: L.sgdyn_compute_coriolis_matrix(self._h, q.shape[0], _ptr(q), _ptr(qd), _ptr(o),
                                                            N.ENV_MAJOR, self._stream(d)),
            qpos, None, self.nv * self.nv)
        return out.view(-1, self.nv, self.nv)

    def compute_inverse_kinematics_batched(self, link_index, target_poses, initial_qpos=None, active_qmask=None,
                                           eps=1e-4, max_iterations=1000, dt=0.1, damp=1e-6):
        """Batched CLIK. target_poses [N, 7] = (x y z qw qx qy qz) FP64 CUDA. Returns
        (q [N, nq], success [N] bool, err [N, 6])."""
        torch = _torch()
        self._require_order()
        self._check_link(link_index)
        tgt = self._check_batch(target_poses, 7, "target_poses")
        n = tgt.shape[0]
        dev = tgt.device
        q0 = self._check_batch(initial_qpos, self.nq_ext, "initial_qpos") if initial_qpos is not None else None
        mask = None
        if active_qmask is not None and len(active_qmask):
            mask = torch.as_tensor(np.asarray(active_qmask, dtype=np.int32).reshape(-1), device=dev)
            if mask.numel() != self.nv:
                raise RuntimeError(f"active_qmask must have {self.nv} entries")
        q = torch.empty(n, self.nq_ext, dtype=torch.float64, device=dev)
        ok = torch.empty(n, dtype=torch.int32, device=dev)
        err = torch.empty(n, 6, dtype=torch.float64, device=dev)
        self._prepare(dev)
        with torch.cuda.device(dev):
            N.check(N.load().sgdyn_compute_inverse_kinematics(
                self._h, n, int(link_index), _ptr(tgt), _ptr(q0), _ptr(mask), float(eps), int(max_iterations),
                float(dt), float(damp), _ptr(q), _ptr(ok), _ptr(err), N.ENV_MAJOR, self._stream(dev)))
        return q, ok.bool(), err

    def compute_passive_force_batched(self, qpos, qvel=None, gravity=True, coriolis_and_centrifugal=True, out=None):
        """PhysxArticulation.compute_passive_force for a whole batch, read straight from
        SAPIEN-style float32 state buffers: qpos / qvel [N, maxDof] (maxDof >= dof, padded
        rows as SAPIEN's GPU system exports them). Returns (or fills `out`) a float32
        [N, maxDof] tensor whose first dof columns hold RNEA(q, qd, 0) with the selected terms,
        computed in FP64."""
        torch = _torch()
        self._require_order()
        if qpos.dtype != torch.float32 or not qpos.is_cuda or qpos.dim() != 2 or qpos.stride(1) != 1:
            raise TypeError("qpos must be a float32 CUDA tensor [N, maxDof] with unit column stride")
        if coriolis_and_centrifugal:
            if qvel is None or qvel.shape != qpos.shape or qvel.stride() != qpos.stride() or qvel.dtype != torch.float32:
                raise TypeError("qvel must be a float32 CUDA tensor laid out like qpos")
        n, width = qpos.shape
        if out is None:
            out = torch.zeros(n, width, dtype=torch.float32, device=qpos.device)
        dev = qpos.device
        self._prepare(dev)
        with torch.cuda.device(dev):
            N.check(N.load().sgdyn_compute_passive_force_f32(
                self._h, n, _ptr(qpos), _ptr(qvel) if coriolis_and_centrifugal else None, qpos.stride(0),
                int(bool(gravity)), int(bool(coriolis_and_centrifugal)), _ptr(out), out.stride(0), self._stream(dev)))
        return out

    # ---- reference single-instance API -----------------------------------
    def compute_forward_kinematics(self, qpos):
        """Compute and cache forward kinematics. After computation, use get_link_pose to
        retrieve the computed pose for a specific link."""
        self._require_order()
        q = self._vec(qpos, self.nq_ext, "qpos")
        if self._link_order_set and self._nlinks > 0 and self._on_host():
            self._fk_cache = self._host_step(N.OP_FK, q)["poses"].reshape(self._nlinks, 7)
        elif self._link_order_set and self._nlinks > 0:
            st = self._stage()
            st.put("q", q)
            self._run1(N.load().sgdyn_compute_forward_kinematics, 1, st.p("q"), st.p("poses"), N.ENV_MAJOR)
            self._fk_cache = st.get("poses").reshape(self._nlinks, 7)
        else:
            self._fk_cache = np.zeros((0, 7))

    def get_link_pose(self, link_index):
        """Given link index, get link pose (in articulation base frame) from forward
        kinematics. Must be called after compute_forward_kinematics."""
        self._check_link(link_index)
        if self._fk_cache is None:
            raise RuntimeError("compute_forward_kinematics must be called before get_link_pose")
        r = self._fk_cache[int(link_index)]
        return Pose(r[:3], r[3:7])

    def compute_full_jacobian(self, qpos):
        """Compute and cache Jacobian for all links"""
        self._require_order()
        self._jac_q = self._vec(qpos, self.nq_ext, "qpos").copy()

    def get_link_jacobian(self, link_index, local=False):
        """Given link index, get the Jacobian. Must be called after compute_full_jacobian.

        Args:
          link_index: index of the link
          local: True for the link (body) frame; False for the world (spatial) frame
        """
        self._check_link(link_index)
        if self._jac_q is None:
            raise RuntimeError("compute_full_jacobian must be called before get_link_jacobian")
        if self._on_host():
            return self._host_link_jacobian(self._jac_q, link_index, local)
        st = self._stage()
        st.put("q", self._jac_q)
        self._run1(N.load().sgdyn_compute_link_jacobian, 1, int(link_index), int(bool(local)), st.p("q"), st.p("J"),
                   N.ENV_MAJOR)
        return st.get("J").reshape(6, self.nv)

    def compute_single_link_local_jacobian(self, qpos, link_index):
        """Compute the link(body) Jacobian for a single link. It is faster than
        compute_full_jacobian followed by get_link_jacobian"""
        self._require_order()
        self._check_link(link_index)
        q = self._vec(qpos, self.nq_ext, "qpos")
        if self._on_host():
            return self._host_link_jacobian(q, link_index, True)
        st = self._stage()
        st.put("q", q)
        self._run1(N.load().sgdyn_compute_single_link_local_jacobian, 1, int(link_index), st.p("q"), st.p("J"),
                   N.ENV_MAJOR)
        return st.get("J").reshape(6, self.nv)

    def _host_link_jacobian(self, q, link_index, local):
        J = np.empty(6 * self.nv)
        N.check(N.load().sgdyn_host_compute_link_jacobian(self._h, 1, int(link_index), int(bool(local)),
                                                          q.ctypes.data_as(ctypes.c_void_p),
                                                          J.ctypes.data_as(ctypes.c_void_p), N.ENV_MAJOR, 1))
        return J.reshape(6, self.nv)

    def compute_generalized_mass_matrix(self, qpos):
        self._require_order()
        q = self._vec(qpos, self.nq_ext, "qpos")
        if self._on_host():
            return self._host_step(N.OP_MASS_MATRIX, q)["M"].reshape(self.nv, self.nv)
        st = self._stage()
        st.put("q", q)
        self._run1(N.load().sgdyn_compute_generalized_mass_matrix, 1, st.p("q"), st.p("M"), N.ENV_MAJOR)
        return st.get("M").reshape(self.nv, self.nv)

    def compute_coriolis_matrix(self, qpos, qvel):
        self._require_order()
        q, qd = self._vec(qpos, self.nq_ext, "qpos"), self._vec(qvel, self.nv, "qvel")
        if self._on_host():
            C = np.empty(self.nv * self.nv)
            N.check(N.load().sgdyn_host_compute_coriolis_matrix(
                self._h, 1, q.ctypes.data_as(ctypes.c_void_p), qd.ctypes.data_as(ctypes.c_void_p),
                C.ctypes.data_as(ctypes.c_void_p), N.ENV_MAJOR, 1))
            return C.reshape(self.nv, self.nv)
        st = self._stage()
        st.put("q", q)
        st.put("qd", qd)
        self._run1(N.load().sgdyn_compute_coriolis_matrix, 1, st.p("q"), st.p("qd"), st.p("M"), N.ENV_MAJOR)
        return st.get("M").reshape(self.nv, self.nv)

    def compute_inverse_dynamics(self, qpos, qvel, qacc):
        self._require_order()
        q, qd, qdd = (self._vec(qpos, self.nq_ext, "qpos"), self._vec(qvel, self.nv, "qvel"),
                      self._vec(qacc, self.nv, "qacc"))
        if self._on_host():
            return self._host_step(N.OP_INVERSE_DYNAMICS, q, qd, qdd)["tau"]
        st = self._stage()
        st.put("q", q)
        st.put("qd", qd)
        st.put("qdd", qdd)
        self._run1(N.load().sgdyn_compute_inverse_dynamics, 1, st.p("q"), st.p("qd"), st.p("qdd"), st.p("out_v"),
                   N.ENV_MAJOR)
        return st.get("out_v")

    def compute_forward_dynamics(self, qpos, qvel, qf):
        self._require_order()
        q, qd, tau = (self._vec(qpos, self.nq_ext, "qpos"), self._vec(qvel, self.nv, "qvel"),
                      self._vec(qf, self.nv, "qf"))
        if self._on_host():
            return self._host_step(N.OP_FORWARD_DYNAMICS, q, qd, tau=tau)["qdd"]
        st = self._stage()
        st.put("q", q)
        st.put("qd", qd)
        st.put("tau", tau)
        self._run1(N.load().sgdyn_compute_forward_dynamics, 1, st.p("q"), st.p("qd"), st.p("tau"), st.p("out_v"),
                   N.ENV_MAJOR)
        return st.get("out_v")

    def compute_inverse_kinematics(self, link_index, pose, initial_qpos=(), active_qmask=(), eps=1e-4,
                                   max_iterations=1000, dt=0.1, damp=1e-6):
        """Compute inverse kinematics with CLIK algorithm.

        Args:
            link_index: index of the link
            pose: target pose of the link in articulation base frame
            initial_qpos: initial qpos to start CLIK
            active_qmask: dof sized integer array, 1 to indicate active joints and 0 for inactive joints, default to all 1s
            max_iterations: number of iterations steps
            dt: iteration step "speed"
            damp: iteration step "damping"
        Returns:
            result: qpos from IK
            success: whether IK is successful
            error: se3 norm error
        """
        self._require_order()
        self._check_link(link_index)
        p = np.asarray(pose.p, dtype=np.float32).astype(np.float64)
        qq = np.asarray(pose.q, dtype=np.float32).astype(np.float64)
        q0v = self._vec(initial_qpos, self.nq_ext, "qpos") if initial_qpos is not None and len(initial_qpos) else None
        m = None
        if active_qmask is not None and len(active_qmask):
            m = np.asarray(active_qmask, dtype=np.int32).reshape(-1)
            if m.size != self.nv:
                raise RuntimeError(f"active_qmask must have {self.nv} entries")
        if self._on_host():
            tgt = np.concatenate([p, qq])
            qo, ok, err = np.empty(self.nq_ext), np.zeros(1, dtype=np.int32), np.empty(6)
            a = lambda x: x.ctypes.data_as(ctypes.c_void_p) if x is not None else None  # noqa: E731
            N.check(N.load().sgdyn_host_compute_inverse_kinematics(
                self._h, 1, int(link_index), a(tgt), a(q0v), a(m), float(eps), int(max_iterations), float(dt),
                float(damp), a(qo), a(ok), a(err), N.ENV_MAJOR, 1))
            return qo, bool(ok[0]), err
        st = self._stage()
        st.put("target", np.concatenate([p, qq]))
        q0 = None
        if q0v is not None:
            st.put("q0", q0v)
            q0 = st.p("q0")
        mask = None
        if m is not None:
            st.inp[: self.nv] = m
            mask = st.ip(0)
        self._run1(N.load().sgdyn_compute_inverse_kinematics, 1, int(link_index), st.p("target"), q0, mask, float(eps),
                   int(max_iterations), float(dt), float(damp), st.p("out_q"), st.ip(self.nv), st.p("err"),
                   N.ENV_MAJOR)
        return st.get("out_q"), bool(st.inp[self.nv]), st.get("err")
