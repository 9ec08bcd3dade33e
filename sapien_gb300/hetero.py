"""Heterogeneous batches: several robot models stepped together in one persistent launch.

    batch = HeteroBatch([arm, quadruped, humanoid], model_of_env)   # plan once
    q = batch.pad_q([q_arm, q_quad, q_hum])                          # padded [N, max_nq]
    out = batch.step(q, qd, qdd, tau)                                # RNEA + ABA + CRBA
    graph = batch.capture(q, qd, qdd, tau, steps=10)                 # CUDA graph of 10 steps
    graph.replay()

Environments are grouped per model into warps (tiles of 32 / L environments for a model
run with L lanes per environment) and the tiles are ordered by descending velocity
dimension; a persistent grid pulls tiles from an atomic counter (see csrc/hetero.cu). The
launch shape (persistent CTAs per SM, warps per CTA, tile order) and the lanes per
environment of each model are chosen by ``sapien_gb300.autotune.tune_batch``.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N

OPS_DYNAMICS = N.OP_MASS_MATRIX | N.OP_INVERSE_DYNAMICS | N.OP_FORWARD_DYNAMICS


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class HeteroBatch:
    def __init__(self, models, model_of_env, device=None):
        self.models = list(models)
        for m in self.models:
            m._require_order()
        self.model_of_env = np.ascontiguousarray(np.asarray(model_of_env, dtype=np.int32))
        self.n = int(self.model_of_env.size)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        L = N.load()
        hs = (ctypes.c_void_p * len(self.models))(*[m._h.value for m in self.models])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            N.check(L.sgdyn_batch_create(hs, len(self.models),
                                         self.model_of_env.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), self.n,
                                         ctypes.byref(h)))
        self._h = h
        n64, nq, nv, nl = ctypes.c_int64(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        N.check(L.sgdyn_batch_info(h, ctypes.byref(n64), ctypes.byref(nq), ctypes.byref(nv), ctypes.byref(nl)))
        self.max_nq, self.max_nv, self.max_nlinks = nq.value, nv.value, nl.value
        self.launch = (4, 1, 0)
        self.lanes = tuple([1] * len(self.models))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                N.load().sgdyn_batch_free(h)
            except Exception:
                pass
            self._h = None

    def set_launch(self, ctas_per_sm, warps_per_cta, order):
        N.check(N.load().sgdyn_batch_set_launch(self._h, int(ctas_per_sm), int(warps_per_cta), int(order)))
        self.launch = (int(ctas_per_sm), int(warps_per_cta), int(order))

    def set_lanes(self, lanes_per_model):
        """Threads per environment for each model (1, 2, 4 or 8): with L > 1, L lanes share an
        environment, the root joints on all of them and the subtrees off them split among
        them, which shortens a wide tree's sequential sweep."""
        lanes = [int(x) for x in lanes_per_model]
        if len(lanes) != len(self.models):
            raise RuntimeError(f"expected {len(self.models)} lane counts")
        arr = (ctypes.c_int * len(lanes))(*lanes)
        with torch.cuda.device(self.device):
            N.check(N.load().sgdyn_batch_set_lanes(self._h, arr))
        self.lanes = tuple(lanes)

    # -- padding helpers ------------------------------------------------------------
    def _pad(self, per_model, width, attr):
        out = torch.zeros(self.n, width, dtype=torch.float64, device=self.device)
        for k, arr in enumerate(per_model):
            idx = np.nonzero(self.model_of_env == k)[0]
            a = torch.as_tensor(np.asarray(arr), dtype=torch.float64, device=self.device)
            if a.shape[0] != idx.size or a.shape[1] != getattr(self.models[k], attr):
                raise RuntimeError(f"model {k}: expected [{idx.size}, {getattr(self.models[k], attr)}]")
            out[torch.as_tensor(idx, device=self.device), : a.shape[1]] = a
        return out

    def pad_q(self, per_model):
        """Per-model [n_k, nq_k] arrays -> padded [N, max_nq] tensor."""
        return self._pad(per_model, self.max_nq, "nq_ext")

    def pad_v(self, per_model):
        """Per-model [n_k, nv_k] arrays -> padded [N, max_nv] tensor."""
        return self._pad(per_model, self.max_nv, "nv")

    def unpad_v(self, t, k):
        """Rows of model k from a padded [N, max_nv] tensor -> [n_k, nv_k]."""
        idx = torch.as_tensor(np.nonzero(self.model_of_env == k)[0], device=t.device)
        return t[idx, : self.models[k].nv]

    def unpad_M(self, t, k):
        idx = torch.as_tensor(np.nonzero(self.model_of_env == k)[0], device=t.device)
        nv = self.models[k].nv
        return t[idx, : nv * nv].reshape(-1, nv, nv)

    # -- stepping ---------------------------------------------------------------------
    def alloc_outputs(self, ops=OPS_DYNAMICS):
        e = lambda w: torch.empty(self.n, w, dtype=torch.float64, device=self.device)  # noqa: E731
        out = {}
        if ops & N.OP_FK:
            out["link_poses"] = e(7 * self.max_nlinks)
        if ops & N.OP_JACOBIAN:
            out["jacobian"] = e(6 * self.max_nv)
        if ops & N.OP_MASS_MATRIX:
            out["mass_matrix"] = e(self.max_nv * self.max_nv)
        if ops & N.OP_INVERSE_DYNAMICS:
            out["qf"] = e(self.max_nv)
        if ops & N.OP_FORWARD_DYNAMICS:
            out["qacc"] = e(self.max_nv)
        return out

    def step(self, q, qd=None, qdd=None, tau=None, ops=OPS_DYNAMICS, out=None):
        """One persistent launch over all environments; returns the (padded) outputs."""
        out = out if out is not None else self.alloc_outputs(ops)
        with torch.cuda.device(self.device):
            N.check(N.load().sgdyn_batch_step(
                self._h, int(ops), _p(q), _p(qd), _p(qdd), _p(tau), _p(out.get("link_poses")), _p(out.get("jacobian")),
                _p(out.get("mass_matrix")), _p(out.get("qf")), _p(out.get("qacc")),
                ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))
        return out

    def integrate(self, q, qd, qdd, dt):
        """Semi-implicit Euler in place on padded rows: qd += dt qdd, then q advanced by
        dt qd with each environment's model (free flyers on SE(3) by their body twist)."""
        with torch.cuda.device(self.device):
            N.check(N.load().sgdyn_batch_integrate(self._h, float(dt), _p(q), _p(qd), _p(qdd),
                                                   ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))

    def rollout_step(self, q, qd, tau, dt, out):
        """One rollout step in place and in one launch: qdd = ABA(q, qd, tau) into
        out["qacc"], then the semi-implicit Euler update of `integrate`, each environment
        right after its own sweep (bitwise the same as `step` + `integrate`)."""
        with torch.cuda.device(self.device):
            N.check(N.load().sgdyn_batch_step_integrate(
                self._h, float(dt), _p(q), _p(qd), _p(tau), _p(out["qacc"]),
                ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))

    def capture_rollout(self, q, qd, tau, dt, steps):
        """Record a whole rollout of `steps` semi-implicit-Euler steps (ABA + integrate per
        step, q / qd updated in place, tau held) into one torch CUDA graph. Replaying it
        advances q and qd by `steps` steps."""
        out = self.alloc_outputs(N.OP_FORWARD_DYNAMICS)
        q0, qd0 = q.clone(), qd.clone()
        self.rollout_step(q, qd, tau, dt, out)  # warm-up outside the capture
        torch.cuda.synchronize(self.device)
        q.copy_(q0)
        qd.copy_(qd0)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(steps):
                    self.rollout_step(q, qd, tau, dt, out)
        torch.cuda.current_stream(self.device).wait_stream(s)
        g.outputs = out
        return g

    def capture(self, q, qd, qdd, tau, steps=1, ops=OPS_DYNAMICS, out=None):
        """Record `steps` consecutive batch steps into a torch CUDA graph (returned with the
        output buffers it writes as graph.outputs)."""
        out = out if out is not None else self.alloc_outputs(ops)
        self.step(q, qd, qdd, tau, ops, out)  # warm-up outside the capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(steps):
                    self.step(q, qd, qdd, tau, ops, out)
        torch.cuda.current_stream(self.device).wait_stream(s)
        g.outputs = out
        return g
