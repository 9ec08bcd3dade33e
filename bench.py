#!/usr/bin/env python
"""Benchmark of the batched articulated-body dynamics step on GB300.

Workload (one "step"): the 9-DoF tree (7 revolute arm joints + 2 prismatic fingers on
the last link), N = 16384 environments per GPU, seeded synthetic float64 inputs; every
step computes, for every environment, forward kinematics (all link poses), the WORLD
Jacobian, the CRBA mass matrix, RNEA inverse dynamics and ABA forward dynamics, i.e.
the five PinocchioModel calls the reference makes per environment.

Our arm: `python bench.py [--gpus N --steps K --warmup W]` (torchrun for N > 1; each rank
owns its own N environments, no collective on the data path: weak scaling).
Reference arm: `python bench.py --impl reference ...` times the CPU oracle (the FP64
restatement of the reference path; the reference itself cannot be built here) on the
same workload with all host threads, on rank 0 only.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ABA/RNEA evals/s at 16k envs; fwd+bwd rollout steps/s vs plain; err<=1e-9"
UNIT = "env-steps/s"
N_ENVS = 16384
WORKLOAD = ("arm9: 9-DoF tree (7 revolute + 2 prismatic fingers), N=16384 envs per GPU, "
            "FK (all link poses) + WORLD Jacobian + CRBA + RNEA + ABA per env per step")

# FP64 thread-instructions (DFMA + DMUL + DADD) per environment-step and DRAM bytes per
# environment of one step (structure-of-arrays buffers; both launches when the step is split),
# from an ncu capture of the model-specialised kernels (run-time compiled) and of the generic
# ones. They hold for the
# kernel source whose digest is KERNEL_SOURCE_SHA256 (kernel_source_digest()); a CPU test
# fails when the source changes, so the figures are re-captured with every kernel change.
KERNEL_COUNTERS = {
    # two launches (FK + Jacobian: 507,392 FP64 warp instructions; CRBA + RNEA + ABA with
    # forward dynamics from the mass matrix: 1,650,688) per 16384 environments (the thread
    # counts with all predicates on, 987.6 + 3223.0 per environment, agree); DRAM bytes as
    # ncu counted them in a cold capture, where most of the 29 MB of results is still held in
    # L2 when the launches end
    "specialised": {"fp64_inst_per_env": 2158080 * 32 / 16384, "dram_bytes_per_env": 8.32e6 / 16384},
}
KERNEL_SOURCE_SHA256 = "49e104c5e570e5883a86511be471883515b1e9846a8d8e5c713b105010c2b432"
KERNEL_HEADERS = ("device_model.h", "kernels.h", "spatial.cuh", "step_kernel.cuh")
STEP_OPS = (3, 28)  # sgdyn_step at N = 16384: FK + Jacobian beside CRBA + RNEA + ABA, two launches


def kernel_source_digest(model, ops=None):
    """SHA-256 of what the step kernels of `model` are compiled from: the run-time-generated
    translation units (their floating-point constants masked: the last bits of the model
    tables differ between host libms, the instruction stream does not) and the device headers
    they include. `ops` defaults to the two launches of the five-op step as bench.py runs it."""
    import hashlib
    import re

    from sapien_gb300 import _native as N

    h = hashlib.sha256()
    for o in (STEP_OPS if ops is None else (ops,)):
        src = ctypes.c_char_p()
        N.check(N.load().sgdyn_jit_source(model._h, o, ctypes.byref(src)))
        h.update(re.sub(rb"[-+]?(?:(?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)", b"#", src.value))
    for name in KERNEL_HEADERS:
        with open(os.path.join(ROOT, "sapien_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def algorithmic_flops(robot):
    """FP64 operations per environment of each op, counted by the oracle's counting scalar
    (local-frame recursions with operations on structural zeros and ones skipped) at one
    seeded input: {op: flops} for fk, jacobian, crba, rnea, aba, the fused five-op step
    (the joint-placement pass they share counted once) and rnea+aba; plus the
    transcendental calls per step."""
    o = _oracle_of(robot)
    q, qd, qdd, tau = robot.sample(1, seed=0)
    c = o.count_ops(q[0], qd[0], qdd[0], tau[0])
    fl = {k: v["add"] + v["mul"] + v["div"] + v["sqrt"] for k, v in c.items()}
    ops = ("fk", "jacobian", "crba", "rnea", "aba")
    out = {k: fl[k] for k in ops}
    out["step"] = sum(fl[k] for k in ops) - (len(ops) - 1) * fl["placements"]
    out["rnea+aba"] = fl["rnea"] + fl["aba"] - fl["placements"]
    out["transcendental_calls_per_step"] = c["placements"]["trig"]
    return out


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_ENVS)
    ap.add_argument("--only-rollout", action="store_true",
                    help="run only the differentiable-rollout workload (for profiling its kernels)")
    ap.add_argument("--only-hetero", choices=["mix", "humanoid"],
                    help="run only the heterogeneous RNEA + ABA + CRBA step, on the 8192-robot mix or on its 1638 "
                         "humanoids alone, at a fixed launch shape (2 CTAs per SM, one warp each) and lanes (1, 1, 4), "
                         "three steps (for profiling its kernel)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the secondary workloads (rollout, heterogeneous batch, IK, derivatives)")
    return ap.parse_args()


def algorithmic_bytes_per_env(nq, nv, nlinks):
    """Compulsory FP64 traffic of one env-step: inputs q, qd, qdd, tau; outputs link poses
    (7 per link), Jacobian 6 x nv, mass matrix nv x nv, tau, qdd."""
    return 8 * (nq + 3 * nv) + 8 * (7 * nlinks + 6 * nv + nv * nv + 2 * nv)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_model():
    """Host CPU name from /proc/cpuinfo (x86 "model name"; Arm implementer / part ids)."""
    try:
        info = open("/proc/cpuinfo").read().splitlines()
    except OSError:
        return "unknown"
    kv = {}
    for line in info:
        if ":" in line:
            k, v = line.split(":", 1)
            kv.setdefault(k.strip(), v.strip())
    if "model name" in kv:
        return kv["model name"]
    if "CPU part" in kv:
        return f"arm implementer {kv.get('CPU implementer', '?')} part {kv['CPU part']}"
    return "unknown"


def time_median(fn, min_reps=5, min_seconds=2.0):
    """Median wall time of fn() over at least min_reps runs and min_seconds."""
    ts, t_start = [], time.perf_counter()
    while len(ts) < min_reps or time.perf_counter() - t_start < min_seconds:
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts)), len(ts)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


PROBE_SRC = os.path.join(ROOT, "bench_fp64_peak.cu")
PROBE_LIB = os.path.join(ROOT, "_bench_build", "libfp64_peak.so")


def build_probe():
    """Compile the FP64-peak microbenchmark (measurement only, not part of the library)."""
    from sapien_gb300.build_native import build_standalone

    return build_standalone(PROBE_SRC, PROBE_LIB)


def fp64_peak_dfma_per_s():
    L = ctypes.CDLL(build_probe())
    L.sgdyn_probe_fp64_dfma_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    v = ctypes.c_double()
    if L.sgdyn_probe_fp64_dfma_rate(5, ctypes.byref(v)) != 0:
        return None
    return v.value


def make_model():
    from sapien_gb300 import PinocchioModel, synthetic

    robot = synthetic.arm_with_fingers()
    pm = PinocchioModel(robot.urdf, [0.0, 0.0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    return robot, pm


def _event_ms(torch, fn, reps=5, warm=2):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def hetero_only(dev, which):
    """The heterogeneous step alone at a fixed launch shape: the 8192-robot mix, or its
    humanoids alone; three steps after one warm-up, CUDA events."""
    import torch

    from sapien_gb300 import PinocchioModel, synthetic
    from sapien_gb300.hetero import OPS_DYNAMICS, HeteroBatch

    robots, moe = synthetic.hetero_mix(8192, seed=0)
    if which == "humanoid":
        moe = np.full(int((moe == 2).sum()), 2, dtype=np.int32)
    models = []
    for r in robots:
        m = PinocchioModel(r.urdf, [0.0, 0.0, -9.81])
        m.set_joint_order(r.joint_names)
        m.set_link_order(r.link_names)
        models.append(m)
    ins = []
    for k, r in enumerate(robots):
        c = int((moe == k).sum())
        ins.append([a[:c] for a in r.sample(max(c, 1), seed=k)])
    hb = HeteroBatch(models, moe, device=dev)
    args = (hb.pad_q([x[0] for x in ins]), hb.pad_v([x[1] for x in ins]), hb.pad_v([x[2] for x in ins]),
            hb.pad_v([x[3] for x in ins]))
    out = hb.alloc_outputs(OPS_DYNAMICS)
    hb.set_launch(2, 1, 0)
    hb.set_lanes([1, 1, 4])
    hb.step(*args, OPS_DYNAMICS, out)
    torch.cuda.synchronize()
    ms = _event_ms(torch, lambda: hb.step(*args, OPS_DYNAMICS, out), reps=3, warm=0)
    return {"workload": f"{len(moe)} envs ({which}), RNEA+ABA+CRBA", "ms_per_step": ms, "launch_shape": [2, 1, 0],
            "lanes_per_env": [1, 1, 4]}


def secondary_workloads(dev, only_rollout=False):
    """The other workloads of the benchmark spec, timed with CUDA events on rank 0:
    differentiable rollout (9-DoF arm, 4096 envs, 200 steps, dt 1/500, q/qd checkpoints
    every 20 steps), heterogeneous batch (8192 mixed robots, RNEA + ABA + CRBA, CUDA-graph
    replay, autotuned launch), batched CLIK (65536 targets, 100 iterations, damping 1e-3)
    and dense derivatives on the floating-base humanoid (8192 envs)."""
    import torch

    from sapien_gb300 import PinocchioModel, autodiff as ad, autotune, synthetic
    from sapien_gb300 import _native as N
    from sapien_gb300.hetero import OPS_DYNAMICS, HeteroBatch

    def model_of(r):
        m = PinocchioModel(r.urdf, [0.0, 0.0, -9.81])
        m.set_joint_order(r.joint_names)
        m.set_link_order(r.link_names)
        return m

    out = {}
    arm = synthetic.arm_with_fingers()
    pm = model_of(arm)
    n, T, K, dt = 4096, 200, 20, 1.0 / 500
    q0, qd0, _, _ = (torch.from_numpy(a).to(dev) for a in arm.sample(n, seed=0))
    tau = torch.from_numpy(np.random.default_rng(1).normal(scale=5.0, size=(T, n, arm.nv))).to(dev)
    fwd = _event_ms(torch, lambda: ad.rollout_forward(pm, q0, qd0, tau, dt))
    fwd_ck = _event_ms(torch, lambda: ad.rollout_forward(pm, q0, qd0, tau, dt, K))
    _, _, qc, qdc = ad.rollout_forward(pm, q0, qd0, tau, dt, K)
    ones = torch.ones_like(q0)
    bwd = _event_ms(torch, lambda: ad.rollout_backward(pm, qc, qdc, tau, dt, K, qT_bar=ones))
    out["rollout"] = {"workload": "arm9, 4096 envs, T=200, dt=1/500, checkpoints every 20 steps",
                      "plain_env_steps_per_s": n * T / (fwd * 1e-3),
                      "fwd_bwd_env_steps_per_s": n * T / ((fwd_ck + bwd) * 1e-3),
                      "fwd_ms": fwd, "fwd_with_checkpoints_ms": fwd_ck, "bwd_ms": bwd,
                      "fwd_bwd_over_plain": (fwd_ck + bwd) / fwd}
    out["rollout"].update(_rollout_parity(torch, ad, arm, pm, q0, qd0, tau, dt, K))
    if only_rollout:
        return out
    robots, moe = synthetic.hetero_mix(8192, seed=0)
    models = [model_of(r) for r in robots]
    ins = [r.sample(int((moe == k).sum()), seed=k) for k, r in enumerate(robots)]
    hb = HeteroBatch(models, moe, device=dev)
    hq, hqd, hqdd, htau = (hb.pad_q([x[0] for x in ins]), hb.pad_v([x[1] for x in ins]),
                           hb.pad_v([x[2] for x in ins]), hb.pad_v([x[3] for x in ins]))
    shape, _ = autotune.tune_batch(hb, hq, hqd, hqdd, htau, OPS_DYNAMICS)
    g = hb.capture(hq, hqd, hqdd, htau, steps=10)
    hms = _event_ms(torch, g.replay, reps=5, warm=1) / 10
    out["hetero"] = {"workload": "8192 envs: 50% 6-DoF arms, 30% 18-DoF quadrupeds, 20% 35-DoF humanoids; "
                                 "RNEA+ABA+CRBA; CUDA-graph replay of 10 steps",
                     "env_steps_per_s": 8192 / (hms * 1e-3), "ms_per_step": hms, "launch_shape": list(shape),
                     "lanes_per_env": list(hb.lanes)}
    out["hetero"].update(_hetero_parity(robots, moe, hb, g.outputs, ins))
    # a whole heterogeneous rollout (ABA + semi-implicit Euler, free flyers on SE(3)) as one graph,
    # with the launch shape and lanes tuned for ABA alone
    rq, rqd, rtau = hq.clone(), hqd.clone(), 0.1 * htau
    rshape, _ = autotune.tune_batch(hb, hq, hqd, hqdd, rtau, N.OP_FORWARD_DYNAMICS)
    rg = hb.capture_rollout(rq, rqd, rtau, 1.0 / 500, 100)
    rms = _event_ms(torch, rg.replay, reps=3, warm=1) / 100
    out["hetero_rollout"] = {"workload": "same 8192-robot mix, 100 semi-implicit-Euler steps (ABA + integrate) "
                                         "captured as one CUDA graph, dt=1/500",
                             "env_steps_per_s": 8192 / (rms * 1e-3), "ms_per_step": rms,
                             "launch_shape": list(rshape), "lanes_per_env": list(hb.lanes)}
    # parity: one replay (100 steps) from the initial state against the oracle's rollout
    rq.copy_(hq)
    rqd.copy_(hqd)
    rg.replay()
    torch.cuda.synchronize()
    out["hetero_rollout"].update(_hetero_rollout_parity(robots, moe, hb, hq, hqd, rtau, rq, rqd, 1.0 / 500, 100))
    nik = 65536
    qik, _, _, _ = arm.sample(nik, seed=3)
    tgt = pm.compute_forward_kinematics_batched(torch.from_numpy(qik).to(dev))[:, arm.ee_link].contiguous()
    ik_ms = _event_ms(torch, lambda: pm.compute_inverse_kinematics_batched(arm.ee_link, tgt, None, None, eps=0.0,
                                                                           max_iterations=100, dt=0.1, damp=1e-3),
                      reps=3, warm=1)
    # parity of a sample against the oracle's CLIK (same targets, fixed 100 iterations)
    from oracle.oracle import Oracle

    q_ik = pm.compute_inverse_kinematics_batched(arm.ee_link, tgt, None, None, eps=0.0, max_iterations=100, dt=0.1,
                                                 damp=1e-3)[0][:256].cpu().numpy()
    t7 = tgt[:256].cpu().numpy()
    t44 = np.zeros((256, 4, 4))
    w, x, y, z = (t7[:, 3 + k] for k in range(4))
    t44[:, 0, :3] = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], 1)
    t44[:, 1, :3] = np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], 1)
    t44[:, 2, :3] = np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1)
    t44[:, :3, 3] = t7[:, :3]
    t44[:, 3, 3] = 1.0
    o = Oracle(arm.urdf)
    o.set_joint_order(arm.joint_names)
    o.set_link_order(arm.link_names)
    q_ref = o.batch_ik(arm.ee_link, t44, None, eps=0.0, max_iterations=100, dt=0.1, damp=1e-3, nthreads=8)[0]
    ik_err = float((np.abs(q_ik - q_ref).max(axis=1) / np.maximum(np.abs(q_ref).max(axis=1), 1e-300)).max())
    out["ik"] = {"workload": "arm9 CLIK, 65536 FK targets, 100 iterations, damping 1e-3",
                 "solves_per_s": nik / (ik_ms * 1e-3), "ms": ik_ms,
                 "max_rel_err_vs_oracle": ik_err, "err_sample": "first 256 targets, joint positions"}
    hum = synthetic.humanoid()
    hm = model_of(hum)
    hq2, hqd2, hqdd2, htau2 = (torch.from_numpy(a).to(dev) for a in hum.sample(8192, seed=0))
    rd = _event_ms(torch, lambda: ad.rnea_derivatives(hm, hq2, hqd2, hqdd2), reps=3, warm=1)
    adr = _event_ms(torch, lambda: ad.aba_derivatives(hm, hq2, hqd2, htau2), reps=3, warm=1)
    out["derivatives"] = {"workload": "humanoid (35 DoF, floating base), 8192 envs, dense dtau/d(q,qd,qdd) and "
                                      "dqdd/d(q,qd,tau)",
                          "rnea_derivatives_evals_per_s": 8192 / (rd * 1e-3),
                          "aba_derivatives_evals_per_s": 8192 / (adr * 1e-3)}
    out["derivatives"].update(_derivative_parity(ad, hum, hm, hq2, hqd2, hqdd2, htau2))
    out["reference_robots"] = _reference_robot_parity(torch, dev)
    out["single_instance"] = _single_instance_latency(arm)
    return out


def _single_instance_latency(arm, calls=2000):
    """The drop-in's one-configuration calls (`PinocchioModel` methods with numpy vectors, as
    the reference's callers make them), answered on the host by the library's sweeps: mean
    wall-clock microseconds per call on this machine's CPU, Python and ctypes included."""
    import time

    from sapien_gb300 import PinocchioModel

    pm = PinocchioModel(arm.urdf, [0.0, 0.0, -9.81])
    pm.set_joint_order(arm.joint_names)
    pm.set_link_order(arm.link_names)
    q, qd, qdd, tau = (a[0].copy() for a in arm.sample(1, seed=5))

    def per_call(fn, n=calls):
        fn()
        t0 = time.perf_counter()
        for _ in range(n):
            fn()
        return (time.perf_counter() - t0) / n * 1e6

    pm.compute_forward_kinematics(q)
    target = pm.get_link_pose(arm.ee_link)
    return {"workload": "arm9, one configuration per call through PinocchioModel (host path)",
            "unit": "us per call",
            "forward_dynamics": per_call(lambda: pm.compute_forward_dynamics(q, qd, tau)),
            "inverse_dynamics": per_call(lambda: pm.compute_inverse_dynamics(q, qd, qdd)),
            "mass_matrix": per_call(lambda: pm.compute_generalized_mass_matrix(q)),
            "forward_kinematics_and_link_pose": per_call(lambda: (pm.compute_forward_kinematics(q),
                                                                  pm.get_link_pose(arm.ee_link))),
            "inverse_kinematics_100_iterations": per_call(
                lambda: pm.compute_inverse_kinematics(arm.ee_link, target, initial_qpos=q * 0.9, eps=0.0,
                                                      max_iterations=100), n=100)}


def _oracle_of(robot):
    from oracle.oracle import Oracle

    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    return o


def _rel(g, r):
    """Largest per-environment normwise relative error (rows = environments)."""
    g = np.asarray(g).reshape(len(g), -1)
    r = np.asarray(r).reshape(len(r), -1)
    return float((np.abs(g - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-300)).max())


def _rollout_parity(torch, ad, arm, pm, q0, qd0, tau, dt, K, sample=64, grad_envs=4, h=1e-6):
    """Final states of the first `sample` environments against the oracle's rollout, and
    the loss gradient (loss = sum |p_ee(q_T) - target|^2) w.r.t. q0 and qd0 of the first
    `grad_envs` environments against central differences of the oracle's rollout."""
    o = _oracle_of(arm)
    s = slice(0, sample)
    qT, qdT, _, _ = ad.rollout_forward(pm, q0[s].contiguous(), qd0[s].contiguous(), tau[:, s].contiguous(), dt, K)
    tau_h = tau[:, s].cpu().numpy()
    targets = np.random.default_rng(2).uniform(-0.5, 0.5, size=(sample, 3))
    rq, rqd, _ = o.rollout(q0[s].cpu().numpy(), qd0[s].cpu().numpy(), tau_h, dt, arm.ee_link, targets, nthreads=8)
    g = slice(0, grad_envs)
    q0t = q0[g].clone().requires_grad_()
    qd0t = qd0[g].clone().requires_grad_()
    qTg, _ = ad.rollout(pm, q0t, qd0t, tau[:, g].contiguous(), dt, checkpoint_every=K)
    tg = torch.from_numpy(targets[g]).to(q0.device)
    ((ad.link_positions(pm, qTg)[:, arm.ee_link] - tg) ** 2).sum().backward()
    qn, qdn, taun = q0[g].cpu().numpy(), qd0[g].cpu().numpy(), tau_h[:, g]

    def loss(a, b):
        return o.rollout(a, b, taun, dt, arm.ee_link, targets[g])[2]

    fq, fqd = np.zeros_like(qn), np.zeros_like(qdn)
    for k in range(qn.shape[1]):
        e = np.zeros(qn.shape[1])
        e[k] = h
        fq[:, k] = (loss(qn + e, qdn) - loss(qn - e, qdn)) / (2 * h)
        fqd[:, k] = (loss(qn, qdn + e) - loss(qn, qdn - e)) / (2 * h)
    return {"max_rel_err_vs_oracle": {"qT": _rel(qT.cpu().numpy(), rq), "qdT": _rel(qdT.cpu().numpy(), rqd)},
            "grad_rel_err_vs_fd": {"q0": _rel(q0t.grad.cpu().numpy(), fq), "qd0": _rel(qd0t.grad.cpu().numpy(), fqd)},
            "err_sample": f"final states of the first {sample} envs; loss gradients of the first {grad_envs} envs vs "
                          f"oracle central differences (h={h:g})"}


def _hetero_parity(robots, moe, hb, outs, ins, sample=256):
    """RNEA / ABA / CRBA of the graph replay against the oracle, up to `sample`
    environments of each robot type."""
    errs = {"rnea": 0.0, "aba": 0.0, "crba": 0.0}
    for k, r in enumerate(robots):
        o = _oracle_of(r)
        q, qd, qdd, tau = (x[:sample] for x in ins[k])
        ref = o.batch_step(q, qd, qdd, tau, ops=4 | 8 | 16, nthreads=8)
        m = len(q)
        errs["rnea"] = max(errs["rnea"], _rel(hb.unpad_v(outs["qf"], k)[:m].cpu().numpy(), ref["tau"]))
        errs["aba"] = max(errs["aba"], _rel(hb.unpad_v(outs["qacc"], k)[:m].cpu().numpy(), ref["qdd"]))
        errs["crba"] = max(errs["crba"], _rel(hb.unpad_M(outs["mass_matrix"], k)[:m].cpu().numpy(), ref["M"]))
    return {"max_rel_err_vs_oracle": errs, "err_sample": f"first {sample} envs of each robot type"}


def _hetero_rollout_parity(robots, moe, hb, q0, qd0, tau, qT, qdT, dt, steps, sample=32):
    """Final q / qd after the captured rollout against the oracle's semi-implicit-Euler
    rollout (SE(3) integrate for free flyers), `sample` environments of each type."""
    eq = eqd = 0.0
    for k, r in enumerate(robots):
        o = _oracle_of(r)
        idx = np.nonzero(moe == k)[0][:sample]
        nq, nv = r.nq_ext, r.nv
        qk, qdk = q0[idx, :nq].cpu().numpy(), qd0[idx, :nv].cpu().numpy()
        tk = np.repeat(tau[idx, :nv].cpu().numpy()[None], steps, axis=0)
        rq, rqd, _ = o.rollout(qk, qdk, tk, dt, 0, np.zeros((len(idx), 3)), nthreads=8)
        eq = max(eq, _rel(qT[idx, :nq].cpu().numpy(), rq))
        eqd = max(eqd, _rel(qdT[idx, :nv].cpu().numpy(), rqd))
    return {"max_rel_err_vs_oracle": {"q": eq, "qd": eqd}, "err_sample": f"first {sample} envs of each robot type"}


def _derivative_parity(ad, robot, pm, q, qd, qdd, tau, envs=2, h=1e-6):
    """Dense derivatives of the first `envs` environments against central differences of
    the oracle's RNEA / ABA (configuration perturbed on the manifold by integrate)."""
    o = _oracle_of(robot)
    s = slice(0, envs)
    dq, dqd, _ = (x.cpu().numpy() for x in ad.rnea_derivatives(pm, q[s], qd[s], qdd[s]))
    aq, aqd, _ = (x.cpu().numpy() for x in ad.aba_derivatives(pm, q[s], qd[s], tau[s]))
    qn, qdn, qddn, taun = (x[s].cpu().numpy() for x in (q, qd, qdd, tau))
    nv = robot.nv
    worst = {"dtau_dq": 0.0, "dtau_dqd": 0.0, "dqdd_dq": 0.0, "dqdd_dqd": 0.0}
    for e in range(envs):
        fd = {k: np.zeros((nv, nv)) for k in worst}
        for k in range(nv):
            d = np.zeros(nv)
            d[k] = h
            qp, qm = o.integrate(qn[e], d), o.integrate(qn[e], -d)
            fd["dtau_dq"][:, k] = (o.compute_inverse_dynamics(qp, qdn[e], qddn[e])
                                   - o.compute_inverse_dynamics(qm, qdn[e], qddn[e])) / (2 * h)
            fd["dqdd_dq"][:, k] = (o.compute_forward_dynamics(qp, qdn[e], taun[e])
                                   - o.compute_forward_dynamics(qm, qdn[e], taun[e])) / (2 * h)
            fd["dtau_dqd"][:, k] = (o.compute_inverse_dynamics(qn[e], qdn[e] + d, qddn[e])
                                    - o.compute_inverse_dynamics(qn[e], qdn[e] - d, qddn[e])) / (2 * h)
            fd["dqdd_dqd"][:, k] = (o.compute_forward_dynamics(qn[e], qdn[e] + d, taun[e])
                                    - o.compute_forward_dynamics(qn[e], qdn[e] - d, taun[e])) / (2 * h)
        for key, got in (("dtau_dq", dq), ("dtau_dqd", dqd), ("dqdd_dq", aq), ("dqdd_dqd", aqd)):
            worst[key] = max(worst[key], _rel(got[e][None], fd[key][None]))
    return {"max_rel_err_vs_fd": worst, "err_sample": f"first {envs} envs, oracle central differences (h={h:g})"}


def _reference_robot_parity(torch, dev, n=1024, sample=256):
    """The reference's own robots (tests/golden: panda, movo_simple, sawyer, fetch, in SAPIEN's
    loader order): per-op largest error of the batched kernels against the oracle, and the
    reference test's movo_simple case (unittest/test_physx/test_articulation.py:75-97)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import reference_robots as rr

    from sapien_gb300 import PinocchioModel

    res = {}
    for name in rr.NAMES:
        r = rr.load(name)
        pm = PinocchioModel(r.urdf, [0.0, 0.0, -9.81])
        pm.set_joint_order(r.joint_names)
        pm.set_link_order(r.link_names)
        o = _oracle_of(r)
        q, qd, qdd, tau = r.sample(n, seed=5)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        dyn = name in rr.DYNAMICS
        ref = o.batch_step(q[:sample], qd[:sample], qdd[:sample], tau[:sample], ops=31 if dyn else 3, nthreads=8)
        P = pm.compute_forward_kinematics_batched(t(q))[:sample].cpu().numpy()
        errs = {"fk_positions": _rel(P[:, :, :3], ref["poses"][:, :, 9:]),
                "jacobian": _rel(pm.compute_full_jacobian_batched(t(q))[:sample].cpu().numpy(), ref["J"])}
        if dyn:
            errs["crba"] = _rel(pm.compute_generalized_mass_matrix_batched(t(q))[:sample].cpu().numpy(), ref["M"])
            errs["rnea"] = _rel(pm.compute_inverse_dynamics_batched(t(q), t(qd), t(qdd))[:sample].cpu().numpy(),
                                ref["tau"])
            errs["aba"] = _rel(pm.compute_forward_dynamics_batched(t(q), t(qd), t(tau))[:sample].cpu().numpy(),
                               ref["qdd"])
        res[name] = {"nv": r.nv, "links": len(r.link_names), "max_rel_err_vs_oracle": errs}
        if name == "movo_simple":
            q0, z, _ = rr.movo_reference_inputs()
            g = pm.compute_inverse_dynamics(q0, z, z)
            pm.compute_forward_kinematics(q0)
            o.compute_forward_kinematics(q0)
            pe = max(float(np.abs(pm.get_link_pose(i).p - o.get_link_pose_matrix(i)[:3, 3]).max())
                     for i in range(len(r.link_names)))
            res[name]["reference_test_case"] = {
                "rnea_q_0_0_rel_err": _rel(g[None], o.compute_inverse_dynamics(q0, z, z)[None]),
                "get_link_pose_max_abs_err_float32": pe}
    res["err_sample"] = f"first {sample} of {n} seeded envs per robot"
    return res


def workload_config(n, nv, nl):
    """The workload as both arms name it (identical dicts, so the two lines compare)."""
    return {"workload": WORKLOAD, "n_envs_per_gpu": n, "nv": nv, "links": nl,
            "layout": "structure of arrays ([cols][n], SGDYN_COL_MAJOR)",
            "l2": "flushed between timed GPU steps (256 MiB write, outside the timed events)"}


CPU_BASELINE_NOTE = ("the oracle: this project's FP64 C++ restatement of the reference path with dense 6x6 "
                     "Plucker algebra (the reference's Pinocchio cannot be built here); slower per call than "
                     "Pinocchio itself, so GPU/CPU ratios against it overstate the speed-up over SAPIEN's CPU path")


def run_reference(args):
    """CPU oracle on the same workload, all host threads, rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.oracle import Oracle
    from sapien_gb300 import synthetic

    robot = synthetic.arm_with_fingers()
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    n = args.n
    q, qd, qdd, tau = robot.sample(n, seed=0)
    cores = host_cores()
    for _ in range(args.warmup):
        o.batch_step(q, qd, qdd, tau, nthreads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.batch_step(q, qd, qdd, tau, nthreads=cores)
    dt = (time.perf_counter() - t0) / args.steps
    value = n / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, robot.nv, len(robot.link_names)),
        "execution": {"parallelism": "host threads over environments (one model per thread)", "threads": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"full workload ({n} envs) per step, {args.steps} steps", "what": CPU_BASELINE_NOTE},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    if args.only_rollout:
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        torch.cuda.set_device(dev)
        print(json.dumps({"secondary": secondary_workloads(dev, only_rollout=True)}), flush=True)
        return
    if args.only_hetero:
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        torch.cuda.set_device(dev)
        print(json.dumps({"hetero_only": hetero_only(dev, args.only_hetero)}), flush=True)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()

    from sapien_gb300 import _native as N
    from sapien_gb300.sharding import aggregate_throughput, max_across_ranks

    robot, pm = make_model()
    n = args.n
    q_h, qd_h, qdd_h, tau_h = robot.sample(n, seed=rank)
    nv, nq, nl = robot.nv, robot.nq_ext, len(robot.link_names)
    # structure-of-arrays buffers ([cols][n], SGDYN_COL_MAJOR): every column coalesced
    soa = lambda a: np.ascontiguousarray(a.reshape(n, -1).T)  # noqa: E731
    q, qd, qdd, tau = (torch.from_numpy(soa(a)).to(dev) for a in (q_h, qd_h, qdd_h, tau_h))
    out_cols = (nl * 7, 6 * nv, nv * nv, nv, nv)
    poses, J, M, tau_o, qdd_o = (torch.empty(c, n, dtype=torch.float64, device=dev) for c in out_cols)
    pm._prepare(dev)
    L = N.load()
    kernel = "specialised" if L.sgdyn_jit_prepare(pm._h, N.OP_ALL) == 0 else "generic"
    counters = KERNEL_COUNTERS.get(kernel)  # None for the generic kernels (not captured)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def step(qq, qqd, qqdd, ttau, ops=N.OP_ALL):
        call(ops, (qq, qqd, qqdd, ttau), (poses, J, M, tau_o, qdd_o))

    def call(ops, ins, outs):
        rc = L.sgdyn_step(pm._h, n, ops, *[P(t) for t in ins], *[P(t) for t in outs], N.COL_MAJOR, sp)
        if rc != 0:
            raise RuntimeError(N.last_error())

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    # sgdyn_step runs the five ops as two concurrent launches (FK + Jacobian beside CRBA +
    # RNEA + ABA) while one warp per 32 environments gives fewer than two warps per FP64
    # scheduler (split mode 2, the default)
    mode = ctypes.c_int()
    N.check(L.sgdyn_step_split(-1, ctypes.byref(mode)))
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    split = mode.value == 1 or (mode.value == 2 and (n + 31) // 32 < 2 * 4 * sms)
    launches_per_step = 2 if split else 1

    # ---- kernel-only timing, inputs resident in HBM ---------------------------------
    for _ in range(args.warmup):
        flush.zero_()
        step(q, qd, qdd, tau)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step(q, qd, qdd, tau)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = max_across_ranks(float(np.mean([a.elapsed_time(b) for a, b in ev])), dist, dev)
    value = aggregate_throughput(n, world, ms * 1e-3)

    # ---- end to end through the C ABI with host buffers ------------------------------
    # Inputs and outputs live in pinned host memory. The C ABI accepts mapped pinned host
    # pointers: the kernel reads the inputs and writes the results in host memory over the
    # host link, so every step's bytes cross it inside the timed region. The same step with
    # explicit cudaMemcpyAsync staging through device buffers is timed beside it.
    pin = lambda a: torch.from_numpy(soa(a)).pin_memory()  # noqa: E731
    ins_h = [pin(q_h), pin(qd_h), pin(qdd_h), pin(tau_h)]
    ins_d = (q, qd, qdd, tau)
    outs_d = (poses, J, M, tau_o, qdd_o)
    outs_h = [torch.empty(o.shape, dtype=torch.float64).pin_memory() for o in outs_d]
    h2d = sum(t.numel() * 8 for t in ins_h)
    d2h = sum(t.numel() * 8 for t in outs_h)

    def e2e_mapped():
        call(N.OP_ALL, ins_h, outs_h)

    def e2e_staged():
        for d, h in zip(ins_d, ins_h):
            d.copy_(h, non_blocking=True)
        step(q, qd, qdd, tau)
        for h, d in zip(outs_h, outs_d):
            h.copy_(d, non_blocking=True)

    def time_e2e(fn):
        for _ in range(args.warmup):
            flush.zero_()
            fn()
        torch.cuda.synchronize()
        ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        barrier()
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush.zero_()
            ev2[k][0].record(stream)
            fn()
            ev2[k][1].record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_across_ranks(float(np.mean([a.elapsed_time(b) for a, b in ev2])), dist, dev)

    ms_e2e = time_e2e(e2e_mapped)
    e2e_value = aggregate_throughput(n, world, ms_e2e * 1e-3)
    ms_e2e_staged = time_e2e(e2e_staged)

    # the host link's own bandwidth (copy-engine copies of the same buffers, each direction
    # alone): the step cannot move its bytes faster than this
    def link_ms(copies):
        for _ in range(2):
            copies()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(5):
            copies()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 5

    d2h_ms = link_ms(lambda: [h.copy_(d, non_blocking=True) for h, d in zip(outs_h, outs_d)])
    h2d_ms = link_ms(lambda: [d.copy_(h, non_blocking=True) for d, h in zip(ins_d, ins_h)])
    # the mapped-host run must give the device run's results bit for bit
    step(q, qd, qdd, tau)
    e2e_mapped()
    torch.cuda.synchronize()
    e2e_identical = all(torch.equal(h, d.cpu()) for h, d in zip(outs_h, outs_d))

    # ---- per-op kernel times (same inputs) -------------------------------------------
    per_op = {}
    for name, ops in (("fk", N.OP_FK), ("jacobian", N.OP_JACOBIAN), ("crba", N.OP_MASS_MATRIX),
                      ("rnea", N.OP_INVERSE_DYNAMICS), ("aba", N.OP_FORWARD_DYNAMICS),
                      ("rnea+aba", N.OP_INVERSE_DYNAMICS | N.OP_FORWARD_DYNAMICS)):
        ts = []
        for k in range(10):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step(q, qd, qdd, tau, ops)
            b.record(stream)
            ts.append((a, b))
        torch.cuda.synchronize()
        t_ms = float(np.mean([a.elapsed_time(b) for a, b in ts[2:]]))
        per_op[name] = {"evals_per_s": n / (t_ms * 1e-3), "us": t_ms * 1e3}

    extras = None
    if rank == 0 and not args.no_extras:
        extras = secondary_workloads(dev)
    barrier()
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- roofline -------------------------------------------------------------------
    peaks, peak_src = measured_peaks()
    alg = algorithmic_bytes_per_env(nq, nv, nl) * n
    achieved_gbs = alg / (ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved_gbs / peaks["hbm_gbs"],
                "traffic": counters["dram_bytes_per_env"] * n if counters else None,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": alg}
    dfma = fp64_peak_dfma_per_s()
    alg = algorithmic_flops(robot)
    roofline_fp64 = None
    if dfma:
        peak_gflops = 2 * dfma / 1e9  # one DFMA = 2 flops
        ach = alg["step"] * n / (ms * 1e-3) / 1e9
        issued = counters["fp64_inst_per_env"] * n / (ms * 1e-3) / 1e9 if counters else None
        roofline_fp64 = {
            "bound": "fp64", "unit": "GFLOP/s", "peak": peak_gflops,
            "peak_source": "measured live: DFMA chain microbenchmark (bench_fp64_peak.cu), 2 flops per DFMA",
            "algorithmic_flops_per_env": alg["step"], "achieved": ach, "frac": ach / peak_gflops,
            "algorithmic_source": "oracle counting scalar: local-frame recursions, operations on structural "
                                  "zeros and ones skipped; the kernels' world-frame sweep needs fewer",
            "issued_inst_per_env": counters["fp64_inst_per_env"] if counters else None,
            "issued_inst_per_s": issued * 1e9 if counters else None,
            "issued_frac": issued / (dfma / 1e9) if counters else None,
            "issued_source": "ncu sass FP64 instruction counts of this kernel source "
                             f"(sha256 {KERNEL_SOURCE_SHA256[:12] or 'unset'}); frac against the DFMA issue peak",
            "source_matches_counters": kernel_source_digest(pm) == KERNEL_SOURCE_SHA256,
            "algorithmic_flops_per_op": alg}
    for name, r in per_op.items():
        r["algorithmic_gflops"] = alg[name] * n / (r["us"] * 1e-6) / 1e9

    # ---- CPU baseline on a bounded sample + parity of that sample --------------------
    from oracle.oracle import Oracle

    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    cores = host_cores()
    S = n  # the whole workload, as the reference arm times it
    o.batch_step(q_h[:256], qd_h[:256], qdd_h[:256], tau_h[:256], nthreads=cores)
    cpu_dt, reps = time_median(lambda: o.batch_step(q_h[:S], qd_h[:S], qdd_h[:S], tau_h[:S], nthreads=cores))
    ref = o.batch_step(q_h[:S], qd_h[:S], qdd_h[:S], tau_h[:S], nthreads=cores)
    S1 = min(n, 512)
    cpu1_dt, _ = time_median(lambda: o.batch_step(q_h[:S1], qd_h[:S1], qdd_h[:S1], tau_h[:S1], nthreads=1),
                             min_seconds=1.0)
    # the product's own sweep compiled for the host (sgdyn_host_step, world-frame algebra),
    # on the same cores: what a structured FP64 CPU implementation reaches, for context
    hout = [np.empty((n, c)) for c in (nl * 7, 6 * nv, nv * nv, nv, nv)]
    hin = [np.ascontiguousarray(a) for a in (q_h, qd_h, qdd_h, tau_h)]
    hp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731

    def host_step():
        N.check(L.sgdyn_host_step(pm._h, n, N.OP_ALL, *[hp(a) for a in hin], *[hp(a) for a in hout], N.ENV_MAJOR,
                                  cores))

    host_step()
    host_dt, host_reps = time_median(host_step)
    step(q, qd, qdd, tau)
    torch.cuda.synchronize()

    def rel(g, r):
        g = g.reshape(g.shape[0], -1)
        r = r.reshape(r.shape[0], -1)
        return float((np.abs(g - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-300)).max())

    first = lambda t, *shape: t[:, :S].T.reshape(S, *shape).cpu().numpy()  # noqa: E731  SoA -> [S, ...]
    errs = {"rnea": rel(first(tau_o, nv), ref["tau"]), "aba": rel(first(qdd_o, nv), ref["qdd"]),
            "crba": rel(first(M, nv, nv), ref["M"]), "jacobian": rel(first(J, 6, nv), ref["J"]),
            "fk_positions": rel(first(poses, nl, 7)[:, :, :3], ref["poses"][:, :, 9:])}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, nv, nl),
        "execution": {"parallelism": f"data-parallel replicas over environments x{world}", "kernel": kernel,
                      "launches_per_step": launches_per_step,
                      "step": "FK+Jacobian and CRBA+RNEA+ABA as two concurrent launches" if split
                      else "one fused launch"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": ms_e2e,
                "transfer": "sgdyn_step on mapped pinned host buffers (SoA): the kernel reads inputs from and "
                            "writes results to host memory over the host link",
                "results_identical_to_device_run": e2e_identical,
                "link": {"d2h_gbs": d2h / (d2h_ms * 1e6), "h2d_gbs": h2d / (h2d_ms * 1e6),
                         "floor_ms": max(d2h_ms, h2d_ms, ms),
                         "frac": max(d2h_ms, h2d_ms, ms) / ms_e2e,
                         "what": "copy-engine bandwidth of the host link for this step's outputs and inputs "
                                 "(each direction alone); floor = the larger of the outputs' transfer time, the "
                                 "inputs' and the device-resident step; frac = floor / e2e ms_per_step"},
                "staged_copies": {"value": aggregate_throughput(n, world, ms_e2e_staged * 1e-3),
                                  "ms_per_step": ms_e2e_staged,
                                  "transfer": "cudaMemcpyAsync host->device, kernel, device->host on one stream"}},
        "gpu_launches": args.steps * launches_per_step,
        "roofline": roofline,
        "roofline_fp64": roofline_fp64,
        "cpu_baseline": {"value": S / cpu_dt, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"the whole workload ({S} envs) per step, median of {reps} repetitions (>= 2 s)",
                         "single_thread_value": S1 / cpu1_dt, "nproc": os.cpu_count(), "cpu_model": cpu_model(),
                         "what": CPU_BASELINE_NOTE,
                         "host_sweep_value": n / host_dt,
                         "host_sweep": f"this library's sweep compiled for the host (sgdyn_host_step), {cores} threads, "
                                       f"the whole workload, median of {host_reps} repetitions (>= 2 s); for context, "
                                       "not the baseline"},
        "per_op_kernel": per_op,
        "max_rel_err_vs_oracle": errs,
        "clocks": clk,
        "secondary": extras,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
