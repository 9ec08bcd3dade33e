"""The header-only C++ drop-in (include/sgdyn_pinocchio_model.hpp, mirroring
sapien::PinocchioModel, pinocchio/pinocchio_model.h:27-130) compiled with g++ against
libsgdyn.so and driven the way a C++ caller of the reference class would; its results
against the oracle, on the CPU (the single-configuration methods run the host sweeps)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle.oracle import Oracle
from sapien_gb300 import synthetic as syn
from sapien_gb300 import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("cpp") / "drop_in_model")
    libdir = os.path.dirname(N.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "drop_in_model.cpp"),
                    "-L", libdir, "-lsgdyn", f"-Wl,-rpath,{libdir}", "-o", out], check=True)
    return out


def _run(program, robot, urdf_path, q, qd, qdd, tau, q0):
    fmt = lambda v: " ".join(repr(float(x)) for x in v)  # noqa: E731
    stdin = "\n".join([urdf_path, " ".join(robot.joint_names), " ".join(robot.link_names), str(robot.ee_link),
                       fmt(q), fmt(qd), fmt(qdd), fmt(tau), fmt(q0)]) + "\n"
    r = subprocess.run([program], input=stdin, capture_output=True, text=True, check=True)
    out = {}
    for line in r.stdout.splitlines():
        k, *v = line.split()
        out[k] = v
    return out


def rel(g, r):
    return np.abs(g - r).max() / max(np.abs(r).max(), 1e-300)


@pytest.mark.parametrize("name", ["arm9", "mixed_chain"])
def test_cpp_drop_in_matches_oracle(program, tmp_path, name):
    robot = {"arm9": syn.arm_with_fingers(sapien_style=True),
             "mixed_chain": syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                                 "continuous", "prismatic"])}[name]
    urdf_path = str(tmp_path / "robot.urdf")
    with open(urdf_path, "w") as f:
        f.write(robot.urdf)
    q, qd, qdd, tau = (a[0] for a in robot.sample(1, seed=8))
    q0 = q + np.random.default_rng(9).normal(scale=0.2, size=q.shape)
    out = _run(program, robot, urdf_path, q, qd, qdd, tau, q0)
    f = lambda k: np.array([float(x) for x in out[k]])  # noqa: E731
    assert out["error_before_order"] == ["runtime_error"]
    assert out["error_bad_name"] == ["invalid_argument"]
    assert out["error_bad_link"] == ["runtime_error"]
    o = Oracle(robot.urdf)
    o.set_joint_order(robot.joint_names)
    o.set_link_order(robot.link_names)
    nv, ee = robot.nv, robot.ee_link
    poses = f("poses").reshape(-1, 7)
    T = o.link_poses(q)
    assert np.abs(poses[:, :3] - T[:, :3, 3]).max() < 1e-6  # float32 poses, as sapien::Pose
    o.compute_full_jacobian(q)
    assert rel(f("jacobian_world").reshape(6, nv), o.get_link_jacobian(ee)) <= 1e-10
    assert rel(f("jacobian_local").reshape(6, nv), o.get_link_jacobian(ee, local=True)) <= 1e-10
    assert rel(f("jacobian_single").reshape(6, nv), o.compute_single_link_local_jacobian(q, ee)) <= 1e-10
    assert rel(f("mass_matrix").reshape(nv, nv), o.compute_generalized_mass_matrix(q)) <= 1e-10
    assert rel(f("coriolis").reshape(nv, nv), o.compute_coriolis_matrix(q, qd)) <= 1e-10
    assert rel(f("inverse_dynamics"), o.compute_inverse_dynamics(q, qd, qdd)) <= 1e-10
    assert rel(f("forward_dynamics"), o.compute_forward_dynamics(q, qd, tau)) <= 1e-8
    # IK to the (float32) end-effector pose, 50 fixed iterations, against the oracle's loop
    p = poses[ee]
    w, x, y, z = p[3:]
    T44 = np.eye(4)
    T44[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                   [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                   [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]]
    T44[:3, 3] = p[:3]
    qr, okr, errr = o.compute_inverse_kinematics(ee, T44, initial_qpos=q0, eps=0.0, max_iterations=50, dt=0.3,
                                                 damp=1e-3)
    assert rel(f("ik_q"), qr) <= 1e-8
    assert int(out["ik_success"][0]) == int(okr)
    rc = f("random_configuration")
    assert rc.shape == (robot.nq_ext,)
    for c, (kind, (lo, hi)) in enumerate(zip(robot.joint_kinds, robot.joint_limits)):
        if kind == syn.CONTINUOUS:
            lo, hi = -np.pi, np.pi
        assert lo <= rc[c] < hi
