"""The reference's own robots on the CPU: SAPIEN's create_pinocchio_model path
(articulation -> exported URDF, python/py_package/wrapper/pinocchio_model.py:317-329 and
urdf_exporter.py:21-152) against the robot's own URDF, in the oracle, and the product's
native articulation source against its URDF builder on the exported text."""
import numpy as np
import pytest

import reference_robots as rr
from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel
from sapien_gb300.articulation import create_pinocchio_model, export_kinematic_chain_urdf
from test_model_builder import parse_table


def _oracle(urdf, joints, links):
    o = Oracle(urdf)
    o.set_joint_order(joints)
    o.set_link_order(links)
    return o


def _exported(robot):
    art = rr.sapien_articulation(robot)
    urdf = export_kinematic_chain_urdf(art, force_fix_root=True)
    joints = [f"joint_{j.child_link.index}" for j in art.active_joints]
    links = [f"link_{l.index}" for l in art.links]
    return art, urdf, joints, links


@pytest.mark.parametrize("name", rr.DYNAMICS)
def test_exported_urdf_path_equals_direct_urdf_in_oracle(name):
    """The model SAPIEN builds from the articulation (dummy links, x axes, principal
    inertias) computes the same link poses, Jacobian, mass matrix, RNEA and ABA as the
    robot's URDF loaded directly, in the loader's joint and link order."""
    r = rr.load(name)
    _, urdf, joints, links = _exported(r)
    assert len(joints) == r.nv and len(links) == len(r.link_names)
    a = _oracle(r.urdf, r.joint_names, r.link_names)
    b = _oracle(urdf, joints, links)
    q, qd, qdd, tau = r.sample(16, seed=3)
    ra, rb = a.batch_step(q, qd, qdd, tau), b.batch_step(q, qd, qdd, tau)
    for k, tol in (("poses", 1e-12), ("J", 1e-12), ("M", 1e-11), ("tau", 1e-11), ("qdd", 1e-9)):
        x, y = ra[k].reshape(16, -1), rb[k].reshape(16, -1)
        err = (np.abs(x - y).max(axis=1) / np.maximum(np.abs(x).max(axis=1), 1e-300)).max()
        assert err <= tol, (k, err)


@pytest.mark.parametrize("name", rr.DYNAMICS)
def test_native_articulation_source_on_reference_robot(name):
    """sgdyn_model_from_articulation builds the tables the URDF builder makes from the
    exported text."""
    r = rr.load(name)
    art, urdf, joints, links = _exported(r)
    native = create_pinocchio_model(art, (0, 0, -9.81))
    ref = PinocchioModel(urdf, [0, 0, -9.81])
    ref.set_joint_order(joints)
    ref.set_link_order(links)
    a, b = parse_table(native.table_bytes()), parse_table(ref.table_bytes())
    assert (a["nj"], a["nv"], a["nq_ext"], a["nlinks"]) == (b["nj"], b["nv"], b["nq_ext"], b["nlinks"])
    for f in ("parent", "kind", "qcol", "vcol", "nv", "ivx"):
        assert np.array_equal(a["joints"][f], b["joints"][f]), f
    for f in ("R", "p", "axis", "m", "h", "I"):
        assert np.abs(a["joints"][f] - b["joints"][f]).max() < 1e-12, f
    assert np.array_equal(a["links"]["joint"], b["links"]["joint"])


def test_movo_reference_case_in_oracle_long_double():
    """unittest/test_physx/test_articulation.py:75-97's inputs: the oracle's double and
    long-double runs agree on every link pose and on the gravity torque."""
    r = rr.load("movo_simple")
    o = _oracle(r.urdf, r.joint_names, r.link_names)
    q, qd, qdd = rr.movo_reference_inputs()
    p64 = o.link_poses(q)
    t64 = o.compute_inverse_dynamics(q, qd, qdd)
    o.set_long_double(True)
    p80 = o.link_poses(q)
    t80 = o.compute_inverse_dynamics(q, qd, qdd)
    assert np.abs(p64 - p80).max() <= 1e-14
    assert np.abs(t64 - t80).max() <= 1e-12 * np.abs(t80).max()
    assert np.abs(t64).max() > 1.0  # gravity acts on the lift and the arm
