"""Native model construction from a SAPIEN-style articulation vs the URDF-export path
(CPU), and the float32 passive-force interop kernel vs the oracle (GPU)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from sapien_gb300 import PinocchioModel
from sapien_gb300.articulation import create_pinocchio_model, export_kinematic_chain_urdf, random_articulation
from test_model_builder import parse_table


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_native_source_matches_urdf_export(seed):
    art = random_articulation(7, seed=seed)
    native = create_pinocchio_model(art, (0, 0, -9.81))
    urdf = export_kinematic_chain_urdf(art, force_fix_root=True)
    ref = PinocchioModel(urdf, [0, 0, -9.81])
    ref.set_joint_order([f"joint_{j.child_link.index}" for j in art.active_joints])
    ref.set_link_order([f"link_{l.index}" for l in art.links])
    a, b = parse_table(native.table_bytes()), parse_table(ref.table_bytes())
    assert (a["nj"], a["nv"], a["nq_ext"], a["nlinks"]) == (b["nj"], b["nv"], b["nq_ext"], b["nlinks"])
    for f in ("parent", "kind", "qcol", "vcol", "nv", "ivx"):
        assert np.array_equal(a["joints"][f], b["joints"][f]), f
    for f in ("R", "p", "axis", "m", "h", "I"):
        assert np.abs(a["joints"][f] - b["joints"][f]).max() < 1e-12, f
    for f in ("R", "p"):
        assert np.abs(a["links"][f] - b["links"][f]).max() < 1e-12, f
    assert np.array_equal(a["links"]["joint"], b["links"]["joint"])
    # an unbounded revolute joint becomes continuous
    kinds = set(int(k) for k in a["joints"]["kind"][1:])
    assert kinds == {1, 2, 3}
    # joint limits reach the model on both paths: equal seeded random configurations
    qa = native.get_random_configuration_batched(64, seed=seed)
    qb = ref.get_random_configuration_batched(64, seed=seed)
    assert np.abs(qa - qb).max() <= 1e-12


def _oracle_for(art):
    o = Oracle(export_kinematic_chain_urdf(art, force_fix_root=True))
    o.set_joint_order([f"joint_{j.child_link.index}" for j in art.active_joints])
    o.set_link_order([f"link_{l.index}" for l in art.links])
    return o


@pytest.mark.gpu
def test_passive_force_on_padded_float32_buffers():
    import torch

    art = random_articulation(7, seed=4)
    pm = create_pinocchio_model(art)
    o = _oracle_for(art)
    n, dof, maxdof = 300, pm.nv, pm.nv + 3
    rng = np.random.default_rng(0)
    qpos = torch.zeros(n, maxdof, dtype=torch.float32)
    qvel = torch.zeros(n, maxdof, dtype=torch.float32)
    qpos[:, :dof] = torch.from_numpy(rng.uniform(-2, 2, (n, dof)).astype(np.float32))
    qvel[:, :dof] = torch.from_numpy(rng.normal(size=(n, dof)).astype(np.float32))
    qf = torch.full((n, maxdof), 7.0, dtype=torch.float32, device="cuda")
    q64, qd64 = qpos[:, :dof].double().numpy(), qvel[:, :dof].double().numpy()
    z = np.zeros(dof)
    cases = {(True, True): lambda e: o.compute_inverse_dynamics(q64[e], qd64[e], z),
             (True, False): lambda e: o.compute_inverse_dynamics(q64[e], z, z),
             (False, True): lambda e: o.compute_inverse_dynamics(q64[e], qd64[e], z) - o.compute_inverse_dynamics(q64[e], z, z)}
    for (g, c), ref in cases.items():
        out = pm.compute_passive_force_batched(qpos.cuda(), qvel.cuda(), gravity=g, coriolis_and_centrifugal=c,
                                               out=qf).cpu().numpy()
        assert np.all(out[:, dof:] == 7.0)  # padding untouched
        R = np.stack([ref(e) for e in range(n)])
        scale = np.maximum(np.abs(R).max(axis=1, keepdims=True), 1e-3)
        assert (np.abs(out[:, :dof] - R) / scale).max() < 2e-6
