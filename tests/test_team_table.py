"""Team tables (several lanes per environment) built on the host, checked without a GPU:
the trunk is a root-connected set that every lane runs, every other joint belongs to exactly
one lane together with its whole subtree, lanes list their joints parents first, and the
attach list holds exactly the trunk joints with a child on a lane."""
import ctypes

import numpy as np
import pytest

from sapien_gb300 import PinocchioModel, synthetic as syn
from sapien_gb300 import _native as N
from test_model_builder import parse_table

ROBOTS = {
    "arm9": lambda: syn.arm_with_fingers(),
    "quadruped": lambda: syn.quadruped(),
    "humanoid": lambda: syn.humanoid(),
    "humanoid_sapien": lambda: syn.humanoid(sapien_style=True),
    "chain7": lambda: syn.serial_chain(7),
}


def team(pm, L):
    p, n = ctypes.POINTER(ctypes.c_int)(), ctypes.c_int()
    N.check(N.load().sgdyn_model_team_table(pm._h, L, ctypes.byref(p), ctypes.byref(n)))
    t = [p[k] for k in range(n.value)]
    Lr, nt, sm, na = t[:4]
    off = 4
    trunk = t[off:off + nt]
    off += nt
    lanes = [t[off + r * sm: off + (r + 1) * sm] for r in range(Lr)]
    off += Lr * sm
    attach = t[off:off + na]
    off += na
    owner = t[off:]
    return Lr, trunk, lanes, attach, owner


@pytest.mark.parametrize("name", list(ROBOTS))
@pytest.mark.parametrize("L", [1, 2, 4, 8])
def test_team_table_invariants(name, L):
    r = ROBOTS[name]()
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    pm.set_joint_order(r.joint_names)
    pm.set_link_order(r.link_names)
    parent = parse_table(pm.table_bytes())["joints"]["parent"]
    nj = len(parent)
    Lr, trunk, lanes, attach, owner = team(pm, L)
    assert Lr == L and len(owner) == nj and owner[0] == -1
    # trunk: sorted, root-connected
    assert trunk == sorted(trunk)
    for j in trunk:
        assert parent[j] == 0 or parent[j] in trunk
        assert owner[j] == -1
    # every other joint on exactly one lane, with its parent on the same lane or in the trunk
    seen = {}
    for role, lst in enumerate(lanes):
        real = [j for j in lst if j > 0]
        assert real == sorted(real) and all(j == 0 for j in lst[len(real):])
        for j in real:
            assert j not in seen and j not in trunk
            seen[j] = role
            assert owner[j] == role
            p = parent[j]
            assert p == 0 or p in trunk or seen.get(p) == role
    assert sorted(list(seen) + trunk) == list(range(1, nj))
    # attach = trunk joints with a child on a lane
    want = sorted({int(parent[j]) for j in seen if parent[j] in trunk})
    assert sorted(attach) == want


def test_team_table_splits_the_humanoid():
    """Four lanes: root + spine in the trunk, the four limbs one per lane."""
    r = syn.humanoid()
    pm = PinocchioModel(r.urdf, [0, 0, -9.81])
    pm.set_joint_order(r.joint_names)
    pm.set_link_order(r.link_names)
    _, trunk, lanes, _, _ = team(pm, 4)
    assert len(trunk) == 4
    assert sorted(len([j for j in lst if j > 0]) for lst in lanes) == [6, 6, 7, 7]
