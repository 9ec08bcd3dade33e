"""CPU checks of the mathematics behind the analytic derivative kernels
(`sapien_gb300/csrc/diff_kernels.cuh`): a numpy restatement of the world-frame column
formulas for dtau/dq, dtau/dqd and M against central differences of the oracle's RNEA, and of
the tree-sparse L^T D L solve (pull-form L^T pass over descendant ranges, ancestor-chain L
pass) against a dense solve. Test infrastructure only."""
import numpy as np
import pytest
from scipy.linalg import expm

from oracle import urdf_model as um
from oracle.oracle import Oracle
from sapien_gb300 import synthetic as syn


def sk(w):
    return np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])


def crm(m):  # motion cross product matrix, (linear, angular) ordering
    X = np.zeros((6, 6))
    X[:3, :3] = sk(m[3:])
    X[:3, 3:] = sk(m[:3])
    X[3:, 3:] = sk(m[3:])
    return X


def crf(m):  # force cross product matrix
    return -crm(m).T


def quat_R(x, y, z, w):
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def rot_axis(a, t):
    K = sk(a)
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K


class WorldModel:
    """World-frame RNEA on the oracle's tree, q / v in tree order (angles for continuous)."""

    def __init__(self, om):
        self.om = om
        self.nj = om.njoints
        self.nvj = [0] + [um._NV[t] for t in om.jtype[1:]]
        self.nqj = [0] + [7 if t == um.JT_FREEFLYER else 1 for t in om.jtype[1:]]
        self.vc = [0] + [int(x) for x in np.cumsum([0] + self.nvj[1:])[:-1]]  # first column per joint
        self.qc = [0] + [int(x) for x in np.cumsum([0] + self.nqj[1:])[:-1]]
        self.nv, self.nq = sum(self.nvj), sum(self.nqj)

    def kinematics(self, q):
        om = self.om
        Rw, pw, S = [np.eye(3)], [np.zeros(3)], [None]
        for j in range(1, self.nj):
            Rp, pp = om.placement[j]
            lam = om.parent[j]
            B, o = Rw[lam] @ Rp, Rw[lam] @ pp + pw[lam]
            t, a, c = om.jtype[j], om.axis[j], self.qc[j]
            if t == um.JT_FREEFLYER:
                Rj, pj = B @ quat_R(*q[c + 3:c + 7]), B @ q[c:c + 3] + o
                Sj = np.zeros((6, 6))
                Sj[:3, :3], Sj[:3, 3:], Sj[3:, 3:] = Rj, sk(pj) @ Rj, Rj
            elif t == um.JT_PRISMATIC:
                Rj, pj = B, o + q[c] * (B @ a)
                Sj = np.zeros((6, 1))
                Sj[:3, 0] = B @ a
            else:
                Rj, pj, w = B @ rot_axis(a, q[c]), o, B @ a
                Sj = np.zeros((6, 1))
                Sj[:3, 0], Sj[3:, 0] = np.cross(pj, w), w
            Rw.append(Rj)
            pw.append(pj)
            S.append(Sj)
        return Rw, pw, S

    def rnea(self, q, qd, qdd):
        om = self.om
        Rw, pw, S = self.kinematics(q)
        v, a, I, f = [np.zeros(6)], [np.concatenate([-om.gravity, np.zeros(3)])], [None], [None]
        for j in range(1, self.nj):
            lam, c, n = om.parent[j], self.vc[j], self.nvj[j]
            vj = v[lam] + S[j] @ qd[c:c + n]
            aj = a[lam] + S[j] @ qdd[c:c + n] + crm(vj) @ (S[j] @ qd[c:c + n])
            Xf = np.zeros((6, 6))
            Xf[:3, :3], Xf[3:, 3:], Xf[3:, :3] = Rw[j], Rw[j], sk(pw[j]) @ Rw[j]
            Ij = Xf @ om.inertia6[j] @ Xf.T
            v.append(vj)
            a.append(aj)
            I.append(Ij)
            f.append(Ij @ aj + crf(vj) @ Ij @ vj)
        F = [None] + [x.copy() for x in f[1:]]
        for j in range(self.nj - 1, 0, -1):
            if om.parent[j] > 0:
                F[om.parent[j]] += F[j]
        tau = np.concatenate([S[j].T @ F[j] for j in range(1, self.nj)])
        return tau, dict(S=S, v=v, a=a, I=I, F=F)

    def integrate(self, q, dv):
        q = q.copy()
        for j in range(1, self.nj):
            c, vc = self.qc[j], self.vc[j]
            if self.om.jtype[j] == um.JT_FREEFLYER:
                T = np.eye(4)
                T[:3, :3], T[:3, 3] = quat_R(*q[c + 3:c + 7]), q[c:c + 3]
                tw = np.zeros((4, 4))
                tw[:3, :3], tw[:3, 3] = sk(dv[vc + 3:vc + 6]), dv[vc:vc + 3]
                T = T @ expm(tw)
                R = T[:3, :3]
                w = np.sqrt(1 + np.trace(R)) / 2
                q[c:c + 3] = T[:3, 3]
                q[c + 3:c + 7] = [(R[2, 1] - R[1, 2]) / (4 * w), (R[0, 2] - R[2, 0]) / (4 * w),
                                  (R[1, 0] - R[0, 1]) / (4 * w), w]
            else:
                q[c] += dv[vc]
        return q

    def is_ancestor(self, i, j):  # strict
        k = self.om.parent[j]
        while k > 0:
            if k == i:
                return True
            k = self.om.parent[k]
        return False

    def analytic(self, q, qd, qdd):
        """The kernels' column formulas: (dtau/dq, dtau/dqd, M)."""
        om, nj = self.om, self.nj
        _, W = self.rnea(q, qd, qdd)
        S, v, a, I, F = W["S"], W["v"], W["a"], W["I"], W["F"]
        Ib = [None] + [I[j].copy() for j in range(1, nj)]
        Db = [None] + [crf(v[j]) @ I[j] - I[j] @ crm(v[j]) for j in range(1, nj)]
        Hb = [None] + [I[j] @ v[j] for j in range(1, nj)]
        for j in range(nj - 1, 0, -1):
            p = om.parent[j]
            if p > 0:
                Ib[p] = Ib[p] + Ib[j]
                Db[p] = Db[p] + Db[j]
                Hb[p] = Hb[p] + Hb[j]
        dq, dqd, M = (np.zeros((self.nv, self.nv)) for _ in range(3))
        for j in range(1, nj):
            lam = om.parent[j]
            for l in range(self.nvj[j]):
                s, c = S[j][:, l], self.vc[j] + l
                u = crm(v[lam]) @ s
                beta = crm(a[lam]) @ s + crm(v[lam]) @ u
                gam = crm(v[lam] + v[j]) @ s
                Phi = crf(s) @ F[j] + Ib[j] @ beta + Db[j] @ u + crf(u) @ Hb[j]
                Psi = Db[j] @ s + crf(s) @ Hb[j] + Ib[j] @ gam
                for i in range(1, nj):
                    r = slice(self.vc[i], self.vc[i] + self.nvj[i])
                    if self.is_ancestor(i, j):
                        dq[r, c], dqd[r, c], M[r, c] = S[i].T @ Phi, S[i].T @ Psi, S[i].T @ Ib[j] @ s
                    elif i == j or self.is_ancestor(j, i):
                        P = Ib[i] @ S[i]
                        Q = np.stack([Db[i] @ S[i][:, k] - crf(S[i][:, k]) @ Hb[i] for k in range(S[i].shape[1])], 1)
                        dq[r, c], dqd[r, c], M[r, c] = P.T @ beta + Q.T @ u, Q.T @ s + P.T @ gam, P.T @ s
        return dq, dqd, M

    def column_tree(self):
        """Per velocity column: parent column and one past its last descendant column."""
        om = self.om
        lam, end = np.full(self.nv, -1), np.zeros(self.nv, dtype=int)
        sub_end = [0] * self.nj
        for j in range(self.nj - 1, 0, -1):
            sub_end[j] = max([j + 1] + [sub_end[k] for k in range(j + 1, self.nj) if om.parent[k] == j])
        for j in range(1, self.nj):
            p = om.parent[j]
            last = self.vc[sub_end[j]] if sub_end[j] < self.nj else self.nv
            for k in range(self.nvj[j]):
                t = self.vc[j] + k
                lam[t] = t - 1 if k > 0 else (self.vc[p] + self.nvj[p] - 1 if p > 0 else -1)
                end[t] = last
        return lam, end


def ltdl_factor(M, lam):
    H, n = np.tril(M).copy(), M.shape[0]
    for k in range(n - 1, -1, -1):
        i = lam[k]
        while i >= 0:
            f = H[k, i] / H[k, k]
            j = i
            while j >= 0:
                H[i, j] -= f * H[k, j]
                j = lam[j]
            H[k, i] = f
            i = lam[i]
    return H


def ltdl_solve(H, lam, end, B):
    B, n = B.copy(), H.shape[0]
    for i in range(n - 1, -1, -1):
        for k in range(i + 1, end[i]):
            B[i] -= H[k, i] * B[k]
    for k in range(n):
        B[k] = B[k] / H[k, k]
        i = lam[k]
        while i >= 0:
            B[k] -= H[k, i] * B[i]
            i = lam[i]
    return B


ROBOTS = {"chain7": lambda: syn.serial_chain(7), "arm9": syn.arm_with_fingers, "quadruped18": syn.quadruped,
          "humanoid": syn.humanoid}


def _case(name, seed):
    robot = ROBOTS[name]()
    om = um.build_model(robot.urdf)
    wm = WorldModel(om)
    rng = np.random.default_rng(seed)
    q = rng.uniform(-1, 1, wm.nq)
    for j in range(1, wm.nj):  # unit quaternions for free flyers
        if om.jtype[j] == um.JT_FREEFLYER:
            c = wm.qc[j]
            q[c + 3:c + 7] /= np.linalg.norm(q[c + 3:c + 7])
    return robot, om, wm, q, rng.normal(size=wm.nv), rng.normal(size=wm.nv)


@pytest.mark.parametrize("name", list(ROBOTS))
def test_column_formulas_match_finite_differences(name):
    robot, om, wm, q, qd, qdd = _case(name, 3)
    o = Oracle(robot.urdf)
    o.set_joint_order(om.joint_names[1:])  # tree order
    tau, _ = wm.rnea(q, qd, qdd)
    assert np.abs(tau - o.compute_inverse_dynamics(q, qd, qdd)).max() <= 1e-12 * np.abs(tau).max()
    dq, dqd, M = wm.analytic(q, qd, qdd)
    h = 1e-6
    fq, fqd = np.zeros_like(dq), np.zeros_like(dqd)
    for c in range(wm.nv):
        e = np.zeros(wm.nv)
        e[c] = h
        fq[:, c] = (wm.rnea(wm.integrate(q, e), qd, qdd)[0] - wm.rnea(wm.integrate(q, -e), qd, qdd)[0]) / (2 * h)
        fqd[:, c] = (wm.rnea(q, qd + e, qdd)[0] - wm.rnea(q, qd - e, qdd)[0]) / (2 * h)
    rel = lambda A, B: np.abs(A - B).max() / np.abs(B).max()
    assert rel(dq, fq) < 1e-7
    assert rel(dqd, fqd) < 1e-7
    assert rel(M, o.compute_generalized_mass_matrix(q)) < 1e-13


@pytest.mark.parametrize("name", list(ROBOTS))
def test_tree_sparse_ltdl_solve(name):
    _, _, wm, q, qd, qdd = _case(name, 5)
    _, _, M = wm.analytic(q, qd, qdd)
    lam, end = wm.column_tree()
    # M's sparsity is the column tree's: nonzero only between ancestor-related columns
    anc = np.zeros_like(M, dtype=bool)
    for k in range(wm.nv):
        i = k
        while i >= 0:
            anc[k, i] = anc[i, k] = True
            i = lam[i]
    assert np.all(M[~anc] == 0)
    assert all(all(anc[k, i] for k in range(i, end[i])) for i in range(wm.nv))  # descendant ranges
    H = ltdl_factor(M, lam)
    B = np.random.default_rng(1).normal(size=(wm.nv, 7))
    X = ltdl_solve(H, lam, end, B)
    assert np.abs(M @ X - B).max() <= 1e-10 * np.abs(B).max() * np.linalg.cond(M)
