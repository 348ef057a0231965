"""CPU oracle of the ADMM-IPC time step (projects/FastIPC/ADMM_IPC.py) -- test infrastructure.

Only tests/ use this module, as the checker of fastipc_gb300.admm; nothing in the product
imports it.  It restates the script with numpy and scipy (and the C oracle's constraint finding,
CCD and intersection check, oracle/ipc_oracle.c):

  initial_guess        ADMM_IPC.py:296-313     AdmmOracle.initial_guess
  compute_filter       :181-268                AdmmOracle.compute_filter
  backup / reuse       :995-1040, 1230-1388    AdmmOracle.find_and_reuse
  global_step + PP..   :388-547                AdmmOracle.global_step (scipy sparse LU)
  solve_system filter  :549-631                AdmmOracle.global_step
  local_elasticity     :633-666                AdmmOracle.local_elasticity
  local_PP .. PEM      :668-960                AdmmOracle.local_rows
  dual_step            :962-994                AdmmOracle.dual_step

Parity unpinned.  The script calls its barrier helpers as functions of a row's relative vectors
with the first vertex at the origin (PP_gradient(op, pos), PT_hessian(op, p0, p1, p2), ...), but
common/math/ipc.py defines those helpers on all the row's points (its PP_gradient returns the
6-vector of both points), so the script does not run against its own library and produces no
golden vectors.  This restatement takes the derivatives the calls intend: with respect to the
vertices at pos_1..pos_{nv-1}, of the row energy at (0, pos_1, ..).  It is pinned to finite
differences and to the GPU path's own conventions only.  Methods differ from the GPU's on
purpose: the barrier derivatives come from the C oracle's forward-mode distance derivatives,
the 3x3 SVD and eigen-decompositions from numpy, the global solve from sparse LU.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import oracle as O

TYPE_NV = (2, 3, 4, 4, 4, 4, 4)
D = O.D


# ----------------------------------------------------------------------------- row energies
def _dist(kind, pts):
    E, g, H = O.distance(kind, pts.reshape(1, 4, 3))
    return E[0], g[0], H[0]


def row_energy(t, X, X0, dhat2, kappa, derivs=True):
    """Barrier energy of one row of list t at vertices X [nv,3] (rest positions X0 [4,3] for the
    mollified lists): E, and with derivs the gradient [3nv] and the Hessian [3nv,3nv] without
    the PSD projection (ipc.py *_energy, *_gradient, *_hessian)."""
    nv = TYPE_NV[t]
    P = np.zeros((4, 3))
    P[:nv] = X
    n = 3 * nv
    if t in (0, 1, 2, 3):                     # PP, PE, PT, EE on the row's own vertices
        d, dg, dH = _dist(t, P)
        dg, dH = dg[:n], dH[:n, :n]
    else:                                     # EEM: EE(a0,a1,b0,b1); PPM: PP(a0,b0); PEM: PE(a0,b0,b1)
        sel = {4: [0, 1, 2, 3], 5: [0, 2], 6: [0, 2, 3]}[t]
        kind = {4: 3, 5: 0, 6: 1}[t]
        Q = np.zeros((4, 3))
        Q[:len(sel)] = P[sel]
        d, g0, H0 = _dist(kind, Q)
        m = 3 * len(sel)
        idx = np.concatenate([3 * np.array(sel)[:, None] + np.arange(3)]).ravel()
        dg, dH = np.zeros(12), np.zeros((12, 12))
        dg[idx] = g0[:m]
        dH[np.ix_(idx, idx)] = H0[:m, :m]
    b, b1, b2 = O.barrier_scalar(np.array([d]), dhat2, kappa)
    b, b1, b2 = b[0], b1[0], b2[0]
    if t < 4:
        if not derivs:
            return b
        return b, b1 * dg, b2 * np.outer(dg, dg) + b1 * dH
    eps = 1e-3 * np.sum((X0[0] - X0[1]) ** 2) * np.sum((X0[2] - X0[3]) ** 2)
    M, Mg, MH = O.mollifier(P.reshape(1, 4, 3), np.array([eps]))
    M, Mg, MH = M[0], Mg[0], MH[0]
    if not derivs:
        return b * M
    g = M * b1 * dg + b * Mg
    H = M * (b2 * np.outer(dg, dg) + b1 * dH) + b1 * (np.outer(dg, Mg) + np.outer(Mg, dg)) + b * MH
    return b * M, g, H


def rel_energy(t, pos, X0, dhat2, kappa, derivs=True):
    """The row energy at (0, pos_1, .., pos_{nv-1}) and its derivatives with respect to pos;
    with derivs also the Frobenius norm of the whole row Hessian there."""
    nv = TYPE_NV[t]
    X = np.vstack([np.zeros((1, 3)), np.asarray(pos).reshape(nv - 1, 3)])
    if not derivs:
        return row_energy(t, X, X0, dhat2, kappa, False)
    E, g, H = row_energy(t, X, X0, dhat2, kappa)
    return E, g[3:], H[3:, 3:], float(np.sqrt((H * H).sum()))


# ----------------------------------------------------------------------------- small solves
def solve_n(A, b):
    """solve_N of common/math/wrapper/wrapper.cpp:90-198: LDL^T with symmetric pivoting (the
    remaining row of largest original diagonal magnitude first), pivots raised to 1e-8, the
    system rebuilt from the factors (in the pivoted order) and solved."""
    def ldlt(A):
        n = len(A)
        a = A.copy()
        dg = np.diag(A).copy()
        perm = []
        for k in range(n):
            p = k + int(np.argmax(np.abs(dg[k:])))
            perm.append(p)
            if p != k:
                a[[k, p]] = a[[p, k]]
                a[:, [k, p]] = a[:, [p, k]]
                dg[[k, p]] = dg[[p, k]]
            d = a[k, k]
            if d == 0.0:
                a[k + 1:, k] = 0.0
                a[k, k + 1:] = 0.0
                continue
            l = a[k + 1:, k] / d
            a[k + 1:, k + 1:] -= np.outer(l, a[k, k + 1:])
            a[k + 1:, k] = l
            a[k, k + 1:] = l
        return np.tril(a, -1) + np.eye(n), np.diag(a).copy(), perm

    A = (np.tril(A) + np.tril(A, -1).T)       # the lower triangle is what the factorisation reads
    L, Dd, _ = ldlt(A)
    F = L @ np.diag(np.maximum(Dd, 1e-8)) @ L.T
    L2, D2, perm = ldlt(F)
    y = np.array(b, dtype=np.float64).copy()
    for k, p in enumerate(perm):
        y[[k, p]] = y[[p, k]]
    y = np.linalg.solve(L2, y)
    y = np.where(D2 != 0, y / np.where(D2 != 0, D2, 1), 0.0)
    y = np.linalg.solve(L2.T, y)
    for k in reversed(range(len(perm))):
        p = perm[k]
        y[[k, p]] = y[[p, k]]
    return y


# ----------------------------------------------------------------------------- fixed-corotated
def fc3_psi(s, la, mu):
    return mu * np.sum((s - 1) ** 2) + la / 2 * (np.prod(s) - 1) ** 2


def fc3_grad(s, la, mu):
    P = np.prod(s)
    noI = np.array([s[1] * s[2], s[2] * s[0], s[0] * s[1]])
    return 2 * mu * (s - 1) + noI * la * (P - 1)


def fc3_hess(s, la, mu):
    P = np.prod(s)
    noI = np.array([s[1] * s[2], s[2] * s[0], s[0] * s[1]])
    H = np.diag(2 * mu + la * noI * noI)
    H[0, 1] = H[1, 0] = la * (s[2] * (P - 1) + noI[0] * noI[1])
    H[0, 2] = H[2, 0] = la * (s[1] * (P - 1) + noI[0] * noI[2])
    H[1, 2] = H[2, 1] = la * (s[0] * (P - 1) + noI[1] * noI[2])
    return H


def svd_rv(F):
    """Rotation-variant SVD: F = U diag(s) V^T with det U = det V = 1 (s[2] < 0 iff det F < 0)."""
    U, s, Vt = np.linalg.svd(F)
    V = Vt.T
    if np.linalg.det(U) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    if np.linalg.det(V) < 0:
        V[:, 2] *= -1
        s[2] *= -1
    return U, s, V


def project_pd(H):
    w, Q = np.linalg.eigh(H)
    if w[0] >= 0:
        return H
    return (Q * np.maximum(w, 0.0)) @ Q.T


# ----------------------------------------------------------------------------- the time step
class AdmmOracle(O.OracleSim):
    """ADMM_IPC.py's time step on the CPU for one scene (fixed-corotated, adaptive kappa without
    the Newton script's factor 10)."""

    def __init__(self, scene, admm_iters=20):
        super().__init__(scene, solver='direct')
        self.kappa /= 10.0
        self.admm_iters = admm_iters
        T = len(self.tets)
        self.W, self.z, self.u = np.zeros(T), np.zeros((T, 9)), np.zeros((T, 9))
        self.vol0 = np.abs(np.linalg.det(self.Dm.reshape(-1, 3, 3))) / 6.0
        self.A = np.linalg.inv(self.Dm.reshape(-1, 3, 3))
        self._empty_rows()

    def _empty_rows(self):
        self.rows_all = np.zeros((0, 4), np.int32)
        self.row_counts = [0] * 7
        self.y, self.r, self.Q = np.zeros((0, 9)), np.zeros((0, 9)), np.zeros(0)

    def _G(self, e):
        A = self.A[e]
        return np.vstack([-A.sum(axis=0), A])          # G[p][j]: shape-function gradients (X2F)

    def _F(self, x, e):
        t = self.tets[e]
        Ds = np.stack([x[t[1]] - x[t[0]], x[t[2]] - x[t[0]], x[t[3]] - x[t[0]]], axis=1)
        return Ds @ self.A[e]

    def initial_guess(self):
        self.compute_xn_and_xTilde()
        for e in range(len(self.tets)):
            self.W[e] = np.sqrt((self.la[e] + self.mu[e] * 2 / 3) * self.dt * self.dt * self.vol0[e])
            self.z[e] = self._F(self.xTilde, e).ravel()
        self.u[:] = 0.0
        self._empty_rows()

    def compute_filter(self, x, x_trial):
        p = np.ascontiguousarray(x_trial - x)
        x = np.ascontiguousarray(x)
        return O.lib().oracle_ccd_step(len(x), O._p(x), O._p(p), len(self.bp), O._p(self.bp, np.int32), len(self.be),
                                       O._p(self.be, np.int32), len(self.bt), O._p(self.bt, np.int32), len(self.tets),
                                       O._p(self.tets, np.int32), D(self.dhat2), D(self.inv_dx), D(0.2), 0)

    def _Q_bounds(self):
        dh = np.sqrt(self.dhat2)

        def fro(d):
            return rel_energy(0, np.full(3, d), np.zeros((4, 3)), self.dhat2, self.kappa)[3]
        return np.sqrt(fro(0.9 * dh)) / 10, np.sqrt(fro(1e-4 * dh)) * 10

    def find_and_reuse(self, alpha):
        old = {}
        off = 0
        for t in range(7):
            for k in range(self.row_counts[t]):
                old[(t, tuple(self.rows_all[off + k]))] = off + k
            off += self.row_counts[t]
        oy, orr, oQ = self.y, self.r, self.Q
        self.find_constraints()
        lists = []
        for t in range(7):
            r4 = np.zeros((len(self.rows[t]), 4), np.int32)
            r4[:, :TYPE_NV[t]] = self.rows[t]
            lists.append(r4)
        self.rows_all = np.concatenate(lists)
        self.row_counts = [len(r) for r in lists]
        n = len(self.rows_all)
        self.y, self.r, self.Q = np.zeros((n, 9)), np.zeros((n, 9)), np.zeros(n)
        minQ, maxQ = self._Q_bounds()
        blend = self.xTilde * alpha + self.x * (1 - alpha)
        c = 0
        for t in range(7):
            nv = TYPE_NV[t]
            for _ in range(self.row_counts[t]):
                ids = self.rows_all[c, :nv]
                key = (t, tuple(self.rows_all[c]))
                if key in old:
                    j = old[key]
                    self.y[c], self.r[c], self.Q[c] = oy[j], orr[j], oQ[j]
                else:
                    pos = (self.x[ids[0]] - self.x[ids[1:]]).ravel()
                    self.y[c, :3 * (nv - 1)] = (blend[ids[0]] - blend[ids[1:]]).ravel()
                    X0 = np.zeros((4, 3))
                    X0[:nv] = self.x0[self.rows_all[c, :nv]] if t >= 4 else 0.0
                    fro = rel_energy(t, pos, X0, self.dhat2, self.kappa)[3]
                    self.Q[c] = min(max(np.sqrt(fro), minQ), maxQ)
                c += 1

    def global_step(self, t_now):
        nV = len(self.x)
        rows, cols, vals = [np.arange(nV)], [np.arange(nV)], [self.m.copy()]
        rhs = self.m[:, None] * self.xTilde
        for e in range(len(self.tets)):
            G = self._G(e)
            w2 = self.W[e] ** 2
            K = w2 * G @ G.T
            tv = self.tets[e]
            rows.append(np.repeat(tv, 4))
            cols.append(np.tile(tv, 4))
            vals.append(K.ravel())
            Fz = (self.z[e] - self.u[e]).reshape(3, 3)
            np.add.at(rhs, tv, w2 * G @ Fz.T)
        c = 0
        for t in range(7):
            nv = TYPE_NV[t]
            EtE = np.eye(nv)
            EtE[0, 0] = nv - 1
            EtE[0, 1:] = EtE[1:, 0] = -1
            for _ in range(self.row_counts[t]):
                ids = self.rows_all[c, :nv]
                q2 = self.Q[c] ** 2
                rows.append(np.repeat(ids, nv))
                cols.append(np.tile(ids, nv))
                vals.append((q2 * EtE).ravel())
                yr = (self.y[c, :3 * (nv - 1)] - self.r[c, :3 * (nv - 1)]).reshape(nv - 1, 3) * q2
                rhs[ids[0]] += yr.sum(axis=0)
                np.add.at(rhs, ids[1:], -yr)
                c += 1
        A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nV, nV)).tocoo()
        mask, target = self.scene.dirichlet(t_now)
        keep = ~(mask[A.row] | mask[A.col])
        moved = mask[A.col] & ~mask[A.row]
        np.add.at(rhs, A.row[moved], -A.data[moved, None] * target[A.col[moved]])
        idx = np.where(mask)[0]
        A = sp.csr_matrix((np.concatenate([A.data[keep], np.ones(len(idx))]),
                           (np.concatenate([A.row[keep], idx]), np.concatenate([A.col[keep], idx]))), shape=(nV, nV))
        rhs[mask] = target[mask]
        lu = spla.splu(A.tocsc())
        sol = np.stack([lu.solve(rhs[:, d]) for d in range(3)], axis=1)
        xx = self.x.copy()
        alpha = self.compute_filter(xx, sol)
        self.x = sol * alpha + xx * (1 - alpha)
        while alpha >= 1e-6 and self.check_collision():
            self.x = (self.x + xx) / 2.0
            alpha /= 2.0
        if alpha < 1e-6:
            self.x = xx
        return alpha

    def local_elasticity(self):
        dt2 = self.dt * self.dt
        for e in range(len(self.tets)):
            U, s0, V = svd_rv(self._F(self.x, e) + self.u[e].reshape(3, 3))
            la, mu, wv, W2 = self.la[e], self.mu[e], dt2 * self.vol0[e], self.W[e] ** 2

            def energy(s):
                return fc3_psi(s, la, mu) * wv + np.sum((s - s0) ** 2) * W2 / 2
            s = s0.copy()
            for _ in range(256):
                g = fc3_grad(s, la, mu) * wv + (s - s0) * W2
                P = project_pd(fc3_hess(s, la, mu)) * wv + np.eye(3) * W2
                p = -np.linalg.inv(P) @ g
                done = p @ p < 1e-6
                alpha, s_0 = 1.0, s.copy()
                E0 = energy(s_0)
                s = s_0 + p
                E = energy(s)
                for _ in range(64):
                    if not E > E0:
                        break
                    alpha *= 0.5
                    s = s_0 + alpha * p
                    E = energy(s)
                if done:
                    break
                if np.array_equal(s, s_0):
                    break           # no movement: every later iteration repeats this one
            self.z[e] = (U @ np.diag(s) @ V.T).ravel()

    def local_rows(self):
        c = 0
        for t in range(7):
            nv = TYPE_NV[t]
            m = 3 * (nv - 1)
            for _ in range(self.row_counts[t]):
                ids = self.rows_all[c, :nv]
                pos = (self.x[ids[0]] - self.x[ids[1:]]).ravel()
                tgt = pos + self.r[c, :m]
                X0 = np.zeros((4, 3))
                if t >= 4:
                    X0[:nv] = self.x0[ids]
                q2 = self.Q[c] ** 2

                def energy(ps):
                    return rel_energy(t, ps, X0, self.dhat2, self.kappa, False) + np.sum((ps - tgt) ** 2) * q2 / 2
                for _ in range(256):
                    _, g, H, _ = rel_energy(t, pos, X0, self.dhat2, self.kappa)
                    g = g + (pos - tgt) * q2
                    P = H + np.eye(m) * q2
                    p = -solve_n(P, g)
                    done = p @ p < 1e-6
                    alpha, p0 = 1.0, pos.copy()
                    E0 = energy(p0)
                    pos = p0 + p
                    E = energy(pos)
                    for _ in range(64):
                        if not E > E0:
                            break
                        alpha *= 0.5
                        pos = p0 + alpha * p
                        E = energy(pos)
                    if done:
                        break
                    if np.array_equal(pos, p0):
                        break       # no movement: every later iteration repeats this one
                self.y[c, :m] = pos
                c += 1

    def dual_step(self):
        for e in range(len(self.tets)):
            self.u[e] += self._F(self.x, e).ravel() - self.z[e]
        c = 0
        for t in range(7):
            nv = TYPE_NV[t]
            m = 3 * (nv - 1)
            for _ in range(self.row_counts[t]):
                ids = self.rows_all[c, :nv]
                self.r[c, :m] += (self.x[ids[0]] - self.x[ids[1:]]).ravel() - self.y[c, :m]
                c += 1

    def admm_iteration(self, f, k):
        alpha = self.compute_filter(self.x, self.xTilde) if k == 0 else 0.0
        self.find_and_reuse(alpha)
        self.global_step(f * self.dt)
        self.local_elasticity()
        self.local_rows()
        self.dual_step()

    def step(self, f):
        self.initial_guess()
        for k in range(self.admm_iters):
            self.admm_iteration(f, k)
        self.v = (self.x - self.xn) / self.dt
        self.newton_iters.append(self.admm_iters)
        return self.admm_iters
