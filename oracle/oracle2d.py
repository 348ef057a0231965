"""CPU oracle for the 2D branch of the FastIPC Newton loop — TEST INFRASTRUCTURE, NOT PRODUCT.

Only tests/ and bench.py's CPU-baseline leg use this module, as the checker.  It restates
``projects/FastIPC/NEWTON_IPC.py`` with ``dim == 2`` in numpy, with methods that differ from
the GPU path on purpose:
  * distances and their derivatives come from the C oracle's forward-mode automatic
    differentiation on points with z = 0 (``oracle.distance``), and the barrier Hessians are
    projected by cyclic Jacobi on the full 4x4 / 6x6 matrix;
  * the 2x2 SVD is numpy's, turned into the rotation-variant convention;
  * the system is assembled from triplets into scipy CSR and solved by sparse LU (standing in
    for CHOLMOD at NEWTON_IPC.py:774);
  * the all-pairs loops are numpy broadcasts.
With ``fast=True`` the element, constraint, CCD and intersection loops run in the C oracle
(``oracle2d_*`` in ipc_oracle.c, OpenMP, a Jacobi 2x2 SVD) for timing; both forms agree.
Every function names the reference lines it follows.
"""
import numpy as np

from . import oracle as O


# ----------------------------------------------------------------------------- element
def svd2(F):
    """Rotation-variant SVD of 2x2 matrices [N,2,2]: U, V rotations, s0 >= |s1|."""
    U, s, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, 1, 2).copy()
    for k in range(len(F)):
        if np.linalg.det(U[k]) < 0:
            U[k][:, 1] *= -1
            s[k, 1] *= -1
        if np.linalg.det(V[k]) < 0:
            V[k][:, 1] *= -1
            s[k, 1] *= -1
    return U, s, V


def fc_psi(s, la, mu):
    """fixed_corotated.py:6-13 (dim 2)."""
    return mu * ((s[:, 0] - 1) ** 2 + (s[:, 1] - 1) ** 2) + la / 2 * (s[:, 0] * s[:, 1] - 1) ** 2


def fc_P_dPdF(F, la, mu):
    """elasticity_first_piola_kirchoff_stress / _derivative (fixed_corotated.py:62-118, dim 2);
    dPdF indexed [j*2+i, s*2+r] as the reference stores it."""
    N = len(F)
    U, s, V = svd2(F)
    J = F[:, 0, 0] * F[:, 1, 1] - F[:, 0, 1] * F[:, 1, 0]
    cof = np.stack([np.stack([F[:, 1, 1], -F[:, 1, 0]], 1), np.stack([-F[:, 0, 1], F[:, 0, 0]], 1)], 1)
    R = U @ np.swapaxes(V, 1, 2)
    P = 2 * mu[:, None, None] * (F - R) + (la * (J - 1))[:, None, None] * cof
    s0, s1 = s[:, 0], s[:, 1]
    pm1 = s0 * s1 - 1
    g0 = 2 * mu * (s0 - 1) + s1 * la * pm1
    g1 = 2 * mu * (s1 - 1) + s0 * la * pm1
    Hs = np.stack([np.stack([2 * mu + la * s1 * s1, la * (pm1 + s1 * s0)], 1),
                   np.stack([la * (pm1 + s1 * s0), 2 * mu + la * s0 * s0], 1)], 1)
    Hs = O.make_pd2(Hs.reshape(N, 4)).reshape(N, 2, 2)
    left = mu - la / 2 * pm1
    right = (g0 + g1) / (2 * np.maximum(s0 + s1, 0.000001))
    B = np.stack([np.stack([left + right, left - right], 1), np.stack([left - right, left + right], 1)], 1)
    B = O.make_pd2(B.reshape(N, 4)).reshape(N, 2, 2)
    M = np.zeros((N, 4, 4))
    M[:, 0, 0], M[:, 0, 3], M[:, 3, 0], M[:, 3, 3] = Hs[:, 0, 0], Hs[:, 0, 1], Hs[:, 1, 0], Hs[:, 1, 1]
    M[:, 1, 1], M[:, 1, 2], M[:, 2, 1], M[:, 2, 2] = B[:, 0, 0], B[:, 0, 1], B[:, 1, 0], B[:, 1, 1]
    dPdF = np.zeros((N, 4, 4))
    # the reference's eight-term sum, term by term
    for j in range(2):
        for i in range(2):
            for ss in range(2):
                for r in range(2):
                    ij, rs = j * 2 + i, ss * 2 + r
                    Ui, Ur, Vj, Vs = U[:, i], U[:, r], V[:, j], V[:, ss]
                    dPdF[:, ij, rs] = (M[:, 0, 0] * Ui[:, 0] * Vj[:, 0] * Ur[:, 0] * Vs[:, 0] +
                                       M[:, 0, 3] * Ui[:, 0] * Vj[:, 0] * Ur[:, 1] * Vs[:, 1] +
                                       M[:, 1, 1] * Ui[:, 0] * Vj[:, 1] * Ur[:, 0] * Vs[:, 1] +
                                       M[:, 1, 2] * Ui[:, 0] * Vj[:, 1] * Ur[:, 1] * Vs[:, 0] +
                                       M[:, 2, 1] * Ui[:, 1] * Vj[:, 0] * Ur[:, 0] * Vs[:, 1] +
                                       M[:, 2, 2] * Ui[:, 1] * Vj[:, 0] * Ur[:, 1] * Vs[:, 0] +
                                       M[:, 3, 0] * Ui[:, 1] * Vj[:, 1] * Ur[:, 0] * Vs[:, 0] +
                                       M[:, 3, 3] * Ui[:, 1] * Vj[:, 1] * Ur[:, 1] * Vs[:, 1])
    return P, dPdF


def elements(tris, x, IB, vol, la, mu, dt):
    """compute_elasticity for dim 2 (NEWTON_IPC.py:568-624): energy [T], gradient [T,6] and
    Hessian [T,6,6] of dt^2 vol0 psi(F), F = [x1-x0, x2-x0] IB."""
    X = x[tris]
    Ds = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]], axis=2)
    F = Ds @ IB
    P, dPdF = fc_P_dPdF(F, la, mu)
    w = dt * dt * vol
    # G [T,4,6]: dF_ij / dx_{a,d}, rows j*2+i
    D = np.stack([-IB[:, 0, :] - IB[:, 1, :], IB[:, 0, :], IB[:, 1, :]], axis=1)    # [T,3(a),2(j)]
    G = np.zeros((len(tris), 4, 6))
    for j in range(2):
        for i in range(2):
            for a in range(3):
                G[:, j * 2 + i, 2 * a + i] = D[:, a, j]
    Pv = np.stack([P[:, 0, 0], P[:, 1, 0], P[:, 0, 1], P[:, 1, 1]], 1)             # vec (j*2+i)
    g = np.einsum('tk,tkn->tn', Pv, G) * w[:, None]
    H = np.einsum('tkn,tkl,tlm->tnm', G, dPdF, G) * w[:, None, None]
    _, s, _ = svd2(F)
    E = fc_psi(s, la, mu) * w
    return E, g, H


# ----------------------------------------------------------------------------- contact
def _pts3(x, rows, nv):
    pts = np.zeros((len(rows), 4, 3))
    for k in range(nv):
        pts[:, k, :2] = x[rows[:, k]]
    return pts


def barrier_rows(type_id, rows, x, dhat2, kappa):
    """PP_g_and_H / PE_g_and_H with 2D points (common/math/ipc.py:67-136): energy [N],
    gradient [N,2nv], projected Hessian [N,2nv,2nv]."""
    nv = 2 if type_id == 0 else 3
    rows = np.asarray(rows).reshape(-1, nv)
    N = len(rows)
    if N == 0:
        return np.zeros(0), np.zeros((0, 2 * nv)), np.zeros((0, 2 * nv, 2 * nv))
    d, dg, dH = O.distance(type_id, _pts3(x, rows, nv))
    keep = np.array([3 * v + c for v in range(nv) for c in range(2)])
    dg, dH = dg[:, keep], dH[:, keep][:, :, keep]
    bE, bg, bH = O.barrier_scalar(d, dhat2, kappa)
    g = bg[:, None] * dg
    H = bH[:, None, None] * np.einsum('ni,nj->nij', dg, dg) + bg[:, None, None] * dH
    return bE, g, O.project_pd(H)


def pe_type(p, e0, e1):
    """PE_type (common/math/distance.py:1757-1768), vectorised."""
    e = e1 - e0
    ratio = np.sum(e * (p - e0), -1) / np.sum(e * e, -1)
    return np.where(ratio < 0, 0, np.where(ratio > 1, 1, 2))


def pe_dist2(p, e0, e1):
    e = e1 - e0
    num = e[..., 1] * p[..., 0] - e[..., 0] * p[..., 1] + e1[..., 0] * e0[..., 1] - e1[..., 1] * e0[..., 0]
    return num * num / np.sum(e * e, -1)


def find_constraints(x, bp, be, dhat2):
    """find_constraints_2D_PE + np.unique (NEWTON_IPC.py:159-179, 348-356): PP [n,2], PE [n,3]."""
    dhat = dhat2 ** 0.5
    p = bp[:, None]
    e0, e1 = be[None, :, 0], be[None, :, 1]
    xp, x0, x1 = x[p], x[e0], x[e1]
    ok = (p != e0) & (p != e1)
    lo, hi = np.minimum(x0, x1), np.maximum(x0, x1)
    ok &= np.all((xp < hi + dhat) & (lo - dhat < xp), axis=-1)
    pp, pe = [], []
    P, E0, E1 = np.broadcast_to(p, ok.shape)[ok], np.broadcast_to(e0, ok.shape)[ok], np.broadcast_to(e1, ok.shape)[ok]
    c = pe_type(x[P], x[E0], x[E1])
    for q, a, b, k in zip(P, E0, E1, c):
        if k < 2:
            o = a if k == 0 else b
            if np.sum((x[q] - x[o]) ** 2) < dhat2:
                pp.append((min(q, o), max(q, o)))
        elif pe_dist2(x[q], x[a], x[b]) < dhat2:
            pe.append((q, a, b))
    PP = np.unique(np.array(pp, dtype=np.int64).reshape(-1, 2), axis=0)
    PE = np.unique(np.array(pe, dtype=np.int64).reshape(-1, 3), axis=0)
    return PP.astype(np.int32), PE.astype(np.int32)


def point_edge_ccd(x0, x1, x2, d0, d1, d2, eta):
    """point_edge_ccd with point_edge_ccd_impl and check_overlap (common/math/ipc.py:415-481)."""
    def overlap(root):
        p0, e0, e1 = x0 + d0 * root, x1 + d1 * root, x2 + d2 * root
        e = e1 - e0
        ratio = np.dot(e, p0 - e0) / np.dot(e, e)
        return 0 <= ratio <= 1

    def impl():
        toc = 1.0
        a = d0[0] * (d2[1] - d1[1]) + d0[1] * (d1[0] - d2[0]) + d2[0] * d1[1] - d2[1] * d1[0]
        b = (x0[0] * (d2[1] - d1[1]) + d0[0] * (x2[1] - x1[1]) + d0[1] * (x1[0] - x2[0]) + x0[1] * (d1[0] - d2[0]) +
             d1[1] * x2[0] + d2[0] * x1[1] - d1[0] * x2[1] - d2[1] * x1[0])
        c = x0[0] * (x2[1] - x1[1]) + x0[1] * (x1[0] - x2[0]) + x2[0] * x1[1] - x2[1] * x1[0]
        roots = []
        if a == 0 and b == 0 and c == 0:
            for xe, de in ((x1, d1), (x2, d2)):
                if np.dot(x0 - xe, d0 - de) < 0:
                    root = np.sqrt(np.dot(x0 - xe, x0 - xe) / np.dot(d0 - de, d0 - de))
                    if 0 < root <= 1:
                        toc = min(toc, root * (1 - eta))
            return toc
        if a == 0:
            if b != 0:
                roots = [-c / b]
        else:
            delta = b * b - 4 * a * c
            if delta == 0:
                roots = [-b / (2 * a)]
            elif delta > 0:
                sq = np.sqrt(delta)
                roots = [(-b - sq) / (2 * a), 2 * c / (-b - sq)] if b > 0 else [2 * c / (-b + sq), (-b + sq) / (2 * a)]
        for root in roots:
            if 0 < root <= 1 and overlap(root):
                toc = min(toc, root * (1 - eta))
        return toc

    k = pe_type(x0, x1, x2)
    dist2 = np.sum((x0 - x1) ** 2) if k == 0 else (np.sum((x0 - x2) ** 2) if k == 1 else pe_dist2(x0, x1, x2))
    mx = max(np.dot(d0, d0), np.dot(d1, d1), np.dot(d2, d2))
    toc = 1.0
    if mx > 0:
        lb = (1 - eta) * np.sqrt(dist2) / (2 * np.sqrt(mx))
        if lb <= 1:
            toc = max(impl(), lb)
    return toc


def ccd_step(x, p, bp, be, dhat2, eta=0.2):
    """compute_filter_2D_PE (NEWTON_IPC.py:361-374)."""
    dhat = dhat2 ** 0.5
    P, E0, E1 = bp[:, None], be[None, :, 0], be[None, :, 1]
    ok = (P != E0) & (P != E1)
    xa, xb, xc = x[P], x[E0], x[E1]
    pa, pb, pc = xa + p[P], xb + p[E0], xc + p[E1]
    lo_p, hi_p = np.minimum(xa, pa), np.maximum(xa, pa)
    lo_e = np.minimum(np.minimum(xb, xc), np.minimum(pb, pc))
    hi_e = np.maximum(np.maximum(xb, xc), np.maximum(pb, pc))
    ok &= np.all((lo_p < hi_e + dhat) & (lo_e - dhat < hi_p), axis=-1)
    alpha = 1.0
    for q, a, b in zip(np.broadcast_to(P, ok.shape)[ok], np.broadcast_to(E0, ok.shape)[ok], np.broadcast_to(E1, ok.shape)[ok]):
        alpha = min(alpha, point_edge_ccd(x[q], x[a], x[b], p[q], p[a], p[b], eta))
    return alpha


def check_collision(x, bp, tris):
    """check_collision_2D with point_inside_triangle (NEWTON_IPC.py:843-854, ipc.py:502-509)."""
    A, B, C = x[tris[:, 0]][None], x[tris[:, 1]][None], x[tris[:, 2]][None]
    cr = lambda u, v: u[..., 0] * v[..., 1] - u[..., 1] * v[..., 0]
    step = max(1, (1 << 22) // max(len(tris), 1))        # points per chunk: bounded memory
    for k in range(0, len(bp), step):
        q = bp[k:k + step]
        P = x[q][:, None, :]
        d1, d2, d3 = cr(P - B, A - B), cr(P - C, B - C), cr(P - A, C - A)
        neg = (d1 < 0) | (d2 < 0) | (d3 < 0)
        pos = (d1 > 0) | (d2 > 0) | (d3 > 0)
        own = (q[:, None] == tris[None, :, 0]) | (q[:, None] == tris[None, :, 1]) | (q[:, None] == tris[None, :, 2])
        if np.any(~(neg & pos) & ~own):
            return True
    return False


# ----------------------------------------------------------------------------- C (OpenMP) versions
def elements_c(tris, x, IB, vol, la, mu, dt):
    """elements() in the C oracle (ipc_oracle.c, oracle2d_elements): a Jacobi 2x2 SVD, OpenMP."""
    tr = np.ascontiguousarray(tris, dtype=np.int32)
    T = len(tr)
    E, g, H = np.zeros(T), np.zeros((T, 6)), np.zeros((T, 6, 6))
    O.lib().oracle2d_elements(T, O._p(tr, np.int32), O._p(O._f64(x)), O._p(O._f64(np.asarray(IB).reshape(T, 4))),
                              O._p(O._f64(vol)), O._p(O._f64(la)), O._p(O._f64(mu)), O.D(dt), O._p(E), O._p(g), O._p(H))
    return E, g, H


def find_constraints_c(x, bp, be, dhat2):
    """find_constraints() in the C oracle (candidate rows from OpenMP threads, then np.unique)."""
    bp32, be32, xx = np.ascontiguousarray(bp, np.int32), np.ascontiguousarray(be, np.int32), O._f64(x)
    cap = 1024
    while True:
        pp, pe, n = np.zeros((cap, 2), np.int32), np.zeros((cap, 3), np.int32), np.zeros(2, np.int32)
        O.lib().oracle2d_find(len(bp32), O._p(bp32, np.int32), len(be32), O._p(be32, np.int32), O._p(xx), O.D(dhat2), cap,
                              O._p(pp, np.int32), O._p(pe, np.int32), O._p(n, np.int32))
        if n.max() <= cap:
            break
        cap = int(n.max()) * 2
    return (np.unique(pp[:n[0]], axis=0).astype(np.int32).reshape(-1, 2),
            np.unique(pe[:n[1]], axis=0).astype(np.int32).reshape(-1, 3))


def ccd_step_c(x, p, bp, be, dhat2, eta=0.2):
    bp32, be32 = np.ascontiguousarray(bp, np.int32), np.ascontiguousarray(be, np.int32)
    L = O.lib()
    L.oracle2d_ccd_step.restype = O.ctypes.c_double
    return float(L.oracle2d_ccd_step(len(bp32), O._p(bp32, np.int32), len(be32), O._p(be32, np.int32), O._p(O._f64(x)),
                                     O._p(O._f64(p)), O.D(dhat2), O.D(eta)))


def check_collision_c(x, bp, tris):
    bp32, tr = np.ascontiguousarray(bp, np.int32), np.ascontiguousarray(tris, np.int32)
    return bool(O.lib().oracle2d_collision(len(bp32), O._p(bp32, np.int32), len(tr), O._p(tr, np.int32), O._p(O._f64(x))))


# ----------------------------------------------------------------------------- driver
class OracleSim2D:
    """NEWTON_IPC.py with dim == 2, one instance per scene (fixed-corotated triangles).
    fast=True runs the element, constraint, CCD and intersection loops in the C oracle (OpenMP
    on all host cores) instead of numpy; the results agree to rounding."""

    def __init__(self, scene, fast=False):
        self.fast = fast
        self.scene = scene
        self.dt, self.gravity = float(scene.dt), float(scene.gravity)
        self.dhat2 = float(scene.dhat) ** 2
        self.tris = np.asarray(scene.tris, np.int64)
        self.bp = np.asarray(scene.boundary_points, np.int64)
        self.be = np.asarray(scene.boundary_edges, np.int64).reshape(-1, 2)
        E, nu = scene.E, scene.nu
        nT = len(self.tris)
        self.la = np.full(nT, E * nu / ((1 + nu) * (1 - 2 * nu)))
        self.mu = np.full(nT, E / (2 * (1 + nu)))
        rest = np.asarray(scene.x, np.float64)
        # compute_restT_and_m (NEWTON_IPC.py:485-494)
        X = rest[self.tris]
        T = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]], axis=2)
        self.vol = np.linalg.det(T) / 2
        self.IB = np.linalg.inv(T)
        self.m = np.zeros(len(rest))
        np.add.at(self.m, self.tris.ravel(), np.repeat(self.vol * scene.rho / 3, 3))
        # compute_adaptive_kappa x 10 (NEWTON_IPC.py:116-124, 943)
        _, _, Hb = O.barrier_scalar(np.array([1e-16]), self.dhat2, 1.0)
        self.kappa = 1e13 * self.m.sum() / len(rest) / (4e-16 * Hb[0]) * 10
        self.mean_edge = float(np.mean(np.linalg.norm(rest[self.be[:, 0]] - rest[self.be[:, 1]], axis=1)))
        self.x = np.array(scene.initial_positions(), np.float64)
        self.v = np.array(scene.v, np.float64)
        self.newton_iters = []

    # NEWTON_IPC.py:497-511
    def compute_xn_and_xTilde(self):
        self.xn = self.x.copy()
        self.xTilde = self.x + self.dt * self.v
        self.xTilde[:, 1] += self.dt * self.dt * self.gravity

    def move_nodes(self, t):
        mask, val = self.scene.dirichlet(t)
        self.x[mask] = val[mask]
        self.xTilde[mask] = val[mask]

    def _elements(self):
        f = elements_c if self.fast else elements
        return f(self.tris, self.x, self.IB, self.vol, self.la, self.mu, self.dt)

    def find_constraints(self):
        f = find_constraints_c if self.fast else find_constraints
        self.PP, self.PE = f(self.x, self.bp, self.be, self.dhat2)
        return len(self.PP), len(self.PE)

    # NEWTON_IPC.py:514-542
    def compute_energy(self):
        e = 0.5 * np.sum(self.m * np.sum((self.x - self.xTilde) ** 2, 1))
        e += np.sum(self._elements()[0])
        for t, rows in ((0, self.PP), (1, self.PE)):
            if len(rows):
                e += np.sum(barrier_rows(t, rows, self.x, self.dhat2, self.kappa)[0])
        return float(e)

    # NEWTON_IPC.py:545-747: triplets (inertia, elasticity, barriers) and rhs = -grad
    def compute_hessian_and_gradient(self):
        import scipy.sparse as sp
        n = 2 * len(self.x)
        rows, cols, vals = [], [], []
        rhs = np.zeros(n)
        dof = np.arange(n)
        rows.append(dof)
        cols.append(dof)
        vals.append(np.repeat(self.m, 2))
        rhs -= np.repeat(self.m, 2) * (self.x - self.xTilde).ravel()

        def load(idx, g, H):
            d = (2 * idx[:, :, None] + np.arange(2)[None, None, :]).reshape(len(idx), -1)
            rows.append(np.repeat(d, d.shape[1], axis=1).ravel())
            cols.append(np.tile(d, (1, d.shape[1])).ravel())
            vals.append(H.reshape(len(idx), -1).ravel())
            np.add.at(rhs, d.ravel(), -g.ravel())
        _, g, H = self._elements()
        load(self.tris, g, H)
        for t, r in ((0, self.PP), (1, self.PE)):
            if len(r):
                _, g, H = barrier_rows(t, r, self.x, self.dhat2, self.kappa)
                load(np.asarray(r, np.int64), g, H)
        self.A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
        self.rhs = rhs

    # NEWTON_IPC.py:750-777
    def solve_system(self, t):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        mask, _ = self.scene.dirichlet(t)
        n = 2 * len(self.x)
        Dm = np.repeat(mask, 2)
        A = self.A.tocoo()
        keep = ~(Dm[A.row] | Dm[A.col])
        A = sp.csr_matrix((A.data * keep, (A.row, A.col)), shape=(n, n))
        idx = np.where(Dm)[0]
        A = A + sp.csr_matrix((np.ones(len(idx)), (idx, idx)), shape=(n, n))
        rhs = self.rhs.copy()
        rhs[Dm] = 0
        self.sol = spla.splu(A.tocsc()).solve(rhs)
        return self.sol

    def compute_intersection_free_step_size(self):
        f = ccd_step_c if self.fast else ccd_step
        return f(self.x, self.sol.reshape(-1, 2), self.bp, self.be, self.dhat2)

    def check_collision(self):
        f = check_collision_c if self.fast else check_collision
        return f(self.x, self.bp, self.tris)

    def apply_sol(self, alpha):
        self.x = self.xPrev + self.sol.reshape(-1, 2) * alpha

    # NEWTON_IPC.py:955-999
    def step(self, f, max_newton=1000, record=None):
        self.compute_xn_and_xTilde()
        self.move_nodes(f * self.dt)
        it = 0
        while True:
            it += 1
            self.find_constraints()
            self.compute_hessian_and_gradient()
            self.solve_system(f * self.dt)
            res = float(np.abs(self.sol).max())
            if record is not None:
                record.append({'PP': self.PP.copy(), 'PE': self.PE.copy(), 'rhs': self.rhs.copy(), 'sol': self.sol.copy(),
                               'residual': res, 'x': self.x.copy()})
            if res < 1e-2 * self.dt or it >= max_newton:
                break
            E0 = self.compute_energy()
            self.xPrev = self.x.copy()
            alpha = self.compute_intersection_free_step_size()
            if record is not None:
                record[-1]['E0'], record[-1]['alpha_ccd'] = E0, alpha
            self.apply_sol(alpha)
            while self.check_collision():
                alpha /= 2.0
                self.apply_sol(alpha)
            self.find_constraints()
            E = self.compute_energy()
            while E > E0:
                alpha *= 0.5
                self.apply_sol(alpha)
                self.find_constraints()
                E = self.compute_energy()
            while self.check_collision():
                alpha /= 2.0
                self.apply_sol(alpha)
            if record is not None:
                record[-1]['alpha'] = alpha
        self.v = (self.x - self.xn) / self.dt
        self.newton_iters.append(it)
        return it
