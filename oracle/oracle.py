"""CPU oracle for the FastIPC Newton inner loop — TEST INFRASTRUCTURE, NOT PRODUCT.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module,
always as the checker.  It wraps ``ipc_oracle.c`` (built into ``oracle/_build`` by
``build()``) and restates the driver of ``projects/FastIPC/NEWTON_IPC.py:934-1003`` in numpy:
every method names the reference function it follows.  The linear solve uses scipy's sparse
LU (exact, standing in for CHOLMOD at ``NEWTON_IPC.py:774``) or, at sizes where a
factorisation is impractical, the C block-Jacobi PCG.
"""
import ctypes
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_build', 'libipc_oracle.so')
TYPES = ['PP', 'PE', 'PT', 'EE', 'EEM', 'PPM', 'PEM']
TYPE_NV = [2, 3, 4, 4, 4, 4, 4]

_lib = None


def build(force=False):
    """Compile ipc_oracle.c (gcc, OpenMP, no FMA contraction so x86 and Arm agree)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    src = os.path.join(HERE, 'ipc_oracle.c')
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + f'.{os.getpid()}.tmp'
        subprocess.check_call(['gcc', '-O2', '-std=gnu11', '-fopenmp', '-ffp-contract=off', '-fPIC', '-shared',
                               src, '-o', tmp, '-lm'])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.oracle_ccd_step.restype = ctypes.c_double
        _lib.oracle_energy.restype = ctypes.c_double
    return _lib


def _p(a, dtype=np.float64):
    if a is None:
        return None
    assert a.dtype == dtype and a.flags['C_CONTIGUOUS'], (a.dtype, dtype)
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


D = ctypes.c_double


# ----------------------------------------------------------------------------- kernels
def barrier_scalar(d, dhat2, kappa):
    d = _f64(d)
    E, g, H = np.empty_like(d), np.empty_like(d), np.empty_like(d)
    lib().oracle_barrier_scalar(len(d), _p(d), D(dhat2), D(kappa), _p(E), _p(g), _p(H))
    return E, g, H


def distance(kind, pts):
    """kind 0 PP, 1 PE, 2 PT, 3 EE, 4 EECN2; pts [N,4,3] -> E [N], g [N,n], H [N,n,n]."""
    pts = _f64(pts).reshape(-1, 4, 3)
    n = 3 * [2, 3, 4, 4, 4][kind]
    N = len(pts)
    E, g, H = np.zeros(N), np.zeros((N, 12)), np.zeros((N, 144))
    lib().oracle_distance(kind, N, _p(pts), _p(E), _p(g), _p(H))
    return E, g[:, :n], H[:, :n * n].reshape(N, n, n)


def mollifier(pts, eps):
    pts, eps = _f64(pts), _f64(eps)
    N = len(pts)
    E, g, H = np.zeros(N), np.zeros((N, 12)), np.zeros((N, 144))
    lib().oracle_mollifier(N, _p(pts), _p(eps), _p(E), _p(g), _p(H))
    return E, g, H.reshape(N, 12, 12)


def types(pts):
    pts = _f64(pts)
    N = len(pts)
    a, b, c = np.zeros(N, np.int32), np.zeros(N, np.int32), np.zeros(N, np.int32)
    lib().oracle_types(N, _p(pts), _p(a, np.int32), _p(b, np.int32), _p(c, np.int32))
    return a, b, c


def barrier_rows(type_id, rows, x, x0, dhat2, kappa, derivs=True):
    """Per-row barrier energy [N], gradient [N,n], projected Hessian [N,n,n] (ipc.py *_g_and_H)."""
    rows = np.zeros((0, 4), np.int32) if len(rows) == 0 else np.asarray(rows)
    r4 = np.zeros((len(rows), 4), np.int32)
    r4[:, :rows.shape[1]] = rows
    x, x0 = _f64(x), _f64(x0)
    N = len(r4)
    n = 3 * TYPE_NV[type_id]
    E = np.zeros(N)
    g = np.zeros((N, 12)) if derivs else None
    H = np.zeros((N, 144)) if derivs else None
    lib().oracle_barrier_rows(type_id, N, _p(r4, np.int32), _p(x), _p(x0), D(dhat2), D(kappa), _p(E), _p(g), _p(H))
    if not derivs:
        return E
    return E, g[:, :n], H[:, :n * n].reshape(N, n, n)


def project_pd(A):
    A = _f64(A)
    N, n = A.shape[0], A.shape[1]
    out = np.zeros_like(A)
    lib().oracle_project_pd(N, n, _p(A), _p(out))
    return out


def make_pd2(A):
    A = _f64(A)
    out = np.zeros_like(A)
    lib().oracle_make_pd2(len(A), _p(A), _p(out))
    return out


def svd3(F):
    F = _f64(F).reshape(-1, 3, 3)
    U, s, V = np.zeros_like(F), np.zeros((len(F), 3)), np.zeros_like(F)
    for i in range(len(F)):
        lib().oracle_svd3(_p(F[i]), _p(U[i]), _p(s[i]), _p(V[i]))
    return U, s, V


def nh_material(F, la, mu):
    F = _f64(F).reshape(-1, 3, 3)
    N = len(F)
    psi, P, dP = np.zeros(N), np.zeros((N, 3, 3)), np.zeros((N, 9, 9))
    lib().oracle_nh_material(N, _p(F), D(la), D(mu), _p(psi), _p(P), _p(dP))
    return psi, P, dP


def elasticity(tets, x, Dm, la, mu, dt, derivs=True):
    tets, x, Dm, la, mu = _i32(tets), _f64(x), _f64(Dm), _f64(la), _f64(mu)
    T = len(tets)
    E = np.zeros(T)
    g = np.zeros((T, 12)) if derivs else None
    H = np.zeros((T, 144)) if derivs else None
    lib().oracle_elasticity(T, _p(tets, np.int32), _p(x), _p(Dm), _p(la), _p(mu), D(dt), _p(E), _p(g), _p(H))
    return (E, g, H.reshape(T, 12, 12)) if derivs else E


def inversion_free(xs, ps, eta=0.2):
    xs, ps = _f64(xs), _f64(ps)
    out = np.zeros(len(xs))
    lib().oracle_inversion_free(len(xs), _p(xs), _p(ps), D(eta), _p(out))
    return out


def ccd(kind, x, p, eta=0.2):
    """kind 0 point-triangle, 1 edge-edge; x, p [N,4,3] -> time of impact [N]"""
    x, p = _f64(x), _f64(p)
    out = np.zeros(len(x))
    lib().oracle_ccd(kind, len(x), _p(x), _p(p), D(eta), _p(out))
    return out


def seg_tri(pts):
    pts = _f64(pts)
    out = np.zeros(len(pts), np.int32)
    lib().oracle_seg_tri(len(pts), _p(pts), _p(out, np.int32))
    return out.astype(bool)


# ----------------------------------------------------------------------------- the simulation
class OracleSim:
    """The reference's Newton driver (NEWTON_IPC.py) on the CPU, for one scene."""

    def __init__(self, scene, solver='direct', pcg_rtol=1e-10, pcg_maxit=100000):
        import scipy.sparse  # noqa: F401
        self.scene = scene
        self.x = _f64(scene.x.copy())
        self.v = _f64(scene.v.copy())
        self.tets = _i32(scene.tets)
        self.bp, self.be, self.bt = _i32(scene.boundary_points), _i32(scene.boundary_edges), _i32(scene.boundary_triangles)
        self.dt = float(scene.dt)
        self.dhat2 = float(scene.dhat) ** 2
        self.gravity = float(scene.gravity)
        self.solver, self.pcg_rtol, self.pcg_maxit = solver, pcg_rtol, pcg_maxit
        self.timings = {}
        self.compute_restT_and_m()
        self.kappa = self.compute_adaptive_kappa() * 10
        self.inv_dx = 1.0 / self.compute_mean_of_boundary_edges()
        self.x0 = self.x.copy()                                           # save_x0
        self.x = _f64(scene.initial_positions().copy())
        self.rows = [np.zeros((0, w), np.int32) for w in TYPE_NV]
        self.newton_iters = []
        self.pcg_iters = []
        if solver == 'bsr':
            self._bsr_pattern()

    # NEWTON_IPC.py:485-494, 145-155
    def compute_restT_and_m(self):
        t = self.tets
        X = self.x
        Dm = np.stack([X[t[:, 1]] - X[t[:, 0]], X[t[:, 2]] - X[t[:, 0]], X[t[:, 3]] - X[t[:, 0]]], axis=2)
        self.Dm = _f64(Dm.reshape(-1, 9))
        det = np.linalg.det(Dm)
        if (det < 0).any():
            raise ValueError('mesh inverted')
        mass = det / 3 / 2 * self.scene.rho / 4
        self.m = np.zeros(len(X))
        for k in range(4):
            np.add.at(self.m, t[:, k], mass)
        E, nu = self.scene.E, self.scene.nu
        self.la = np.full(len(t), E * nu / ((1 + nu) * (1 - 2 * nu)))
        self.mu = np.full(len(t), E / (2 * (1 + nu)))

    # NEWTON_IPC.py:116-124
    def compute_adaptive_kappa(self):
        _, _, H_b = barrier_scalar(np.array([1.0e-16]), self.dhat2, 1.0)
        return 1.0e13 * self.m.sum() / len(self.m) / (4.0e-16 * H_b[0])

    # NEWTON_IPC.py:127-134
    def compute_mean_of_boundary_edges(self):
        e = self.be
        return float(np.linalg.norm(self.x[e[:, 0]] - self.x[e[:, 1]], axis=1).sum() / len(e))

    def _tic(self, k):
        self.timings.setdefault(k, 0.0)
        self.timings[k] -= time.perf_counter()

    def _toc(self, k):
        self.timings[k] += time.perf_counter()

    # NEWTON_IPC.py:497-511
    def compute_xn_and_xTilde(self):
        self.xn = self.x.copy()
        self.xTilde = self.x + self.dt * self.v
        self.xTilde[:, 1] += self.dt * self.dt * self.gravity

    def move_nodes(self, t):
        mask, val = self.scene.dirichlet(t)
        self.x[mask] = val[mask]
        self.xTilde[mask] = val[mask]

    # NEWTON_IPC.py:337-357
    def find_constraints(self):
        self._tic('Find constraints')
        counts = np.zeros(7, np.int32)
        L = lib()
        L.oracle_find_constraints(len(self.x), _p(self.x), _p(self.x0), len(self.bp), _p(self.bp, np.int32),
                                  len(self.be), _p(self.be, np.int32), len(self.bt), _p(self.bt, np.int32),
                                  D(self.dhat2), D(self.inv_dx), _p(counts, np.int32))
        rows = []
        for k in range(7):
            r = np.zeros((counts[k], 4), np.int32)
            L.oracle_get_rows(k, _p(r, np.int32))
            rows.append(r[:, :TYPE_NV[k]])
        self.rows = rows
        self._toc('Find constraints')
        return rows

    # NEWTON_IPC.py:514-542
    def compute_energy(self, x=None):
        x = self.x if x is None else x
        counts = np.array([len(r) for r in self.rows], np.int32)
        allr = np.zeros((int(counts.sum()), 4), np.int32)
        o = 0
        for r in self.rows:
            allr[o:o + len(r), :r.shape[1]] = r
            o += len(r)
        return lib().oracle_energy(len(x), _p(_f64(x)), _p(self.xTilde), _p(self.m), len(self.tets), _p(self.tets, np.int32),
                                   _p(self.Dm), _p(self.la), _p(self.mu), D(self.dt), _p(self.x0), _p(counts, np.int32),
                                   _p(allr, np.int32), D(self.dhat2), D(self.kappa))

    # static 3x3 block pattern of inertia + elasticity (large scenes: solver='bsr')
    def _bsr_pattern(self):
        nV, t = len(self.x), self.tets.astype(np.int64)
        pairs = (t[:, :, None] * nV + t[:, None, :]).reshape(-1)
        keys = np.unique(np.concatenate([pairs, np.arange(nV, dtype=np.int64) * (nV + 1)]))
        self.bsr_keys = keys
        self.bsr_rp = np.ascontiguousarray(np.searchsorted(keys, np.arange(nV + 1, dtype=np.int64) * nV).astype(np.int64))
        self.bsr_ci = np.ascontiguousarray((keys % nV).astype(np.int32))
        self.bsr_pos16 = np.ascontiguousarray(np.searchsorted(keys, pairs).astype(np.int64))
        self.bsr_diag = np.ascontiguousarray(np.searchsorted(keys, np.arange(nV, dtype=np.int64) * (nV + 1)).astype(np.int64))

    def _assemble_bsr(self):
        nV = len(self.x)
        n = 3 * nV
        rhs = -(np.repeat(self.m, 3) * (self.x - self.xTilde).ravel())
        _, g, H = elasticity(self.tets, self.x, self.Dm, self.la, self.mu, self.dt)
        dof = (3 * self.tets[:, :, None] + np.arange(3)).reshape(-1, 12)
        np.add.at(rhs, dof, -g)
        val = np.zeros((len(self.bsr_keys), 9))
        lib().oracle_bsr_accumulate(len(self.tets), _p(self.bsr_pos16, np.int64), _p(_f64(H)), _p(val))
        val[self.bsr_diag, 0] += self.m
        val[self.bsr_diag, 4] += self.m
        val[self.bsr_diag, 8] += self.m
        ck, cv = [], []
        for k in range(7):
            r = self.rows[k]
            if len(r) == 0:
                continue
            _, gb, Hb = barrier_rows(k, r, self.x, self.x0, self.dhat2, self.kappa)
            nv = r.shape[1]
            dof = (3 * r[:, :, None] + np.arange(3)).reshape(-1, 3 * nv)
            np.add.at(rhs, dof, -gb)
            ck.append((r[:, :, None].astype(np.int64) * nV + r[:, None, :]).reshape(-1))
            cv.append(Hb.reshape(-1, nv, 3, nv, 3).transpose(0, 1, 3, 2, 4).reshape(-1, 9))
        if ck:
            ck, cv = np.concatenate(ck), np.concatenate(cv)
            uk, inv = np.unique(ck, return_inverse=True)
            cva = np.zeros((len(uk), 9))
            np.add.at(cva, inv.ravel(), cv)
        else:
            uk, cva = np.zeros(0, np.int64), np.zeros((0, 9))
        self.c_rp = np.ascontiguousarray(np.searchsorted(uk, np.arange(nV + 1, dtype=np.int64) * nV).astype(np.int64))
        self.c_ci = np.ascontiguousarray((uk % nV).astype(np.int32))
        self.c_va = np.ascontiguousarray(cva)
        self.bsr_val = val
        self.rhs = rhs

    # NEWTON_IPC.py:558-747: inertia, elasticity, barriers -> (CSR matrix, rhs)
    def compute_hessian_and_gradient(self):
        if self.solver == 'bsr':
            self._tic('Build System')
            self._assemble_bsr()
            self._toc('Build System')
            return None, self.rhs
        import scipy.sparse as sp
        self._tic('Build System')
        n = 3 * len(self.x)
        rhs = -(np.repeat(self.m, 3) * (self.x - self.xTilde).ravel())
        rows_l, cols_l, vals_l = [np.arange(n)], [np.arange(n)], [np.repeat(self.m, 3)]
        _, g, H = elasticity(self.tets, self.x, self.Dm, self.la, self.mu, self.dt)
        dof = (3 * self.tets[:, :, None] + np.arange(3)).reshape(-1, 12)
        np.add.at(rhs, dof, -g)
        rows_l.append(np.repeat(dof, 12, axis=1).ravel())
        cols_l.append(np.tile(dof, (1, 12)).ravel())
        vals_l.append(H.ravel())
        for k in range(7):
            r = self.rows[k]
            if len(r) == 0:
                continue
            _, gb, Hb = barrier_rows(k, r, self.x, self.x0, self.dhat2, self.kappa)
            nd = 3 * r.shape[1]
            dof = (3 * r[:, :, None] + np.arange(3)).reshape(-1, nd)
            np.add.at(rhs, dof, -gb)
            rows_l.append(np.repeat(dof, nd, axis=1).ravel())
            cols_l.append(np.tile(dof, (1, nd)).ravel())
            vals_l.append(Hb.ravel())
        A = sp.csr_matrix((np.concatenate(vals_l), (np.concatenate(rows_l), np.concatenate(cols_l))), shape=(n, n))
        A.sort_indices()
        self.A, self.rhs = A, rhs
        self._toc('Build System')
        return A, rhs

    # NEWTON_IPC.py:750-777
    def solve_system(self, t):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        self._tic('Solve System')
        mask, _ = self.scene.dirichlet(t)
        n = 3 * len(self.x)
        Dm = np.repeat(mask, 3)
        rhs = self.rhs.copy()
        if self.solver == 'bsr':
            fixed = np.ascontiguousarray(mask.astype(np.uint8))
            sol = np.zeros(n)
            it = lib().oracle_bsr_pcg(len(self.x), _p(self.bsr_rp, np.int64), _p(self.bsr_ci, np.int32), _p(self.bsr_val),
                                      _p(self.c_rp, np.int64), _p(self.c_ci, np.int32), _p(self.c_va),
                                      _p(self.bsr_diag, np.int64), _p(_f64(rhs)), _p(fixed, np.uint8), D(self.pcg_rtol),
                                      self.pcg_maxit, _p(sol))
            self.pcg_iters.append(it)
            self.sol = sol
        elif self.solver == 'direct':
            A = self.A.tocoo()
            keep = ~(Dm[A.row] | Dm[A.col])
            A = sp.csr_matrix((A.data * keep, (A.row, A.col)), shape=(n, n))
            idx = np.where(Dm)[0]
            A = A + sp.csr_matrix((np.ones(len(idx)), (idx, idx)), shape=(n, n))
            rhs[Dm] = 0
            self.sol = spla.splu(A.tocsc()).solve(rhs)
            self.pcg_iters.append(0)
        else:
            fixed = np.ascontiguousarray(mask.astype(np.uint8))
            indptr = np.ascontiguousarray(self.A.indptr.astype(np.int64))
            indices = _i32(self.A.indices)
            sol = np.zeros(n)
            it = lib().oracle_pcg(n, _p(indptr, np.int64), _p(indices, np.int32), _p(_f64(self.A.data)), _p(_f64(rhs)),
                                  _p(fixed, np.uint8), D(self.pcg_rtol), self.pcg_maxit, _p(sol))
            self.pcg_iters.append(it)
            self.sol = sol
        self._toc('Solve System')
        return self.sol

    # NEWTON_IPC.py:456-468
    def compute_intersection_free_step_size(self, p=None):
        p = _f64((self.sol if p is None else p).reshape(-1, 3))
        return lib().oracle_ccd_step(len(self.x), _p(self.x), _p(p), len(self.bp), _p(self.bp, np.int32), len(self.be),
                                     _p(self.be, np.int32), len(self.bt), _p(self.bt, np.int32), len(self.tets),
                                     _p(self.tets, np.int32), D(self.dhat2), D(self.inv_dx), D(0.2), 1)

    # NEWTON_IPC.py:881-886
    def check_collision(self):
        return bool(lib().oracle_check_collision(_p(self.x), len(self.be), _p(self.be, np.int32), len(self.bt),
                                                 _p(self.bt, np.int32), D(self.dhat2), D(self.inv_dx)))

    def apply_sol(self, alpha):
        self.x = _f64(self.xPrev + self.sol.reshape(-1, 3) * alpha)

    # NEWTON_IPC.py:955-999, one time step; returns the Newton iteration count
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
                record.append({'rows': [r.copy() for r in self.rows], 'rhs': self.rhs.copy(), 'sol': self.sol.copy(),
                               'residual': res, 'x': self.x.copy()})
            if res < 1e-2 * self.dt or it >= max_newton:
                break
            self._tic('Line Search')
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
            self._toc('Line Search')
        self.v = (self.x - self.xn) / self.dt                             # compute_v
        self.newton_iters.append(it)
        return it
