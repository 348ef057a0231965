"""The 2D IPC Newton driver on one GB300: projects/FastIPC/NEWTON_IPC.py with dim == 2.

``NewtonIPC2D`` holds positions and velocities as CUDA FP64 tensors [V,2] and keeps the
reference's function names: ``compute_xn_and_xTilde``, ``move_nodes``, ``find_constraints``
(find_constraints_2D_PE), ``compute_hessian_and_gradient``, ``solve_system``,
``output_residual``, ``compute_energy``, ``save_xPrev``, ``compute_intersection_free_step_size``
(compute_filter_2D_PE), ``apply_sol``, ``check_collision`` (check_collision_2D), ``compute_v``;
``step`` is NEWTON_IPC.py:955-999.  The material is the reference's default fixed-corotated
model.  Every call goes to the fipc2d_* entry points of libfastipc.so; there is no other
compute path.  As in the 3D driver, the direction comes from PCG (``pcg_rtol``) instead of
CHOLMOD, and the Newton and line-search loops are bounded.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from ._native import FastIPCError, check, dptr, hptr
from .newton import Timer

D = ctypes.c_double
F64 = torch.float64


class NewtonIPC2D:
    def __init__(self, scene, device='cuda:0', pcg_rtol=1e-10, pcg_maxit=100000, eta=0.2, max_newton=500, max_halvings=64):
        self.scene = scene
        self.device = torch.device(device)
        torch.cuda.set_device(self.device)
        self.dt, self.gravity = float(scene.dt), float(scene.gravity)
        self.dhat2 = float(scene.dhat) ** 2
        self.eta = eta
        self.pcg_rtol, self.pcg_maxit = pcg_rtol, pcg_maxit
        self.max_newton, self.max_halvings = max_newton, max_halvings
        self.timer = Timer()
        rest = np.ascontiguousarray(scene.x, dtype=np.float64)
        tris = np.ascontiguousarray(scene.tris, dtype=np.int32)
        nT = len(tris)
        E, nu = scene.E, scene.nu
        lam = np.full(nT, E * nu / ((1 + nu) * (1 - 2 * nu)))
        mu = np.full(nT, E / (2 * (1 + nu)))
        bp = np.ascontiguousarray(scene.boundary_points, dtype=np.int32)
        be = np.ascontiguousarray(scene.boundary_edges, dtype=np.int32).reshape(-1)
        ctx = ctypes.c_void_p()
        check(N.lib().fipc2d_ctx_create(ctypes.byref(ctx), len(rest), nT, hptr(tris), hptr(rest), hptr(lam), hptr(mu),
                                        D(scene.rho), len(bp), hptr(bp), len(be) // 2, hptr(be), D(self.dhat2), D(self.dt)),
              'fipc2d_ctx_create')
        self.ctx = ctx
        self.nV, self.nT = len(rest), nT
        kap, me = D(), D()
        check(N.lib().fipc2d_ctx_params(ctx, ctypes.byref(kap), ctypes.byref(me)), 'fipc2d_ctx_params')
        self.kappa, self.mean_edge = kap.value, me.value
        dev = self.device
        self.x = torch.tensor(scene.initial_positions(), dtype=F64, device=dev).contiguous()
        self.v = torch.tensor(scene.v, dtype=F64, device=dev).contiguous()
        self.xn = torch.zeros_like(self.x)
        self.xTilde = torch.zeros_like(self.x)
        self.xPrev = torch.zeros_like(self.x)
        self.data_sol = torch.zeros_like(self.x)
        self.fixed = torch.zeros(self.nV, dtype=torch.uint8, device=dev)
        self.target = torch.zeros_like(self.x)
        self._dir_key = None
        self.counts = [0, 0]
        self.newton_iters, self.pcg_iters, self.alphas = [], [], []

    def close(self):
        if getattr(self, 'ctx', None):
            torch.cuda.synchronize(self.device)
            N.lib().fipc2d_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _s(self):
        return N.stream()

    def set_kappa(self, kappa):
        self.kappa = float(kappa)
        check(N.lib().fipc2d_ctx_set_kappa(self.ctx, D(self.kappa)), 'fipc2d_ctx_set_kappa')

    def mass(self):
        m = np.zeros(self.nV)
        check(N.lib().fipc2d_ctx_mass(self.ctx, hptr(m)), 'fipc2d_ctx_mass')
        return m

    def _dirichlet(self, t):
        if self._dir_key == t:
            return
        mask, val = self.scene.dirichlet(t)
        self.fixed.copy_(torch.from_numpy(np.ascontiguousarray(mask.astype(np.uint8))))
        self.target.copy_(torch.from_numpy(np.ascontiguousarray(val, dtype=np.float64)))
        self._dir_key = t

    # ------------------------------------------------------------------ NEWTON_IPC.py surface
    def compute_xn_and_xTilde(self):
        check(N.lib().fipc2d_compute_xn_and_xtilde(self.nV, dptr(self.x, F64), dptr(self.v, F64), D(self.dt), D(self.gravity),
                                                   dptr(self.xn, F64), dptr(self.xTilde, F64), self._s()), 'compute_xn_and_xTilde')

    def move_nodes(self, t):
        self._dirichlet(t)
        check(N.lib().fipc2d_move_nodes(self.nV, dptr(self.fixed, torch.uint8), dptr(self.target, F64), dptr(self.x, F64),
                                        dptr(self.xTilde, F64), self._s()), 'move_nodes')

    def find_constraints(self):
        with self.timer('Find constraints'):
            c = (ctypes.c_int * 2)()
            check(N.lib().fipc2d_find_constraints(self.ctx, dptr(self.x, F64), c, self._s()), 'find_constraints')
            self.counts = list(c)
        return self.counts

    def constraints(self):
        """(PP [n,2], PE [n,3]) as numpy arrays, lexicographically sorted."""
        out = []
        for t, w in ((0, 2), (1, 3)):
            n = self.counts[t]
            r = torch.zeros((max(n, 1), 4), dtype=torch.int32, device=self.device)
            check(N.lib().fipc2d_get_constraints(self.ctx, t, dptr(r, torch.int32), self._s()), 'get_constraints')
            out.append(r[:n, :w].cpu().numpy())
        return tuple(out)

    def compute_hessian_and_gradient(self):
        with self.timer('Build System'):
            check(N.lib().fipc2d_compute_hessian_and_gradient(self.ctx, dptr(self.x, F64), dptr(self.xTilde, F64), self._s()),
                  'compute_hessian_and_gradient')

    def export_system(self):
        """(A before the Dirichlet edit as scipy BSR with 2x2 blocks, rhs) on the host (tests)."""
        import scipy.sparse as sp
        nnz = ctypes.c_int()
        check(N.lib().fipc2d_system_nnzb(self.ctx, ctypes.byref(nnz)), 'system_nnzb')
        dev = self.device
        rp = torch.zeros(self.nV + 1, dtype=torch.int32, device=dev)
        ci = torch.zeros(max(nnz.value, 1), dtype=torch.int32, device=dev)
        va = torch.zeros((max(nnz.value, 1), 4), dtype=F64, device=dev)
        rhs = torch.zeros(2 * self.nV, dtype=F64, device=dev)
        check(N.lib().fipc2d_export_system(self.ctx, dptr(rp), dptr(ci), dptr(va), dptr(rhs), self._s()), 'export_system')
        n = nnz.value
        A = sp.bsr_matrix((va[:n].cpu().numpy().reshape(-1, 2, 2), ci[:n].cpu().numpy(), rp.cpu().numpy()),
                          shape=(2 * self.nV, 2 * self.nV))
        return A, rhs.cpu().numpy()

    def solve_system(self, t):
        with self.timer('Solve System'):
            self._dirichlet(t)
            it = ctypes.c_int()
            check(N.lib().fipc2d_solve_system(self.ctx, dptr(self.fixed, torch.uint8), D(self.pcg_rtol), self.pcg_maxit,
                                              dptr(self.data_sol, F64), ctypes.byref(it), self._s()), 'solve_system')
            self.pcg_iters.append(it.value)

    def output_residual(self):
        r = D()
        check(N.lib().fipc2d_output_residual(self.ctx, dptr(self.data_sol, F64), ctypes.byref(r), self._s()), 'output_residual')
        return r.value

    def compute_energy(self):
        e = D()
        check(N.lib().fipc2d_compute_energy(self.ctx, dptr(self.x, F64), dptr(self.xTilde, F64), ctypes.byref(e), self._s()),
              'compute_energy')
        return e.value

    def save_xPrev(self):
        self.xPrev.copy_(self.x)

    def compute_intersection_free_step_size(self):
        a = D()
        check(N.lib().fipc2d_compute_intersection_free_step_size(self.ctx, dptr(self.x, F64), dptr(self.data_sol, F64),
                                                                 D(self.eta), ctypes.byref(a), self._s()),
              'compute_intersection_free_step_size')
        return a.value

    def apply_sol(self, alpha):
        check(N.lib().fipc2d_apply_sol(self.nV, dptr(self.xPrev, F64), dptr(self.data_sol, F64), D(alpha), dptr(self.x, F64),
                                       self._s()), 'apply_sol')

    def check_collision(self):
        h = ctypes.c_int()
        check(N.lib().fipc2d_check_collision(self.ctx, dptr(self.x, F64), ctypes.byref(h), self._s()), 'check_collision')
        return bool(h.value)

    def compute_v(self):
        check(N.lib().fipc2d_compute_v(self.nV, dptr(self.x, F64), dptr(self.xn, F64), D(self.dt), dptr(self.v, F64), self._s()),
              'compute_v')

    def set_state(self, x, v):
        """Positions and velocities [V,2] (host or device), as the restart of NEWTON_IPC.py:949-953
        loads them."""
        self.x.copy_(torch.as_tensor(np.asarray(x, dtype=np.float64) if not isinstance(x, torch.Tensor) else x).reshape(-1, 2))
        self.v.copy_(torch.as_tensor(np.asarray(v, dtype=np.float64) if not isinstance(v, torch.Tensor) else v).reshape(-1, 2))

    def run(self, n_frames, directory=None, start_frame=0):
        """The reference's main loop for dim 2 (NEWTON_IPC.py:947-1003) for n_frames time steps.
        With a directory, the state after every step goes to caches/%06d.p as the reference
        writes it (pickled [x, v]); start_frame > 0 restarts from caches/{start_frame:06d}.p.
        The 2D write_image draws into a window and is not reproduced.  Returns the Newton
        iteration count of every step."""
        from . import frames
        if start_frame > 0 and directory is None:
            raise FastIPCError(5, 'a restart (start_frame > 0) reads caches/%06d.p from a directory')
        writer = frames.FrameWriter(directory, None, self.nV, obj=False, cache=True, dim=2) if directory is not None else None
        try:
            if start_frame > 0:
                x, v = frames.load_cache(frames.cache_path(directory, start_frame))
                self.set_state(x, v)
            its = []
            for f in range(start_frame, start_frame + n_frames):
                its.append(self.step(f))
                if writer is not None:
                    writer.submit(f + 1, self.x, self.v)
            if writer is not None:
                writer.flush()
        finally:
            if writer is not None:
                writer.close()
        return its

    # ------------------------------------------------------------------ the time step
    def step(self, f, record=None):
        """One time step (NEWTON_IPC.py:955-999); returns the Newton iteration count."""
        with self.timer('Time Step'):
            self.compute_xn_and_xTilde()
            self.move_nodes(f * self.dt)
            it = 0
            while True:
                it += 1
                self.find_constraints()
                self.compute_hessian_and_gradient()
                self.solve_system(f * self.dt)
                res = self.output_residual()
                if record is not None:
                    record.append({'counts': list(self.counts), 'residual': res})
                if res < 1e-2 * self.dt:
                    break
                if it >= self.max_newton:
                    raise FastIPCError(2, f'Newton did not converge in {self.max_newton} iterations')
                with self.timer('Line Search'):
                    E0 = self.compute_energy()
                    self.save_xPrev()
                    alpha = self.compute_intersection_free_step_size()
                    alpha_ccd = alpha
                    self.apply_sol(alpha)
                    k = 0
                    while self.check_collision():
                        alpha /= 2.0
                        self.apply_sol(alpha)
                        k += 1
                        if k > self.max_halvings:
                            raise FastIPCError(2, 'line search: collision halving limit')
                    self.find_constraints()
                    E = self.compute_energy()
                    while E > E0:
                        alpha *= 0.5
                        self.apply_sol(alpha)
                        self.find_constraints()
                        E = self.compute_energy()
                        k += 1
                        if k > self.max_halvings:
                            raise FastIPCError(2, 'line search: energy halving limit')
                    while self.check_collision():
                        alpha /= 2.0
                        self.apply_sol(alpha)
                        k += 1
                        if k > self.max_halvings:
                            raise FastIPCError(2, 'line search: collision halving limit')
                    self.alphas.append(alpha)
                    if record is not None:
                        record[-1].update({'E0': E0, 'alpha_ccd': alpha_ccd, 'alpha': alpha, 'E': E})
            self.compute_v()
        self.newton_iters.append(it)
        return it
