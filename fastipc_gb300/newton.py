"""The IPC Newton driver on one GB300, with the call surface of projects/FastIPC/NEWTON_IPC.py.

``NewtonIPC`` holds the simulation state as CUDA FP64 tensors ([V,3], vertex-major) and keeps
the reference's function names and semantics: ``compute_xn_and_xTilde``, ``move_nodes``,
``find_constraints``, ``compute_hessian_and_gradient``, ``solve_system``, ``output_residual``,
``compute_energy``, ``save_xPrev``, ``compute_intersection_free_step_size``, ``apply_sol``,
``check_collision``, ``compute_v``; ``step`` is the time-step loop body of
NEWTON_IPC.py:955-999.  Every call goes to libfastipc.so; there is no other compute path.

Differences from the reference, by design:
  * the Newton direction comes from PCG (``pcg_rtol``) instead of CHOLMOD; ``solver='direct'``
    uses a sparse Cholesky factorisation as the reference does, and a PCG solve that reaches
    ``pcg_maxit`` falls back to it (``direct_fallback``);
  * the Newton and line-search loops are bounded (``max_newton``, ``max_halvings``) and raise
    ``FastIPCError`` instead of spinning forever (NEWTON_IPC.py:961, 983, 988, 993 are
    unbounded).
"""
import ctypes
import time

import numpy as np
import torch

from . import _native as N
from ._native import FastIPCError, check, dptr, hptr

TYPES = ['PP', 'PE', 'PT', 'EE', 'EEM', 'PPM', 'PEM']
TYPE_NV = [2, 3, 4, 4, 4, 4, 4]
D = ctypes.c_double
F64 = torch.float64


class Timer:
    """Named wall-clock sections with the reference's names (common/utils/timer.py)."""

    def __init__(self):
        self.total = {}

    def __call__(self, name):
        timer = self

        class _S:
            def __enter__(self_):
                self_.t = time.perf_counter()

            def __exit__(self_, *a):
                timer.total[name] = timer.total.get(name, 0.0) + time.perf_counter() - self_.t
        return _S()


class NewtonIPC:
    def __init__(self, scene, device='cuda:0', pcg_rtol=1e-10, pcg_maxit=200000, eta=0.2, inversion_filter=True,
                 max_newton=500, max_halvings=64, pcg_warm_start=False, coarse_agg=None, device_dirichlet=True,
                 solver='pcg', direct_fallback=True):
        self.scene = scene
        self.device = torch.device(device)
        torch.cuda.set_device(self.device)
        self.dt = float(scene.dt)
        self.gravity = float(scene.gravity)
        self.dhat2 = float(scene.dhat) ** 2
        self.eta = eta
        self.pcg_rtol, self.pcg_maxit = pcg_rtol, pcg_maxit
        # 'pcg' (default) or 'direct' (sparse Cholesky, the reference's exact solve); with
        # direct_fallback a PCG solve that reaches pcg_maxit is redone by the direct solver
        if solver not in ('pcg', 'direct'):
            raise FastIPCError(5, f'unknown solver {solver!r}')
        self.solver, self.direct_fallback = solver, direct_fallback
        self.direct_solves = 0
        self.inversion_filter = inversion_filter
        self.max_newton, self.max_halvings = max_newton, max_halvings
        self.timer = Timer()
        L = N.lib()
        rest = np.ascontiguousarray(scene.x, dtype=np.float64)
        tets = np.ascontiguousarray(scene.tets, dtype=np.int32)
        nT = len(tets)
        E, nu = scene.E, scene.nu
        lam = np.full(nT, E * nu / ((1 + nu) * (1 - 2 * nu)))
        mu = np.full(nT, E / (2 * (1 + nu)))
        bp = np.ascontiguousarray(scene.boundary_points, dtype=np.int32)
        be = np.ascontiguousarray(scene.boundary_edges, dtype=np.int32).reshape(-1)
        bt = np.ascontiguousarray(scene.boundary_triangles, dtype=np.int32).reshape(-1)
        ctx = ctypes.c_void_p()
        check(L.fipc_ctx_create(ctypes.byref(ctx), len(rest), nT, hptr(tets), hptr(rest), hptr(lam), hptr(mu),
                                D(scene.rho), len(bp), hptr(bp), len(be) // 2, hptr(be), len(bt) // 3, hptr(bt),
                                D(self.dhat2), D(self.dt)), 'fipc_ctx_create')
        self.ctx = ctx
        self.nV, self.nT = len(rest), nT
        kap, idx, nnzb = D(), D(), ctypes.c_int()
        check(L.fipc_ctx_params(ctx, ctypes.byref(kap), ctypes.byref(idx), ctypes.byref(nnzb)), 'fipc_ctx_params')
        self.kappa, self.inv_dx, self.nnzb = kap.value, idx.value, nnzb.value
        if coarse_agg is not None:
            self.set_preconditioner(coarse_agg)
        dev = self.device
        self.x = torch.tensor(scene.initial_positions(), dtype=F64, device=dev).contiguous()
        self.v = torch.tensor(scene.v, dtype=F64, device=dev).contiguous()
        self.xn = torch.zeros_like(self.x)
        self.xTilde = torch.zeros_like(self.x)
        self.xPrev = torch.zeros_like(self.x)
        self.data_sol = torch.zeros_like(self.x)
        self.counts = [0] * 7
        self._dir_key = None
        self.fixed = torch.zeros(self.nV, dtype=torch.uint8, device=dev)
        self.target = torch.zeros_like(self.x)
        # the Dirichlet schedule on the device (fipc_dirichlet_script) when the scene gives it as
        # rigid motions of vertex groups; otherwise scene.dirichlet(t) runs on the host
        self._script = None
        if device_dirichlet and getattr(scene, 'dirichlet_motion', None) is not None:
            self._script = (torch.tensor(rest, dtype=F64, device=dev).contiguous(),
                            torch.tensor(np.asarray(scene.dirichlet_groups, dtype=np.int32), device=dev).contiguous(),
                            torch.tensor(np.asarray(scene.dirichlet_motion, dtype=np.float64), device=dev).reshape(-1, 10).contiguous())
        self.newton_iters = []
        self.pcg_iters = []
        self.alphas = []
        # optional PCG initial guess: the direction of the same Newton iteration of the
        # previous time step (the solution is unchanged up to the PCG tolerance)
        self.pcg_warm_start = pcg_warm_start
        self._dir_hist = {}
        self._newton_k = 0
        # optional Newton initial guess hook, called as initial_guess(sim, f) after move_nodes
        # (the reference starts every step from x^n; see fastipc_gb300.learned)
        self.initial_guess = None
        # displacement of the step before the last one (v * dt holds the last one)
        self.dx_prev = torch.zeros_like(self.x)

    def close(self):
        if getattr(self, 'ctx', None):
            torch.cuda.synchronize(self.device)
            N.lib().fipc_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ state helpers
    def _s(self):
        return N.stream()

    def set_kappa(self, kappa=None, inv_dx=None):
        """Override the adaptive kappa / hash cell (the reference's module globals)."""
        self.kappa = self.kappa if kappa is None else float(kappa)
        self.inv_dx = self.inv_dx if inv_dx is None else float(inv_dx)
        check(N.lib().fipc_ctx_set_params(self.ctx, D(self.kappa), D(self.inv_dx)), 'fipc_ctx_set_params')

    def set_preconditioner(self, agg_rows):
        """0: block-Jacobi PCG; a multiple of 128: add the rigid-body coarse space of every run of
        agg_rows consecutive vertices.  Either switches the multigrid preconditioner off."""
        check(N.lib().fipc_ctx_set_preconditioner(self.ctx, int(agg_rows)), 'fipc_ctx_set_preconditioner')

    def set_multigrid(self, on=True, h=0.0):
        """The multigrid preconditioner (the default for scenes of at least 1000 vertices): on or
        off; h is the first aggregation box's cell (0: the spatial hash's)."""
        check(N.lib().fipc_ctx_set_multigrid(self.ctx, int(bool(on)), D(h)), 'fipc_ctx_set_multigrid')

    def set_multigrid_fp32(self, on=True):
        """FP32 level-0 smoothing products in the multigrid V-cycle (on, the default) or FP64 (off)."""
        check(N.lib().fipc_ctx_set_multigrid_fp32(self.ctx, int(bool(on))), 'fipc_ctx_set_multigrid_fp32')

    def multigrid(self):
        """Levels of the multigrid hierarchy in use (0: off) and nodes per level."""
        lv, nodes = ctypes.c_int(), (ctypes.c_int * 8)()
        check(N.lib().fipc_ctx_multigrid(self.ctx, ctypes.byref(lv), nodes), 'fipc_ctx_multigrid')
        return {'levels': lv.value, 'nodes': [nodes[k] for k in range(lv.value)]}

    def preconditioner(self):
        a, n = ctypes.c_int(), ctypes.c_int()
        check(N.lib().fipc_ctx_preconditioner(self.ctx, ctypes.byref(a), ctypes.byref(n)), 'fipc_ctx_preconditioner')
        return {'agg_rows': a.value, 'coarse_dofs': n.value}

    def mass(self):
        m = np.zeros(self.nV)
        check(N.lib().fipc_ctx_mass(self.ctx, hptr(m)), 'fipc_ctx_mass')
        return m

    def _dirichlet(self, t):
        # settings['dirichlet'](t) is a function of t only: evaluate once per distinct t
        if self._dir_key == t:
            return
        if self._script is not None:
            xr, grp, mot = self._script
            check(N.lib().fipc_dirichlet_script(self.nV, dptr(xr, F64), dptr(grp, torch.int32), len(mot), dptr(mot, F64), D(t),
                                                dptr(self.fixed, torch.uint8), dptr(self.target, F64), self._s()),
                  'dirichlet_script')
            self._dir_key = t
            return
        mask, val = self.scene.dirichlet(t)
        self.fixed.copy_(torch.from_numpy(np.ascontiguousarray(mask.astype(np.uint8))))
        self.target.copy_(torch.from_numpy(np.ascontiguousarray(val, dtype=np.float64)))
        self._dir_key = t

    # ------------------------------------------------------------------ NEWTON_IPC.py surface
    def compute_xn_and_xTilde(self):
        check(N.lib().fipc_compute_xn_and_xtilde(self.nV, dptr(self.x, F64), dptr(self.v, F64), D(self.dt), D(self.gravity),
                                                 dptr(self.xn, F64), dptr(self.xTilde, F64), self._s()),
              'compute_xn_and_xTilde')

    def move_nodes(self, t):
        self._dirichlet(t)
        check(N.lib().fipc_move_nodes(self.nV, dptr(self.fixed, torch.uint8), dptr(self.target, F64), dptr(self.x, F64),
                                      dptr(self.xTilde, F64), self._s()), 'move_nodes')

    def find_constraints(self):
        with self.timer('Find constraints'):
            c = (ctypes.c_int * 7)()
            check(N.lib().fipc_find_constraints(self.ctx, dptr(self.x, F64), c, self._s()), 'find_constraints')
            self.counts = list(c)
        return self.counts

    def constraints(self):
        """The seven lists (canonical order) as numpy arrays of width 2/3/4."""
        out = []
        for t in range(7):
            n = self.counts[t]
            r = torch.zeros((max(n, 1), 4), dtype=torch.int32, device=self.device)
            check(N.lib().fipc_get_constraints(self.ctx, t, dptr(r, torch.int32), self._s()), 'get_constraints')
            out.append(r[:n, :TYPE_NV[t]].cpu().numpy())
        return out

    def compute_hessian_and_gradient(self):
        with self.timer('Build System'):
            check(N.lib().fipc_compute_hessian_and_gradient(self.ctx, dptr(self.x, F64), dptr(self.xTilde, F64), self._s()),
                  'compute_hessian_and_gradient')

    def export_system(self):
        """(elastic BSR, contact BSR, rhs) as host scipy matrices + vector (tests)."""
        import scipy.sparse as sp
        L = N.lib()
        ne, nc = ctypes.c_int(), ctypes.c_int()
        check(L.fipc_system_sizes(self.ctx, ctypes.byref(ne), ctypes.byref(nc)), 'system_sizes')
        dev = self.device
        rp = torch.zeros(self.nV + 1, dtype=torch.int32, device=dev)
        ci = torch.zeros(max(ne.value, 1), dtype=torch.int32, device=dev)
        va = torch.zeros((max(ne.value, 1), 9), dtype=F64, device=dev)
        crp = torch.zeros(self.nV + 1, dtype=torch.int32, device=dev)
        cci = torch.zeros(max(nc.value, 1), dtype=torch.int32, device=dev)
        cva = torch.zeros((max(nc.value, 1), 9), dtype=F64, device=dev)
        rhs = torch.zeros(3 * self.nV, dtype=F64, device=dev)
        check(L.fipc_export_system(self.ctx, dptr(rp), dptr(ci), dptr(va), dptr(crp), dptr(cci), dptr(cva), dptr(rhs),
                                   self._s()), 'export_system')
        n = self.nV

        def bsr(rp, ci, va, nnz):
            return sp.bsr_matrix((va[:nnz].cpu().numpy().reshape(-1, 3, 3), ci[:nnz].cpu().numpy(), rp.cpu().numpy()),
                                 shape=(3 * n, 3 * n))
        return bsr(rp, ci, va, ne.value), bsr(crp, cci, cva, nc.value), rhs.cpu().numpy()

    def solve_system(self, t):
        with self.timer('Solve System'):
            self._dirichlet(t)
            it = ctypes.c_int()
            guess = self.pcg_warm_start and self._newton_k in self._dir_hist
            if guess:
                self.data_sol.copy_(self._dir_hist[self._newton_k])
                self.data_sol[self.fixed.bool()] = 0.0
            if self.solver == 'direct':
                self._solve_direct()
                self.pcg_iters.append(0)
            else:
                st = N.lib().fipc_solve_system(self.ctx, dptr(self.fixed, torch.uint8), D(self.pcg_rtol), self.pcg_maxit,
                                               int(guess), dptr(self.data_sol, F64), ctypes.byref(it), self._s())
                if st == 2 and self.direct_fallback:      # PCG stopped at pcg_maxit
                    self._solve_direct()
                else:
                    check(st, 'solve_system')
                self.pcg_iters.append(it.value)
            if self.pcg_warm_start:
                self._dir_hist[self._newton_k] = self.data_sol.clone()
            self._newton_k += 1

    def _solve_direct(self):
        check(N.lib().fipc_solve_system_direct(self.ctx, dptr(self.fixed, torch.uint8), dptr(self.data_sol, F64), None, self._s()),
              'solve_system_direct')
        self.direct_solves += 1

    def direct_stats(self):
        """The last direct solve: fronts, front storage (doubles), factorisation flops and the host
        analysis time (ms)."""
        nf, nd, fl, ms = ctypes.c_int(), ctypes.c_longlong(), D(), D()
        check(N.lib().fipc_direct_stats(self.ctx, ctypes.byref(nf), ctypes.byref(nd), ctypes.byref(fl), ctypes.byref(ms)),
              'fipc_direct_stats')
        return {'fronts': nf.value, 'front_doubles': nd.value, 'flops': fl.value, 'analyse_ms': ms.value}

    def output_residual(self):
        r = D()
        check(N.lib().fipc_output_residual(self.ctx, dptr(self.data_sol, F64), ctypes.byref(r), self._s()), 'output_residual')
        return r.value

    def compute_energy(self):
        e = D()
        check(N.lib().fipc_compute_energy(self.ctx, dptr(self.x, F64), dptr(self.xTilde, F64), ctypes.byref(e), self._s()),
              'compute_energy')
        return e.value

    def save_xPrev(self):
        self.xPrev.copy_(self.x)

    def compute_intersection_free_step_size(self):
        a = D()
        check(N.lib().fipc_compute_intersection_free_step_size(self.ctx, dptr(self.x, F64), dptr(self.data_sol, F64), D(self.eta),
                                                               int(self.inversion_filter), ctypes.byref(a), self._s()),
              'compute_intersection_free_step_size')
        return a.value

    def apply_sol(self, alpha):
        check(N.lib().fipc_apply_sol(self.nV, dptr(self.xPrev, F64), dptr(self.data_sol, F64), D(alpha), dptr(self.x, F64),
                                     self._s()), 'apply_sol')

    def check_collision(self):
        h = ctypes.c_int()
        check(N.lib().fipc_check_collision(self.ctx, dptr(self.x, F64), ctypes.byref(h), self._s()), 'check_collision')
        return bool(h.value)

    def compute_v(self):
        check(N.lib().fipc_compute_v(self.nV, dptr(self.x, F64), dptr(self.xn, F64), D(self.dt), dptr(self.v, F64), self._s()),
              'compute_v')

    def set_state(self, x, v):
        """Positions and velocities [V,3] (host or device), as the restart of NEWTON_IPC.py:949-953
        loads them."""
        self.x.copy_(torch.as_tensor(np.asarray(x, dtype=np.float64) if not isinstance(x, torch.Tensor) else x).reshape(-1, 3))
        self.v.copy_(torch.as_tensor(np.asarray(v, dtype=np.float64) if not isinstance(v, torch.Tensor) else v).reshape(-1, 3))

    # ------------------------------------------------------------------ the main loop
    def run(self, n_frames, directory=None, start_frame=0, obj=True, cache=True):
        """The reference's main loop (NEWTON_IPC.py:947-1003) for n_frames time steps.  With a
        directory, frame 0 and every frame after a step go to objs/%06d.obj and
        caches/%06d.p as the reference writes them (through ``frames.FrameWriter``, off the
        simulation stream); start_frame > 0 restarts from caches/{start_frame:06d}.p.  Returns
        the Newton iteration count of every step."""
        from . import frames
        if start_frame > 0 and directory is None:
            raise FastIPCError(5, 'a restart (start_frame > 0) reads caches/%06d.p from a directory')
        writer = None
        if directory is not None and (obj or cache):
            writer = frames.FrameWriter(directory, self.scene.boundary_triangles, self.nV, obj=obj, cache=cache)
        try:
            if writer is not None:
                writer.submit(0, self.x, self.v, cache=False)   # write_image(0) (NEWTON_IPC.py:947)
            if start_frame > 0:
                if writer is not None:
                    writer.flush()
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
            self._newton_k = 0
            if self.initial_guess is not None:
                self.initial_guess(self, f)
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
            torch.mul(self.v, self.dt, out=self.dx_prev)
            self.compute_v()
        self.newton_iters.append(it)
        return it
