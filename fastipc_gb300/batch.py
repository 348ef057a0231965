"""Batched scenes: many independent IPC scenes stepped together on one GPU.

``BatchNewtonIPC`` runs the reference driver's Newton loop (``NEWTON_IPC.py:955-999``) for every
scene at once.  Each scene keeps its own convergence test, CCD step, collision halving and
energy backtracking; a scene that has converged takes no further updates while the others
iterate.  The union mesh lives in one batch context of libfastipc.so: per-element kernels run
over all scenes in one launch, and per-scene quantities (hash cell, kappa, energy, residual,
step size, PCG scalars) come back as device arrays with one entry per scene.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from ._native import FastIPCError, check, dptr, hptr
from .newton import Timer

F64 = torch.float64
D = ctypes.c_double


def concat_scenes(scenes):
    """Union arrays and per-scene offsets of a list of scenes (vertex ids made global)."""
    voff, toff, eoff = [0], [0], [0]
    xs, x0s, vs, tets, bps, bes, bts, lam, mu = [], [], [], [], [], [], [], [], []
    for sc in scenes:
        o = voff[-1]
        xs.append(np.asarray(sc.initial_positions(), np.float64))
        x0s.append(np.asarray(sc.x, np.float64))
        vs.append(np.asarray(sc.v, np.float64))
        tets.append(np.asarray(sc.tets, np.int64) + o)
        bps.append(np.asarray(sc.boundary_points, np.int64) + o)
        bes.append(np.asarray(sc.boundary_edges, np.int64).reshape(-1, 2) + o)
        bts.append(np.asarray(sc.boundary_triangles, np.int64).reshape(-1, 3) + o)
        nT = len(sc.tets)
        lam.append(np.full(nT, sc.E * sc.nu / ((1 + sc.nu) * (1 - 2 * sc.nu))))
        mu.append(np.full(nT, sc.E / (2 * (1 + sc.nu))))
        voff.append(o + len(sc.x))
        toff.append(toff[-1] + nT)
        eoff.append(eoff[-1] + len(bes[-1]))
    cat = lambda a, dt: np.ascontiguousarray(np.concatenate(a).astype(dt))
    return {'x': cat(xs, np.float64), 'x0': cat(x0s, np.float64), 'v': cat(vs, np.float64), 'tets': cat(tets, np.int32),
            'bp': cat(bps, np.int32), 'be': cat(bes, np.int32), 'bt': cat(bts, np.int32), 'lam': cat(lam, np.float64),
            'mu': cat(mu, np.float64), 'voff': np.array(voff, np.int32), 'toff': np.array(toff, np.int32),
            'eoff': np.array(eoff, np.int32)}


class BatchNewtonIPC:
    def __init__(self, scenes, device='cuda:0', pcg_rtol=1e-10, pcg_maxit=200000, eta=0.2, inversion_filter=True,
                 max_newton=500, max_halvings=64, device_dirichlet=True):
        if len(scenes) < 2:
            raise FastIPCError(5, 'a batch needs at least two scenes (use NewtonIPC for one)')
        first = scenes[0]
        for sc in scenes:
            if (sc.dt, sc.dhat, sc.rho, sc.gravity) != (first.dt, first.dhat, first.rho, first.gravity):
                raise FastIPCError(5, 'scenes of a batch share dt, d-hat, density and gravity')
        self.scenes = scenes
        self.S = len(scenes)
        self.device = torch.device(device)
        torch.cuda.set_device(self.device)
        self.dt, self.gravity = float(first.dt), float(first.gravity)
        self.dhat2 = float(first.dhat) ** 2
        self.eta, self.inversion_filter = eta, inversion_filter
        self.pcg_rtol, self.pcg_maxit = pcg_rtol, pcg_maxit
        self.max_newton, self.max_halvings = max_newton, max_halvings
        self.timer = Timer()
        u = concat_scenes(scenes)
        self.voff = u['voff']
        self.nV, self.nT = len(u['x']), len(u['tets'])
        ctx = ctypes.c_void_p()
        check(N.lib().fipc_batch_create(ctypes.byref(ctx), self.S, hptr(u['voff']), hptr(u['toff']), hptr(u['eoff']), self.nV,
                                        self.nT, hptr(u['tets']), hptr(u['x0']), hptr(u['lam']), hptr(u['mu']), D(first.rho),
                                        len(u['bp']), hptr(u['bp']), len(u['be']), hptr(u['be']), len(u['bt']), hptr(u['bt']),
                                        D(self.dhat2), D(self.dt)), 'fipc_batch_create')
        self.ctx = ctx
        self.kappa, self.inv_dx = np.zeros(self.S), np.zeros(self.S)
        check(N.lib().fipc_batch_params(ctx, None, hptr(self.kappa), hptr(self.inv_dx)), 'fipc_batch_params')
        dev = self.device
        self.x = torch.tensor(u['x'], dtype=F64, device=dev)
        self.v = torch.tensor(u['v'], dtype=F64, device=dev)
        self.xn, self.xTilde, self.xPrev = (torch.zeros_like(self.x) for _ in range(3))
        self.data_sol = torch.zeros_like(self.x)
        self.fixed = torch.zeros(self.nV, dtype=torch.uint8, device=dev)
        self.target = torch.zeros_like(self.x)
        self._dir_key = None
        # the scenes' Dirichlet schedules on the device when every scene gives one as rigid
        # motions of vertex groups (group ids offset per scene)
        self._script = None
        if device_dirichlet and all(getattr(sc, 'dirichlet_motion', None) is not None for sc in scenes):
            grp, mot, g0 = [], [], 0
            for sc in scenes:
                gs = np.asarray(sc.dirichlet_groups, dtype=np.int32)
                grp.append(np.where(gs >= 0, gs + g0, -1).astype(np.int32))
                m = np.asarray(sc.dirichlet_motion, dtype=np.float64).reshape(-1, 10)
                mot.append(m)
                g0 += len(m)
            self._script = (torch.tensor(u['x0'], dtype=F64, device=dev).contiguous(),
                            torch.tensor(np.concatenate(grp), device=dev).contiguous(),
                            torch.tensor(np.concatenate(mot), dtype=F64, device=dev).contiguous())
        S = self.S
        self.E0 = torch.zeros(S, dtype=F64, device=dev)
        self.E = torch.zeros(S, dtype=F64, device=dev)
        self.alpha = torch.zeros(S, dtype=F64, device=dev)
        self.res = torch.zeros(S, dtype=F64, device=dev)
        self.hit = torch.zeros(S, dtype=torch.int32, device=dev)
        self.iters = torch.zeros(S, dtype=torch.int32, device=dev)
        self.active_d = torch.ones(S, dtype=torch.uint8, device=dev)
        self.counts = [0] * 7
        # scene of every vertex (device), for per-scene selections on the host side
        self.v_scene = torch.repeat_interleave(torch.arange(S, device=dev), torch.from_numpy(np.diff(self.voff).astype(np.int64)).to(dev))
        # optional Newton initial guess hook, called as initial_guess(sim, f) after move_nodes;
        # dx_prev: the displacement of the step before the last one (for such hooks)
        self.initial_guess = None
        self.dx_prev = torch.zeros_like(self.x)
        self.newton_iters = []     # per step: numpy [S]
        self.pcg_iters = []        # per solve: numpy [S]

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

    def _s(self):
        return N.stream()

    def scene_slice(self, s):
        return slice(int(self.voff[s]), int(self.voff[s + 1]))

    def _dirichlet(self, t):
        if self._dir_key == t:
            return
        if self._script is not None:
            xr, grp, mot = self._script
            check(N.lib().fipc_dirichlet_script(self.nV, dptr(xr, F64), dptr(grp, torch.int32), len(mot), dptr(mot, F64), D(t),
                                                dptr(self.fixed, torch.uint8), dptr(self.target, F64), self._s()),
                  'dirichlet_script')
            self._dir_key = t
            return
        masks, vals = zip(*(sc.dirichlet(t) for sc in self.scenes))
        self.fixed.copy_(torch.from_numpy(np.concatenate(masks).astype(np.uint8)))
        self.target.copy_(torch.from_numpy(np.ascontiguousarray(np.concatenate(vals), dtype=np.float64)))
        self._dir_key = t

    # ------------------------------------------------------------------ per-call surface
    def compute_xn_and_xTilde(self):
        check(N.lib().fipc_compute_xn_and_xtilde(self.nV, dptr(self.x, F64), dptr(self.v, F64), D(self.dt), D(self.gravity),
                                                 dptr(self.xn, F64), dptr(self.xTilde, F64), self._s()), 'compute_xn_and_xTilde')

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
        from .newton import TYPE_NV
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

    def solve_system(self, t, active=None):
        """Directions of the scenes with active[s] (numpy bool [S], default all); 0 elsewhere."""
        with self.timer('Solve System'):
            self._dirichlet(t)
            if active is None:
                self.active_d.fill_(1)
            else:
                self.active_d.copy_(torch.from_numpy(np.asarray(active, np.uint8)))
            nf = ctypes.c_int()
            st = N.lib().fipc_batch_solve_system(self.ctx, dptr(self.fixed, torch.uint8), dptr(self.active_d, torch.uint8),
                                                 D(self.pcg_rtol), self.pcg_maxit, 0, dptr(self.data_sol, F64),
                                                 dptr(self.iters, torch.int32), ctypes.byref(nf), self._s())
            check(st, 'batch_solve_system')
            self.pcg_iters.append(self.iters.cpu().numpy())

    def output_residual(self):
        check(N.lib().fipc_batch_output_residual(self.ctx, dptr(self.data_sol, F64), dptr(self.res, F64), self._s()),
              'batch_output_residual')
        return self.res.cpu().numpy()

    def compute_energy(self, out=None):
        out = self.E if out is None else out
        check(N.lib().fipc_batch_compute_energy(self.ctx, dptr(self.x, F64), dptr(self.xTilde, F64), dptr(out, F64), self._s()),
              'batch_compute_energy')
        return out

    def save_xPrev(self):
        self.xPrev.copy_(self.x)

    def compute_intersection_free_step_size(self):
        check(N.lib().fipc_batch_step_size(self.ctx, dptr(self.x, F64), dptr(self.data_sol, F64), D(self.eta),
                                           int(self.inversion_filter), dptr(self.alpha, F64), self._s()), 'batch_step_size')
        return self.alpha

    def apply_sol(self):
        check(N.lib().fipc_batch_apply_sol(self.ctx, dptr(self.xPrev, F64), dptr(self.data_sol, F64), dptr(self.alpha, F64),
                                           dptr(self.x, F64), self._s()), 'batch_apply_sol')

    def check_collision(self):
        check(N.lib().fipc_batch_check_collision(self.ctx, dptr(self.x, F64), dptr(self.hit, torch.int32), self._s()),
              'batch_check_collision')
        return self.hit.cpu().numpy() != 0

    def compute_v(self):
        check(N.lib().fipc_compute_v(self.nV, dptr(self.x, F64), dptr(self.xn, F64), D(self.dt), dptr(self.v, F64), self._s()),
              'compute_v')

    def pcg_shape(self):
        tr, grid, nt, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        check(N.lib().fipc_batch_pcg_shape(self.ctx, ctypes.byref(tr), ctypes.byref(grid), ctypes.byref(nt), ctypes.byref(ms)),
              'batch_pcg_shape')
        return {'tile_rows': tr.value, 'grid': grid.value, 'tiles': nt.value, 'spmv_ms': ms.value}

    # ------------------------------------------------------------------ the time step
    def _halve(self, mask):
        """alpha[s] /= 2 for the scenes in mask (numpy bool), then x = xPrev + alpha p."""
        m = torch.from_numpy(mask).to(self.device)
        self.alpha.copy_(torch.where(m, self.alpha * 0.5, self.alpha))
        self.apply_sol()

    def step(self, f):
        """One time step of every scene; returns the Newton iteration counts [S]."""
        S = self.S
        with self.timer('Time Step'):
            self.compute_xn_and_xTilde()
            self.move_nodes(f * self.dt)
            if self.initial_guess is not None:
                self.initial_guess(self, f)
            active = np.ones(S, bool)
            its = np.zeros(S, np.int64)
            while True:
                its[active] += 1
                self.find_constraints()
                self.compute_hessian_and_gradient()
                self.solve_system(f * self.dt, active)
                res = self.output_residual()
                active &= ~(res < 1e-2 * self.dt)
                if not active.any():
                    break
                if its.max() >= self.max_newton:
                    raise FastIPCError(2, f'Newton did not converge in {self.max_newton} iterations')
                with self.timer('Line Search'):
                    self.compute_energy(self.E0)
                    self.save_xPrev()
                    self.compute_intersection_free_step_size()
                    act = torch.from_numpy(active).to(self.device)
                    self.alpha.copy_(torch.where(act, self.alpha, torch.zeros_like(self.alpha)))
                    self.apply_sol()
                    k = 0
                    while True:
                        bad = self.check_collision() & active
                        if not bad.any():
                            break
                        self._halve(bad)
                        k += 1
                        if k > self.max_halvings:
                            raise FastIPCError(2, 'line search: collision halving limit')
                    self.find_constraints()
                    self.compute_energy()
                    while True:
                        bad = (self.E > self.E0).cpu().numpy() & active
                        if not bad.any():
                            break
                        self._halve(bad)
                        self.find_constraints()
                        self.compute_energy()
                        k += 1
                        if k > self.max_halvings:
                            raise FastIPCError(2, 'line search: energy halving limit')
                    while True:
                        bad = self.check_collision() & active
                        if not bad.any():
                            break
                        self._halve(bad)
                        k += 1
                        if k > self.max_halvings:
                            raise FastIPCError(2, 'line search: collision halving limit')
            torch.mul(self.v, self.dt, out=self.dx_prev)
            self.compute_v()
        self.newton_iters.append(its)
        return its
