"""ADMM-IPC on the GPU: the alternating-direction variant of the IPC time step
(projects/FastIPC/ADMM_IPC.py), driven from Python over libfastipc.so.

`AdmmIPC.step(f)` follows the script's main loop (ADMM_IPC.py:1471-1526): initial_guess, then
a fixed number of ADMM iterations (20 in the script), each of them
  1. the CCD step toward xTilde (first iteration only; it seeds the new rows' y),
  2. backup of the rows and their variables, find_constraints, reuse_admm_variables,
  3. the global step (one SPD solve for x, Dirichlet vertices at their targets),
  4. the global filter: the CCD step from the previous x to the solution, then halving toward
     the previous x while any edge crosses a triangle,
  5. the local steps (per tet, per row) and the dual step;
and compute_v.  Every kernel runs on the GPU (fipc_admm_* and the Newton path's constraint
finding, CCD and intersection check on the same context); the loop control is here.

The script uses kappa from the adaptive rule without the Newton script's factor 10
(ADMM_IPC.py:1459 against NEWTON_IPC.py:943) and fixed-corotated elasticity; both are set
here.  Its local loops are unbounded; here they stop after 256 Newton iterations or 64 halvings
(a constraint row whose unprojected Hessian is indefinite can take regularised steps that never
fall below the tolerance), and `local_detail` records which bounds the last local step reached
(bits 1 / 2: a tet's Newton / halving bound, 4 / 8: a row's).
"""
import ctypes

import torch

from . import _native as N
from ._native import FastIPCError, check, dptr
from .newton import NewtonIPC

F64 = torch.float64
D = ctypes.c_double
TYPE_NV = (2, 3, 4, 4, 4, 4, 4)


class AdmmIPC(NewtonIPC):
    def __init__(self, scene, device='cuda:0', admm_iters=20, pcg_rtol=1e-10, pcg_maxit=200000, eta=0.2):
        super().__init__(scene, device=device, pcg_rtol=pcg_rtol, pcg_maxit=pcg_maxit, eta=eta, inversion_filter=False,
                         direct_fallback=False)
        # compute_adaptive_kappa without the factor 10 of the Newton script
        self.set_kappa(self.kappa / 10.0)
        self.admm_iters = admm_iters
        dev = self.device
        self.W = torch.zeros(self.nT, dtype=F64, device=dev)
        self.z = torch.zeros((self.nT, 9), dtype=F64, device=dev)
        self.u = torch.zeros((self.nT, 9), dtype=F64, device=dev)
        self._empty_rows()
        self.global_iters = []
        self.filter_alphas = []

    def _empty_rows(self):
        dev = self.device
        self.rows_all = torch.zeros((0, 4), dtype=torch.int32, device=dev)
        self.row_counts = [0] * 7
        self.y = torch.zeros((0, 9), dtype=F64, device=dev)
        self.r = torch.zeros((0, 9), dtype=F64, device=dev)
        self.Q = torch.zeros(0, dtype=F64, device=dev)

    @staticmethod
    def _p(t):
        return dptr(t) if t.numel() > 0 else None

    # ------------------------------------------------------------------ the script's kernels
    def admm_initial_guess(self):
        """initial_guess of the script (ADMM_IPC.py:296-313; renamed here because the Newton
        driver's `initial_guess` is its warm-start hook): xn, xTilde, W, z, u, and no
        constraint rows."""
        self.compute_xn_and_xTilde()
        check(N.lib().fipc_admm_init(self.ctx, dptr(self.xTilde, F64), dptr(self.W, F64), dptr(self.z, F64), dptr(self.u, F64),
                                     self._s()), 'fipc_admm_init')
        self._empty_rows()

    def compute_filter(self, x, x_trial):
        """compute_filter (ADMM_IPC.py:258-268): the point-triangle and edge-edge CCD step from x
        toward x_trial (no inversion filter)."""
        p = (x_trial - x).contiguous()
        a = D()
        check(N.lib().fipc_compute_intersection_free_step_size(self.ctx, dptr(x, F64), dptr(p, F64), D(self.eta), 0, ctypes.byref(a),
                                                               self._s()), 'compute_filter')
        return a.value

    def find_and_reuse(self, alpha):
        """backup_admm_variables, find_constraints, reuse_admm_variables (ADMM_IPC.py:995-1388)."""
        old = (self.rows_all, list(self.row_counts), self.y, self.r, self.Q)
        counts = self.find_constraints()
        lists = []
        for t in range(7):
            n = counts[t]
            rt = torch.zeros((max(n, 1), 4), dtype=torch.int32, device=self.device)
            check(N.lib().fipc_get_constraints(self.ctx, t, dptr(rt, torch.int32), self._s()), 'get_constraints')
            lists.append(rt[:n])
        self.rows_all = torch.cat(lists).contiguous()
        self.row_counts = list(counts)
        n = len(self.rows_all)
        self.y = torch.zeros((n, 9), dtype=F64, device=self.device)
        self.r = torch.zeros((n, 9), dtype=F64, device=self.device)
        self.Q = torch.zeros(n, dtype=F64, device=self.device)
        oc = (ctypes.c_int * 7)(*old[1])
        check(N.lib().fipc_admm_reuse(self.ctx, D(alpha), dptr(self.x, F64), dptr(self.xTilde, F64), oc, self._p(old[0]), self._p(old[2]),
                                      self._p(old[3]), self._p(old[4]), self._p(self.y), self._p(self.r), self._p(self.Q), self._s()),
              'fipc_admm_reuse')

    def global_step(self, t):
        """global_step + solve_system (ADMM_IPC.py:388-631): the solution with the Dirichlet
        targets of time t, then the global filter; returns the filter's step."""
        self._dirichlet(t)
        xx = self.x.clone()
        sol = self.x.clone()
        fx = self.fixed.bool()
        sol[fx] = self.target[fx]
        it = ctypes.c_int()
        check(N.lib().fipc_admm_global(self.ctx, dptr(self.xTilde, F64), dptr(self.W, F64), dptr(self.z, F64), dptr(self.u, F64),
                                       self._p(self.y), self._p(self.r), self._p(self.Q), dptr(self.fixed, torch.uint8), D(self.pcg_rtol),
                                       self.pcg_maxit, dptr(sol, F64), ctypes.byref(it), self._s()), 'fipc_admm_global')
        self.global_iters.append(it.value)
        alpha = self.compute_filter(xx, sol)
        self.x.copy_(sol * alpha + xx * (1 - alpha))
        while alpha >= 1e-6 and self.check_collision():
            self.x.copy_((self.x + xx) / 2.0)
            alpha /= 2.0
        if alpha < 1e-6:
            self.x.copy_(xx)
        self.filter_alphas.append(alpha)
        return alpha

    def local_step(self):
        """local_elasticity and local_PP .. local_PEM (ADMM_IPC.py:633-960)."""
        detail = ctypes.c_int()
        st = N.lib().fipc_admm_local(self.ctx, dptr(self.x, F64), dptr(self.W, F64), dptr(self.z, F64), dptr(self.u, F64),
                                     self._p(self.y), self._p(self.r), self._p(self.Q), ctypes.byref(detail), self._s())
        self.local_detail = detail.value
        check(st, 'fipc_admm_local')

    def dual_step(self):
        """dual_step (ADMM_IPC.py:962-994)."""
        check(N.lib().fipc_admm_dual(self.ctx, dptr(self.x, F64), dptr(self.z, F64), dptr(self.u, F64), self._p(self.y),
                                     self._p(self.r), self._s()), 'fipc_admm_dual')

    # ------------------------------------------------------------------ the time step
    def admm_iteration(self, f, k):
        """ADMM iteration k of time step f (ADMM_IPC.py:1477-1519)."""
        alpha = self.compute_filter(self.x, self.xTilde) if k == 0 else 0.0
        self.find_and_reuse(alpha)
        self.global_step(f * self.dt)
        self.local_step()
        self.dual_step()

    def step(self, f, record=None):
        """One time step (ADMM_IPC.py:1472-1521); returns the number of ADMM iterations."""
        with self.timer('Time Step'):
            self.admm_initial_guess()
            for k in range(self.admm_iters):
                self.admm_iteration(f, k)
                if record is not None:
                    record.append({'x': self.x.cpu().numpy(), 'counts': list(self.row_counts)})
            self.compute_v()
        self.newton_iters.append(self.admm_iters)
        return self.admm_iters

    def state(self):
        """The ADMM variables as numpy arrays (tests)."""
        return {'x': self.x.cpu().numpy(), 'W': self.W.cpu().numpy(), 'z': self.z.cpu().numpy(), 'u': self.u.cpu().numpy(),
                'rows': self.rows_all.cpu().numpy(), 'counts': list(self.row_counts), 'y': self.y.cpu().numpy(),
                'r': self.r.cpu().numpy(), 'Q': self.Q.cpu().numpy()}


__all__ = ['AdmmIPC', 'FastIPCError']
