"""The two-level PCG preconditioner (block-Jacobi + rigid-body coarse space) on the GB300: the
Newton direction is the same as with block-Jacobi alone (both solve the reference's system to
the tolerance), with fewer iterations on a long bar.  (The multigrid preconditioner, the default,
is checked in test_gpu_multigrid.py; set_preconditioner switches it off.)

Bars: directions within 1e-8 relative at rtol 1e-12; at least 2x fewer PCG iterations."""
import numpy as np
import pytest

from fastipc_gb300 import scenes
from fastipc_gb300.newton import NewtonIPC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def bar():
    sc = scenes.predeform(scenes.twisted_bar(nx=60, ny=6, nz=6, size=(0.3, 0.05, 0.05), seed=3), 2e-4, 3)
    sim = NewtonIPC(sc, pcg_rtol=1e-12)
    sim.compute_xn_and_xTilde()
    sim.move_nodes(sim.dt)
    sim.find_constraints()
    sim.compute_hessian_and_gradient()
    yield sim
    sim.close()


def solve(sim, agg):
    sim.set_preconditioner(agg)
    sim.solve_system(sim.dt)
    return sim.data_sol.clone(), sim.pcg_iters[-1]


def test_default_is_multigrid_with_two_level_configured(bar):
    """Multigrid is in use at creation; the two-level coarse space stays configured (2048-vertex
    runs) and takes over when set_preconditioner selects it."""
    assert bar.multigrid()['levels'] >= 2
    p = bar.preconditioner()
    assert p['agg_rows'] == 2048 and p['coarse_dofs'] == 6 * ((bar.nV + 2047) // 2048)


@pytest.mark.parametrize('agg', [128, 256, 512])
def test_same_direction_fewer_iterations(bar, agg):
    ref, it_j = solve(bar, 0)
    d, it_c = solve(bar, agg)
    scale = ref.abs().max().item()
    assert (d - ref).abs().max().item() <= 1e-8 * scale
    assert it_c * 2 <= it_j, (it_c, it_j)
    n_agg = (bar.nV + agg - 1) // agg
    assert bar.preconditioner() == {'agg_rows': agg, 'coarse_dofs': 6 * n_agg}


def test_rejects_bad_sizes(bar):
    from fastipc_gb300._native import FastIPCError
    with pytest.raises(FastIPCError):
        bar.set_preconditioner(100)            # not a multiple of 128
    bar.set_preconditioner(2048)


def test_full_step_matches_block_jacobi():
    sc = scenes.predeform(scenes.twisted_bar(nx=40, ny=5, nz=5, size=(0.2, 0.05, 0.05), seed=4), 2e-4, 4)
    a = NewtonIPC(sc, pcg_rtol=1e-12, coarse_agg=0)
    b = NewtonIPC(sc, pcg_rtol=1e-12, coarse_agg=128)
    for f in range(3):
        assert a.step(f) == b.step(f)
    ext = float(np.ptp(sc.x, axis=0).max())
    assert (a.x - b.x).abs().max().item() <= 1e-9 * ext
    assert sum(b.pcg_iters) < sum(a.pcg_iters)
    a.close()
    b.close()


@pytest.mark.parametrize('n', [32, 96, 544, 800])
def test_dense_spd_inverse(n):
    """the symmetric block-sweep inverse of the coarse solves against numpy (1e-10 relative),
    exactly symmetric"""
    import ctypes
    import torch
    from fastipc_gb300 import _native as NN
    rng = np.random.default_rng(n)
    M = rng.normal(size=(n, n))
    A = M @ M.T + 0.1 * n * np.eye(n)
    d = torch.from_numpy(A.copy()).cuda()
    work = torch.empty(1024 + 64 * n, dtype=torch.float64, device='cuda')
    assert NN.lib().fipc_dense_spd_inverse(n, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(work.data_ptr()), NN.stream()) == 0
    ref = np.linalg.inv(A)
    out = d.cpu().numpy()
    assert np.abs(out - ref).max() <= 1e-10 * np.abs(ref).max()
    assert np.array_equal(out, out.T)
    assert NN.lib().fipc_dense_spd_inverse(100, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(work.data_ptr()), NN.stream()) != 0
