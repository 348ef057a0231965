"""The oracle's Newton driver against the reference's own driver (NEWTON_IPC.py run through
the Taichi stand-in) on a small two-cube drop with contact (no GPU).

Bars: constraint sets exact after canonical (lexicographic) sorting; gradient (rhs) and the
assembled Hessian 1e-9 relative to their largest entry; energy 1e-10 relative; CCD step
1e-6; positions after every step 1e-6 relative to the scene extent.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from fastipc_gb300 import scenes
from oracle import oracle as O


@pytest.fixture(scope='module')
def run(newton_golden):
    g = newton_golden
    scene = scenes.predeform(scenes.two_cubes(n=int(g['n']), seed=int(g['seed'])), float(g['predeform']), int(g['seed']))
    sim = O.OracleSim(scene, solver='direct')
    rec = []
    xs = []
    for f in range(int(g['steps'])):
        sim.step(f, record=rec)
        xs.append(sim.x.copy())
    sim.x_steps = np.array(xs)
    return sim, rec


def test_setup(newton_golden, run):
    sim, _ = run
    g = newton_golden
    np.testing.assert_allclose(sim.m, g['mass'], rtol=1e-13)
    assert abs(sim.kappa / float(g['kappa']) - 1) < 1e-12
    assert abs(sim.inv_dx / float(g['inv_dx']) - 1) < 1e-12


def test_iterations(newton_golden, run):
    g = newton_golden
    sim, rec = run
    n_it = sum(1 for k in g.files if k.endswith('_residual'))
    for i in range(n_it):
        k = f'it{i}_'
        r = rec[i]
        for t, name in enumerate(O.TYPES):
            np.testing.assert_array_equal(r['rows'][t], g[k + name], err_msg=f'iteration {i} {name}')
        scale = np.abs(g[k + 'rhs']).max()
        assert np.abs(r['rhs'] - g[k + 'rhs']).max() <= 1e-9 * scale, i
        assert abs(r['residual'] - float(g[k + 'residual'])) <= 1e-9 * float(g[k + 'residual']), i
        if k + 'E0' in g.files:
            assert abs(r['E0'] - float(g[k + 'E0'])) <= 1e-10 * abs(float(g[k + 'E0'])), i
            assert abs(r['alpha_ccd'] - float(g[k + 'alpha_ccd'])) <= 1e-6, i
            assert abs(r['alpha'] - float(g[k + 'alpha'])) <= 1e-6, i


def test_matrices(newton_golden, run):
    """The assembled system (before the Dirichlet edit) matches the reference's triplets."""
    g = newton_golden
    sim, rec = run
    # re-assemble at the recorded iterates and compare
    for i in (0, 2, 5):
        k = f'it{i}_'
        if k + 'A_data' not in g.files:
            continue
        n = 3 * len(sim.x)
        A_ref = sp.csr_matrix((g[k + 'A_data'], g[k + 'A_indices'], g[k + 'A_indptr']), shape=(n, n))
        sim.x = rec[i]['x'].copy()
        sim.xTilde = g[k + 'xtilde']
        sim.rows = [r.copy() for r in rec[i]['rows']]
        A, rhs = sim.compute_hessian_and_gradient()
        diff = abs(A - A_ref).max()
        assert diff <= 1e-9 * abs(A_ref).max(), (i, diff)


def test_positions(newton_golden, run):
    g = newton_golden
    sim, _ = run
    assert list(sim.newton_iters) == list(g['newton_iters'])
    ext = np.abs(g['x_init']).max()
    np.testing.assert_allclose(sim.x_steps, g['x_steps'], atol=1e-6 * ext, rtol=0)
