"""The 2D oracle against the reference's own 2D driver (NEWTON_IPC.py with dim == 2, run
through the Taichi stand-in; fixture tests/golden/newton2d_two_squares_n3.npz) on two squares
with a fixed ground segment (no GPU): all 32 Newton iterations of six steps, point-edge and
point-point contact, CCD-limited line searches.

Bars: constraint lists exact; gradient and assembled Hessian 1e-9 relative to their largest
entry; energy 1e-10 relative; CCD step 1e-6; Newton iteration counts equal; positions after
every step 1e-6 relative to the scene extent.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from fastipc_gb300 import scenes
from oracle import oracle2d as O2


def golden_scene2d(g):
    return scenes.predeform(scenes.two_squares_2d(n=int(g['n']), seed=int(g['seed'])), float(g['predeform']), int(g['seed']))


@pytest.fixture(scope='module')
def run(newton2d_golden):
    g = newton2d_golden
    sim = O2.OracleSim2D(golden_scene2d(g))
    rec, xs = [], []
    for f in range(int(g['steps'])):
        sim.step(f, record=rec)
        xs.append(sim.x.copy())
    sim.x_steps = np.array(xs)
    return sim, rec


def test_scene_matches_fixture(newton2d_golden):
    g = newton2d_golden
    sc = golden_scene2d(g)
    np.testing.assert_array_equal(sc.tris, g['tris'])
    np.testing.assert_array_equal(sc.boundary_edges, g['bedges'])
    np.testing.assert_array_equal(sc.x, g['x_rest'])
    np.testing.assert_array_equal(sc.initial_positions(), g['x_init'])


def test_boundary_matches_reference(newton2d_golden):
    """scenes.find_boundary_2d against the reference's graph_tools.find_boundary (run on the
    same triangles when the fixture was made): the same points and the same oriented edges in
    the same order."""
    g = newton2d_golden
    for tris, pts, edges in ((g['tris'], g['ref_bpoints'], g['ref_bedges']),
                             (g['stack_tris'], g['stack_ref_bpoints'], g['stack_ref_bedges'])):
        bp, be = scenes.find_boundary_2d(tris)
        np.testing.assert_array_equal(bp, pts)
        np.testing.assert_array_equal(be, edges.reshape(-1, 2))
    sc = golden_scene2d(g)
    n = len(g['ref_bedges'])
    np.testing.assert_array_equal(sc.boundary_edges[:n], g['ref_bedges'].reshape(-1, 2))


def test_setup(newton2d_golden, run):
    sim, _ = run
    g = newton2d_golden
    np.testing.assert_allclose(sim.m, g['mass'], rtol=1e-13)
    assert abs(sim.kappa / float(g['kappa']) - 1) < 1e-12
    assert abs(sim.mean_edge / float(g['mean_edge']) - 1) < 1e-12


def test_iterations(newton2d_golden, run):
    g = newton2d_golden
    _, rec = run
    n_it = sum(1 for k in g.files if k.endswith('_residual'))
    assert n_it >= 10
    n_pe = 0
    for i in range(n_it):
        k = f'it{i}_'
        r = rec[i]
        np.testing.assert_array_equal(r['PP'], g[k + 'PP'].reshape(-1, 2), err_msg=f'iteration {i} PP')
        np.testing.assert_array_equal(r['PE'], g[k + 'PE'].reshape(-1, 3), err_msg=f'iteration {i} PE')
        n_pe += len(r['PE'])
        scale = np.abs(g[k + 'rhs']).max()
        assert np.abs(r['rhs'] - g[k + 'rhs']).max() <= 1e-9 * scale, i
        assert abs(r['residual'] - float(g[k + 'residual'])) <= 1e-9 * float(g[k + 'residual']), i
        if k + 'E0' in g.files:
            assert abs(r['E0'] - float(g[k + 'E0'])) <= 1e-10 * abs(float(g[k + 'E0'])), i
            assert abs(r['alpha_ccd'] - float(g[k + 'alpha_ccd'])) <= 1e-6, i
            assert abs(r['alpha'] - float(g[k + 'alpha'])) <= 1e-6, i
    assert n_pe > 0   # contact is exercised


def test_later_iterations_with_point_point_rows(newton2d_golden, run):
    """The iterations after the first twelve (fixture keys xt{i}_), which include the
    point-point rows of steps 3-4, evaluated at the reference's own iterates: lists, system,
    direction, energy and CCD step."""
    g = newton2d_golden
    sim, _ = run
    n = 2 * len(sim.x)
    extra = sorted(int(k[2:].split('_')[0]) for k in g.files if k.startswith('xt') and k.endswith('_res'))
    assert len(extra) >= 10
    n_pp = 0
    for i in extra:
        k = f'xt{i}_'
        sim.x, sim.xTilde = g[k + 'x'].copy(), g[k + 'xtilde']
        sim.find_constraints()
        np.testing.assert_array_equal(sim.PP, g[k + 'PP'].reshape(-1, 2), err_msg=f'iteration {i} PP')
        np.testing.assert_array_equal(sim.PE, g[k + 'PE'].reshape(-1, 3), err_msg=f'iteration {i} PE')
        n_pp += len(sim.PP)
        sim.compute_hessian_and_gradient()
        A_ref = sp.csr_matrix((g[k + 'A_data'], g[k + 'A_indices'], g[k + 'A_indptr']), shape=(n, n))
        assert abs(sim.A - A_ref).max() <= 1e-9 * abs(A_ref).max(), i
        assert np.abs(sim.rhs - g[k + 'rhs']).max() <= 1e-9 * np.abs(g[k + 'rhs']).max(), i
        sol = sim.solve_system(0.0)
        assert np.abs(sol - g[k + 'sol']).max() <= 1e-8 * np.abs(g[k + 'sol']).max(), i
        if k + 'E0' in g.files:
            assert abs(sim.compute_energy() - float(g[k + 'E0'])) <= 1e-10 * abs(float(g[k + 'E0'])), i
            sim.sol = g[k + 'sol']
            assert abs(sim.compute_intersection_free_step_size() - float(g[k + 'alpha_ccd'])) <= 1e-6, i
    assert n_pp > 0


def test_matrices(newton2d_golden, run):
    g = newton2d_golden
    sim, rec = run
    n = 2 * len(sim.x)
    for i in range(12):
        k = f'it{i}_'
        if k + 'A_data' not in g.files:
            continue
        A_ref = sp.csr_matrix((g[k + 'A_data'], g[k + 'A_indices'], g[k + 'A_indptr']), shape=(n, n))
        sim.x = g[k + 'x'].copy()
        sim.xTilde = g[k + 'xtilde']
        sim.PP, sim.PE = g[k + 'PP'].reshape(-1, 2), g[k + 'PE'].reshape(-1, 3)
        sim.compute_hessian_and_gradient()
        assert abs(sim.A - A_ref).max() <= 1e-9 * abs(A_ref).max(), i
        assert np.abs(sim.rhs - g[k + 'rhs']).max() <= 1e-9 * np.abs(g[k + 'rhs']).max(), i


def test_positions(newton2d_golden, run):
    g = newton2d_golden
    sim, _ = run
    assert list(sim.newton_iters) == list(g['newton_iters'])
    ext = np.abs(g['x_init']).max()
    np.testing.assert_allclose(sim.x_steps, g['x_steps'], atol=1e-6 * ext, rtol=0)


def test_svd2_convention():
    """numpy's SVD turned rotation-variant: U, V rotations, s0 >= |s1|, s1 < 0 iff det F < 0."""
    rng = np.random.default_rng(2)
    F = rng.normal(size=(200, 2, 2))
    U, s, V = O2.svd2(F)
    np.testing.assert_allclose(U @ (s[:, :, None] * np.swapaxes(V, 1, 2)), F, atol=1e-13)
    assert np.all(np.linalg.det(U) > 0) and np.all(np.linalg.det(V) > 0)
    assert np.all(s[:, 0] >= np.abs(s[:, 1]))
    assert np.all((s[:, 1] < 0) == (np.linalg.det(F) < 0))


def test_c_oracle_matches_numpy_oracle(newton2d_golden):
    """The C (OpenMP) 2D loops against the numpy ones: elements (Jacobi against numpy SVD,
    1e-11 relative), constraint lists (exact), CCD step and intersection flag, at the
    reference's own iterates and at random deformations."""
    g = newton2d_golden
    sim = O2.OracleSim2D(golden_scene2d(g))
    rng = np.random.default_rng(12)
    states = [g[f'it{i}_x'] for i in (0, 5, 11)] + [g['x_rest'] + rng.normal(size=g['x_rest'].shape) * s for s in (1e-3, 8e-3)]
    for x in states:
        a = O2.elements(sim.tris, x, sim.IB, sim.vol, sim.la, sim.mu, sim.dt)
        b = O2.elements_c(sim.tris, x, sim.IB, sim.vol, sim.la, sim.mu, sim.dt)
        for u, v in zip(a, b):
            assert np.abs(u - v).max() <= 1e-11 * max(np.abs(u).max(), 1e-300)
        np.testing.assert_array_equal(O2.find_constraints(x, sim.bp, sim.be, sim.dhat2)[0],
                                      O2.find_constraints_c(x, sim.bp, sim.be, sim.dhat2)[0])
        np.testing.assert_array_equal(O2.find_constraints(x, sim.bp, sim.be, sim.dhat2)[1],
                                      O2.find_constraints_c(x, sim.bp, sim.be, sim.dhat2)[1])
        p = rng.normal(size=x.shape) * 2e-3
        assert abs(O2.ccd_step(x, p, sim.bp, sim.be, sim.dhat2) - O2.ccd_step_c(x, p, sim.bp, sim.be, sim.dhat2)) <= 1e-12
        assert O2.check_collision(x, sim.bp, sim.tris) == O2.check_collision_c(x, sim.bp, sim.tris)
    x = g['x_rest'].copy()
    x[len(x) // 2:-2, 1] -= 0.05
    assert O2.check_collision_c(x, sim.bp, sim.tris) and O2.check_collision(x, sim.bp, sim.tris)


def test_c_oracle_trajectory(newton2d_golden):
    g = newton2d_golden
    sim = O2.OracleSim2D(golden_scene2d(g), fast=True)
    xs = []
    for f in range(int(g['steps'])):
        sim.step(f)
        xs.append(sim.x.copy())
    assert list(sim.newton_iters) == list(g['newton_iters'])
    np.testing.assert_allclose(np.array(xs), g['x_steps'], atol=1e-6 * np.abs(g['x_init']).max(), rtol=0)
