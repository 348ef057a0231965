"""The full Newton path on the GB300 (NewtonIPC over libfastipc.so) against the reference's own
driver (golden fixture from NEWTON_IPC.py run through the Taichi stand-in) and the oracle.

Bars: constraint lists exact after canonical sorting; assembled Hessian and gradient 1e-9
relative to their largest entry; energy 1e-10 relative; CCD step 1e-6; Newton iteration counts
equal; positions after every step within 1e-6 of the scene extent; reruns bitwise equal."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from fastipc_gb300 import scenes
from fastipc_gb300.newton import NewtonIPC
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def golden_scene(g):
    return scenes.predeform(scenes.two_cubes(n=int(g['n']), seed=int(g['seed'])), float(g['predeform']), int(g['seed']))


@pytest.fixture(scope='module')
def sim(newton_golden):
    s = NewtonIPC(golden_scene(newton_golden), pcg_rtol=1e-12)
    yield s
    s.close()


def iters(g):
    return sorted(int(k[2:].split('_')[0]) for k in g.files if k.endswith('_residual'))


def test_setup(newton_golden, sim):
    g = newton_golden
    np.testing.assert_allclose(sim.mass(), g['mass'], rtol=1e-13)
    assert abs(sim.kappa / float(g['kappa']) - 1) < 1e-12
    assert abs(sim.inv_dx / float(g['inv_dx']) - 1) < 1e-12


def set_state(sim, g, i):
    sim.x.copy_(torch.from_numpy(g[f'it{i}_x']))
    sim.xTilde.copy_(torch.from_numpy(g[f'it{i}_xtilde']))


def test_find_constraints(newton_golden, sim):
    g = newton_golden
    for i in iters(g):
        set_state(sim, g, i)
        sim.find_constraints()
        rows = sim.constraints()
        for t, name in enumerate(O.TYPES):
            np.testing.assert_array_equal(rows[t], g[f'it{i}_{name}'].reshape(-1, O.TYPE_NV[t]), err_msg=f'it {i} {name}')


def test_system(newton_golden, sim):
    g = newton_golden
    n = 3 * sim.nV
    for i in iters(g):
        set_state(sim, g, i)
        sim.find_constraints()
        sim.compute_hessian_and_gradient()
        Ael, Act, rhs = sim.export_system()
        assert np.abs(rhs - g[f'it{i}_rhs']).max() <= 1e-9 * np.abs(g[f'it{i}_rhs']).max(), i
        if f'it{i}_A_data' in g.files:
            A_ref = sp.csr_matrix((g[f'it{i}_A_data'], g[f'it{i}_A_indices'], g[f'it{i}_A_indptr']), shape=(n, n))
            diff = abs((Ael + Act).tocsr() - A_ref).max()
            assert diff <= 1e-9 * abs(A_ref).max(), (i, diff)


def test_energy_ccd_solve(newton_golden, sim):
    g = newton_golden
    for i in iters(g):
        if f'it{i}_E0' not in g.files:
            continue
        set_state(sim, g, i)
        sim.find_constraints()
        E0 = sim.compute_energy()
        assert abs(E0 - float(g[f'it{i}_E0'])) <= 1e-10 * abs(float(g[f'it{i}_E0'])), i
        sim.data_sol.copy_(torch.from_numpy(g[f'it{i}_sol'].reshape(-1, 3)))
        a = sim.compute_intersection_free_step_size()
        assert abs(a - float(g[f'it{i}_alpha_ccd'])) <= 1e-6, (i, a, float(g[f'it{i}_alpha_ccd']))
        # the PCG direction against the reference's exact solve
        sim.compute_hessian_and_gradient()
        sim.solve_system(0.0)
        sol = sim.data_sol.cpu().numpy().ravel()
        ref = g[f'it{i}_sol']
        assert np.abs(sol - ref).max() <= 1e-7 * np.abs(ref).max(), i


def test_newton_trajectory(newton_golden):
    g = newton_golden
    s = NewtonIPC(golden_scene(g), pcg_rtol=1e-12)
    xs = []
    for f in range(int(g['steps'])):
        s.step(f)
        xs.append(s.x.cpu().numpy().copy())
        assert not s.check_collision()
    s.close()
    assert list(s.newton_iters) == list(g['newton_iters'])
    ext = np.abs(g['x_init']).max()
    np.testing.assert_allclose(np.array(xs), g['x_steps'], atol=1e-6 * ext, rtol=0)


def test_determinism(newton_golden):
    g = newton_golden
    out = []
    for _ in range(2):
        s = NewtonIPC(golden_scene(g), pcg_rtol=1e-12)
        s.step(0)
        out.append(s.x.cpu().numpy().copy())
        s.close()
    assert np.array_equal(out[0], out[1])


def test_collision_detects_intersection(newton_golden):
    g = newton_golden
    s = NewtonIPC(golden_scene(g))
    x = s.x.cpu().numpy()
    lower = x[:, 1] < 0.1 + 1e-9
    upper = ~lower
    assert not s.check_collision()
    x2 = x.copy()
    x2[upper, 1] -= 0.05          # push the upper cube half-way into the lower one
    s.x.copy_(torch.from_numpy(x2))
    hit = s.check_collision()
    from oracle.oracle import lib as olib, _p
    be, bt = np.ascontiguousarray(s.scene.boundary_edges, np.int32), np.ascontiguousarray(s.scene.boundary_triangles, np.int32)
    ref = bool(olib().oracle_check_collision(_p(np.ascontiguousarray(x2)), len(be), _p(be, np.int32), len(bt), _p(bt, np.int32),
                                             O.D(s.dhat2), O.D(s.inv_dx)))
    assert hit == ref == True  # noqa: E712
    s.close()


def test_two_cubes_8_vs_oracle():
    """The configuration-0 mesh size (2 x 8^3 hexes, 6144 tets): three steps against the oracle."""
    scene = scenes.predeform(scenes.two_cubes(n=8, seed=1), 2e-4, 1)
    s = NewtonIPC(scene, pcg_rtol=1e-12)
    o = O.OracleSim(scene, solver='direct')
    for f in range(3):
        s.step(f)
        o.step(f)
        assert s.newton_iters[-1] == o.newton_iters[-1]
        np.testing.assert_allclose(s.x.cpu().numpy(), o.x, atol=1e-6 * 0.2, rtol=0)
    s.find_constraints()
    o.find_constraints()
    for t in range(7):
        np.testing.assert_array_equal(s.constraints()[t], o.rows[t])
    s.close()


def test_twisted_bar_small_vs_oracle():
    """Twisted-bar scene family (rotating Dirichlet ends, E=1e6, nu=0.45) at 4 x 4 x 40 hexes,
    pre-deformed so that no element sits exactly at rest (where the reference's projected
    Neo-Hookean Hessian depends on the sign of rounding noise)."""
    scene = scenes.predeform(scenes.twisted_bar(nx=40, ny=4, nz=4, size=(0.1, 0.01, 0.01), seed=2), 5e-5, 2)
    s = NewtonIPC(scene, pcg_rtol=1e-12)
    o = O.OracleSim(scene, solver='direct')
    for f in range(3):
        s.step(f)
        o.step(f)
        assert s.newton_iters[-1] == o.newton_iters[-1]
        np.testing.assert_allclose(s.x.cpu().numpy(), o.x, atol=1e-6 * 0.05, rtol=0)
    s.close()
