"""The direct solve of the Newton system (fipc_solve_system_direct: the reference's CHOLMOD
role, NEWTON_IPC.py:758-776) on the GB300 against the reference's own exact solves
(tests/golden/newton_two_cubes_n3.npz), and the PCG fallback to it.

Bars: direction 1e-9 relative to its largest entry (both sides factorise exactly); Newton
iteration counts equal; positions after every step within 1e-6 of the scene extent; the
fallback reproduces the direct solver bit for bit.
"""
import numpy as np
import pytest
import torch

from fastipc_gb300 import scenes
from fastipc_gb300.newton import NewtonIPC

pytestmark = pytest.mark.gpu


def golden_scene(g):
    return scenes.predeform(scenes.two_cubes(n=int(g['n']), seed=int(g['seed'])), float(g['predeform']), int(g['seed']))


def iters(g):
    return sorted(int(k[2:].split('_')[0]) for k in g.files if k.endswith('_residual'))


def test_direct_direction_vs_reference(newton_golden):
    g = newton_golden
    sim = NewtonIPC(golden_scene(g), solver='direct')
    try:
        for i in iters(g):
            sim.x.copy_(torch.from_numpy(g[f'it{i}_x']))
            sim.xTilde.copy_(torch.from_numpy(g[f'it{i}_xtilde']))
            sim.find_constraints()
            sim.compute_hessian_and_gradient()
            sim._dir_key = None
            sim.solve_system(0.0)
            sol = sim.data_sol.cpu().numpy().ravel()
            ref = g[f'it{i}_sol']
            assert np.abs(sol - ref).max() <= 1e-9 * np.abs(ref).max(), i
        assert sim.direct_solves == len(iters(g))
    finally:
        sim.close()


def test_direct_trajectory_vs_reference(newton_golden):
    g = newton_golden
    sim = NewtonIPC(golden_scene(g), solver='direct')
    try:
        xs = []
        for f in range(int(g['steps'])):
            sim.step(f)
            xs.append(sim.x.cpu().numpy().copy())
        assert list(sim.newton_iters) == list(g['newton_iters'])
        ext = np.abs(g['x_init']).max()
        np.testing.assert_allclose(np.array(xs), g['x_steps'], atol=1e-6 * ext, rtol=0)
    finally:
        sim.close()


def test_pcg_fallback_to_direct(newton_golden):
    """A PCG capped at 2 iterations stops at its limit every time; each solve is redone by the
    direct solver, so the steps equal the direct solver's bit for bit."""
    g = newton_golden
    out = []
    for kw in ({'solver': 'direct'}, {'pcg_maxit': 2, 'direct_fallback': True}):
        sim = NewtonIPC(golden_scene(g), **kw)
        try:
            for f in range(2):
                sim.step(f)
            out.append(sim.x.cpu().numpy().tobytes())
            assert sim.direct_solves == sum(sim.newton_iters) > 0
        finally:
            sim.close()
    assert out[0] == out[1]


@pytest.mark.parametrize('case', ['lattice_216', 'bar_100'])
def test_direct_matches_tight_pcg_on_large_scenes(case):
    """Full-size lattice at its first ground contact and a 240k-tet bar a few steps into its
    twist: hundreds to thousands of fronts over a dozen tree levels.  The direct direction
    agrees with PCG at relative residual 1e-12 to 1e-8 of its largest entry."""
    if case == 'lattice_216':
        scene = scenes.predeform(scenes.cube_lattice(m=6, n=6, seed=0), 1e-4, 0)
    else:
        scene = scenes.twisted_bar(nx=100, ny=20, nz=20, size=(0.25, 0.05, 0.05), seed=1)
    sim = NewtonIPC(scene, pcg_rtol=1e-8)
    try:
        f = 0
        while f < 40:
            sim.step(f)
            f += 1
            if case == 'bar_100' and f == 4:
                break
            if case == 'lattice_216' and sum(sim.counts) > 0:
                break
        sim.compute_xn_and_xTilde()
        sim.move_nodes(f * sim.dt)
        sim.find_constraints()
        sim.compute_hessian_and_gradient()
        sim.pcg_rtol, sim.pcg_maxit = 1e-12, 100000
        sim.solve_system(f * sim.dt)
        p_pcg = sim.data_sol.cpu().numpy().copy()
        sim.solver = 'direct'
        sim.solve_system(f * sim.dt)
        p_dir = sim.data_sol.cpu().numpy().copy()
        assert np.abs(p_dir - p_pcg).max() <= 1e-8 * np.abs(p_pcg).max()
        fixed = sim.fixed.cpu().numpy().astype(bool)
        assert np.all(p_dir.reshape(-1, 3)[fixed] == 0.0)
    finally:
        sim.close()
