"""The multigrid preconditioner of the PCG direction solve on the GB300 (csrc/mg.cu, set-up from
csrc/mg_plan.h), against the same PCG with the two-level additive preconditioner on the same
assembled systems:

* a 20 x 20 x 100-hex twisted bar (240k tets) a few steps into its twist, and the 216-cube
  lattice at its first ground contact (contact blocks at every level): the directions at relative
  residual 1e-12 agree to 1e-8 of their largest entry, Dirichlet entries are 0, and multigrid
  PCG needs under a third of the iterations;
* the solve is deterministic: two solves of the same system give the same bits;
* switching multigrid off and on through the C ABI restores the other preconditioner.
"""
import numpy as np
import pytest

from fastipc_gb300 import scenes
from fastipc_gb300.newton import NewtonIPC

pytestmark = pytest.mark.gpu


def _state(case):
    if case == 'lattice':
        scene = scenes.predeform(scenes.cube_lattice(m=6, n=6, seed=0), 1e-4, 0)
    else:
        scene = scenes.twisted_bar(nx=100, ny=20, nz=20, size=(0.25, 0.05, 0.05), seed=1)
    sim = NewtonIPC(scene, pcg_rtol=1e-8)
    f = 0
    while f < 40:
        sim.step(f)
        f += 1
        if case == 'bar' and f == 4:
            break
        if case == 'lattice' and sum(sim.counts) > 0:
            break
    sim.compute_xn_and_xTilde()
    sim.move_nodes(f * sim.dt)
    sim.find_constraints()
    sim.compute_hessian_and_gradient()
    return sim, f


def _solve(sim, f, rtol=1e-12):
    sim.pcg_rtol, sim.pcg_maxit = rtol, 200000
    sim.data_sol.zero_()
    sim.solve_system(f * sim.dt)
    return sim.data_sol.cpu().numpy().copy(), sim.pcg_iters[-1]


@pytest.mark.parametrize('case', ['bar', 'lattice'])
def test_multigrid_direction_vs_two_level(case):
    sim, f = _state(case)
    try:
        mg = sim.multigrid()
        assert mg['levels'] >= 3, mg
        if case == 'lattice':
            assert sum(sim.counts) > 0
        p_mg, it_mg = _solve(sim, f)
        p_mg2, _ = _solve(sim, f)
        assert p_mg.tobytes() == p_mg2.tobytes()          # deterministic
        sim.set_preconditioner(2048)                      # the additive two-level preconditioner
        assert sim.multigrid()['levels'] == 0
        sim.compute_hessian_and_gradient()                # offsets at the current positions
        p_cs, it_cs = _solve(sim, f)
        assert np.abs(p_mg - p_cs).max() <= 1e-8 * np.abs(p_cs).max()
        fixed = sim.fixed.cpu().numpy().astype(bool)
        assert np.all(p_mg.reshape(-1, 3)[fixed] == 0.0)
        assert it_mg * 3 < it_cs, (it_mg, it_cs)
        sim.set_multigrid(True)
        assert sim.multigrid()['levels'] == mg['levels']
        sim.compute_hessian_and_gradient()
        p_again, _ = _solve(sim, f)
        assert p_again.tobytes() == p_mg.tobytes()
    finally:
        sim.close()


@pytest.mark.parametrize('case', ['bar', 'lattice'])
def test_fp32_smoothing_products(case):
    """FP32 level-0 smoothing products (the default): the same direction as the FP64 cycle (1e-8
    of its largest entry at relative residual 1e-12), at most 10% more PCG iterations, bitwise
    reproducible."""
    sim, f = _state(case)
    try:
        sim.set_multigrid_fp32(False)
        p64, it64 = _solve(sim, f)
        sim.set_multigrid_fp32(True)
        p32, it32 = _solve(sim, f)
        p32b, _ = _solve(sim, f)
        assert p32.tobytes() == p32b.tobytes()
        assert np.abs(p32 - p64).max() <= 1e-8 * np.abs(p64).max()
        assert it32 <= 1.1 * it64 + 2, (it32, it64)
        sim.set_multigrid_fp32(False)
        p64b, _ = _solve(sim, f)
        assert p64b.tobytes() == p64.tobytes()
        sim.set_multigrid_fp32(True)
    finally:
        sim.close()
