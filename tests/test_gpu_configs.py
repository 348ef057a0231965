"""Parity at the benchmark configurations' full sizes: the GPU path against the CPU oracle,
both started from the same mid-trajectory state.

* The 960k-tet twisted bar (the headline workload; 176,841 vertices, 960,000 tets): the GPU runs
  150 of the configuration's 200 steps from t = 0.  The configured twist (4 pi between the end
  faces after 200 steps) stays below the roughly 15 rad at which this bar buckles into a coil
  (Greenhill's clamped-rod torque 2.86 pi EI / L over GJ), and the run confirms it: the
  constraint lists are empty on every step (they stayed empty through 450 steps on a GB300).
  At step 150 the lists must equal the oracle's bit for bit (both empty), the
  incremental-potential energy agree within 1e-10 relative, the right-hand side (minus the
  gradient) within 1e-9 of its largest entry, and the CCD step size on the GPU's own direction
  within 1e-6.  Then both take two whole time steps from that state with tight solves (PCG
  relative residual 1e-11 on both sides): equal Newton iteration counts and positions within
  1e-6 of the bar's length.  Contact at full size is covered by the next two cases.
* The 216-cube lattice drop (74,096 vertices, 279,942 tets), started a seeded 0.1 mm away from
  rest (at an exactly undeformed element the reference's projected Neo-Hookean Hessian depends
  on the sign of rounding noise): the same checks at its first ground contact, and two steps.
* The three largest scenes of the 512-scene batch (about 48k tets each), pre-deformed the same
  way, stepped together in one batch context: every scene against the oracle running it alone,
  over fourteen steps (a rotated lowest cube starts up to 39 mm above the ground, about nine
  steps of free fall), which include every scene's first contacts: equal Newton counts per
  step and positions within 1e-6 of the scene's extent.

The line search compares energies E and E0 that, near convergence, agree to about as many
digits as the two implementations' rounding; a case where the two sides halve differently would
end both inside the Newton tolerance, and is reported by the assertion message if it happens.
"""
import numpy as np
import pytest

from fastipc_gb300 import scenes
from fastipc_gb300.newton import NewtonIPC
from oracle import oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

RTOL = 1e-11


def _compare_state(sim, o, f):
    """sim and o hold the same (x, v) at the start of step f: compare the first Newton
    iterate's lists, energy, right-hand side and CCD step."""
    dt = sim.dt
    sim.compute_xn_and_xTilde()
    sim.move_nodes(f * dt)
    o.compute_xn_and_xTilde()
    o.move_nodes(f * dt)
    # the Dirichlet targets come from the device schedule on one side and the per-vertex loop on
    # the other (equal within 1e-14 m); the comparison below starts from identical inputs
    np.testing.assert_allclose(sim.xTilde.cpu().numpy(), o.xTilde, rtol=0, atol=1e-13)
    o.x, o.xn, o.xTilde = sim.x.cpu().numpy().copy(), sim.xn.cpu().numpy().copy(), sim.xTilde.cpu().numpy().copy()
    counts = sim.find_constraints()
    o.find_constraints()
    lists = sim.constraints()
    for t in range(7):
        np.testing.assert_array_equal(lists[t], o.rows[t], err_msg=f'list {t}')
    E, E_o = sim.compute_energy(), o.compute_energy()
    assert abs(E - E_o) <= 1e-10 * abs(E_o), (E, E_o)
    sim.compute_hessian_and_gradient()
    _, _, rhs = sim.export_system()
    _, rhs_o = o.compute_hessian_and_gradient()
    assert np.abs(rhs - rhs_o).max() <= 1e-9 * np.abs(rhs_o).max()
    sim.solve_system(f * dt)
    p = sim.data_sol.cpu().numpy().copy()
    sim.save_xPrev()
    a = sim.compute_intersection_free_step_size()
    a_o = o.compute_intersection_free_step_size(p=p)
    assert abs(a - a_o) <= 1e-6, (a, a_o)
    return counts


def _two_steps(sim, o, x, v, f, extent):
    sim.set_state(x, v)
    o.x, o.v = x.copy(), v.copy()
    for k in (f, f + 1):
        it = sim.step(k)
        it_o = o.step(k)
        dev = float(np.abs(sim.x.cpu().numpy() - o.x).max())
        assert it == it_o, (k, it, it_o, dev)
        assert dev <= 1e-6 * extent, (k, dev)
        assert not sim.check_collision()


def test_twisted_bar_960k_mid_run_vs_oracle():
    scene = scenes.twisted_bar(nx=400, ny=20, nz=20, size=(1.0, 0.05, 0.05), seed=0)
    assert scene.n_tets == 960000
    sim = NewtonIPC(scene, pcg_rtol=1e-6, pcg_warm_start=True)
    f = 0
    while f < 150:
        sim.step(f)
        f += 1
        assert sum(sim.counts) == 0, f'self-contact at step {f}'
    x, v = sim.x.cpu().numpy().copy(), sim.v.cpu().numpy().copy()
    sim.pcg_rtol, sim.pcg_warm_start = RTOL, False
    o = O.OracleSim(scene, solver='bsr', pcg_rtol=RTOL, pcg_maxit=400000)
    o.x, o.v = x.copy(), v.copy()
    _compare_state(sim, o, f)
    _two_steps(sim, o, x, v, f, extent=1.0)
    sim.close()


def test_lattice_216_cubes_at_ground_contact_vs_oracle():
    scene = scenes.predeform(scenes.cube_lattice(m=6, n=6, seed=0), 1e-4, 0)
    sim = NewtonIPC(scene, pcg_rtol=1e-8)
    f = 0
    while f < 40:
        sim.step(f)
        f += 1
        if sum(sim.counts) > 0:
            break
    assert sum(sim.counts) > 0, 'no ground contact in 40 steps'
    x, v = sim.x.cpu().numpy().copy(), sim.v.cpu().numpy().copy()
    sim.pcg_rtol = RTOL
    o = O.OracleSim(scene, solver='bsr', pcg_rtol=RTOL, pcg_maxit=400000)
    o.x, o.v = x.copy(), v.copy()
    _compare_state(sim, o, f)
    ext = float(np.ptp(scene.x[:-8], axis=0).max())
    _two_steps(sim, o, x, v, f, extent=ext)
    sim.close()


def test_three_largest_batch_scenes_vs_oracle():
    from fastipc_gb300.batch import BatchNewtonIPC
    sizes = [scenes.cube_stack(s).n_tets for s in range(512)]
    pick = sorted(np.argsort(sizes)[-3:].tolist())
    scs = [scenes.predeform(scenes.cube_stack(int(s)), 1e-4, int(s)) for s in pick]
    assert min(sc.n_tets for sc in scs) > 30000
    batch = BatchNewtonIPC(scs, pcg_rtol=1e-12)
    oracles = [O.OracleSim(sc, solver='bsr', pcg_rtol=1e-12, pcg_maxit=400000) for sc in scs]
    contact = [False] * len(scs)
    for f in range(14):
        its = batch.step(f)
        for k, (sc, o) in enumerate(zip(scs, oracles)):
            it_o = o.step(f)
            xb = batch.x[batch.scene_slice(k)].cpu().numpy()
            ext = float(np.ptp(sc.x[:-8], axis=0).max())
            dev = float(np.abs(xb - o.x).max())
            assert int(its[k]) == it_o, (pick[k], f, int(its[k]), it_o, dev)
            assert dev <= 1e-6 * ext, (pick[k], f, dev)
            contact[k] |= sum(len(r) for r in o.rows) > 0
    assert all(contact), contact
    batch.close()
