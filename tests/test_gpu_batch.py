"""Batched scenes on the GB300: a batch context must give every scene what the scene gets alone
in its own context (NewtonIPC), since the scenes are independent.

Bars, from one state: kappa, hash cell and constraint lists identical; per-scene energy 1e-12
relative; PCG directions 1e-8 relative at rtol 1e-12 (different summation order); CCD steps
1e-6.  Over whole steps the line search compares energies that agree to rounding, and near
convergence E and E0 agree to about as many digits, so the two runs may halve differently:
their Newton iteration counts agree within one per step and they end within the Newton
tolerance (|p|inf < 1e-2 dt = 1e-4 m) of each other."""
import numpy as np
import pytest
import torch

from fastipc_gb300 import scenes
from fastipc_gb300.batch import BatchNewtonIPC
from fastipc_gb300.newton import NewtonIPC

pytestmark = pytest.mark.gpu


def small_scenes():
    out = [scenes.predeform(scenes.two_cubes(n=2, seed=1), 5e-4, 1),
           scenes.cube_stack(3, max_cubes=2, max_hex=4),
           scenes.predeform(scenes.two_cubes(n=3, seed=2), 5e-4, 2),
           scenes.cube_stack(8, max_cubes=3, max_hex=3)]
    return out


@pytest.fixture(scope='module')
def pair():
    sc = small_scenes()
    batch = BatchNewtonIPC(sc, pcg_rtol=1e-12)
    singles = [NewtonIPC(s, pcg_rtol=1e-12) for s in sc]
    yield batch, singles
    batch.close()
    for s in singles:
        s.close()


def test_per_scene_parameters(pair):
    batch, singles = pair
    for s, one in enumerate(singles):
        assert batch.kappa[s] == one.kappa
        assert batch.inv_dx[s] == one.inv_dx


def _advance_to_contact(batch, singles):
    # move both to the state after move_nodes of step 0 and a few plain steps of the singles
    for one in singles:
        for f in range(2):
            one.step(f)
    x = torch.cat([one.x for one in singles])
    v = torch.cat([one.v for one in singles])
    batch.x.copy_(x)
    batch.v.copy_(v)
    for one in singles:
        one.compute_xn_and_xTilde()
        one.move_nodes(2 * one.dt)
    batch.compute_xn_and_xTilde()
    batch.move_nodes(2 * batch.dt)


def test_constraints_energy_direction_and_step(pair):
    batch, singles = pair
    _advance_to_contact(batch, singles)
    batch.find_constraints()
    lists_b = batch.constraints()
    total = 0
    for s, one in enumerate(singles):
        one.find_constraints()
        total += sum(one.counts)
        lists_1 = one.constraints()
        sl = batch.scene_slice(s)
        for t in range(7):
            rb = lists_b[t]
            mine = rb[(rb[:, 0] >= sl.start) & (rb[:, 0] < sl.stop)] - sl.start
            np.testing.assert_array_equal(mine, lists_1[t])
    assert total > 0, 'the scenes should be in contact'
    assert sum(batch.counts) == total
    E = batch.compute_energy().cpu().numpy()
    for s, one in enumerate(singles):
        e1 = one.compute_energy()
        assert abs(E[s] - e1) <= 1e-12 * abs(e1)
    batch.compute_hessian_and_gradient()
    batch.solve_system(2 * batch.dt)
    shape = batch.pcg_shape()
    assert shape['tile_rows'] in (64, 128, 256) and shape['grid'] > 0
    res = batch.output_residual()
    alpha = batch.compute_intersection_free_step_size().cpu().numpy()
    for s, one in enumerate(singles):
        one.compute_hessian_and_gradient()
        one.solve_system(2 * one.dt)
        d1 = one.data_sol
        db = batch.data_sol[batch.scene_slice(s)]
        assert (db - d1).abs().max().item() <= 1e-8 * d1.abs().max().item()
        assert abs(res[s] - one.output_residual()) <= 1e-8 * one.output_residual()
        a1 = one.compute_intersection_free_step_size()
        # the step is a min over exact per-pair tests, so the same direction gives the same bits;
        # directions agree to 1e-8 here
        assert abs(alpha[s] - a1) <= 1e-6 * a1


def test_inactive_scene_gets_zero_direction(pair):
    batch, _ = pair
    batch.compute_hessian_and_gradient()
    active = np.array([True, False, True, False])
    batch.solve_system(2 * batch.dt, active)
    for s in (1, 3):
        assert batch.data_sol[batch.scene_slice(s)].abs().max().item() == 0.0
    assert batch.pcg_iters[-1][1] == 0


def test_full_steps_match_single_scenes():
    """Whole steps: the single scenes run block-Jacobi PCG, as the batch does.  The two sides sum
    in different orders, and a Newton iteration whose |p|inf lands within rounding of the
    tolerance can end the loop on one side and not the other; each step may therefore differ by
    one Newton iteration, and the positions agree within the Newton tolerance."""
    sc = small_scenes()
    batch = BatchNewtonIPC(sc, pcg_rtol=1e-12)
    singles = [NewtonIPC(s, pcg_rtol=1e-12, coarse_agg=0) for s in sc]
    for f in range(4):
        its = batch.step(f)
        for s, one in enumerate(singles):
            assert abs(one.step(f) - int(its[s])) <= 1, (s, f)
    for s, one in enumerate(singles):
        xb = batch.x[batch.scene_slice(s)]
        ext = (one.x.max(0).values - one.x.min(0).values).max().item()
        assert (xb - one.x).abs().max().item() <= 2e-4 * max(ext, 1.0)
        assert not one.check_collision()
    assert not batch.check_collision().any()
    batch.close()
    for s in singles:
        s.close()


def test_batched_start_choice_matches_single_scenes():
    """BatchLearnedStart picks, for every scene, the start that LearnedStart picks for the scene
    alone (here the filtered inertial guess against x^n).  On the first step of two free cubes
    the candidates' energies differ clearly, so the choices must agree exactly, and the steps end
    within a few Newton tolerances of each other.  Later steps check the invariants only."""
    from fastipc_gb300.learned import BatchLearnedStart, LearnedStart
    sc = [scenes.two_cubes(n=2, seed=1), scenes.two_cubes(n=3, seed=2)]
    batch = BatchNewtonIPC(sc, pcg_rtol=1e-12)
    hook = BatchLearnedStart(kind='inertial')
    batch.initial_guess = hook
    singles = []
    for s in sc:
        one = NewtonIPC(s, pcg_rtol=1e-12)
        one.initial_guess = LearnedStart(kind='inertial')
        singles.append(one)
    batch.step(0)
    for one in singles:
        one.step(0)
    for name in ('plain', 'inertial'):
        assert hook.chosen[name] == sum(one.initial_guess.chosen[name] for one in singles)
    for k, one in enumerate(singles):
        # the Newton loops that follow meet contact near-ties, so their paths may differ (14
        # against 16 iterations seen for the n=3 pair); each stops once its last direction is
        # below 1e-4 m, so the two ends lie within a few tolerances of each other
        assert (batch.x[batch.scene_slice(k)] - one.x).abs().max().item() <= 5e-4
    for f in range(1, 3):
        batch.step(f)
        assert not batch.check_collision().any()
    assert sum(hook.chosen.values()) == 3 * len(sc)
    batch.close()
    for one in singles:
        one.close()
