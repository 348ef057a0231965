"""Scenes whose boundary mixes fine bodies with a few large triangles (a ground box under cube
stacks): triangles and edges whose box covers more than 256 hash cells bypass the grid and are
tested against every primitive of their scene.  The constraint lists, the CCD step and the
intersection check must equal the oracle's, which hashes every primitive.

Bars: constraint lists exact; CCD step 1e-12 relative; intersection flag equal."""
import numpy as np
import pytest
import torch

from fastipc_gb300 import scenes
from fastipc_gb300.batch import BatchNewtonIPC
from fastipc_gb300.newton import NewtonIPC
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def on_ground(sc, s):
    ground = set(range(len(sc.x) - 8, len(sc.x)))
    s.find_constraints()
    return any(int(v) in ground for r in s.constraints() for v in r.ravel())


def settled(seed, max_steps=30):
    """the stack stepped until its lowest cube is within d-hat of the ground box"""
    sc = scenes.cube_stack(seed, max_cubes=3, max_hex=5)
    s = NewtonIPC(sc, pcg_rtol=1e-12)
    for f in range(max_steps):
        s.step(f)
        if on_ground(sc, s):
            break
    return sc, s


@pytest.mark.parametrize('seed', [5, 6])
def test_lists_ccd_and_collision_match_oracle(seed):
    sc, s = settled(seed)
    o = O.OracleSim(sc, solver='bsr')
    x = s.x.cpu().numpy()
    o.x = x.copy()
    s.find_constraints()
    o.find_constraints()
    ground = set(range(len(sc.x) - 8, len(sc.x)))
    touches_ground = False
    for t in range(7):
        r = s.constraints()[t]
        np.testing.assert_array_equal(r, o.rows[t])
        touches_ground |= any(int(v) in ground for v in r.ravel())
    assert touches_ground, 'the stack should rest on the ground box'
    # a direction that pushes everything down into the ground
    rng = np.random.default_rng(seed)
    p = np.zeros_like(x)
    p[:-8, 1] = -2e-3
    p[:-8] += rng.uniform(-2e-4, 2e-4, (len(x) - 8, 3))
    s.data_sol.copy_(torch.from_numpy(p))
    a_gpu = s.compute_intersection_free_step_size()
    a_ref = o.compute_intersection_free_step_size(p)
    assert a_ref < 1.0
    assert abs(a_gpu - a_ref) <= 1e-12 * a_ref
    # positions pushed through the ground intersect; the filtered step does not
    s.x.copy_(torch.from_numpy(x + p * 1.0))
    o.x = x + p * 1.0
    assert s.check_collision() == o.check_collision() == True  # noqa: E712
    s.x.copy_(torch.from_numpy(x + p * a_gpu))
    o.x = x + p * a_gpu
    assert s.check_collision() == o.check_collision() == False  # noqa: E712
    s.close()


def test_batch_of_stacks_matches_single_scenes():
    scs = [scenes.cube_stack(k, max_cubes=3, max_hex=5) for k in (5, 6, 7)]
    singles = []
    for sc in scs:
        s = NewtonIPC(sc, pcg_rtol=1e-12)
        for f in range(4):
            s.step(f)
        singles.append(s)
    b = BatchNewtonIPC(scs, pcg_rtol=1e-12)
    b.x.copy_(torch.cat([s.x for s in singles]))
    b.find_constraints()
    rows = b.constraints()
    for k, s in enumerate(singles):
        s.find_constraints()
        sl = b.scene_slice(k)
        for t in range(7):
            r = rows[t]
            np.testing.assert_array_equal(r[(r[:, 0] >= sl.start) & (r[:, 0] < sl.stop)] - sl.start, s.constraints()[t])
    b.close()
    for s in singles:
        s.close()
