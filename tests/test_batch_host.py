"""Host side of batched scenes: the cube-stack generator and the union arrays (CPU only)."""
import numpy as np

from fastipc_gb300 import scenes
from fastipc_gb300.batch import concat_scenes


def test_cube_stack_sizes_and_gaps():
    sizes = []
    for seed in range(40):
        sc = scenes.cube_stack(seed)
        k = sc.meta['cubes']
        assert 1 <= k <= 8
        sizes.append(sc.n_tets)
        mask, _ = sc.dirichlet(0.0)
        assert mask.sum() == 8 and mask[-8:].all()              # the ground box only
        # cubes above the ground top (y = 0) with at least the gap
        assert sc.x[:-8, 1].min() >= 2e-3 - 1e-12
    assert min(sizes) >= 168 and max(sizes) <= 48006


def test_concat_offsets_and_global_ids():
    sc = [scenes.two_cubes(n=2, seed=1), scenes.cube_stack(3, max_cubes=2, max_hex=4), scenes.two_cubes(n=3, seed=2)]
    u = concat_scenes(sc)
    nv = [s.n_verts for s in sc]
    assert list(u['voff']) == [0, nv[0], nv[0] + nv[1], sum(nv)]
    assert list(u['toff']) == list(np.cumsum([0] + [s.n_tets for s in sc]))
    for s, one in enumerate(sc):
        v0, v1 = u['voff'][s], u['voff'][s + 1]
        t0, t1 = u['toff'][s], u['toff'][s + 1]
        np.testing.assert_array_equal(u['tets'][t0:t1] - v0, one.tets)
        e0, e1 = u['eoff'][s], u['eoff'][s + 1]
        np.testing.assert_array_equal(u['be'][e0:e1] - v0, one.boundary_edges)
        np.testing.assert_array_equal(u['x'][v0:v1], one.initial_positions())
        assert ((u['tets'][t0:t1] >= v0) & (u['tets'][t0:t1] < v1)).all()
