"""ADMM-IPC on the GB300 (fastipc_gb300.admm over fipc_admm_*) against the CPU ADMM oracle
(oracle/admm_oracle.py; parity unpinned to the reference, whose ADMM script does not run against
its own library -- see the oracle's header).

Scene: two 3^3-hex cubes, the upper one dropping into contact (a seeded 0.3 mm start off rest).
* Iteration by iteration from shared states: before every ADMM iteration the oracle takes the
  GPU's state (x, W, z, u, the rows and their y, r, Q); after it, the lists must be equal, y, r,
  Q, z and u within 1e-8 relative to their largest entry and x within 1e-9 of the scene extent.
  The GPU solves the global system by PCG (relative residual 1e-12), the oracle by sparse LU.
* Two whole time steps run independently: positions within 1e-6 of the extent, no edge crossing
  a triangle.
"""
import numpy as np
import pytest

from fastipc_gb300 import scenes
from fastipc_gb300.admm import AdmmIPC
from oracle.admm_oracle import AdmmOracle

pytestmark = pytest.mark.gpu


def scene():
    return scenes.predeform(scenes.two_cubes(n=3, seed=1), 3e-4, 1)


def _sync(o, st, sim):
    o.x = st['x'].copy()
    o.xn = sim.xn.cpu().numpy().copy()
    o.xTilde = sim.xTilde.cpu().numpy().copy()
    o.W, o.z, o.u = st['W'].copy(), st['z'].copy(), st['u'].copy()
    o.rows_all, o.row_counts = st['rows'].copy(), list(st['counts'])
    o.y, o.r, o.Q = st['y'].copy(), st['r'].copy(), st['Q'].copy()


def _close(a, b, rel):
    assert a.shape == b.shape
    if b.size:
        scale = max(np.abs(b).max(), 1e-300)
        assert np.abs(a - b).max() <= rel * scale, (np.abs(a - b).max(), scale)


def test_admm_iterations_vs_oracle():
    sc = scene()
    ext = float(np.ptp(sc.x, axis=0).max())
    sim = AdmmIPC(sc, pcg_rtol=1e-12)
    o = AdmmOracle(sc)
    assert abs(o.kappa - sim.kappa) <= 1e-12 * o.kappa
    rows_seen = 0
    for f in range(2):
        sim.admm_initial_guess()
        o.x, o.v = sim.x.cpu().numpy().copy(), sim.v.cpu().numpy().copy()
        o.initial_guess()
        np.testing.assert_allclose(o.W, sim.W.cpu().numpy(), rtol=1e-12)
        np.testing.assert_allclose(o.z, sim.z.cpu().numpy(), rtol=0, atol=1e-12)
        for k in range(sim.admm_iters):
            _sync(o, sim.state(), sim)
            sim.admm_iteration(f, k)
            o.admm_iteration(f, k)
            st = sim.state()
            assert st['counts'] == o.row_counts, (f, k)
            np.testing.assert_array_equal(st['rows'], o.rows_all)
            rows_seen += len(o.rows_all)
            for name, rel in (('y', 1e-8), ('r', 1e-8), ('Q', 1e-8), ('z', 1e-8), ('u', 1e-8)):
                _close(st[name], getattr(o, name), rel)
            assert np.abs(st['x'] - o.x).max() <= 1e-9 * ext, (f, k)
        sim.compute_v()
    assert rows_seen > 0
    sim.close()


def test_admm_steps_vs_oracle():
    sc = scene()
    ext = float(np.ptp(sc.x, axis=0).max())
    sim = AdmmIPC(sc, pcg_rtol=1e-12)
    o = AdmmOracle(sc)
    for f in range(2):
        sim.step(f)
        o.step(f)
        assert np.abs(sim.x.cpu().numpy() - o.x).max() <= 1e-6 * ext, f
        assert not sim.check_collision()
    sim.close()
