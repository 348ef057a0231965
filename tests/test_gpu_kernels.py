"""Element kernels on the GB300 through the C ABI, against the reference's golden vectors and
the oracle.  Bars: energy 1e-10 relative; gradient/Hessian 1e-9 relative to the largest entry
of each array; CCD time of impact 1e-6 absolute; classifications exact."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.gpu_util import D, cu, lib, p, rel, stream

pytestmark = pytest.mark.gpu


def barrier_gpu(t, X, X0, dh2, kappa):
    N = len(X)
    x = cu(X.reshape(-1, 3))
    x0 = cu(X0.reshape(-1, 3))
    rows = cu((np.arange(N)[:, None] * 4 + np.arange(4)[None, :]).astype(np.int32))
    E = torch.zeros(N, dtype=torch.float64, device='cuda')
    g = torch.zeros((N, 12), dtype=torch.float64, device='cuda')
    H = torch.zeros((N, 16, 9), dtype=torch.float64, device='cuda')
    assert lib().fipc_barrier_rows(t, N, p(rows), p(x), p(x0), D(dh2), D(kappa), p(E), p(g), p(H), stream()) == 0
    torch.cuda.synchronize()
    nv = O.TYPE_NV[t]
    Hb = H.cpu().numpy().reshape(N, 4, 4, 3, 3)[:, :nv, :nv].transpose(0, 1, 3, 2, 4).reshape(N, 3 * nv, 3 * nv)
    return E.cpu().numpy(), g.cpu().numpy()[:, :3 * nv], Hb


@pytest.mark.parametrize('t', range(7))
def test_barrier_rows_golden(unit_golden, t):
    g = unit_golden
    name = O.TYPES[t]
    E, gr, H = barrier_gpu(t, g[f'bar_{name}_x'], g[f'bar_{name}_x0'], float(g['bar_dhat2']), float(g['bar_kappa']))
    np.testing.assert_allclose(E, g[f'bar_{name}_E'], rtol=1e-10)
    assert rel(gr, g[f'bar_{name}_g']) < 1e-9
    assert rel(H, g[f'bar_{name}_H']) < 1e-9


@pytest.mark.parametrize('t', range(7))
def test_barrier_rows_random_vs_oracle(t):
    rng = np.random.default_rng(500 + t)
    N = 2000
    X = rng.uniform(-1, 1, (N, 1, 3)) + rng.normal(size=(N, 4, 3)) * 4e-4
    if t >= 4:
        d = rng.normal(size=(N, 3)) * 3e-3
        X[:, 1] = X[:, 0] + d
        X[:, 3] = X[:, 2] + d * 1.05 + rng.normal(size=(N, 3)) * 3e-5   # ~1e-2 rad: inside the mollifier band
    X0 = X.copy()
    X0[:, 1] = X0[:, 0] + (X[:, 1] - X[:, 0]) * 4
    X0[:, 3] = X0[:, 2] + (X[:, 3] - X[:, 2]) * 4
    dh2, kappa = 1e-6, 1e8
    E, gr, H = barrier_gpu(t, X, X0, dh2, kappa)
    nv = O.TYPE_NV[t]
    rows = (np.arange(N)[:, None] * 4 + np.arange(nv)[None, :]).astype(np.int32)
    Eo, go, Ho = O.barrier_rows(t, rows, X.reshape(-1, 3), X0.reshape(-1, 3), dh2, kappa)
    act = Eo != 0
    assert act.sum() > 100
    np.testing.assert_allclose(E, Eo, rtol=1e-10, atol=0)
    assert rel(gr[act], go[act]) < 1e-9
    assert rel(H[act], Ho[act]) < 1e-9


def test_elasticity_vs_oracle():
    rng = np.random.default_rng(11)
    N = 5000
    rest = rng.normal(size=(N, 4, 3)) * 0.002
    rest[:, 1:] += np.eye(3) * 0.02
    X = rest + rng.normal(size=(N, 4, 3)) * np.array([1e-4, 1e-3, 3e-3])[rng.integers(0, 3, N)][:, None, None]
    Dm = np.stack([rest[:, 1] - rest[:, 0], rest[:, 2] - rest[:, 0], rest[:, 3] - rest[:, 0]], axis=2)
    Ds = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], axis=2)
    ok = (np.linalg.det(Ds) / np.linalg.det(Dm) > 0.2) & (np.linalg.det(Dm) > 0)
    X, Dm = X[ok], Dm[ok]
    N = len(X)
    la, mu, dt = 1e6 * 0.45 / (1.45 * 0.1), 1e6 / 2.9, 0.01
    tets = np.arange(4 * N, dtype=np.int32).reshape(N, 4)
    vol = np.linalg.det(Dm) / 6
    x, t = cu(X.reshape(-1, 3)), cu(tets)
    dminv, v = cu(np.linalg.inv(Dm).reshape(N, 9)), cu(vol)
    lam, muv = cu(np.full(N, la)), cu(np.full(N, mu))
    E = torch.zeros(N, dtype=torch.float64, device='cuda')
    g = torch.zeros((N, 12), dtype=torch.float64, device='cuda')
    Hu = torch.zeros((N, 90), dtype=torch.float64, device='cuda')
    assert lib().fipc_elasticity(N, p(t), p(x), p(dminv), p(v), p(lam), p(muv), D(dt), p(E), p(g), p(Hu), stream()) == 0
    torch.cuda.synchronize()
    Eo, go, Ho = O.elasticity(tets, X.reshape(-1, 3), Dm.reshape(N, 9), np.full(N, la), np.full(N, mu), dt)
    np.testing.assert_allclose(E.cpu().numpy(), Eo, rtol=1e-10, atol=1e-12 * np.abs(Eo).max())
    assert rel(g.cpu().numpy(), go) < 1e-9
    H = np.zeros((N, 12, 12))
    hu = Hu.cpu().numpy().reshape(N, 10, 3, 3)
    b = 0
    for a in range(4):
        for c in range(a, 4):
            H[:, 3 * a:3 * a + 3, 3 * c:3 * c + 3] = hu[:, b]
            H[:, 3 * c:3 * c + 3, 3 * a:3 * a + 3] = hu[:, b].transpose(0, 2, 1)
            b += 1
    assert rel(H, Ho) < 1e-9


@pytest.mark.parametrize('kind,name', [(0, 'pt'), (1, 'ee')])
def test_ccd_pairs_golden(unit_golden, kind, name):
    g = unit_golden
    xq, pq = cu(g[f'ccd_{name}_x']), cu(g[f'ccd_{name}_p'])
    n = len(g[f'ccd_{name}_x'])
    toc = torch.zeros(n, dtype=torch.float64, device='cuda')
    assert lib().fipc_ccd_pairs(kind, n, p(xq), p(pq), D(0.2), p(toc), stream()) == 0
    torch.cuda.synchronize()
    assert np.abs(toc.cpu().numpy() - g[f'ccd_{name}_toc']).max() < 1e-6


def test_inversion_free_golden(unit_golden):
    g = unit_golden
    xs, ps = cu(g['cubic_x']), cu(g['cubic_p'])
    n = len(g['cubic_x'])
    out = torch.zeros(n, dtype=torch.float64, device='cuda')
    assert lib().fipc_inversion_free_pairs(n, p(xs), p(ps), D(0.2), p(out), stream()) == 0
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy() - g['cubic_t']).max() < 1e-6


def test_argument_errors_are_reported():
    """Invalid arguments return status 5 without launching anything."""
    assert lib().fipc_barrier_rows(9, 1, None, None, None, D(1e-6), D(1.0), None, None, None, stream()) == 5
    assert lib().fipc_ccd_pairs(3, 1, None, None, D(0.2), None, stream()) == 5
