"""The ADMM oracle's building blocks on the CPU (oracle/admm_oracle.py), pinned where the
reference itself cannot run (its ADMM script calls barrier helpers with signatures its own
library no longer has):

* the relative-coordinate barrier derivatives against central differences of the row energy,
  for every list type, near and inside d-hat, mollified rows with an active mollifier;
* the fixed-corotated sigma-space gradient and Hessian against central differences;
* the oracle's solve_N against libfastipc's host export of the same function (which itself is
  checked against the reference's a.so in test_scalar_abi.py).
"""
import ctypes

import numpy as np
import pytest

from oracle import admm_oracle as A

DH2, KAPPA = 1e-6, 1e4


def _case(rng, t):
    nv = A.TYPE_NV[t]
    pos = rng.normal(size=(nv - 1, 3)) * 4e-4
    X0 = np.zeros((4, 3))
    if t >= 4:   # nearly parallel rest edges: a small eps keeps the mollifier active
        X0 = np.array([[0, 0, 0], [1e-2, 0, 0], [0, 3e-4, 1e-4], [1e-2, 3e-4, 1.1e-4]])
    return pos.ravel(), X0


@pytest.mark.parametrize('t', range(7))
def test_relative_barrier_derivatives(t):
    rng = np.random.default_rng(30 + t)
    hit = 0
    for _ in range(20):
        pos, X0 = _case(rng, t)
        E, g, H, fro = A.rel_energy(t, pos, X0, DH2, KAPPA)
        if E == 0.0:
            continue
        hit += 1
        h = 1e-9
        for i in range(len(pos)):
            d = np.zeros_like(pos)
            d[i] = h
            Ep = A.rel_energy(t, pos + d, X0, DH2, KAPPA, False)
            Em = A.rel_energy(t, pos - d, X0, DH2, KAPPA, False)
            assert abs((Ep - Em) / (2 * h) - g[i]) <= 1e-5 * np.abs(g).max() + 1e-12
            gp = A.rel_energy(t, pos + d, X0, DH2, KAPPA)[1]
            gm = A.rel_energy(t, pos - d, X0, DH2, KAPPA)[1]
            assert np.abs((gp - gm) / (2 * h) - H[:, i]).max() <= 1e-4 * np.abs(H).max() + 1e-9
        assert np.allclose(H, H.T, rtol=0, atol=1e-9 * np.abs(H).max())
        assert fro >= np.sqrt((H * H).sum()) * (1 - 1e-12)
    assert hit >= 5


def test_fixed_corotated_sigma_derivatives():
    rng = np.random.default_rng(5)
    la, mu = 1.2e5, 3.5e4
    for _ in range(20):
        s = rng.uniform(0.6, 1.4, 3) * rng.choice([1, 1, -1], 3)
        g, H = A.fc3_grad(s, la, mu), A.fc3_hess(s, la, mu)
        h = 1e-6
        for i in range(3):
            d = np.zeros(3)
            d[i] = h
            assert abs((A.fc3_psi(s + d, la, mu) - A.fc3_psi(s - d, la, mu)) / (2 * h) - g[i]) <= 1e-6 * np.abs(g).max() + 1e-6
            assert np.abs((A.fc3_grad(s + d, la, mu) - A.fc3_grad(s - d, la, mu)) / (2 * h) - H[:, i]).max() <= 1e-5 * np.abs(H).max()


def test_solve_n_matches_the_library_export():
    from fastipc_gb300.build import LIB, build
    build()
    so = ctypes.CDLL(LIB)
    rng = np.random.default_rng(9)
    for n in (3, 6, 9):
        f = getattr(so, f'solve_{n}')
        f.argtypes = [ctypes.c_double] * (n * n + n) + [ctypes.POINTER(ctypes.c_double)] * n
        f.restype = None
        for k in range(60):
            G = rng.normal(size=(n, n))
            M = G @ G.T + (0.5 if k % 2 == 0 else -1.0) * np.eye(n)
            b = rng.normal(size=n)
            outs = [ctypes.c_double() for _ in range(n)]
            f(*M.ravel().tolist(), *b.tolist(), *[ctypes.byref(o) for o in outs])
            ref = np.array([o.value for o in outs])
            mine = A.solve_n(M, b)
            tol = 1e-10 if k % 2 == 0 else 1e-4
            assert np.abs(mine - ref).max() <= tol * np.abs(ref).max(), (n, k)
