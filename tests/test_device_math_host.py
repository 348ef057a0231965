"""The GPU kernels' math headers, compiled for the host with g++, against the oracle and the
reference's golden vectors (no GPU).  This checks the product's formulas (reduced-coordinate
barrier derivatives and projection, Neo-Hookean mode assembly, CTCD) before any device run.
Tolerances as in test_oracle_golden: 1e-9 relative to the largest entry; CCD 1e-6.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'native', 'math_host.cpp')
OUT = os.path.join(HERE, 'native', '_build', 'math_host.so')


@pytest.fixture(scope='module')
def hc():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + f'.{os.getpid()}'
    subprocess.check_call(['g++', '-O2', '-std=c++17', '-ffp-contract=off', '-fPIC', '-shared', SRC, '-o', tmp])
    os.replace(tmp, OUT)
    return ctypes.CDLL(OUT)


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = np.maximum(np.abs(b).reshape(len(b), -1).max(axis=1), 1e-300)
    return (np.abs(a - b).reshape(len(b), -1).max(axis=1) / scale).max()


@pytest.mark.parametrize('t', range(7))
def test_barrier_rows_vs_golden(hc, unit_golden, t):
    g = unit_golden
    name = O.TYPES[t]
    X, X0 = g[f'bar_{name}_x'], g[f'bar_{name}_x0']
    N = len(X)
    nv = O.TYPE_NV[t]
    rows = np.ascontiguousarray((np.arange(N)[:, None] * 4 + np.arange(4)[None, :]).astype(np.int32))
    x = np.ascontiguousarray(X.reshape(-1, 3))
    x0 = np.ascontiguousarray(X0.reshape(-1, 3))
    E, gr, H = np.zeros(N), np.zeros((N, 12)), np.zeros((N, 144))
    hc.hc_barrier_rows(t, N, P(rows), P(x), P(x0), ctypes.c_double(float(g['bar_dhat2'])),
                       ctypes.c_double(float(g['bar_kappa'])), P(E), P(gr), P(H))
    n = 3 * nv
    np.testing.assert_allclose(E, g[f'bar_{name}_E'], rtol=1e-10)
    assert rel(gr[:, :n], g[f'bar_{name}_g']) < 1e-9
    assert rel(H[:, :n * n].reshape(N, n, n), g[f'bar_{name}_H']) < 1e-9


@pytest.mark.parametrize('t', range(7))
def test_barrier_rows_vs_oracle_random(hc, t):
    """Random contact-scale rows, including configurations with strongly indefinite Hessians."""
    rng = np.random.default_rng(100 + t)
    N = 200
    base = rng.uniform(-1, 1, (N, 1, 3))
    X = base + rng.normal(size=(N, 4, 3)) * 4e-4
    if t >= 4:
        d = rng.normal(size=(N, 3)) * 3e-3
        X[:, 1] = X[:, 0] + d
        X[:, 3] = X[:, 2] + d * 1.05 + rng.normal(size=(N, 3)) * 3e-5   # ~1e-2 rad: inside the mollifier band
    X0 = X.copy()
    X0[:, 1] = X0[:, 0] + (X[:, 1] - X[:, 0]) * 4
    X0[:, 3] = X0[:, 2] + (X[:, 3] - X[:, 2]) * 4
    x = np.ascontiguousarray(X.reshape(-1, 3))
    x0 = np.ascontiguousarray(X0.reshape(-1, 3))
    rows = np.ascontiguousarray((np.arange(N)[:, None] * 4 + np.arange(4)[None, :]).astype(np.int32))
    dh2, kappa = 1e-6, 1e8
    E, gr, H = np.zeros(N), np.zeros((N, 12)), np.zeros((N, 144))
    hc.hc_barrier_rows(t, N, P(rows), P(x), P(x0), ctypes.c_double(dh2), ctypes.c_double(kappa), P(E), P(gr), P(H))
    nv = O.TYPE_NV[t]
    Eo, go, Ho = O.barrier_rows(t, rows[:, :nv], x, x0, dh2, kappa)
    n = 3 * nv
    active = Eo != 0
    assert active.sum() > 10
    np.testing.assert_allclose(E, Eo, rtol=1e-10, atol=0)
    assert rel(gr[active, :n], go[active]) < 1e-9
    assert rel(H[active, :n * n].reshape(-1, n, n), Ho[active]) < 1e-9


def test_sym_eig(hc):
    rng = np.random.default_rng(7)
    for n in (2, 3, 6, 9):
        A = rng.normal(size=(50, n, n))
        A = np.ascontiguousarray((A + A.transpose(0, 2, 1)) / 2)
        w, V = np.zeros((50, n)), np.zeros((50, n, n))
        hc.hc_sym_eig(50, n, P(A), P(w), P(V))
        np.testing.assert_allclose(w, np.linalg.eigvalsh(A), atol=1e-12)
        rec = np.einsum('bij,bj,bkj->bik', V, w, V)
        np.testing.assert_allclose(rec, A, atol=1e-12)


def test_svd3(hc, unit_golden):
    F = np.ascontiguousarray(unit_golden['svd_in'])
    N = len(F)
    U, s, V = np.zeros((N, 3, 3)), np.zeros((N, 3)), np.zeros((N, 3, 3))
    hc.hc_svd3(N, P(F), P(U), P(s), P(V))
    np.testing.assert_allclose(np.einsum('nij,nj,nkj->nik', U, s, V), F, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(U), 1, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(V), 1, atol=1e-12)
    np.testing.assert_allclose(np.abs(s), np.sort(np.linalg.svd(F, compute_uv=False), axis=1)[:, ::-1], rtol=1e-12, atol=1e-14)


def test_nh_element_vs_oracle(hc):
    rng = np.random.default_rng(3)
    N = 300
    rest = rng.normal(size=(N, 4, 3)) * 0.002
    rest[:, 1:] += np.eye(3) * 0.02
    X = rest + rng.normal(size=(N, 4, 3)) * np.array([1e-4, 1e-3, 4e-3])[rng.integers(0, 3, N)][:, None, None]
    Dm = np.stack([rest[:, 1] - rest[:, 0], rest[:, 2] - rest[:, 0], rest[:, 3] - rest[:, 0]], axis=2)
    Ds = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], axis=2)
    ok = (np.linalg.det(Ds) / np.linalg.det(Dm) > 0.2) & (np.linalg.det(Dm) > 0)
    rest, X, Dm = rest[ok], X[ok], Dm[ok]
    N = len(X)
    IB = np.ascontiguousarray(np.linalg.inv(Dm).reshape(N, 9))
    la, mu, dt = 1e6 * 0.45 / (1.45 * 0.1), 1e6 / 2.9, 0.01
    vol = np.linalg.det(Dm) / 6
    E, g, H = np.zeros(N), np.zeros((N, 12)), np.zeros((N, 144))
    Xc = np.ascontiguousarray(X.reshape(N, 12))
    for i in range(N):   # per-element weight dt^2 vol0
        hc.hc_nh_element(1, P(Xc[i:i + 1].copy()), P(IB[i:i + 1].copy()), ctypes.c_double(la), ctypes.c_double(mu),
                         ctypes.c_double(dt * dt * vol[i]), P(E[i:]), P(g[i:]), P(H[i:]))
    tets = np.arange(4 * N, dtype=np.int32).reshape(N, 4)
    Eo, go, Ho = O.elasticity(tets, X.reshape(-1, 3), Dm.reshape(N, 9), np.full(N, la), np.full(N, mu), dt)
    np.testing.assert_allclose(E, Eo, rtol=1e-10, atol=1e-12 * np.abs(Eo).max())
    assert rel(g, go) < 1e-9
    assert rel(H.reshape(N, 12, 12), Ho) < 1e-9


@pytest.mark.parametrize('kind,name', [(0, 'pt'), (1, 'ee')])
def test_ccd_vs_golden(hc, unit_golden, kind, name):
    g = unit_golden
    x, p = np.ascontiguousarray(g[f'ccd_{name}_x']), np.ascontiguousarray(g[f'ccd_{name}_p'])
    toc = np.zeros(len(x))
    hc.hc_ccd(kind, len(x), P(x), P(p), ctypes.c_double(0.2), P(toc))
    assert np.abs(toc - g[f'ccd_{name}_toc']).max() < 1e-6


def test_types_and_segments(hc, unit_golden):
    g = unit_golden
    pts = np.ascontiguousarray(g['type_pts'])
    pt, ee = np.zeros(len(pts), np.int32), np.zeros(len(pts), np.int32)
    hc.hc_types(len(pts), P(pts), P(pt), P(ee))
    np.testing.assert_array_equal(pt, g['PT_type'])
    np.testing.assert_array_equal(ee, g['EE_type'])
    seg = np.ascontiguousarray(g['seg_pts'])
    hit = np.zeros(len(seg), np.int32)
    hc.hc_seg_tri(len(seg), P(seg), P(hit))
    np.testing.assert_array_equal(hit.astype(bool), g['seg_hit'])


def test_inversion_free(hc, unit_golden):
    g = unit_golden
    xs, ps = np.ascontiguousarray(g['cubic_x']), np.ascontiguousarray(g['cubic_p'])
    out = np.zeros(len(xs))
    hc.hc_inversion(len(xs), P(xs), P(ps), ctypes.c_double(0.2), P(out))
    assert np.abs(out - g['cubic_t']).max() < 1e-6


@pytest.mark.parametrize('eta', [0.1, 0.2])
def test_inversion_early_out_is_exact(hc, unit_golden, eta):
    """A tet whose volume polynomial provably stays positive over the step's range is skipped:
    every skipped tet's inversion-free step is >= 1 (golden cases and 40k random tets with
    vertex motions from 1e-4 to 3 of the tet's size)."""
    g = unit_golden
    rng = np.random.default_rng(5)
    n = 40000
    X = rng.normal(size=(n, 4, 3))
    vol = np.einsum('ij,ij->i', np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), X[:, 3] - X[:, 0])
    X[vol < 0, 3] = 2 * X[vol < 0, 0] - X[vol < 0, 3]      # positive orientation
    rs = 10.0 ** rng.uniform(-4, 0.5, size=n)
    Pm = rng.normal(size=(n, 4, 3)) * rs[:, None, None] + rng.normal(size=(n, 1, 3))
    xs = np.ascontiguousarray(np.concatenate([np.reshape(g['cubic_x'], (-1, 12)), X.reshape(n, 12)]))
    ps = np.ascontiguousarray(np.concatenate([np.reshape(g['cubic_p'], (-1, 12)), Pm.reshape(n, 12)]))
    out = np.zeros(len(xs))
    skip = np.zeros(len(xs), np.int32)
    hc.hc_inversion(len(xs), P(xs), P(ps), ctypes.c_double(eta), P(out))
    hc.hc_inversion_skip(len(xs), P(xs), P(ps), ctypes.c_double(eta), P(skip))
    s = skip.astype(bool)
    assert np.all(out[s] >= 1.0)
    small = np.concatenate([np.zeros(len(xs) - n, bool), rs < 1e-2])
    assert s[small].mean() > 0.5
    assert (out[~s] < 1.0).any()
