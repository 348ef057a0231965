"""The 2D device math (fc2d.cuh), compiled for the host with g++, against the 2D oracle and
the reference's native a.so (no GPU): fixed-corotated triangles, 2D barrier rows, point-edge
CCD, point-in-triangle and the 2x2 SVD.  Bars: 1e-9 relative to the largest entry; CCD 1e-6.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from fastipc_gb300 import scenes
from oracle import oracle2d as O2

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'native', 'math2d_host.cpp')
OUT = os.path.join(HERE, 'native', '_build', 'math2d_host.so')
D = ctypes.c_double


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


def test_svd2_convention(hc):
    rng = np.random.default_rng(5)
    F = np.ascontiguousarray(rng.normal(size=(300, 2, 2)))
    U, s, V = np.zeros_like(F), np.zeros((300, 2)), np.zeros_like(F)
    hc.h2_svd2(300, P(F), P(U), P(s), P(V))
    np.testing.assert_allclose(U @ (s[:, :, None] * np.swapaxes(V, 1, 2)), F, atol=1e-14)
    _, s_o, _ = O2.svd2(F)
    np.testing.assert_allclose(s, s_o, rtol=1e-12, atol=1e-14)
    assert np.all(np.abs(np.linalg.det(U) - 1) < 1e-14) and np.all(np.abs(np.linalg.det(V) - 1) < 1e-14)


@pytest.mark.parametrize('scale', [0.02, 0.3])
def test_elements_vs_oracle(hc, scale):
    """Random deformations around rest, compressed, stretched and inverted triangles."""
    rng = np.random.default_rng(11)
    sc = scenes.two_squares_2d(n=4, seed=1, segment=False)
    sim = O2.OracleSim2D(sc)
    x = sc.x + rng.normal(size=sc.x.shape) * scale * 0.025
    T = len(sc.tris)
    E_o, g_o, H_o = O2.elements(sim.tris, x, sim.IB, sim.vol, sim.la, sim.mu, sc.dt)
    X = np.ascontiguousarray(x[sc.tris])
    IB = np.ascontiguousarray(sim.IB.reshape(T, 4))
    w = np.ascontiguousarray(sc.dt ** 2 * sim.vol)
    E, g, H = np.zeros(T), np.zeros((T, 6)), np.zeros((T, 36))
    hc.h2_elements(T, P(X), P(IB), P(np.ascontiguousarray(sim.la)), P(np.ascontiguousarray(sim.mu)), P(w), P(E), P(g), P(H))
    # H [T][a*3+b][d*2+e] -> full [T][2a+d][2b+e]
    Hf = H.reshape(T, 3, 3, 2, 2).transpose(0, 1, 3, 2, 4).reshape(T, 6, 6)
    np.testing.assert_allclose(E, E_o, rtol=1e-10, atol=1e-14 * np.abs(E_o).max())
    assert rel(g, g_o) < 1e-9
    assert rel(Hf, H_o) < 1e-9
    if scale > 0.1:
        Xe = x[sc.tris]
        det = (Xe[:, 1, 0] - Xe[:, 0, 0]) * (Xe[:, 2, 1] - Xe[:, 0, 1]) - (Xe[:, 2, 0] - Xe[:, 0, 0]) * (Xe[:, 1, 1] - Xe[:, 0, 1])
        assert (det < 0).any()        # inverted triangles are covered


@pytest.mark.parametrize('t', [0, 1])
def test_barrier_vs_oracle(hc, t):
    rng = np.random.default_rng(7 + t)
    N, nv, dh2, kappa = 400, 2 + t, 1e-6, 1.3e9
    X = np.zeros((N, 3, 2))
    X[:, 0] = rng.uniform(-1, 1, (N, 2))
    X[:, 1:nv] = X[:, :1] + rng.normal(size=(N, nv - 1, 2)) * (4e-4 if t == 0 else 2e-3)
    if t == 1:      # a point close to the edge's interior
        u = rng.uniform(0.1, 0.9, N)[:, None]
        nrm = np.stack([-(X[:, 2, 1] - X[:, 1, 1]), X[:, 2, 0] - X[:, 1, 0]], 1)
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        X[:, 0] = X[:, 1] + u * (X[:, 2] - X[:, 1]) + nrm * rng.uniform(1e-5, 9e-4, N)[:, None]
    X = np.ascontiguousarray(X)
    E, g, H = np.zeros(N), np.zeros((N, 6)), np.zeros((N, 36))
    hc.h2_barrier(t, N, P(X), D(dh2), D(kappa), P(E), P(g), P(H))
    rows = np.arange(N * 3).reshape(N, 3)[:, :nv]
    E_o, g_o, H_o = O2.barrier_rows(t, rows, X.reshape(-1, 2), dh2, kappa)
    n = 2 * nv
    Hf = H[:, :4 * nv * nv].reshape(N, nv, nv, 2, 2).transpose(0, 1, 3, 2, 4).reshape(N, n, n)
    live = E_o > 0
    assert live.sum() > N // 4
    np.testing.assert_allclose(E, E_o, rtol=1e-10, atol=0)
    assert rel(g[live, :n], g_o[live]) < 1e-9
    assert rel(Hf[live], H_o[live]) < 1e-9


def test_ccd_vs_oracle(hc):
    rng = np.random.default_rng(3)
    N = 3000
    xq = rng.uniform(-1, 1, (N, 3, 2)) * 0.01
    pq = rng.normal(size=(N, 3, 2)) * 0.01
    # special cases: collinear motion along the edge line, parallel edge, zero motion
    xq[:10] = [[0.5, 0.0], [0.0, 0.0], [1.0, 0.0]]
    pq[:10] = [[-0.6, 0.0], [0.0, 0.0], [0.0, 0.0]]
    pq[10:20] = 0.0
    xq[20:30] = [[0.2, 0.5], [0.0, 0.0], [1.0, 0.0]]
    pq[20:30] = [[0.0, -1.0], [0.0, 0.0], [0.0, 0.0]]
    xq, pq = np.ascontiguousarray(xq), np.ascontiguousarray(pq)
    toc = np.zeros(N)
    hc.h2_ccd(N, P(xq), P(pq), D(0.2), P(toc))
    ref = np.array([O2.point_edge_ccd(xq[i, 0], xq[i, 1], xq[i, 2], pq[i, 0], pq[i, 1], pq[i, 2], 0.2) for i in range(N)])
    np.testing.assert_allclose(toc, ref, atol=1e-12, rtol=1e-12)
    assert (ref < 1).sum() > 100
    np.testing.assert_allclose(toc[20], 0.5 * 0.8, rtol=1e-14)


def test_point_in_triangle(hc):
    rng = np.random.default_rng(9)
    N = 2000
    pts = np.ascontiguousarray(rng.uniform(-1, 1, (N, 4, 2)))
    pts[:5] = [[0.0, 0.0], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]      # on a vertex: inside
    out = np.zeros(N, np.int32)
    hc.h2_in_tri(N, P(pts), P(out))
    x = pts.reshape(-1, 2)
    tris = np.arange(4 * N).reshape(N, 4)[:, 1:]
    ref = np.array([O2.check_collision(x, np.array([4 * i]), tris[i:i + 1] * 0 + np.array([[4 * i + 1, 4 * i + 2, 4 * i + 3]]))
                    for i in range(N)])
    np.testing.assert_array_equal(out.astype(bool), ref)
    assert out[:5].all() and 0 < out.sum() < N
