"""The multigrid preconditioner's set-up (fastipc_gb300/csrc/mg_plan.h: box aggregation per body,
coarse patterns, Galerkin contribution lists, contact patterns per level), driven by a host
restatement of the V-cycle and of CG (tests/native/mg_host.cpp) with the GPU kernels' algebra
(rigid-mode prolongation, damped block-Jacobi smoothing with power-iteration weights, dense
coarsest inverse).  No GPU.

On Newton matrices the oracle assembles (a short twisted bar, a cube lattice on its ground,
with random SPD couplings between random vertex pairs passed as contact blocks, and random
extra Dirichlet vertices): the solution equals scipy's sparse LU to 1e-8 of its largest entry
at relative residual 1e-10, Dirichlet entries are exactly 0, and CG needs fewer than a third of
the iterations block-Jacobi CG needs.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from fastipc_gb300 import scenes
from test_mf_host import _bsr, _contact, _reference, _system

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'native', 'mg_host.cpp')
OUT = os.path.join(HERE, 'native', '_build', 'mg_host.so')


@pytest.fixture(scope='module')
def mg():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + f'.{os.getpid()}'
    subprocess.check_call(['g++', '-O2', '-std=c++17', '-fPIC', '-shared', SRC, '-o', tmp])
    os.replace(tmp, OUT)
    return ctypes.CDLL(OUT)


def P(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _block_jacobi_iterations(A, b, mask, rtol):
    D = np.repeat(mask, 3)
    A = A.tocoo()
    keep = ~(D[A.row] | D[A.col])
    n = A.shape[0]
    idx = np.where(D)[0]
    M = sp.csr_matrix((np.concatenate([A.data[keep], np.ones(len(idx))]),
                       (np.concatenate([A.row[keep], idx]), np.concatenate([A.col[keep], idx]))), shape=(n, n))
    bb = b.copy()
    bb[D] = 0
    Bm = sp.bsr_matrix(M, blocksize=(3, 3))
    diag = np.zeros((n // 3, 3, 3))
    for i in range(n // 3):
        for k in range(Bm.indptr[i], Bm.indptr[i + 1]):
            if Bm.indices[k] == i:
                diag[i] = Bm.data[k]
    inv = np.linalg.inv(diag)
    it = [0]

    def cb(_):
        it[0] += 1
    spla.cg(M, bb, rtol=rtol, maxiter=20000, M=spla.LinearOperator((n, n), matvec=lambda r: np.einsum('kij,kj->ki', inv, r.reshape(-1, 3)).ravel()),
            callback=cb)
    return it[0]


CASES = {
    'bar': (lambda: scenes.twisted_bar(nx=40, ny=4, nz=4, size=(0.4, 0.04, 0.04), seed=0), 0.01),
    'lattice': (lambda: scenes.predeform(scenes.cube_lattice(m=2, n=3, seed=0), 1e-4, 0), 0.1 / 3),
}


@pytest.mark.parametrize('name', sorted(CASES))
def test_multigrid_cg_vs_sparse_lu(mg, name):
    make, h = CASES[name]
    scene = make()
    A, rhs, mask, x = _system(scene)
    rng = np.random.default_rng(3)
    nV = len(x)
    Ac = _contact(nV, x, rng, max(4, nV // 20))
    mask = mask.copy()
    mask[rng.choice(nV, max(1, nV // 50), replace=False)] = True
    rp, ci, ev = _bsr(A)
    crp, cci, cv = _bsr(Ac)
    fixed = np.ascontiguousarray(mask.astype(np.uint8))
    x0 = np.ascontiguousarray(scene.x, dtype=np.float64)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    b = np.ascontiguousarray(rhs, dtype=np.float64)
    info = np.zeros(1 + 2 * 8)
    mg.mg_host_plan(nV, P(x0), P(rp), P(ci), ctypes.c_double(h), P(info))
    assert info[0] >= 2, 'no coarse level'
    sol = np.zeros(3 * nV)
    om = np.zeros(8)
    it = mg.mg_host_pcg(nV, P(rp), P(ci), P(ev), P(crp), P(cci), P(cv), P(fixed), P(xx), P(x0), ctypes.c_double(h), P(b),
                        ctypes.c_double(1e-10), 4000, P(sol), P(om))
    assert it > 0
    ref = _reference(A + Ac, rhs, mask)
    assert np.abs(sol - ref).max() <= 1e-8 * np.abs(ref).max()
    assert np.all(sol.reshape(-1, 3)[mask] == 0.0)
    assert np.all((om[:int(info[0]) - 1] > 0.1) & (om[:int(info[0]) - 1] < 1.0))
    bj = _block_jacobi_iterations(A + Ac, rhs, mask, 1e-10)
    assert it * 3 < bj, (it, bj)


def test_aggregates_stay_inside_bodies(mg):
    """The lattice's cubes are separate components: with no contact pattern the level-1 static
    pattern couples no two aggregates of different cubes, so its blocks per row stay at most
    the box neighbourhood of one body."""
    scene = scenes.cube_lattice(m=2, n=3, seed=0)
    A, rhs, mask, x = _system(scene)
    rp, ci, _ = _bsr(A)
    info = np.zeros(1 + 2 * 8)
    x0 = np.ascontiguousarray(scene.x, dtype=np.float64)
    mg.mg_host_plan(len(x0), P(x0), P(rp), P(ci), ctypes.c_double(0.1 / 3), P(info))
    n1, nnz1 = int(info[2]), int(info[1 + 8 + 1])
    cubes = 8 + 1
    assert n1 >= cubes            # at least one aggregate per body
    assert nnz1 <= 27 * n1        # a box neighbourhood per row


def test_line_aggregates_keep_translations_only(mg):
    """Level-1 aggregates of one or two vertices, or of collinear vertices, have a rank-deficient
    rotation block (the rotation about their line moves nothing): the plan keeps their
    translations only.  Every other aggregate keeps its rotations; on the two-cube scene, whose
    box grid leaves single vertices and vertex pairs at the cubes' edges, both kinds occur."""
    scene = scenes.predeform(scenes.two_cubes(n=8, seed=1), 2e-4, 1)
    A, rhs, mask, x = _system(scene)
    rp, ci, _ = _bsr(A)
    x0 = np.ascontiguousarray(scene.x, dtype=np.float64)
    be = scene.boundary_edges
    h = float(np.median(np.linalg.norm(x0[be[:, 0]] - x0[be[:, 1]], axis=1)))
    rot = np.zeros(len(x0), np.int32)
    mem = np.zeros(len(x0), np.int32)
    n = mg.mg_host_level1(len(x0), P(x0), P(rp), P(ci), ctypes.c_double(h), P(rot), P(mem))
    rot, mem = rot[:n], mem[:n]
    assert n > 0
    assert np.all(rot[mem <= 2] == 0)
    assert np.all(mem[rot == 0] <= 9)          # only thin slivers lose their rotations
    assert (rot == 1).sum() > 0.8 * n
