"""The multifrontal direct solve's analysis (fastipc_gb300/csrc/mf_plan.h: nested-dissection
ordering, assembly tree, front structures, extend-add maps, scatter destinations and the panel
task tables), driven by a host restatement of the numeric phase (tests/native/mf_host.cpp) that
runs the same tasks in the GPU's launch order.  No GPU: the solutions are compared with scipy's
sparse LU on the same Dirichlet-edited systems, to 1e-10 relative to the largest entry.

Systems: the Newton matrices the oracle assembles for small scenes (a cube pair, a short
twisted bar, a 2x2 cube lattice with its ground), with an extra "contact" pattern of random SPD
couplings between random vertex pairs passed as the second block matrix, as the context's
contact blocks are; Dirichlet masks from the scenes plus random extra fixed vertices.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from fastipc_gb300 import scenes
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'native', 'mf_host.cpp')
OUT = os.path.join(HERE, 'native', '_build', 'mf_host.so')


@pytest.fixture(scope='module')
def mf():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + f'.{os.getpid()}'
    subprocess.check_call(['g++', '-O2', '-std=c++17', '-fPIC', '-shared', SRC, '-o', tmp])
    os.replace(tmp, OUT)
    return ctypes.CDLL(OUT)


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _bsr(A):
    B = sp.bsr_matrix(A, blocksize=(3, 3))
    B.sort_indices()
    return (np.ascontiguousarray(B.indptr, np.int32), np.ascontiguousarray(B.indices, np.int32),
            np.ascontiguousarray(B.data.reshape(-1, 9)))


def _contact(nV, x, rng, n_pairs):
    """Random SPD couplings between vertex pairs: k (e e^T) on [[I, -I], [-I, I]] blocks."""
    rows, cols, vals = [], [], []
    for _ in range(n_pairs):
        a, b = rng.choice(nV, 2, replace=False)
        e = rng.normal(size=3)
        K = np.outer(e, e) + 0.1 * np.eye(3)
        for (i, j, s) in ((a, a, 1), (b, b, 1), (a, b, -1), (b, a, -1)):
            for r in range(3):
                for c in range(3):
                    rows.append(3 * i + r)
                    cols.append(3 * j + c)
                    vals.append(s * K[r, c])
    return sp.csr_matrix((vals, (rows, cols)), shape=(3 * nV, 3 * nV))


def _system(scene, steps=0):
    o = O.OracleSim(scene, solver='direct')
    for f in range(steps):
        o.step(f)
    o.compute_xn_and_xTilde()
    o.move_nodes(steps * o.dt)
    o.find_constraints()
    A, rhs = o.compute_hessian_and_gradient()
    mask, _ = scene.dirichlet(steps * o.dt)
    return A.tocsr(), rhs, mask.astype(bool), o.x.copy()


def _reference(A, rhs, mask):
    D = np.repeat(mask, 3)
    A = A.tocoo()
    keep = ~(D[A.row] | D[A.col])
    n = A.shape[0]
    idx = np.where(D)[0]
    M = sp.csr_matrix((np.concatenate([A.data[keep], np.ones(len(idx))]),
                       (np.concatenate([A.row[keep], idx]), np.concatenate([A.col[keep], idx]))), shape=(n, n))
    b = rhs.copy()
    b[D] = 0
    return spla.spsolve(M.tocsc(), b)


def _solve(mf, Ae, Ac, rhs, mask, x):
    nV = len(x)
    rp, ci, ev = _bsr(Ae)
    if Ac is None:
        crp = cci = cv = None
    else:
        crp, cci, cv = _bsr(Ac)
    fixed = np.ascontiguousarray(mask.astype(np.uint8))
    sol = np.zeros(3 * nV)
    info = np.zeros(5)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    b = np.ascontiguousarray(rhs, dtype=np.float64)
    st = mf.mf_host_solve(nV, P(rp), P(ci), P(ev), P(crp) if crp is not None else None, P(cci) if cci is not None else None,
                          P(cv) if cv is not None else None, P(fixed), P(xx), P(b), P(sol), P(info))
    return st, sol, info


CASES = {
    'cubes': lambda: scenes.predeform(scenes.two_cubes(n=3, seed=1), 3e-4, 1),
    'bar': lambda: scenes.twisted_bar(nx=24, ny=3, nz=3, size=(0.24, 0.03, 0.03), seed=0),
    'lattice': lambda: scenes.predeform(scenes.cube_lattice(m=2, n=3, seed=0), 1e-4, 0),
}


@pytest.mark.parametrize('name', sorted(CASES))
def test_direct_solve_plan_vs_sparse_lu(mf, name):
    scene = CASES[name]()
    A, rhs, mask, x = _system(scene)
    rng = np.random.default_rng(7)
    nV = len(x)
    Ac = _contact(nV, x, rng, max(4, nV // 20))
    mask = mask.copy()
    mask[rng.choice(nV, max(1, nV // 50), replace=False)] = True
    st, sol, info = _solve(mf, A, Ac, rhs, mask, x)
    assert st == 0
    ref = _reference(A + Ac, rhs, mask)
    assert np.abs(sol - ref).max() <= 1e-10 * np.abs(ref).max()
    assert np.all(sol.reshape(-1, 3)[mask] == 0.0)
    assert info[0] > 1 and info[3] >= 1     # a real tree, not one dense front


def test_direct_solve_without_contact_pattern(mf):
    A, rhs, mask, x = _system(CASES['cubes']())
    st, sol, _ = _solve(mf, A, None, rhs, mask, x)
    assert st == 0
    ref = _reference(A, rhs, mask)
    assert np.abs(sol - ref).max() <= 1e-10 * np.abs(ref).max()


def test_direct_solve_reports_an_indefinite_matrix(mf):
    A, rhs, mask, x = _system(CASES['cubes']())
    A = A - 1e3 * sp.identity(A.shape[0], format='csr') * abs(A.diagonal()).max()
    st, _, _ = _solve(mf, A, None, rhs, mask, x)
    assert st == 2


def test_direct_solve_all_fixed(mf):
    A, rhs, mask, x = _system(CASES['cubes']())
    st, sol, info = _solve(mf, A, None, rhs, np.ones(len(x), bool), x)
    assert st == 0 and info[0] == 0
    assert np.all(sol == 0.0)
