"""The CPU oracle against golden vectors from the reference's own code (no GPU).

The fixtures come from tests/golden/gen_golden.py: the reference's Python kernels run through
a numpy Taichi stand-in, and its native a.so built from source.  Tolerances: distances,
barrier and Neo-Hookean quantities 1e-9 relative to the largest entry of each array;
types and constraint sets exact; CCD time of impact 1e-6 absolute.
"""
import numpy as np
import pytest

from oracle import oracle as O


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = np.maximum(np.abs(b).reshape(len(b), -1).max(axis=1), 1e-300)
    return (np.abs(a - b).reshape(len(b), -1).max(axis=1) / scale).max()


@pytest.mark.parametrize('kind,name', [(0, 'PP_3D'), (1, 'PE_3D'), (2, 'PT_3D'), (3, 'EE_3D'), (4, 'EECN2')])
def test_distance_derivatives(unit_golden, kind, name):
    g = unit_golden
    E, gr, H = O.distance(kind, g['dist_pts'])
    assert rel(E[:, None], g[f'{name}_E'][:, None]) < 1e-10
    assert rel(gr, g[f'{name}_g']) < 1e-9
    assert rel(H, g[f'{name}_H']) < 1e-9


def test_types(unit_golden):
    g = unit_golden
    pt, ee, pe = O.types(g['type_pts'])
    np.testing.assert_array_equal(pt, g['PT_type'])
    np.testing.assert_array_equal(ee, g['EE_type'])
    np.testing.assert_array_equal(pe, g['PE_type'])


def test_barrier_scalar(unit_golden):
    g = unit_golden
    E, gg, H = O.barrier_scalar(g['barrier_d'], float(g['barrier_dhat2']), 1.0)
    np.testing.assert_allclose(E, g['barrier_E'], rtol=1e-12, atol=0)
    np.testing.assert_allclose(gg, g['barrier_g'], rtol=1e-12, atol=0)
    np.testing.assert_allclose(H, g['barrier_H'], rtol=1e-12, atol=0)


def test_mollifier(unit_golden):
    g = unit_golden
    E, gr, H = O.mollifier(g['moll_pts'], g['moll_eps'])
    np.testing.assert_allclose(E, g['M_E'], rtol=1e-10)
    assert rel(gr, g['M_g']) < 1e-9
    assert rel(H, g['M_H']) < 1e-9


@pytest.mark.parametrize('t', range(7))
def test_barrier_rows(unit_golden, t):
    g = unit_golden
    name = O.TYPES[t]
    X, X0 = g[f'bar_{name}_x'], g[f'bar_{name}_x0']
    nv = O.TYPE_NV[t] if t < 4 else 4
    N = len(X)
    x = X.reshape(-1, 3)
    x0 = X0.reshape(-1, 3)
    rows = (np.arange(N)[:, None] * 4 + np.arange(nv)[None, :]).astype(np.int32)
    kappa, dh2 = float(g['bar_kappa']), float(g['bar_dhat2'])
    E, gr, H = O.barrier_rows(t, rows, x, x0, dh2, kappa)
    np.testing.assert_allclose(E, g[f'bar_{name}_E'], rtol=1e-10)
    assert rel(gr, g[f'bar_{name}_g']) < 1e-9
    assert rel(H, g[f'bar_{name}_H']) < 1e-9


@pytest.mark.parametrize('n', [3, 6, 9, 12])
def test_project_pd(unit_golden, n):
    g = unit_golden
    out = O.project_pd(g[f'ppd{n}_in'])
    assert rel(out, g[f'ppd{n}_out']) < 1e-10


def test_make_pd2(unit_golden):
    g = unit_golden
    out = O.make_pd2(g['mpd_in'])
    assert rel(out, g['mpd_out']) < 1e-12


def test_svd3(unit_golden):
    g = unit_golden
    F = g['svd_in']
    U, s, V = O.svd3(F)
    ref_s = np.abs(g['svd_out'][:, 9:18].reshape(-1, 3, 3)[:, [0, 1, 2], [0, 1, 2]])
    np.testing.assert_allclose(np.sort(np.abs(s), axis=1), np.sort(ref_s, axis=1), rtol=1e-10, atol=1e-13)
    rec = np.einsum('nij,nj,nkj->nik', U, s, V)
    np.testing.assert_allclose(rec, F, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(U), 1.0, atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(V), 1.0, atol=1e-12)


def test_neo_hookean(unit_golden):
    g = unit_golden
    psi, P, dP = O.nh_material(g['nh_F'], float(g['nh_la']), float(g['nh_mu']))
    np.testing.assert_allclose(psi, g['nh_energy'], rtol=1e-9, atol=1e-9 * np.abs(g['nh_energy']).max())
    assert rel(P, g['nh_P']) < 1e-10
    assert rel(dP, g['nh_dPdF']) < 1e-9


def test_inversion_free_cubic(unit_golden):
    g = unit_golden
    t = O.inversion_free(g['cubic_x'], g['cubic_p'])
    # Cardano with complex cube roots is ill-conditioned near repeated roots; the CCD bar is 1e-6
    assert np.abs(t - g["cubic_t"]).max() < 1e-6


@pytest.mark.parametrize('kind,name', [(0, 'pt'), (1, 'ee')])
def test_ccd(unit_golden, kind, name):
    g = unit_golden
    toc = O.ccd(kind, g[f'ccd_{name}_x'], g[f'ccd_{name}_p'])
    ref = g[f'ccd_{name}_toc']
    assert np.abs(toc - ref).max() < 1e-6, np.abs(toc - ref).max()


def test_segment_triangle(unit_golden):
    g = unit_golden
    np.testing.assert_array_equal(O.seg_tri(g['seg_pts']), g['seg_hit'])
