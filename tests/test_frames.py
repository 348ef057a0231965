"""Per-frame output, restart files and the Dirichlet schedule as rigid motions, on the CPU.

* fipc_write_obj against the reference's own write loop (NEWTON_IPC.py:926-931, restated
  below in Python): byte-identical text, including negative zero, rounding ties, tiny and huge
  magnitudes and a mesh large enough to be formatted in several chunks.
* caches/%06d.p: the pickle the reference writes (NEWTON_IPC.py:1002) and reads back
  (:951-953).
* FrameWriter on host arrays: the same files as direct writes; a write error surfaces.
* The rigid-motion form of each scene's Dirichlet schedule (what fipc_dirichlet_script
  evaluates, restated in numpy here) against the scene's per-vertex loop in the form of
  reader.py:170-185.
"""
import os
import pickle

import numpy as np
import pytest

from fastipc_gb300 import frames, scenes
from fastipc_gb300._native import FastIPCError
from fastipc_gb300.build import build


@pytest.fixture(scope='module', autouse=True)
def _lib():
    build()


def reference_obj_text(x, tris):
    # NEWTON_IPC.py:926-931, statement for statement
    out = []
    for i in range(len(x)):
        out.append('v %.6f %.6f %.6f\n' % (x[i, 0], x[i, 1], x[i, 2]))
    for [p0, p1, p2] in tris:
        out.append('f %d %d %d\n' % (p0 + 1, p1 + 1, p2 + 1))
    return ''.join(out).encode()


def edge_values():
    v = [0.0, -0.0, 5e-7, -5e-7, 2.5e-7, 1.5e-6, 0.0000005, 0.1234565, -0.1234565, 1e-300, -1e-300, 123456.7890125,
         1e15 + 0.5, -2.0 ** 60, 1e300, -1e300, 0.9999995, 9.9999995, np.nextafter(0.5, 1), np.nextafter(-0.5, 0)]
    return np.array(v, dtype=np.float64)


def test_obj_bytes_match_reference_writer(tmp_path):
    rng = np.random.default_rng(3)
    scale = 10.0 ** rng.integers(-9, 13, size=(60000, 1))
    x = rng.normal(size=(60000, 3)) * scale
    ev = edge_values()
    x[:len(ev), 0] = ev
    x[:len(ev), 1] = ev[::-1]
    x[:len(ev), 2] = -ev
    tris = rng.integers(0, len(x), size=(30000, 3)).astype(np.int32)
    path = str(tmp_path / 'a.obj')
    frames.write_obj(path, x, tris)
    assert open(path, 'rb').read() == reference_obj_text(x, tris)


def test_obj_small_and_empty(tmp_path):
    sc = scenes.two_cubes(n=2, seed=1)
    path = str(tmp_path / 'b.obj')
    frames.write_obj(path, sc.x, sc.boundary_triangles)
    assert open(path, 'rb').read() == reference_obj_text(sc.x, sc.boundary_triangles)
    frames.write_obj(path, np.zeros((0, 3)), np.zeros((0, 3), np.int32))
    assert open(path, 'rb').read() == b''


def test_obj_io_error_is_reported(tmp_path):
    with pytest.raises(FastIPCError) as e:
        frames.write_obj(str(tmp_path / 'missing' / 'c.obj'), np.zeros((1, 3)), np.zeros((0, 3), np.int32))
    assert e.value.status == 6


def test_cache_is_the_reference_pickle(tmp_path):
    rng = np.random.default_rng(0)
    x, v = rng.normal(size=(17, 3)), rng.normal(size=(17, 3))
    path = str(tmp_path / '000003.p')
    frames.save_cache(path, x, v)
    # the reference's restart: [x_, v_] = pickle.load(open(..., 'rb'))
    [x_, v_] = pickle.load(open(path, 'rb'))
    assert x_.dtype == np.float64 and x_.shape == (17, 3)
    assert np.array_equal(x_, x) and np.array_equal(v_, v)
    x2, v2 = frames.load_cache(path)
    assert np.array_equal(x2, x) and np.array_equal(v2, v)


def test_frame_writer_host_arrays(tmp_path):
    sc = scenes.two_cubes(n=2, seed=2)
    rng = np.random.default_rng(1)
    d = str(tmp_path / 'run')
    w = frames.FrameWriter(d, sc.boundary_triangles, len(sc.x), depth=2)
    states = [(sc.x + rng.normal(size=sc.x.shape) * 1e-3, rng.normal(size=sc.x.shape)) for _ in range(5)]
    w.submit(0, *states[0], cache=False)
    for f in range(1, 5):
        w.submit(f, *states[f])
    w.flush()
    w.close()
    assert not os.path.exists(frames.cache_path(d, 0))
    for f in range(5):
        assert open(frames.obj_path(d, f), 'rb').read() == reference_obj_text(states[f][0], sc.boundary_triangles)
    for f in range(1, 5):
        x, v = frames.load_cache(frames.cache_path(d, f))
        assert np.array_equal(x, states[f][0]) and np.array_equal(v, states[f][1])


def test_frame_writer_reports_errors(tmp_path):
    sc = scenes.two_cubes(n=2, seed=2)
    d = str(tmp_path / 'run')
    w = frames.FrameWriter(d, sc.boundary_triangles, len(sc.x), cache=False)
    os.rmdir(os.path.join(d, 'objs'))
    w.submit(1, sc.x, sc.v)
    with pytest.raises(FastIPCError):
        w.flush()
    with pytest.raises(FastIPCError):
        w.close()


def script_targets(x_rest, groups, motion, t):
    """The rigid-motion schedule fipc_dirichlet_script evaluates (Rodrigues' rotation about
    the axis through the centre, then the translation), restated in numpy."""
    mask = groups >= 0
    tgt = x_rest.copy()
    g = groups[mask]
    m = motion[g]
    c, a, om, u = m[:, 0:3], m[:, 3:6], m[:, 6], m[:, 7:10]
    r = x_rest[mask] - c
    s, co = np.sin(om * t)[:, None], np.cos(om * t)[:, None]
    ad = np.sum(a * r, axis=1, keepdims=True) * (1 - co)
    tgt[mask] = c + r * co + np.cross(a, r) * s + a * ad + u * t
    return mask, tgt


@pytest.mark.parametrize('t', [0.0, 0.01, 0.37, 2.0, 11.3])
def test_twist_script_matches_loop_schedule(t):
    sc = scenes.twisted_bar(nx=6, ny=3, nz=3, seed=4)
    mask, tgt = script_targets(sc.x, sc.dirichlet_groups, sc.dirichlet_motion, t)
    ref_mask, ref_tgt = sc.dirichlet(t)
    assert np.array_equal(mask, ref_mask)
    assert mask.sum() == 2 * 4 * 4
    np.testing.assert_allclose(tgt, ref_tgt, rtol=0, atol=1e-15)
    # and in the reference's own per-vertex form (reader.py:170-185)
    for i in np.flatnonzero(mask)[:8]:
        a, b, c = sc.x[i]
        ang = np.arctan2(b, c) + np.pi * t * (1 if a < 0 else -1)
        rad = np.sqrt(b * b + c * c)
        np.testing.assert_allclose(tgt[i], [a, rad * np.sin(ang), rad * np.cos(ang)], rtol=0, atol=1e-15)


@pytest.mark.parametrize('make', [lambda: scenes.two_cubes(n=3, seed=5), lambda: scenes.cube_stack(7),
                                  lambda: scenes.cube_lattice(m=2, n=2, seed=1)])
def test_static_script_is_exact(make):
    sc = make()
    for t in (0.0, 0.05, 3.0):
        mask, tgt = script_targets(sc.x, sc.dirichlet_groups, sc.dirichlet_motion, t)
        ref_mask, ref_tgt = sc.dirichlet(t)
        assert np.array_equal(mask, ref_mask)
        assert np.array_equal(tgt, ref_tgt)


def test_frame_writer_2d_caches(tmp_path):
    """dim 2: caches only, [V,2] arrays as the reference's 2D driver pickles them."""
    rng = np.random.default_rng(8)
    d = str(tmp_path / 'run2d')
    w = frames.FrameWriter(d, None, 11, obj=False, dim=2)
    states = [(rng.normal(size=(11, 2)), rng.normal(size=(11, 2))) for _ in range(3)]
    for f, (x, v) in enumerate(states, start=1):
        w.submit(f, x, v)
    w.flush()
    w.close()
    assert not os.path.exists(os.path.join(d, 'objs'))
    for f, (x, v) in enumerate(states, start=1):
        x2, v2 = frames.load_cache(frames.cache_path(d, f))
        assert x2.shape == (11, 2) and np.array_equal(x2, x) and np.array_equal(v2, v)
    with pytest.raises(ValueError):
        frames.FrameWriter(d, None, 11, obj=True, dim=2)
