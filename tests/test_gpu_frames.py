"""Device Dirichlet schedule, per-frame output and restart on the GB300.

* fipc_dirichlet_script (through NewtonIPC and the batch context) against each scene's
  schedule in the reference's per-vertex form (reader.py:170-185): masks equal, targets exact
  for fixed masks and within 1e-14 m for the rotating bar ends.
* NewtonIPC.run writes the reference's objs/%06d.obj and caches/%06d.p (NEWTON_IPC.py:947,
  1000-1002); a restart from caches/000002.p (:949-953) reproduces the uninterrupted run's
  later frames bit for bit.
"""
import os
import shutil

import numpy as np
import pytest
import torch

from fastipc_gb300 import frames, scenes
from fastipc_gb300.batch import BatchNewtonIPC
from fastipc_gb300.newton import NewtonIPC

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('which', ['bar', 'cubes'])
def test_dirichlet_script_matches_schedule(which):
    sc = scenes.twisted_bar(nx=12, ny=4, nz=4, seed=3) if which == 'bar' else scenes.two_cubes(n=3, seed=2)
    sim = NewtonIPC(sc)
    try:
        assert sim._script is not None
        for t in (0.0, 0.01, 0.37, 2.0):
            sim._dirichlet(t)
            torch.cuda.synchronize()
            mask, tgt = sc.dirichlet(t)
            assert np.array_equal(sim.fixed.cpu().numpy().astype(bool), mask)
            got = sim.target.cpu().numpy()
            if which == 'bar':
                np.testing.assert_allclose(got, tgt, rtol=0, atol=1e-14)
            else:
                assert np.array_equal(got, tgt)
    finally:
        sim.close()


def test_batch_dirichlet_script_matches_schedules():
    scs = [scenes.cube_stack(s, max_cubes=2, max_hex=4) for s in range(3)]
    b = BatchNewtonIPC(scs)
    try:
        assert b._script is not None
        b._dirichlet(0.2)
        torch.cuda.synchronize()
        masks, vals = zip(*(sc.dirichlet(0.2) for sc in scs))
        assert np.array_equal(b.fixed.cpu().numpy().astype(bool), np.concatenate(masks))
        assert np.array_equal(b.target.cpu().numpy(), np.concatenate(vals))
    finally:
        b.close()


def test_device_schedule_steps_like_host_schedule():
    sc = scenes.twisted_bar(nx=12, ny=4, nz=4, seed=3)
    out = []
    for dev in (True, False):
        sim = NewtonIPC(sc, pcg_rtol=1e-12, device_dirichlet=dev)
        try:
            for f in range(3):
                sim.step(f)
            out.append(sim.x.cpu().numpy())
        finally:
            sim.close()
    np.testing.assert_allclose(out[0], out[1], rtol=0, atol=1e-12)


def test_run_writes_frames_and_restarts_exactly(tmp_path):
    sc = scenes.two_cubes(n=3, seed=1)
    d1, d2 = str(tmp_path / 'a'), str(tmp_path / 'b')
    sim = NewtonIPC(sc, pcg_rtol=1e-12)
    try:
        sim.run(4, directory=d1)
        x4, v4 = sim.x.cpu().numpy(), sim.v.cpu().numpy()
    finally:
        sim.close()
    assert not os.path.exists(frames.cache_path(d1, 0))
    for f in range(5):
        assert os.path.exists(frames.obj_path(d1, f))
    xc, vc = frames.load_cache(frames.cache_path(d1, 4))
    assert np.array_equal(xc, x4) and np.array_equal(vc, v4)
    lines = open(frames.obj_path(d1, 4)).read().splitlines()
    assert len(lines) == len(x4) + len(sc.boundary_triangles)
    np.testing.assert_allclose(np.array([[float(t) for t in l.split()[1:]] for l in lines[:len(x4)]]), x4, atol=5.1e-7)
    # restart from frame 2 in a fresh directory holding only that cache
    os.makedirs(os.path.join(d2, 'caches'))
    shutil.copy(frames.cache_path(d1, 2), frames.cache_path(d2, 2))
    sim = NewtonIPC(sc, pcg_rtol=1e-12)
    try:
        sim.run(2, directory=d2, start_frame=2)
    finally:
        sim.close()
    for f in (3, 4):
        assert open(frames.obj_path(d2, f), 'rb').read() == open(frames.obj_path(d1, f), 'rb').read()
        a, b = frames.load_cache(frames.cache_path(d1, f)), frames.load_cache(frames.cache_path(d2, f))
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
