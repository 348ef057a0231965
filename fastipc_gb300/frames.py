"""Per-frame output and restart of the driver (NEWTON_IPC.py:900-931, 947-953, 1000-1002).

The reference writes, after every time step f, ``objs/{f:06d}.obj`` (positions and boundary
triangles, ``write_image``) and ``caches/{f:06d}.p`` (``pickle.dump([x, v])``), and restarts
from such a cache when ``start_frame > 0``.  Both files have the reference's exact format
here: the OBJ text comes from ``fipc_write_obj`` (byte-identical to the reference's ``'%.6f'``
formatting) and the cache is the same pickled list of two float64 [V,3] arrays, so either side
can read the other's frames.

``FrameWriter`` keeps the output off the simulation stream: a frame is snapshotted on the
device (a few microseconds of HBM copy), copied to pinned host memory on a side stream, and
formatted and written by a worker thread while the next time step runs.
"""
import os
import pickle
import queue
import threading

import numpy as np
import torch

from . import _native as N
from ._native import check, hptr


def obj_path(directory, f):
    return os.path.join(directory, 'objs', f'{f:06d}.obj')


def cache_path(directory, f):
    return os.path.join(directory, 'caches', f'{f:06d}.p')


def write_obj(path, x, triangles):
    """One OBJ frame (NEWTON_IPC.py:926-931) from host arrays x [V,3] and triangles [F,3]."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
    check(N.lib().fipc_write_obj(os.fsencode(path), len(x), hptr(x), len(t), hptr(t)), f'write_obj {path}')


def save_cache(path, x, v):
    """caches/%06d.p as the reference writes it (NEWTON_IPC.py:1002): pickle of [x, v]."""
    with open(path, 'wb') as fh:
        pickle.dump([np.asarray(x, dtype=np.float64), np.asarray(v, dtype=np.float64)], fh)


def load_cache(path):
    """[x, v] from a cache file (NEWTON_IPC.py:951-953)."""
    with open(path, 'rb') as fh:
        x, v = pickle.load(fh)
    return np.asarray(x, dtype=np.float64), np.asarray(v, dtype=np.float64)


class FrameWriter:
    """Asynchronous writer of the reference's per-frame files.

    ``submit(f, x, v)`` returns as soon as the frame is queued; ``flush()`` waits for every
    queued frame and re-raises the first error a write met.  ``depth`` frames can be in
    flight; a further submit waits for the oldest one.  x and v may be CUDA or CPU tensors (or
    numpy arrays) of shape [V, dim].  With dim 2 only caches are written: the reference's 2D
    write_image draws into a window instead of writing a file.
    """

    def __init__(self, directory, triangles, n_verts, obj=True, cache=True, depth=2, dim=3):
        if dim not in (2, 3):
            raise ValueError('dim must be 2 or 3')
        if dim == 2 and obj:
            raise ValueError('OBJ frames are written for 3D scenes only')
        self.directory = directory
        self.obj, self.cache = obj, cache
        self.dim = dim
        self.tris = None if triangles is None else np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
        self.n = int(n_verts)
        for sub, on in (('objs', obj), ('caches', cache)):
            if on:
                os.makedirs(os.path.join(directory, sub), exist_ok=True)
        self.cuda = torch.cuda.is_available()
        pin = self.cuda
        self._host = [(torch.empty((self.n, dim), dtype=torch.float64, pin_memory=pin),
                       torch.empty((self.n, dim), dtype=torch.float64, pin_memory=pin)) for _ in range(depth)]
        self._dev = [None] * depth          # device snapshots, made on first CUDA submit
        self._free = queue.Queue()
        for k in range(depth):
            self._free.put(k)
        self._jobs = queue.Queue()
        self._error = None
        self._copy_stream = None
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()

    def submit(self, f, x, v, obj=None, cache=None):
        """Queue frame f; obj / cache override the writer's defaults for this frame (the
        reference writes no cache for frame 0)."""
        if self._error is not None:
            raise self._error
        k = self._free.get()
        hx, hv = self._host[k]
        done = None
        if isinstance(x, torch.Tensor) and x.is_cuda:
            if self._dev[k] is None:
                self._dev[k] = (torch.empty((self.n, self.dim), dtype=torch.float64, device=x.device),
                                torch.empty((self.n, self.dim), dtype=torch.float64, device=x.device))
            if self._copy_stream is None:
                self._copy_stream = torch.cuda.Stream(device=x.device)
            dx, dv = self._dev[k]
            main = torch.cuda.current_stream(x.device)
            dx.copy_(x.reshape(-1, self.dim))   # snapshot on the simulation stream
            dv.copy_(v.reshape(-1, self.dim))
            snap = torch.cuda.Event()
            snap.record(main)
            with torch.cuda.stream(self._copy_stream):
                self._copy_stream.wait_event(snap)
                hx.copy_(dx, non_blocking=True)
                hv.copy_(dv, non_blocking=True)
                done = torch.cuda.Event()
                done.record(self._copy_stream)
        else:
            hx.copy_(torch.as_tensor(np.asarray(x, dtype=np.float64)).reshape(-1, self.dim))
            hv.copy_(torch.as_tensor(np.asarray(v, dtype=np.float64)).reshape(-1, self.dim))
        self._jobs.put((f, k, done, self.obj if obj is None else obj, self.cache if cache is None else cache))

    def _run(self):
        while True:
            job = self._jobs.get()
            if job is None:
                self._jobs.task_done()
                return
            f, k, done, obj, cache = job
            try:
                if done is not None:
                    done.synchronize()
                hx, hv = self._host[k]
                xn, vn = hx.numpy(), hv.numpy()
                if obj:
                    write_obj(obj_path(self.directory, f), xn, self.tris)
                if cache:
                    save_cache(cache_path(self.directory, f), xn.copy(), vn.copy())
            except Exception as e:   # reported by the next submit() or flush()
                if self._error is None:
                    self._error = e
            finally:
                self._free.put(k)
                self._jobs.task_done()

    def flush(self):
        self._jobs.join()
        if self._error is not None:
            raise self._error

    def close(self):
        if self._thread.is_alive():
            self._jobs.put(None)
            self._thread.join()
        if self._error is not None:
            raise self._error

