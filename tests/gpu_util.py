"""Helpers for the GPU tests: device tensors, the C-ABI library, tolerances."""
import ctypes

import numpy as np

D = ctypes.c_double


def lib():
    from fastipc_gb300 import _native
    return _native.lib()


def cu(a, dtype=None):
    import torch
    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a).to('cuda:0')
    return t if dtype is None else t.to(dtype)


def p(t):
    return ctypes.c_void_p(t.data_ptr())


def stream():
    from fastipc_gb300 import _native
    return _native.stream()


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = np.maximum(np.abs(b).reshape(len(b), -1).max(axis=1), 1e-300)
    return (np.abs(a - b).reshape(len(b), -1).max(axis=1) / scale).max()
