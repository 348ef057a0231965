"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every function that
include/fastipc.h declares (no compute calls)."""
import ctypes
import os
import re

from fastipc_gb300 import _native
from fastipc_gb300.build import build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'include', 'fastipc.h')
ASO_HEADER = os.path.join(os.path.dirname(HEADER), 'fastipc_aso.h')


def declared():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(fipc(?:2d)?_[a-z0-9_]+)\s*\(', src)))


def test_header_matches_binding():
    assert declared() == sorted(_native.EXPORTS)


def test_library_exports_all_symbols():
    lib = ctypes.CDLL(build())
    for name in declared():
        assert hasattr(lib, name), name


def test_library_exports_the_aso_functions():
    """include/fastipc_aso.h: the scalar functions with the reference a.so's signatures."""
    src = re.sub(r'/\*.*?\*/', '', open(ASO_HEADER).read(), flags=re.S)
    names = sorted(set(re.findall(r'\bvoid\s+([a-z_0-9]+)\s*\(', src)))
    assert len(names) == 17
    lib = ctypes.CDLL(build())
    for name in names:
        assert hasattr(lib, name), name


def test_status_strings():
    lib = ctypes.CDLL(build())
    lib.fipc_status_string.restype = ctypes.c_char_p
    assert lib.fipc_status_string(0) == b'ok'
    assert lib.fipc_status_string(5) == b'invalid argument'


def test_2d_entry_points_reject_misaligned_positions():
    """The 2D kernels read a vertex as one 16-byte load: a position array that does not start on
    a 16-byte boundary is rejected with status 5 before anything reaches the device (host logic
    only, no compute call)."""
    import numpy as np
    lib = ctypes.CDLL(build())
    buf = np.zeros(64, dtype=np.float64)
    base = buf.ctypes.data
    odd = ctypes.c_void_p(base + (8 if base % 16 == 0 else 0))     # 8 mod 16
    tris = np.zeros(3, dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.fipc2d_elements(1, P(tris), odd, P(buf), P(buf), P(buf), P(buf), ctypes.c_double(0.01), None, None, None,
                               None) == 5
    assert lib.fipc2d_barrier_rows(0, 1, P(tris), odd, ctypes.c_double(1e-6), ctypes.c_double(1.0), None, None, None,
                                   None) == 5
