"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every function that
include/fastipc.h declares (no compute calls)."""
import ctypes
import os
import re

from fastipc_gb300 import _native
from fastipc_gb300.build import build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'include', 'fastipc.h')


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


def test_status_strings():
    lib = ctypes.CDLL(build())
    lib.fipc_status_string.restype = ctypes.c_char_p
    assert lib.fipc_status_string(0) == b'ok'
    assert lib.fipc_status_string(5) == b'invalid argument'
