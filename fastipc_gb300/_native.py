"""ctypes binding of libfastipc.so (include/fastipc.h).

The library is the only compute path: importing this module never falls back to anything
else, and every entry point raises ``FastIPCError`` when the library is missing or a call
returns a non-zero status.
"""
import ctypes
import os

from .build import LIB

_lib = None

STATUS = {0: 'ok', 1: 'capacity exceeded', 2: 'iteration limit reached', 3: 'non-finite value', 4: 'CUDA error',
          5: 'invalid argument', 6: 'file I/O error'}

# symbols declared in include/fastipc.h
EXPORTS = [
    'fipc_elasticity', 'fipc_barrier_rows', 'fipc_ccd_pairs', 'fipc_inversion_free_pairs', 'fipc_compute_xn_and_xtilde',
    'fipc_move_nodes', 'fipc_dirichlet_script', 'fipc_apply_sol', 'fipc_compute_v', 'fipc_ctx_create', 'fipc_ctx_destroy', 'fipc_ctx_params',
    'fipc_ctx_set_params', 'fipc_ctx_mass', 'fipc_ctx_set_x0', 'fipc_find_constraints', 'fipc_get_constraints',
    'fipc_compute_hessian_and_gradient', 'fipc_system_sizes', 'fipc_export_system', 'fipc_solve_system',
    'fipc_output_residual', 'fipc_compute_energy', 'fipc_compute_intersection_free_step_size', 'fipc_check_collision',
    'fipc_launch_count', 'fipc_status_string', 'fipc_profile_enable', 'fipc_profile_read', 'fipc_fp64_fma_probe',
    'fipc_compute_energy_noalloc', 'fipc_mlp_param_count', 'fipc_mlp_forward', 'fipc_mlp_backward', 'fipc_mlp_mse',
    'fipc_mlp_adam', 'fipc_mlp_features', 'fipc_batch_create', 'fipc_batch_params', 'fipc_batch_compute_energy',
    'fipc_batch_output_residual', 'fipc_batch_step_size', 'fipc_batch_check_collision', 'fipc_batch_apply_sol',
    'fipc_batch_solve_system', 'fipc_batch_pcg_shape', 'fipc_ctx_set_preconditioner', 'fipc_ctx_preconditioner', 'fipc_ctx_set_multigrid', 'fipc_ctx_multigrid', 'fipc_ctx_set_multigrid_fp32', 'fipc_mlp_smooth', 'fipc_dense_spd_inverse',
    'fipc_write_obj', 'fipc_solve_system_direct', 'fipc_direct_stats', 'fipc_admm_init', 'fipc_admm_reuse', 'fipc_admm_global', 'fipc_admm_local',
    'fipc_admm_dual', 'fipc2d_ctx_create', 'fipc2d_ctx_destroy', 'fipc2d_ctx_params', 'fipc2d_ctx_set_kappa', 'fipc2d_ctx_mass',
    'fipc2d_compute_xn_and_xtilde', 'fipc2d_move_nodes', 'fipc2d_apply_sol', 'fipc2d_compute_v', 'fipc2d_elements',
    'fipc2d_barrier_rows', 'fipc2d_ccd_pairs', 'fipc2d_find_constraints', 'fipc2d_get_constraints',
    'fipc2d_compute_hessian_and_gradient', 'fipc2d_system_nnzb', 'fipc2d_export_system', 'fipc2d_solve_system',
    'fipc2d_output_residual', 'fipc2d_compute_energy', 'fipc2d_compute_intersection_free_step_size', 'fipc2d_check_collision',
]


class FastIPCError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__(f'{what}: {STATUS.get(status, status)} (status {status})')


def lib():
    """Load libfastipc.so (built by fastipc_gb300.build.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise FastIPCError(4, f'libfastipc.so not built at {LIB}; run fastipc_gb300.build.build()')
        L = ctypes.CDLL(LIB)
        for name in EXPORTS:
            getattr(L, name).restype = ctypes.c_int
        L.fipc_launch_count.restype = ctypes.c_longlong
        L.fipc_status_string.restype = ctypes.c_char_p
        _lib = L
    return _lib


def check(status, what):
    if status != 0:
        raise FastIPCError(status, what)


def dptr(t, dtype=None):
    """Device pointer of a contiguous CUDA tensor (checked)."""
    import torch
    if t is None:
        return None
    if not t.is_cuda:
        raise FastIPCError(5, 'expected a CUDA tensor')
    if not t.is_contiguous():
        raise FastIPCError(5, 'expected a contiguous tensor')
    if dtype is not None and t.dtype != dtype:
        raise FastIPCError(5, f'expected dtype {dtype}, got {t.dtype}')
    _ = torch
    return ctypes.c_void_p(t.data_ptr())


def hptr(a):
    """Host pointer of a contiguous numpy array."""
    assert a.flags['C_CONTIGUOUS']
    return a.ctypes.data_as(ctypes.c_void_p)


def stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def launch_count():
    return int(lib().fipc_launch_count())
