"""ctypes binding of libwotg.so (the C ABI declared in include/wotg.h).

There is no CPU fallback: every compute entry point of ``wot_gb300`` goes
through this module, and loading fails loudly when the library has not been
built (``python -m wot_gb300._build``) or when no CUDA device is present.
"""
from __future__ import annotations

import ctypes
import logging
import os

import numpy as np

logger = logging.getLogger('wot')

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'libwotg.so')

WOTG_OK = 0
WOTG_MAX_ITER = 1
WOTG_NONFINITE = 2
WOTG_BADARG = 3
WOTG_CUDA_ERROR = 4
WOTG_WORKSPACE = 5
WOTG_TOO_LARGE = 6

SOLVER_DUALITY_GAP = 0
SOLVER_FIXED_ITERS = 1

# Every symbol include/wotg.h declares (checked by the CPU test suite).
EXPORTS = (
    'wotg_version', 'wotg_last_error', 'wotg_cost_sqeuclidean', 'wotg_cost_from_f64',
    'wotg_median_workspace_bytes', 'wotg_median', 'wotg_solve_workspace_bytes',
    'wotg_compute_transport_matrix', 'wotg_apply_coupling_f64', 'wotg_launch_count',
    'wotg_lse_matvec_workspace_bytes', 'wotg_lse_matvec', 'wotg_noalloc_scratch_bytes',
    'wotg_compute_transport_matrix_noalloc', 'wotg_problem_workspace_bytes', 'wotg_tc_selftest',
    'wotg_lse_points_workspace_bytes', 'wotg_lse_points', 'wotg_transpose_cost', 'wotg_batch_workspace_bytes',
    'wotg_solve_batched', 'wotg_lse_matvec_multi_workspace_bytes', 'wotg_lse_matvec_multi',
    'wotg_coupling_from_potentials', 'wotg_ot_adjoint_workspace_bytes', 'wotg_ot_adjoint',
    'wotg_refine_potentials', 'wotg_exp2_rate', 'wotg_lse_points_timing', 'wotg_lse_points_bounded',
    'wotg_batch_pass_timing', 'wotg_gemm_f64', 'wotg_csr_count', 'wotg_csr_fill',
    'wotg_csr_transpose_workspace_bytes', 'wotg_csr_transpose', 'wotg_spmm_centred', 'wotg_gram_workspace_bytes',
    'wotg_gram_f64', 'wotg_vecmat_workspace_bytes', 'wotg_vecmat_f64', 'wotg_apply_points_workspace_bytes',
    'wotg_apply_points', 'wotg_exp2_fma', 'wotg_batch_replay_profile',
)


class Params(ctypes.Structure):
    _fields_ = [('epsilon', ctypes.c_double), ('lambda1', ctypes.c_double), ('lambda2', ctypes.c_double),
                ('epsilon0', ctypes.c_double), ('tau', ctypes.c_double), ('tolerance', ctypes.c_double),
                ('max_iter', ctypes.c_double), ('batch_size', ctypes.c_int32),
                ('scaling_iter', ctypes.c_int32), ('inner_iter_max', ctypes.c_int32),
                ('extra_iter', ctypes.c_int32), ('growth_iters', ctypes.c_int32), ('solver', ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [('iterations', ctypes.c_int64), ('absorptions', ctypes.c_int64), ('checks', ctypes.c_int64),
                ('gap', ctypes.c_double), ('final_epsilon', ctypes.c_double),
                ('hit_max_iter', ctypes.c_int32), ('exact_rows', ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


FORM_MATERIALIZED = 0
FORM_ONTHEFLY = 1


class Problem(ctypes.Structure):
    _fields_ = [('I', ctypes.c_int64), ('J', ctypes.c_int64), ('C', ctypes.c_void_p), ('ldc', ctypes.c_int64),
                ('cost_scale', ctypes.c_double), ('G', ctypes.c_void_p), ('X', ctypes.c_void_p),
                ('ldx', ctypes.c_int64), ('Y', ctypes.c_void_p), ('ldy', ctypes.c_int64), ('d', ctypes.c_int32),
                ('form', ctypes.c_int32)]


class Pair(ctypes.Structure):
    _fields_ = [('I', ctypes.c_int64), ('J', ctypes.c_int64), ('C', ctypes.c_void_p), ('ldc', ctypes.c_int64),
                ('CT', ctypes.c_void_p), ('ldct', ctypes.c_int64), ('cost_scale', ctypes.c_double),
                ('G', ctypes.c_void_p)]


class Item(ctypes.Structure):
    _fields_ = [('pair', ctypes.c_int32), ('reserved_', ctypes.c_int32), ('params', Params),
                ('row_offset', ctypes.c_int64), ('col_offset', ctypes.c_int64), ('growth_offset', ctypes.c_int64)]


_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load libwotg.so and declare its signatures; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _LIB_PATH
    if not os.path.exists(path):
        raise ImportError('libwotg.so is not built (%s); run `python -m wot_gb300._build` '
                          '(wot_gb300 has no CPU fallback)' % path)
    lib = ctypes.CDLL(path)
    vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
    sig = {
        'wotg_version': (ctypes.c_char_p, []),
        'wotg_last_error': (ctypes.c_char_p, []),
        'wotg_cost_sqeuclidean': (ctypes.c_int, [vp, i64, i64, vp, i64, i64, i32, vp, i64, vp]),
        'wotg_cost_from_f64': (ctypes.c_int, [vp, i64, i64, vp, i64, vp]),
        'wotg_median_workspace_bytes': (ctypes.c_size_t, []),
        'wotg_median': (ctypes.c_int, [vp, i64, i64, i64, ctypes.POINTER(dbl), vp, ctypes.c_size_t, vp]),
        'wotg_solve_workspace_bytes': (ctypes.c_size_t, [i64, i64, i64]),
        'wotg_problem_workspace_bytes': (ctypes.c_size_t, [ctypes.POINTER(Problem)]),
        'wotg_tc_selftest': (ctypes.c_int, [vp, vp, vp, ctypes.c_uint32, ctypes.c_uint32, i32, vp, vp]),
        'wotg_lse_points_workspace_bytes': (ctypes.c_size_t, [i64, i64, i32]),
        'wotg_lse_points': (ctypes.c_int, [vp, i64, i64, vp, i64, i64, i32, dbl, vp, vp, vp, ctypes.c_size_t, vp]),
        'wotg_csr_count': (ctypes.c_int, [vp, i64, i64, i64, vp, vp, vp]),
        'wotg_csr_fill': (ctypes.c_int, [vp, i64, i64, i64, vp, vp, vp, vp]),
        'wotg_csr_transpose_workspace_bytes': (ctypes.c_size_t, [i64, i64]),
        'wotg_csr_transpose': (ctypes.c_int, [vp, vp, vp, i64, i64, vp, vp, vp, vp, ctypes.c_size_t, vp]),
        'wotg_spmm_centred': (ctypes.c_int, [vp, vp, vp, i64, vp, i32, vp, vp, vp, vp, vp]),
        'wotg_gram_workspace_bytes': (ctypes.c_size_t, [i64, i32]),
        'wotg_gram_f64': (ctypes.c_int, [vp, i64, i32, vp, vp, ctypes.c_size_t, vp]),
        'wotg_vecmat_workspace_bytes': (ctypes.c_size_t, [i64, i32]),
        'wotg_vecmat_f64': (ctypes.c_int, [vp, vp, i64, i32, vp, vp, ctypes.c_size_t, vp]),
        'wotg_apply_points_workspace_bytes': (ctypes.c_size_t, [i64, i64, i32]),
        'wotg_apply_points': (ctypes.c_int, [vp, i64, i64, vp, i64, i64, i32, dbl, vp, vp, vp, i64, i32, vp, vp,
                                             ctypes.c_size_t, vp]),
        'wotg_gemm_f64': (ctypes.c_int, [vp, i64, vp, i64, vp, vp, i64, i64, i64, i64, vp]),
        'wotg_batch_pass_timing': (ctypes.c_int, [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                                  ctypes.POINTER(ctypes.c_int32)]),
        'wotg_lse_points_bounded': (ctypes.c_int, [vp, i64, i64, vp, i64, i64, i32, dbl, vp, vp, ctypes.c_uint32,
                                                   vp, ctypes.c_size_t, vp]),
        'wotg_compute_transport_matrix': (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(Params),
                                                         vp, vp, vp, vp, vp, ctypes.POINTER(Stats),
                                                         vp, ctypes.c_size_t, vp]),
        'wotg_apply_coupling_f64': (ctypes.c_int, [vp, i64, i64, vp, i32, i32, i32, vp, vp]),
        'wotg_launch_count': (ctypes.c_ulonglong, []),
        'wotg_noalloc_scratch_bytes': (ctypes.c_size_t, []),
        'wotg_compute_transport_matrix_noalloc': (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(Params),
                                                                 vp, vp, vp, vp, vp, ctypes.POINTER(Stats), vp]),
        'wotg_transpose_cost': (ctypes.c_int, [vp, i64, i64, i64, vp, i64, vp]),
        'wotg_batch_workspace_bytes': (ctypes.c_size_t, [ctypes.POINTER(Pair), i32, ctypes.POINTER(Item), i32]),
        'wotg_solve_batched': (ctypes.c_int, [ctypes.POINTER(Pair), i32, ctypes.POINTER(Item), i32, vp, vp, vp, vp,
                                              ctypes.POINTER(Stats), ctypes.POINTER(i32), vp, ctypes.c_size_t, vp]),
        'wotg_lse_matvec_multi_workspace_bytes': (ctypes.c_size_t, [i64, i32]),
        'wotg_lse_matvec_multi': (ctypes.c_int, [vp, i64, i64, i64, vp, i64, ctypes.POINTER(ctypes.c_float), i32,
                                                 vp, i64, vp, ctypes.c_size_t, vp]),
        'wotg_coupling_from_potentials': (ctypes.c_int, [vp, i64, i64, i64, dbl, dbl, vp, vp, dbl, vp, vp]),
        'wotg_ot_adjoint_workspace_bytes': (ctypes.c_size_t, [i64, i64]),
        'wotg_exp2_rate': (ctypes.c_int, [ctypes.POINTER(dbl), vp]),
        'wotg_exp2_fma': (ctypes.c_int, [vp, vp, i64, vp]),
        'wotg_batch_replay_profile': (i32, [vp, vp, i32]),
        'wotg_lse_points_timing': (ctypes.c_int, [vp, i64, i64, vp, i64, i64, i32, dbl, vp, i32, i32,
                                                  ctypes.POINTER(ctypes.c_float), vp, ctypes.c_size_t, vp]),
        'wotg_refine_potentials': (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(Params), dbl, i32, vp, vp,
                                                  ctypes.POINTER(Stats), vp, ctypes.c_size_t, vp]),
        'wotg_ot_adjoint': (ctypes.c_int, [vp, i64, i64, vp, i64, i64, i32, dbl, dbl, dbl, dbl, vp, vp, vp, vp, vp,
                                           vp, ctypes.POINTER(dbl), vp, ctypes.c_size_t, vp]),
        'wotg_lse_matvec_workspace_bytes': (ctypes.c_size_t, [i64, i64, i64]),
        'wotg_lse_matvec': (ctypes.c_int, [vp, i64, i64, i64, vp, ctypes.c_float, i32, vp, vp, ctypes.c_size_t,
                                           vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, what: str) -> int:
    """Map a wotg_status to the reference's exceptions / warnings."""
    if status == WOTG_OK:
        return status
    if status == WOTG_MAX_ITER:
        logger.warning("Reached max_iter with duality gap still above threshold. Returning")
        return status
    if status == WOTG_NONFINITE:
        raise RuntimeError("Overflow encountered in duality gap computation, please report this incident")
    if status == WOTG_BADARG:
        raise ValueError('%s: invalid arguments' % what)
    if status == WOTG_WORKSPACE:
        raise ValueError('%s: workspace missing or too small' % what)
    if status == WOTG_TOO_LARGE:
        raise ValueError(load().wotg_last_error().decode())
    msg = load().wotg_last_error().decode()
    raise RuntimeError('%s: CUDA error: %s' % (what, msg))


def require_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError('wot_gb300 needs a CUDA device (GB300, sm_103a); no CPU fallback exists')
    load()
    return torch


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def stream_handle(torch_mod=None):
    import torch
    return torch.cuda.current_stream().cuda_stream


def round_up(n: int, m: int) -> int:
    return (n + m - 1) // m * m


def to_numpy_f64(x) -> np.ndarray:
    return np.asarray(x, dtype=np.float64)
