"""ctypes binding of libmusg.so (the C ABI declared in include/musg.h).

The library is built in-tree by ``muspectre_gb300.build`` (``__graft_entry__.build()``).
There is no CPU fallback: if the library is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libmusg.so')

# status codes (include/musg.h)
OK, ERR_RUNTIME, ERR_PROJECTION, ERR_SOLVER, ERR_CONVERGENCE, ERR_SHAPE, ERR_CUDA, ERR_MEMORY, ERR_ARGUMENT, \
    ERR_NONFINITE = range(10)
FINITE_STRAIN, SMALL_STRAIN = 0, 1
FLAG_ALLOW_EVEN = 1
PRECISION_FP64, PRECISION_MIXED = 0, 1
LAW_LE1, LAW_LE2, LAW_LE3, LAW_LE4, LAW_HEP1, LAW_GENERIC = 1, 2, 3, 4, 5, 6
PROJ_SMALL_STRAIN, PROJ_FINITE_STRAIN_FAST, PROJ_FINITE_STRAIN = 0, 1, 2


class ProjectionError(RuntimeError):
    """ProjectionError (src/fft/projection_base.hh)."""


class SolverError(RuntimeError):
    """SolverError (src/solver/solver_common.hh:80-83)."""


class ConvergenceError(SolverError):
    """ConvergenceError (src/solver/solver_common.hh:86-88)."""


class CudaError(RuntimeError):
    """A CUDA runtime failure inside libmusg."""


class ResultInfo(C.Structure):
    _fields_ = [('success', C.c_int), ('status', C.c_int), ('nb_it', C.c_uint), ('nb_fev', C.c_uint),
                ('message', C.c_char * 64), ('hom_stress', C.c_double * 9)]


class Request(C.Structure):
    _fields_ = [('dim', C.c_int), ('resolutions', C.c_int * 3), ('lengths', C.c_double * 3),
                ('formulation', C.c_int), ('flags', C.c_int), ('nb_materials', C.c_int),
                ('laws', C.POINTER(C.c_int)), ('params', C.POINTER(C.c_double)),
                ('phase', C.POINTER(C.c_ubyte)), ('per_pixel', C.POINTER(C.c_double)),
                ('per_pixel_stride', C.c_int), ('nb_steps', C.c_int), ('load_steps', C.POINTER(C.c_double))]


class ServerResult(C.Structure):
    _fields_ = [('id', C.c_longlong), ('success', C.c_int), ('nb_steps_done', C.c_int), ('nb_it', C.c_uint),
                ('nb_fev', C.c_uint), ('stress', C.c_double * 9), ('latency_s', C.c_double),
                ('service_s', C.c_double), ('batched_with', C.c_int), ('message', C.c_char * 64)]


class ServerStats(C.Structure):
    _fields_ = [('submitted', C.c_longlong), ('completed', C.c_longlong), ('batches', C.c_longlong),
                ('budget', C.c_ulonglong), ('in_use', C.c_ulonglong), ('peak_in_use', C.c_ulonglong),
                ('queued', C.c_longlong)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_LL = C.POINTER(C.c_longlong)

_SIGNATURES = {
    'musg_last_error': (C.c_char_p, []),
    'musg_version': (C.c_int, []),
    'musg_selftest_wait_timeout': (C.c_int, [C.c_double, C.POINTER(C.c_int)]),
    'musg_device_count': (C.c_int, [_I]),
    'musg_set_device': (C.c_int, [C.c_int]),
    'musg_cell_create': (C.c_int, [C.c_int, _I, _D, C.c_int, C.c_int, C.POINTER(_P)]),
    'musg_cell_destroy': (C.c_int, [_P]),
    'musg_cell_sizes': (C.c_int, [_P, _LL, _LL]),
    'musg_cell_set_stream': (C.c_int, [_P, _P]),
    'musg_material_create': (C.c_int, [_P, C.c_int, C.c_char_p, _D, C.c_int, _I]),
    'musg_material_add_pixels': (C.c_int, [_P, C.c_int, _LL, C.c_longlong, _D, C.c_int]),
    'musg_material_size': (C.c_int, [_P, C.c_int, _LL]),
    'musg_cell_initialise': (C.c_int, [_P, C.c_int]),
    'musg_cell_tuning': (C.c_int, [_P, _I, _LL]),
    'musg_cell_set_uniform_strain': (C.c_int, [_P, _D]),
    'musg_cell_get_strain': (C.c_int, [_P, _D]),
    'musg_cell_set_strain': (C.c_int, [_P, _D]),
    'musg_cell_get_stress': (C.c_int, [_P, _D]),
    'musg_cell_evaluate_stress_tangent': (C.c_int, [_P, _D, _D]),
    'musg_cell_apply_projection': (C.c_int, [_P, _D]),
    'musg_cell_directional_stiffness': (C.c_int, [_P, _D, _D]),
    'musg_cell_cg_operator': (C.c_int, [_P, C.c_int, _D, _D]),
    'musg_cell_save_history_variables': (C.c_int, [_P]),
    'musg_cell_homogenised_stress': (C.c_int, [_P, _D]),
    'musg_cell_get_internal': (C.c_int, [_P, C.c_char_p, _D, C.c_longlong, _I]),
    'musg_cell_checkpoint_size': (C.c_int, [_P, C.POINTER(C.c_ulonglong)]),
    'musg_cell_checkpoint_save': (C.c_int, [_P, _P, C.c_ulonglong]),
    'musg_cell_checkpoint_load': (C.c_int, [_P, _P, C.c_ulonglong]),
    'musg_solver_cg_create': (C.c_int, [_P, C.c_double, C.c_uint, C.c_int, C.c_int, C.POINTER(_P)]),
    'musg_solver_destroy': (C.c_int, [_P]),
    'musg_solver_set_inner_tol': (C.c_int, [_P, C.c_double]),
    'musg_solver_set_line_search': (C.c_int, [_P, C.c_int]),
    'musg_solver_set_incremental_residual': (C.c_int, [_P, C.c_int]),
    'musg_probe_fp64_fma': (C.c_int, [C.POINTER(C.c_double)]),
    'musg_solver_get_counter': (C.c_int, [_P, C.POINTER(C.c_uint)]),
    'musg_solver_reset_counter': (C.c_int, [_P]),
    'musg_solver_has_converged': (C.c_int, [_P, _I]),
    'musg_solver_solve': (C.c_int, [_P, _D, _D]),
    'musg_newton_cg': (C.c_int, [_P, _D, C.c_int, _P, C.c_double, C.c_double, C.c_int, C.POINTER(ResultInfo), _D,
                                 _D]),
    'musg_de_geus': (C.c_int, [_P, _D, C.c_int, _P, C.c_double, C.c_double, C.c_int, C.POINTER(ResultInfo), _D,
                               _D]),
    'musg_batch_create': (C.c_int, [C.POINTER(_P), C.c_int, C.c_double, C.c_uint, C.c_int, C.POINTER(_P)]),
    'musg_batch_destroy': (C.c_int, [_P]),
    'musg_batch_set_inner_tol': (C.c_int, [_P, C.c_double]),
    'musg_batch_newton_cg': (C.c_int, [_P, _D, C.c_int, C.c_double, C.c_double, C.POINTER(ResultInfo), _D]),
    'musg_launch_count': (C.c_int, [C.POINTER(C.c_ulonglong)]),
    'musg_solver_profile': (C.c_int, [_P, C.c_int, _D, _I]),
    'musg_solver_kernel_name': (C.c_char_p, [_P, C.c_int]),
    'musg_fft_create': (C.c_int, [C.c_int, _I, C.c_int, C.POINTER(_P)]),
    'musg_fft_destroy': (C.c_int, [_P]),
    'musg_fft_forward': (C.c_int, [_P, _D, _D]),
    'musg_fft_inverse': (C.c_int, [_P, _D, _D]),
    'musg_projection_create': (C.c_int, [C.c_int, _I, _D, C.c_int, C.c_int, C.POINTER(_P)]),
    'musg_projection_destroy': (C.c_int, [_P]),
    'musg_projection_apply': (C.c_int, [_P, _D]),
    'musg_projection_get_operator': (C.c_int, [_P, _D, _LL, _LL]),
    'musg_request_bytes': (C.c_int, [C.POINTER(Request), C.c_int, C.POINTER(C.c_ulonglong)]),
    'musg_server_create': (C.c_int, [C.c_ulonglong, C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_double,
                                     C.POINTER(_P)]),
    'musg_server_submit': (C.c_int, [_P, C.POINTER(Request), _LL]),
    'musg_server_close': (C.c_int, [_P]),
    'musg_server_cancel_waiting': (C.c_int, [_P, _LL]),
    'musg_server_cancel_running': (C.c_int, [_P, _LL]),
    'musg_solver_set_stop_flag': (C.c_int, [_P, _I]),
    'musg_batch_set_stop_flag': (C.c_int, [_P, _I]),
    'musg_server_wait': (C.c_int, [_P, C.c_longlong, C.c_double, C.POINTER(ServerResult)]),
    'musg_server_get_stats': (C.c_int, [_P, C.POINTER(ServerStats)]),
    'musg_server_destroy': (C.c_int, [_P]),
    'musg_server_admit': (C.c_int, [_P, _LL, C.c_int, _I, C.POINTER(C.c_ulonglong)]),
    'musg_server_release': (C.c_int, [_P, C.c_ulonglong]),
    'musg_projection_apply_noalloc': (C.c_int, [C.c_int, _I, _D, C.c_int, C.c_int, _P, _P, _P]),
}

_lib = None


def lib():
    """The loaded library; raises when it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError('libmusg.so is not built (%s); run `python -c "import __graft_entry__ as g; g.build()"` '
                               'or `python -m muspectre_gb300.build`' % LIB_PATH)
        handle = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(rc):
    if rc == OK:
        return
    msg = lib().musg_last_error().decode('utf-8', 'replace')
    if rc == ERR_PROJECTION:
        raise ProjectionError(msg)
    if rc == ERR_CONVERGENCE:
        raise ConvergenceError(msg)
    if rc == ERR_SOLVER:
        raise SolverError(msg)
    if rc in (ERR_CUDA, ERR_MEMORY):
        raise CudaError(msg)
    if rc == ERR_ARGUMENT:
        raise ValueError(msg)
    raise RuntimeError(msg)


def dptr(a):
    return a.ctypes.data_as(_D) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_I)


def llptr(a):
    return a.ctypes.data_as(_LL)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def launch_count():
    n = C.c_ulonglong(0)
    check(lib().musg_launch_count(C.byref(n)))
    return n.value


def probe_fp64_fma():
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    t = C.c_double(0.0)
    check(lib().musg_probe_fp64_fma(C.byref(t)))
    return t.value


def selftest_wait_timeout(limit_ms=5.0):
    """Self-test of the bounded mbarrier waits of the TMA-fed passes: True when a wait
    that nothing completes gave up after ``limit_ms`` and the host saw the fault word
    (musg_selftest_wait_timeout)."""
    out = C.c_int(0)
    check(lib().musg_selftest_wait_timeout(float(limit_ms), C.byref(out)))
    return bool(out.value)


def device_count():
    n = C.c_int(0)
    check(lib().musg_device_count(C.byref(n)))
    return n.value
