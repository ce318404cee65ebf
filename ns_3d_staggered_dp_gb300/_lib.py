"""ctypes binding of libns_gpu.so (the C ABI declared in include/ns_gpu.h).

There is no CPU fallback: if the library is missing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libns_gpu.so")

NS_OK = 0
STATUS = {0: "NS_OK", 1: "NS_ERR_SHAPE", 2: "NS_ERR_CUDA", 3: "NS_ERR_NONFINITE", 4: "NS_ERR_TIMEOUT",
          5: "NS_ERR_UNSUPPORTED_BC", 6: "NS_ERR_ARG", 7: "NS_ERR_NOMEM", 8: "NS_ERR_IO"}


class NSConfig(C.Structure):
    """Mirror of ``ns_config`` (include/ns_gpu.h)."""
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("nu", C.c_double), ("dt", C.c_double),
        ("scheme", C.c_int),
        ("bc", C.c_int * 3), ("pbc", C.c_int * 3),
        ("dp_flag", C.c_int), ("gauge", C.c_int),
        ("mean_dp", C.c_double),
        ("cn_periodic_closure", C.c_int),
        ("use_graph", C.c_int),
        ("poisson_z", C.c_int),
        ("keep_sweeps", C.c_int),
        ("reserved", C.c_int * 6),
    ]


class NSKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("ms", C.c_double), ("launches", C.c_longlong)]


class NSDiag(C.Structure):
    _fields_ = [("max_div", C.c_double), ("probe", C.c_double), ("steps_done", C.c_longlong),
                ("euler_start_pending", C.c_int), ("reserved", C.c_int)]


class NSSubdomain(C.Structure):
    """Mirror of ``ns_subdomain``."""
    _fields_ = [("x0", C.c_int), ("y0", C.c_int), ("z0", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("nz", C.c_int), ("sub_tstep", C.c_int), ("reserved", C.c_int)]


class NSBatchConfig(C.Structure):
    """Mirror of ``ns_batch_config``."""
    _fields_ = [
        ("scheme", C.c_int), ("bc", C.c_int), ("pbc", C.c_int), ("restart", C.c_int), ("n_slots", C.c_int),
        ("mode", C.c_int), ("use_graph", C.c_int),
        ("nu", C.c_double), ("dt0", C.c_double), ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("grid", C.c_int * 16), ("using_ustar", C.c_int), ("dp_flag", C.c_int), ("reserved", C.c_int * 6),
    ]


# Every entry point of include/ns_gpu.h with its ctypes signature.
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    "ns_config_default": (C.c_int, [C.POINTER(NSConfig), C.c_int, C.c_int, C.c_int]),
    "ns_create": (C.c_int, [C.POINTER(NSConfig), C.POINTER(C.c_void_p)]),
    "ns_destroy": (C.c_int, [C.c_void_p]),
    "ns_last_error": (C.c_char_p, [C.c_void_p]),
    "ns_status_string": (C.c_char_p, [C.c_int]),
    "ns_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ns_synchronize": (C.c_int, [C.c_void_p]),
    "ns_set_state": (C.c_int, [C.c_void_p] + [_DP] * 7),
    "ns_get_state": (C.c_int, [C.c_void_p] + [_DP] * 7),
    "ns_set_faces": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(_DP)]),
    "ns_step": (C.c_int, [C.c_void_p, C.c_int]),
    "ns_set_mean_dp": (C.c_int, [C.c_void_p, C.c_double]),
    "ns_step_host": (C.c_int, [C.c_void_p] + [_DP] * 14),
    "ns_get_diag": (C.c_int, [C.c_void_p, C.POINTER(NSDiag)]),
    "ns_get_stage": (C.c_int, [C.c_void_p] + [_DP] * 4),
    "ns_get_sweeps": (C.c_int, [C.c_void_p] + [_DP] * 6),
    "ns_tgv": (C.c_int, [_DP, C.c_int, _DP, C.c_int, C.c_int, C.c_double, C.c_double] + [_DP] * 4),
    "ns_cal_conv": (C.c_int, [C.c_void_p] + [_DP] * 6),
    "ns_cal_diff": (C.c_int, [C.c_void_p] + [_DP] * 6),
    "ns_poisson": (C.c_int, [C.c_void_p, _DP, _DP]),
    "ns_adi": (C.c_int, [C.c_void_p, _DP, _DP, _DP]),
    "ns_profile": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(NSKernelTime), C.c_int, C.POINTER(C.c_int)]),
    "ns_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "ns_poisson_fft_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                         C.c_double, C.c_void_p]),
    "ns_version": (C.c_char_p, []),
    "ns_selftest_wait_timeout": (C.c_int, [C.c_double, _DP]),
    "ns_batch_config_default": (None, [C.POINTER(NSBatchConfig)]),
    "ns_batch_create": (C.c_int, [C.POINTER(NSBatchConfig), C.POINTER(NSSubdomain), C.c_int, C.POINTER(C.c_void_p)]),
    "ns_batch_destroy": (C.c_int, [C.c_void_p]),
    "ns_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "ns_batch_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ns_batch_init_from_parent": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ns_batch_set_state": (C.c_int, [C.c_void_p, C.c_int] + [_DP] * 7),
    "ns_batch_get_state": (C.c_int, [C.c_void_p, C.c_int] + [_DP] * 7),
    "ns_batch_capture": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_double]),
    "ns_batch_set_snapshot": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, C.POINTER(_DP), C.c_double]),
    "ns_batch_get_snapshot": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(_DP), _DP]),
    "ns_batch_set_sweep_faces": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(_DP)]),
    "ns_batch_get_sweep_faces": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(_DP)]),
    "ns_batch_advance": (C.c_int, [C.c_void_p, C.c_double]),
    "ns_batch_max_div": (C.c_int, [C.c_void_p, C.c_int, _DP]),
    "ns_batch_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "ns_batch_autotune": (C.c_int, [C.c_void_p, C.c_int]),
    "ns_batch_get_config": (C.c_int, [C.c_void_p, C.POINTER(NSBatchConfig)]),
    "ns_batch_profile": (C.c_int, [C.c_void_p, C.c_int, _DP]),
    "ns_spline_weights": (C.c_int, [_DP, C.c_int, C.c_double, C.POINTER(C.c_int), _DP]),
    "ns_error_metrics": (C.c_int, [C.c_void_p] + [_DP] * 5),
    "ns_batch_error_metrics": (C.c_int, [C.c_void_p, C.c_void_p, _DP]),
    "ns_write_err_csv": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _DP]),
    "ns_spectrum": (C.c_int, [C.c_void_p, _DP, _DP, C.POINTER(C.c_longlong), _DP]),
    "ns_adj_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "ns_adj_backward": (C.c_int, [C.c_void_p] + [_DP] * 9),
    "ns_vel_bc": (C.c_int, [C.c_void_p, _DP, _DP, _DP]),
    "ns_correct": (C.c_int, [C.c_void_p] + [_DP] * 8),
    # HDF5 files of the reference (host-only)
    "ns_h5_create": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    "ns_h5_open": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    "ns_h5_flush": (C.c_int, [C.c_void_p]),
    "ns_h5_close": (C.c_int, [C.c_void_p]),
    "ns_h5_last_error": (C.c_char_p, [C.c_void_p]),
    "ns_h5_group": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ns_h5_attr_int": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int]),
    "ns_h5_attr_double": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_double]),
    "ns_h5_attr_string": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p]),
    "ns_h5_write_double": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_longlong), _DP]),
    "ns_h5_dims": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "ns_h5_read_double": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_longlong), _DP]),
    "ns_h5_get_attr_int": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_longlong)]),
    "ns_h5_get_attr_double": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, _DP]),
    "ns_h5_get_attr_string": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]),
    "ns_h5_members": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_longlong, C.POINTER(C.c_longlong)]),
    "ns_h5_write_state": (C.c_int, [C.c_void_p, C.c_char_p, C.c_double, C.c_int, C.c_int]),
    "ns_h5_read_state": (C.c_int, [C.c_void_p, C.c_char_p, _DP, C.POINTER(C.c_int)]),
}

_lib = None


def load(path: str | None = None):
    """Load libns_gpu.so (build it first with ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libns_gpu.so not found at {p}: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
