"""ctypes binding of the C ABI in include/owt_gpu.h.

There is no fallback: if ``libowt_gpu.so`` has not been built, loading fails
with an error that says how to build it.
"""
import ctypes as C
import os

import numpy as np

from .build import LIB

FIELDS = ["velx", "vely", "velz", "vorx", "vory", "vorz", "lmbx", "lmby", "lmbz", "Hv", "Hg",
          "vely_0", "vely_1", "vely_2", "vory_0", "vory_1", "vory_2",
          "Hv_0", "Hv_1", "Hv_2", "Hg_0", "Hg_1", "Hg_2"]
MEANS = ["lmbx_mean_0", "lmbx_mean_1", "lmbx_mean_2", "lmbz_mean_0", "lmbz_mean_1", "lmbz_mean_2",
         "velx_mean_0", "velx_mean_1", "velx_mean_2", "velz_mean_0", "velz_mean_1", "velz_mean_2"]
ROUTINES = {"get_vor_from_vel": 0, "Lamb_vec": 1, "nonlinear_source": 2, "solve_friction_force": 3,
            "time_Integration": 4}
PREC = {"fp64": 0, "mixed": 1}

OK = 0
STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NUMERIC", 4: "STATE", 5: "NOMEM"}


class OwtParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("dkx", C.c_double), ("dkz", C.c_double), ("alpha_mesh", C.c_double),
                ("nu", C.c_double), ("NX", C.c_int64), ("NY", C.c_int64), ("NZ", C.c_int64),
                ("precision", C.c_int32), ("device", C.c_int32), ("fd_order", C.c_int32)]


class OwtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{STATUS.get(code, code)}] {msg}")
        self.code = code


_lib = None
_dp = C.POINTER(C.c_double)
_h = C.c_void_p


def load(path=LIB):
    """Load libowt_gpu.so (once) and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`")
    L = C.CDLL(path)
    sig = {
        "owt_create": ([C.POINTER(OwtParams), C.POINTER(_h)], C.c_int),
        "owt_destroy": ([_h], C.c_int),
        "owt_last_error": ([_h], C.c_char_p),
        "owt_init_fields": ([_h, _dp, _dp, _dp], C.c_int),
        "owt_init_seeded": ([_h, C.c_uint64, C.c_double], C.c_int),
        "owt_band_factor_selftest": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
        "owt_convert_selftest": ([C.c_int64, C.c_uint64, C.POINTER(C.c_int64)], C.c_int),
        "owt_time_integration": ([_h, C.c_int64], C.c_int),
        "owt_call": ([_h, C.c_int], C.c_int),
        "owt_synchronize": ([_h], C.c_int),
        "owt_get_field": ([_h, C.c_int, _dp], C.c_int),
        "owt_set_field": ([_h, C.c_int, _dp], C.c_int),
        "owt_get_mean": ([_h, C.c_int, _dp], C.c_int),
        "owt_set_mean": ([_h, C.c_int, _dp], C.c_int),
        "owt_get_friction": ([_h, _dp], C.c_int),
        "owt_set_friction": ([_h, _dp], C.c_int),
        "owt_set_precision": ([_h, C.c_int], C.c_int),
        "owt_use_graph": ([_h, C.c_int], C.c_int),
        "owt_get_step": ([_h, C.POINTER(C.c_int64)], C.c_int),
        "owt_get_stream": ([_h, C.POINTER(C.c_void_p)], C.c_int),
        "owt_get_launch_count": ([_h, C.POINTER(C.c_int64)], C.c_int),
        "owt_get_grid": ([_h, _dp], C.c_int),
        "owt_dy_apply": ([_h, C.c_int, _dp, _dp], C.c_int),
        "owt_fourier2physical": ([_h, _dp, _dp], C.c_int),
        "owt_time_integration_host": ([_h, C.POINTER(_dp), _dp, _dp, _dp, _dp, _dp], C.c_int),
        "owt_physical2fourier": ([_h, _dp, _dp], C.c_int),
        "owt_enqueue_stage": ([_h, C.c_int], C.c_int),
        "owt_set_option": ([_h, C.c_int, C.c_int64], C.c_int),
        "owt_get_info": ([_h, C.c_int, C.POINTER(C.c_int64)], C.c_int),
        "owt_tuning_report": ([_h], C.c_char_p),
        "owt_setup_report": ([_h], C.c_char_p),
        "owt_statistics": ([_h, _dp], C.c_int),
        "owt_batch_create": ([C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)], C.c_int),
        "owt_batch_step": ([C.c_void_p, C.c_int64], C.c_int),
        "owt_batch_synchronize": ([C.c_void_p], C.c_int),
        "owt_batch_destroy": ([C.c_void_p], C.c_int),
        "owt_batch_get_stream": ([C.c_void_p, C.POINTER(C.c_void_p)], C.c_int),
        "owt_batch_get_launch_count": ([C.c_void_p, C.POINTER(C.c_int64)], C.c_int),
        "owt_batch_get_step_launches": ([C.c_void_p, C.POINTER(C.c_int64)], C.c_int),
        "owt_batch_tuning_report": ([C.c_void_p], C.c_char_p),
        "owt_checkpoint_bytes": ([_h, C.POINTER(C.c_int64)], C.c_int),
        "owt_checkpoint_save": ([_h, C.c_void_p, C.c_int64], C.c_int),
        "owt_checkpoint_load": ([_h, C.c_void_p, C.c_int64], C.c_int),
        "owt_dy1_noalloc": ([C.c_int64, C.c_int64, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "owt_state_keep": ([_h], C.c_int),
        "owt_state_restore": ([_h], C.c_int),
        "owt_set_wall_velocity": ([_h, _dp, _dp], C.c_int),
        "owt_get_wall_velocity": ([_h, _dp, _dp], C.c_int),
        "owt_drag_forward": ([_h, C.c_int64, C.c_int64, _dp], C.c_int),
        "owt_drag_backward": ([_h, C.c_double, _dp, _dp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def dptr(a):
    return a.ctypes.data_as(_dp)
