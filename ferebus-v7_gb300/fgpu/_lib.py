"""ctypes binding of libfgpu.so (the C-ABI in include/fgpu.h).

The library is loaded from the package's ``_lib`` folder, where
``fgpu.build.build_library()`` puts it.  There is no fallback: if the shared
library is missing or was built for another machine, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB_PATH

_lib = None

# every symbol include/fgpu.h declares
EXPORTS = (
    "fgpu_create", "fgpu_nparams", "fgpu_loglik", "fgpu_loglik_batch", "fgpu_grad",
    "fgpu_plan_create", "fgpu_plan_run_device", "fgpu_plan_run", "fgpu_plan_destroy",
    "fgpu_destroy", "fgpu_last_error", "fgpu_version", "fgpu_last_launch_count",
    "fgpu_plan_set_profiling", "fgpu_plan_stage_times", "fgpu_loglik_noalloc",
    "fgpu_set_trailing_update", "fgpu_diag_exp", "fgpu_plan_waves", "fgpu_plan_partition",
    "fgpu_diag_wait", "fgpu_set_build_mode", "fgpu_diag_exp_fixed",
)

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)


class FgpuError(RuntimeError):
    """A negative status returned by the engine (argument, CUDA or allocation error)."""

    def __init__(self, code, msg):
        super().__init__(f"fgpu error {code}: {msg}")
        self.code = code


def load(path=None):
    """Load libfgpu.so once and declare the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run fgpu.build.build_library() (the CUDA engine has no CPU fallback)")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.fgpu_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, c_double_p, c_double_p, c_double_p,
                                c_int_p, C.c_int, C.c_int, C.c_double, C.c_int]
    lib.fgpu_create.restype = C.c_int
    lib.fgpu_nparams.argtypes = [vp]
    lib.fgpu_nparams.restype = C.c_int
    lib.fgpu_loglik.argtypes = [vp, c_double_p, C.c_int, c_double_p, c_int_p, c_double_p]
    lib.fgpu_loglik.restype = C.c_int
    lib.fgpu_loglik_batch.argtypes = [C.POINTER(vp), C.c_int, C.POINTER(c_double_p), c_double_p, c_int_p]
    lib.fgpu_loglik_batch.restype = C.c_int
    lib.fgpu_grad.argtypes = [vp, c_double_p, C.c_int, c_double_p, c_double_p, c_int_p]
    lib.fgpu_grad.restype = C.c_int
    lib.fgpu_plan_create.argtypes = [C.POINTER(vp), C.POINTER(vp), C.c_int, C.c_int]
    lib.fgpu_plan_create.restype = C.c_int
    lib.fgpu_plan_run_device.argtypes = [vp, vp, vp, vp, vp]
    lib.fgpu_plan_run_device.restype = C.c_int
    lib.fgpu_plan_run.argtypes = [vp, c_double_p, c_double_p, c_int_p]
    lib.fgpu_plan_run.restype = C.c_int
    lib.fgpu_plan_destroy.argtypes = [vp]
    lib.fgpu_plan_destroy.restype = None
    lib.fgpu_destroy.argtypes = [vp]
    lib.fgpu_destroy.restype = None
    lib.fgpu_last_error.argtypes = []
    lib.fgpu_last_error.restype = C.c_char_p
    lib.fgpu_version.argtypes = []
    lib.fgpu_version.restype = C.c_char_p
    lib.fgpu_last_launch_count.argtypes = []
    lib.fgpu_last_launch_count.restype = C.c_longlong
    lib.fgpu_plan_set_profiling.argtypes = [vp, C.c_int]
    lib.fgpu_plan_set_profiling.restype = C.c_int
    lib.fgpu_plan_stage_times.argtypes = [vp, c_double_p, c_int_p]
    lib.fgpu_plan_stage_times.restype = C.c_int
    lib.fgpu_loglik_noalloc.argtypes = [C.c_int, C.c_int, vp, vp, vp, c_int_p, C.c_int, C.c_int, C.c_double,
                                        C.c_int, vp, vp, vp, vp]
    lib.fgpu_loglik_noalloc.restype = C.c_int
    lib.fgpu_set_trailing_update.argtypes = [C.c_int]
    lib.fgpu_set_trailing_update.restype = C.c_int
    lib.fgpu_diag_exp.argtypes = [c_double_p, c_double_p, C.c_int]
    lib.fgpu_diag_exp.restype = C.c_int
    lib.fgpu_plan_waves.argtypes = [vp, c_int_p, C.POINTER(C.c_longlong)]
    lib.fgpu_plan_waves.restype = C.c_int
    lib.fgpu_plan_partition.argtypes = [C.POINTER(C.c_longlong), C.c_int, C.c_longlong, c_int_p, c_int_p]
    lib.fgpu_plan_partition.restype = C.c_int
    lib.fgpu_diag_wait.argtypes = [C.c_int, C.c_int]
    lib.fgpu_diag_wait.restype = C.c_int
    lib.fgpu_diag_exp_fixed.argtypes = [C.POINTER(C.c_ulonglong), C.c_int, c_double_p, C.c_int]
    lib.fgpu_diag_exp_fixed.restype = C.c_int
    lib.fgpu_set_build_mode.argtypes = [C.c_int]
    lib.fgpu_set_build_mode.restype = C.c_int
    _lib = lib
    return lib


def check(rc):
    if rc < 0:
        raise FgpuError(rc, _lib.fgpu_last_error().decode())
    return rc
