"""The C-ABI library: it builds for sm_103a, loads, exports every symbol
include/fgpu.h declares, and reports errors without a GPU (no compute)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "fgpu.h")).read()
    return sorted(set(re.findall(r"\b(fgpu_[a-z_]+)\s*\(", src)))


def test_header_declarations_match_binding():
    from fgpu._lib import EXPORTS
    assert sorted(EXPORTS) == declared_symbols()


def test_library_exports_every_declared_symbol(lib):
    from fgpu.build import LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    for sym in declared_symbols():
        assert sym in exported, sym
        assert getattr(lib, sym) is not None


def test_version_string(lib):
    assert b"sm_103a" in lib.fgpu_version()


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_create_without_device_fails_cleanly(lib):
    from fgpu import _lib
    X = np.asfortranarray(np.random.default_rng(0).normal(size=(10, 2)))
    y = np.zeros(10)
    ks = (C.c_int * 4)(1, 2, 1, 2)
    h = C.c_void_p()
    rc = lib.fgpu_create(C.byref(h), 10, 2, X.ctypes.data_as(_lib.c_double_p), y.ctypes.data_as(_lib.c_double_p),
                         y.ctypes.data_as(_lib.c_double_p), ks, 4, 0, 1e-10, 0)
    assert rc == -4 and h.value is None
    assert b"device" in lib.fgpu_last_error()


def test_argument_errors_need_no_device(lib):
    from fgpu import _lib
    h = C.c_void_p()
    y = np.zeros(4)
    ks = (C.c_int * 3)(1, 1, 1)
    dp = y.ctypes.data_as(_lib.c_double_p)
    assert lib.fgpu_create(C.byref(h), 0, 1, dp, dp, dp, ks, 3, 0, 0.0, 0) == -1
    assert lib.fgpu_create(C.byref(h), 4, 1, dp, dp, dp, ks, 3, 7, 0.0, 0) == -1
    assert lib.fgpu_create(C.byref(h), 4, 1, dp, dp, None, ks, 3, 0, 0.0, 0) == -1
    assert lib.fgpu_loglik(None, dp, 1, None, None, None) == -1
    assert lib.fgpu_plan_create(C.byref(h), None, 0, 1) == -1
    assert b"NULL" in lib.fgpu_last_error() or b"bad" in lib.fgpu_last_error()
    for mode in (0, 1, 2):
        assert lib.fgpu_plan_set_profiling(None, mode) == -1
    assert b"NULL" in lib.fgpu_last_error()
