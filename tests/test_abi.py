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


_C_HOST = r"""
#include "fgpu.h"
#include <stdio.h>
#include <string.h>
int main(void) {
  long long bytes[4] = {40, 30, 20, 10};
  int wave_of[4], nwaves = 0;
  if (strstr(fgpu_version(), "sm_103a") == NULL) return 2;
  if (fgpu_plan_partition(bytes, 4, 50, wave_of, &nwaves) != 0) return 3;
  printf("%d %d %d %d %d\n", nwaves, wave_of[0], wave_of[1], wave_of[2], wave_of[3]);
  if (fgpu_loglik(NULL, NULL, 0, NULL, NULL, NULL) != FGPU_EINVAL) return 4;
  printf("%s\n", fgpu_last_error());
  return 0;
}
"""


@pytest.mark.parametrize("compiler", [["gcc", "-std=c99", "-x", "c"], ["g++", "-std=c++17", "-x", "c++"]])
def test_header_serves_a_c_host(lib, tmp_path, compiler):
    """A plain C (and a C++) program includes include/fgpu.h with every
    warning an error, links libfgpu.so and calls host-only entry points:
    the wave partition (40, 30, 20, 10 bytes under a budget of 50: waves
    0 | 1 1 | 2) and an argument error."""
    import shutil
    from fgpu.build import LIB_DIR
    if shutil.which(compiler[0]) is None:
        pytest.skip(f"{compiler[0]} not installed")
    src = tmp_path / "host.c"
    src.write_text(_C_HOST)
    exe = tmp_path / "host"
    cmd = [*compiler, "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"), str(src),
           "-x", "none", "-L", LIB_DIR, "-lfgpu", f"-Wl,-rpath,{LIB_DIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    lines = r.stdout.splitlines()
    assert lines[0] == "3 0 1 1 2"
    assert lines[1] == "NULL argument"


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
