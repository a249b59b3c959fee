"""Build recipe for the oracle's C restatement (oracle/ref_cpu.c -> oracle/_ref/libref_cpu.so).

TEST / BENCHMARK INFRASTRUCTURE ONLY.  FEREBUS-v7 itself is Fortran and is
not buildable on these machines (no Fortran compiler; its toml-f submodule is
absent), so there is no ``oracle/_ref`` build of the reference sources; the
library built here is the restatement ("port") used as the timed CPU
baseline and by ``bench.py --impl reference``.  Output goes to
``oracle/_ref/`` (git-ignored, shipped to the GPU machine with the tree).
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_cpu.so")
SRC = os.path.join(HERE, "ref_cpu.c")


def build_ref(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", LIB, SRC, "-ldl", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the CPU restatement failed:\n" + r.stdout + r.stderr)
    return LIB


def openblas_path():
    """scipy's bundled OpenBLAS (provides dgemv / dpotrf / dpotrs)."""
    import scipy
    base = os.path.dirname(scipy.__file__)
    cands = glob.glob(os.path.join(base, "..", "scipy.libs", "libscipy_openblas*.so*"))
    cands += glob.glob(os.path.join(base, ".dylibs", "libscipy_openblas*"))
    if not cands:
        raise FileNotFoundError("no scipy_openblas library found")
    return os.path.abspath(cands[0])


class RefCPU:
    """ctypes handle on one data set in the C restatement."""

    def __init__(self, X, y, mu, kspec, likelihood, noise, optimise_noise=False):
        import numpy as np
        lib = C.CDLL(build_ref())
        lib.ref_load_blas.argtypes = [C.c_char_p]
        lib.ref_create.restype = C.c_void_p
        lib.ref_create.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                   C.c_int, C.c_double, C.c_int]
        lib.ref_loglik_batch.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_int]
        lib.ref_destroy.argtypes = [C.c_void_p]
        lib.ref_last_error.restype = C.c_char_p
        if lib.ref_load_blas(openblas_path().encode()) != 0:
            raise RuntimeError(lib.ref_last_error().decode())
        self.lib = lib
        self.X = np.asfortranarray(X, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.mu = np.ascontiguousarray(mu if mu is not None else np.zeros(len(y)), dtype=np.float64)
        self.ks = np.ascontiguousarray(kspec, dtype=np.int32)
        n, d = self.X.shape
        self.h = lib.ref_create(n, d, self.X.ctypes.data, self.y.ctypes.data, self.mu.ctypes.data,
                                self.ks.ctypes.data, len(self.ks), likelihood, noise, 1 if optimise_noise else 0)
        if not self.h:
            raise MemoryError(lib.ref_last_error().decode())

    def loglik_batch(self, thetas, nthreads):
        import numpy as np
        th = np.ascontiguousarray(thetas, dtype=np.float64)
        S = th.shape[0]
        ll = np.empty(S)
        info = np.empty(S, dtype=np.int32)
        rc = self.lib.ref_loglik_batch(self.h, S, th.ctypes.data, th.shape[1], ll.ctypes.data, info.ctypes.data,
                                       nthreads)
        if rc != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())
        return ll, info

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = None


if __name__ == "__main__":
    print(build_ref(force=True))
