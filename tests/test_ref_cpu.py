"""The C restatement of the reference's OpenMP CPU path (oracle/ref_cpu.c,
built by oracle/build_ref.py) -- the timed CPU baseline and the reference
arm of the benchmark -- against the golden fixtures, on the CPU.

It is one more FP64 evaluation of the reference's formulas (its own
distance tensors, dgemv, dpotrf / dpotrs from the same OpenBLAS), so it is
held to the engine's bar (conftest.parity_tol against the extended-precision
value) on every fixture whose kernel it implements (rbf and periodic leaves,
sums and products: the benchmark shapes), runs its particles on two OpenMP
threads, and reports a non-positive-definite K with the LAPACK pivot column.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_case, parity_tol
from oracle import gpr_oracle as O

RESTATED = {O.RBF, O.PERIODIC}


def _restated(name):
    c = load_case(name)
    return all(n[1] in RESTATED for n in O.parse_kspec([int(v) for v in c["kspec"]]) if n[0] == "leaf")


@pytest.mark.parametrize("name", [n for n in golden_cases() if _restated(n)])
def test_c_restatement_meets_the_parity_bar(name):
    from oracle.build_ref import RefCPU
    c = load_case(name)
    ref = RefCPU(c["X"], c["y"], c["mu"], [int(v) for v in c["kspec"]], int(c["likelihood"]), float(c["noise"]),
                 bool(c["optimise_noise"]))
    try:
        ll, info = ref.loglik_batch(np.asarray(c["thetas"]), 2)
    finally:
        ref.close()
    for k in range(len(ll)):
        assert info[k] == int(c["info"][k]), (k, info[k], c["info"][k])
        if info[k] != 0:
            continue
        tol = parity_tol(float(c["ll_exact"][k]), float(c["ll"][k]), float(c["fp64_err"][k]))
        assert abs(ll[k] - c["ll_exact"][k]) <= tol, (k, ll[k], c["ll_exact"][k], tol)


def test_unrestated_kernels_are_an_error():
    from oracle.build_ref import RefCPU
    c = load_case("rbf_plus_constant")
    ref = RefCPU(c["X"], c["y"], c["mu"], [int(v) for v in c["kspec"]], int(c["likelihood"]), float(c["noise"]))
    try:
        with pytest.raises(RuntimeError, match="not in the CPU restatement"):
            ref.loglik_batch(np.asarray(c["thetas"][:1]), 1)
    finally:
        ref.close()
