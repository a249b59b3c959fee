"""fgpu: GB300 engine for FEREBUS-v7's GPR log-likelihood hot path.

The compute path is the CUDA library ``libfgpu.so`` (C-ABI, include/fgpu.h).
This package holds the host-side mirror of the reference's interface
(``GaussianProcessRegressor`` cost function, batched swarm evaluation), the
kernel-expression parser, the nvcc build and seeded synthetic inputs.
"""
from .kernel_spec import (CONSTANT, LINEAR, PERIODIC, PROD, RBF, RBF_CYCLIC, SUM, build_kspec,
                          nparams, parse_expression)
from .gpr import (CONCENTRATED, MARGINAL, Engine, GaussianProcessRegressor, IterResult, Plan,
                  loglik_batch)

__all__ = [
    "RBF", "PERIODIC", "RBF_CYCLIC", "LINEAR", "CONSTANT", "SUM", "PROD", "build_kspec", "nparams",
    "parse_expression", "MARGINAL", "CONCENTRATED", "Engine", "GaussianProcessRegressor",
    "IterResult", "Plan", "loglik_batch",
]
