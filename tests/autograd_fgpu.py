"""torch.autograd.Function over the engine's likelihood and FP64 adjoint
(test harness only: the product's interface is the C-ABI).

``loglik(theta, engine)`` returns logL(theta) as a 0-d float64 tensor; its
backward multiplies the incoming gradient by d logL / d theta from
``fgpu_grad`` (1/2 tr((alpha alpha^T / s - K^-1) dK/dtheta), FP64, including
the noise parameter when it is optimised).
"""
import numpy as np
import torch


class _LogLik(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, engine):
        ll, g, info = engine.grad(theta.detach().cpu().numpy().astype(np.float64))
        if info != 0:
            raise ValueError(f"K is not positive definite (info={info})")
        ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
        return torch.tensor(ll, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None


def loglik(theta, engine):
    return _LogLik.apply(theta, engine)
