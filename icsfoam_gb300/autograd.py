"""PyTorch autograd binding of the residual source and its exact derivatives.

``residual(case, W)`` returns the residual source R V (the vector
``ics_residual`` computes) for the conservative state ``W`` [N, 5] as a
differentiable torch function: its backward pass is the exact vector-Jacobian
product ``ics_vjp`` (boundary values held at the case's current ones), so a
scalar functional of the residual can be back-propagated to the state, e.g.
for an adjoint right-hand side.  ``jvp(case, W, v)`` is the forward-mode
product ``ics_jvp``.

Device tensors are passed to the library by pointer after the current torch
stream has been synchronised; the library synchronises its own stream before
returning, so no copy goes through the host on the backward pass.
"""

from __future__ import annotations

import numpy as np
import torch


def _set_state(case, W: torch.Tensor):
    case.set_conservative(W.detach().to("cpu", torch.float64).numpy())


class _Residual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, W, case):
        _set_state(case, W)
        src = torch.from_numpy(case.residual()).to(W.device)
        ctx.case = case
        ctx.save_for_backward(W.detach().clone())
        return src

    @staticmethod
    def backward(ctx, g):
        (W,) = ctx.saved_tensors
        case = ctx.case
        _set_state(case, W)
        u = g.detach().to(torch.float64).contiguous()
        if u.is_cuda:
            out = torch.empty_like(u)
            torch.cuda.current_stream(u.device).synchronize()
            case.vjp_device(u.data_ptr(), out.data_ptr())
        else:
            out = torch.from_numpy(case.vjp(u.numpy()))
        return out.to(W.dtype), None


def residual(case, W: torch.Tensor) -> torch.Tensor:
    """Residual source R V of ``case`` at state ``W`` [N, 5] (differentiable)."""
    if W.shape != (case.N, 5):
        raise ValueError("W must be [n_cells, 5]")
    return _Residual.apply(W, case)


def jvp(case, W: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    """d(R V)/dW v at ``W`` (forward mode, exact)."""
    _set_state(case, W)
    vv = v.detach().to(torch.float64).contiguous()
    if vv.is_cuda:
        out = torch.empty_like(vv)
        torch.cuda.current_stream(vv.device).synchronize()
        case.jvp_device(vv.data_ptr(), out.data_ptr())
        return out
    return torch.from_numpy(case.jvp(np.asarray(vv.numpy())))
