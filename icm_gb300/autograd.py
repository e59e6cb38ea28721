"""torch.autograd bindings of the GB300 engine.

``equity(stacks, payouts, Q=256, node_terms=False)`` returns the equities
as a torch tensor that autograd differentiates with respect to both inputs:
the forward pass is the GPU equity solve (``icm_equity``), the backward pass
the GPU adjoint passes (``icm_gb300_equity_vjp``) with the incoming gradient
as cotangent.  ``node_terms=True`` also differentiates the quadrature nodes'
dependence on max S, making the gradient the exact derivative of the
forward's Q-node formula.
Tensors may live on any device; the library's C ABI takes host arrays, so
values are copied through host memory (FP64).
"""
from __future__ import annotations

import numpy as np
import torch

import icm_gb300 as _icm


def _host(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


class ICMEquity(torch.autograd.Function):
    """equity = ICM(stacks, payouts); VJPs with respect to both."""

    @staticmethod
    def forward(ctx, stacks, payouts, Q=256, node_terms=False):
        ctx.save_for_backward(stacks, payouts)
        ctx.Q = int(Q)
        ctx.node_terms = bool(node_terms)
        eq = _icm.equity(_host(stacks), _host(payouts), Q=ctx.Q)
        return torch.from_numpy(eq).to(device=stacks.device, dtype=stacks.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        stacks, payouts = ctx.saved_tensors
        gS, gP = _icm.equity_vjp(_host(stacks), _host(payouts), _host(grad_out), Q=ctx.Q,
                                 node_terms=ctx.node_terms)
        gS_t = torch.from_numpy(gS).to(device=stacks.device, dtype=stacks.dtype)
        gP_t = torch.from_numpy(gP).to(device=payouts.device, dtype=payouts.dtype)
        return (gS_t if ctx.needs_input_grad[0] else None,
                gP_t if ctx.needs_input_grad[1] else None, None, None)


def equity(stacks: torch.Tensor, payouts: torch.Tensor, Q: int = 256, node_terms: bool = False) -> torch.Tensor:
    """Differentiable ICM equities (FP64)."""
    return ICMEquity.apply(stacks, payouts, Q, node_terms)
