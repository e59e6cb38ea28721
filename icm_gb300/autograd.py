"""torch.autograd bindings of the GB300 engine.

``equity(stacks, payouts, Q=256, node_terms=False)`` returns the equities
as a torch tensor that autograd differentiates with respect to both inputs:
the forward pass is the GPU equity solve, the backward pass the GPU adjoint
passes with the incoming gradient as cotangent.  ``node_terms=True`` also
differentiates the quadrature nodes' dependence on max S, making the
gradient the exact derivative of the forward's Q-node formula.

CUDA tensors on the library's device stay there: payouts, equities,
cotangents and gradients go through the stream-ordered device entry points
(icm_gb300_plan_equity_dev, icm_gb300_vjp_run_dev) on torch's current
stream; only the stacks are read on the host, where the engine sorts the
players.  Other tensors (CPU, or another device) go through host arrays
(``icm_equity``, ``icm_gb300_equity_vjp``).  All values are FP64.
"""
from __future__ import annotations

import numpy as np
import torch

import icm_gb300 as _icm


def _host(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


def _on_library_device(*ts: torch.Tensor) -> bool:
    """True when every tensor is a CUDA tensor on the device the library runs on."""
    if not all(t.is_cuda for t in ts):
        return False
    import ctypes
    from ._lib import lib
    _icm._auto_init()
    dev = ctypes.c_int(-1)
    lib().icm_gb300_current_device(ctypes.byref(dev))
    return all(t.device.index == dev.value for t in ts)


def _dev64(t: torch.Tensor) -> torch.Tensor:
    return t.detach().to(torch.float64).contiguous()


class ICMEquity(torch.autograd.Function):
    """equity = ICM(stacks, payouts); VJPs with respect to both."""

    @staticmethod
    def forward(ctx, stacks, payouts, Q=256, node_terms=False):
        ctx.save_for_backward(stacks, payouts)
        ctx.Q = int(Q)
        ctx.node_terms = bool(node_terms)
        if _on_library_device(stacks, payouts):
            P = _dev64(payouts)
            out = torch.empty(stacks.shape[0], dtype=torch.float64, device=stacks.device)
            plan = _icm.GpuPlan(_host(stacks), P.shape[0])
            try:
                plan.equity_device(P.data_ptr(), out.data_ptr(), torch.cuda.current_stream(stacks.device).cuda_stream,
                                   Q=ctx.Q)
            finally:
                plan.close()   # waits for the plan's own work (its buffers are freed)
            return out.to(stacks.dtype)
        eq = _icm.equity(_host(stacks), _host(payouts), Q=ctx.Q)
        return torch.from_numpy(eq).to(device=stacks.device, dtype=stacks.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        stacks, payouts = ctx.saved_tensors
        if _on_library_device(stacks, payouts, grad_out):
            P, C = _dev64(payouts), _dev64(grad_out)
            gS = torch.empty(stacks.shape[0], dtype=torch.float64, device=stacks.device)
            gP = torch.empty(P.shape[0], dtype=torch.float64, device=stacks.device)
            plan = _icm.VjpPlan(_host(stacks), P.shape[0])
            try:
                plan.run_device(P.data_ptr(), C.data_ptr(), gS.data_ptr(), gP.data_ptr(),
                                torch.cuda.current_stream(stacks.device).cuda_stream, Q=ctx.Q,
                                node_terms=ctx.node_terms)
            finally:
                plan.close()
            gS_t, gP_t = gS.to(stacks.dtype), gP.to(payouts.dtype)
        else:
            gS, gP = _icm.equity_vjp(_host(stacks), _host(payouts), _host(grad_out), Q=ctx.Q,
                                     node_terms=ctx.node_terms)
            gS_t = torch.from_numpy(gS).to(device=stacks.device, dtype=stacks.dtype)
            gP_t = torch.from_numpy(gP).to(device=payouts.device, dtype=payouts.dtype)
        return (gS_t if ctx.needs_input_grad[0] else None,
                gP_t if ctx.needs_input_grad[1] else None, None, None)


def equity(stacks: torch.Tensor, payouts: torch.Tensor, Q: int = 256, node_terms: bool = False) -> torch.Tensor:
    """Differentiable ICM equities (FP64)."""
    return ICMEquity.apply(stacks, payouts, Q, node_terms)
