"""Quadrature nodes partitioned over the ranks of a torch.distributed group.

The Q quadrature nodes of one solve are independent: rank r of W solves the
contiguous node range node_ranges(Q, W, node_work(S, Q))[r] (equal work:
nodes at low y have long zero prefixes and cost less) on its own GPU (one plan,
icm_gb300_plan_equity_nodes) and one all-reduce sums the partial equities in
FP64.  The result equals the single-GPU equities to rounding (the all-reduce
adds the ranks' partial sums; a single GPU adds the nodes one by one).  This
is the multi-GPU form of the node loop: no data moves between GPUs during a
solve, only the final n-vector.

Batches of independent tournaments need no exchange at all: give each rank
its own tournaments (icm_gb300.equity_batched on each)."""
from __future__ import annotations

import numpy as np


def node_ranges(Q: int, world: int, weights=None):
    """Contiguous node ranges [b, e) of Q nodes over world ranks.

    Without weights the sizes differ by at most one (earlier ranks take the
    larger ones).  With per-node weights (node_work) rank r's range ends at
    the first node where the running weight reaches (r + 1) / world of the
    total, so the ranks' work differs by at most one node's weight."""
    if Q < 1 or world < 1:
        raise ValueError(f"need Q >= 1 and world >= 1, got Q={Q}, world={world}")
    if weights is None:
        base, extra = divmod(Q, world)
        out, b = [], 0
        for r in range(world):
            e = b + base + (1 if r < extra else 0)
            out.append((b, e))
            b = e
        return out
    w = np.asarray(weights, dtype=np.float64)
    if w.shape != (Q,) or np.any(w < 0):
        raise ValueError("weights must be Q non-negative numbers")
    cum = np.cumsum(w)
    total = float(cum[-1])
    out, b = [], 0
    for r in range(world):
        if r == world - 1:
            e = Q
        elif total <= 0.0:
            e = b
        else:
            e = int(np.searchsorted(cum, total * (r + 1) / world, side="left")) + 1
            e = min(max(e, b), Q)
        out.append((b, e))
        b = e
    return out


def node_work(stacks, Q: int):
    """Per node of the rule, the players outside its zero prefix (the tree
    work the engine does at that node; 0 for skipped nodes of weight 0), from
    the library's own node rule on the host (icm_gb300_node_work)."""
    import ctypes
    from ._lib import ICMError, lib
    S = np.ascontiguousarray(stacks, dtype=np.float64)
    out = np.zeros(int(Q), dtype=np.int32)
    if lib().icm_gb300_node_work(len(S), S.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(Q),
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return out


def _gpu_partial(stacks, payouts, Q, q_begin, q_end):
    from . import GpuPlan
    plan = GpuPlan(stacks, len(payouts))
    try:
        return plan.equity(payouts, Q=Q, nodes=(q_begin, q_end))
    finally:
        plan.close()


def equity(stacks, payouts, Q: int = 256, group=None, partial=None, balance=True):
    """Equities of one tournament with the nodes split over the group's ranks.

    Every rank passes the same stacks, payouts and Q and receives the full
    equities.  ``partial(stacks, payouts, Q, q_begin, q_end)`` computes one
    rank's part (default: a plan on this rank's current GPU).  balance=True
    cuts the node ranges by node_work (equal work per rank), else by node
    count.  NCCL groups reduce on the current CUDA device, others (gloo) on
    the host."""
    import torch
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    weights = node_work(stacks, Q) if balance else None
    qb, qe = node_ranges(int(Q), world, weights)[rank]
    part = (partial or _gpu_partial)(np.asarray(stacks, dtype=np.float64), np.asarray(payouts, dtype=np.float64),
                                     int(Q), qb, qe)
    t = torch.from_numpy(np.ascontiguousarray(part, dtype=np.float64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
