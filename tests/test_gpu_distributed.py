"""The node-range entry point (icm_gb300_plan_equity_nodes) on the GPU: the
parts of a partition of [0, Q) add up to the full equities (to rounding:
1e-12 relative, the full run adds the nodes one by one), the whole range
equals the full run bit for bit, an empty range gives zeros, invalid ranges
fail; and the distributed driver on a one-rank gloo group."""
import os
import socket

import numpy as np
import pytest

from tests.conftest import max_rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(300, 300), (5000, 300), (40000, 40000)])
def test_node_ranges_add_up(gpu_icm, n, k):
    from icm_gb300._lib import IcmGpuOptions
    from icm_gb300.distributed import node_ranges
    rng = np.random.default_rng(n)
    S = 10.0 ** (5 * rng.random(n))
    P = 0.9 ** np.arange(k)
    for opts in (None, IcmGpuOptions(enable_graphs=1)):
        plan = gpu_icm.GpuPlan(S, k, opts)
        full = plan.equity(P)
        assert np.array_equal(plan.equity(P, nodes=(0, 256)), full)
        for W in (2, 3, 7):
            parts = [plan.equity(P, nodes=r) for r in node_ranges(256, W)]
            assert max_rel(np.sum(parts, axis=0), full, floor=1e-300) < 1e-12, W
        assert np.array_equal(plan.equity(P, nodes=(9, 9)), np.zeros(n))
        for bad in ((5, 3), (-1, 2), (0, 257)):
            with pytest.raises(gpu_icm.ICMError):
                plan.equity(P, nodes=bad)
        assert np.array_equal(plan.equity(P), full)   # the plan is unchanged by the failures
        plan.close()


@pytest.mark.parametrize("backend", ["gloo", "nccl"])
def test_distributed_one_rank(gpu_icm, backend):
    """One rank: its range is [0, Q) and the all-reduce (on the host for gloo,
    on the device for NCCL) leaves the equities unchanged."""
    import torch
    import torch.distributed as dist
    from icm_gb300 import distributed as D
    if backend == "nccl" and not dist.is_nccl_available():
        pytest.skip("no NCCL in this torch build")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    if backend == "nccl":
        torch.cuda.set_device(0)
    dist.init_process_group(backend, rank=0, world_size=1)
    try:
        rng = np.random.default_rng(2)
        S = 1e4 * np.exp(rng.standard_normal(3000))
        P = 0.8 ** np.arange(200)
        assert np.array_equal(D.equity(S, P), gpu_icm.gpu_equity(S, P))
    finally:
        dist.destroy_process_group()
