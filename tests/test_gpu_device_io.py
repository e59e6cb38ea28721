"""Stream-ordered runs on device memory (icm_gb300_plan_equity_dev,
icm_gb300_vjp_run_dev) against the host-array entry points, and the autograd
binding on CUDA tensors against its host path.  The same kernels run on the
same inputs, so results are compared bit for bit."""
import numpy as np
import pytest

from icm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _cuda(a):
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device="cuda:0")


@pytest.mark.parametrize("case", ["small", "dropin_20000", "trunc"])
def test_plan_equity_device_matches_host(gpu_icm, case):
    if case == "small":
        S, P = W.plain_small(n=300, k=40)
    elif case == "dropin_20000":
        S, P, _ = W.dropin(n=20000)
    else:
        rng = np.random.default_rng(4)
        S, P = 1e4 * np.exp(rng.standard_normal(9000)), W.geometric_payout(1200, 0.99)
    plan = gpu_icm.GpuPlan(S, len(P))
    ref = plan.equity(P)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):   # the caller's own stream, not the default one
        Pd = _cuda(P)
        out = torch.full((len(S),), float("nan"), dtype=torch.float64, device="cuda:0")
        for _ in range(2):   # a second run on the same buffers
            plan.equity_device(Pd.data_ptr(), out.data_ptr(), side.cuda_stream)
        got = out.cpu()   # ordered after the run on this stream
    plan.close()
    assert np.array_equal(got.numpy(), ref)


@pytest.mark.parametrize("node_terms", [False, True])
def test_vjp_run_device_matches_host(gpu_icm, node_terms):
    S, P, cot = W.vjp(n=6000, k=700)
    plan = gpu_icm.VjpPlan(S, len(P))
    gS, gP = plan.run(P, cot, node_terms=node_terms)
    Pd, Cd = _cuda(P), _cuda(cot)
    dS = torch.empty(len(S), dtype=torch.float64, device="cuda:0")
    dP = torch.empty(len(P), dtype=torch.float64, device="cuda:0")
    plan.run_device(Pd.data_ptr(), Cd.data_ptr(), dS.data_ptr(), dP.data_ptr(),
                    torch.cuda.current_stream().cuda_stream, node_terms=node_terms)
    plan.close()
    assert np.array_equal(dS.cpu().numpy(), gS) and np.array_equal(dP.cpu().numpy(), gP)


def test_device_entry_points_reject_host_memory(gpu_icm):
    S, P = W.plain_small(n=200, k=20)
    plan = gpu_icm.GpuPlan(S, len(P))
    out = torch.empty(len(S), dtype=torch.float64, device="cuda:0")
    host = np.ascontiguousarray(P)
    with pytest.raises(gpu_icm.ICMError, match="not device memory"):
        plan.equity_device(host.ctypes.data, out.data_ptr(), 0)
    plan.close()


def test_autograd_on_cuda_tensors_matches_host_path(gpu_icm):
    from icm_gb300.autograd import equity
    S, P, cot = W.vjp(n=3000, k=400)
    res = {}
    for dev in ("cpu", "cuda:0"):
        s = torch.tensor(S, dtype=torch.float64, device=dev, requires_grad=True)
        p = torch.tensor(P, dtype=torch.float64, device=dev, requires_grad=True)
        e = equity(s, p)
        assert e.device == s.device
        (e * torch.tensor(cot, dtype=torch.float64, device=dev)).sum().backward()
        res[dev] = (e.detach().cpu().numpy(), s.grad.cpu().numpy(), p.grad.cpu().numpy())
    for a, b in zip(res["cpu"], res["cuda:0"]):
        assert np.array_equal(a, b)
