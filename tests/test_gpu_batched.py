"""Batched tournaments (work lists per tree-level step, CUDA-graph replay)
through the C ABI: every tournament's equities equal a single-tournament
solve bit for bit, and the oracle within 1e-9."""
import numpy as np
import pytest

from tests.conftest import max_rel
from icm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def default_config(gpu_icm):
    gpu_icm.configure()
    yield
    gpu_icm.configure()


def _uneven(seed, count, n_hi=3000):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.choice([1, 2, 3, 7, 8, 9, 16, 17, 33, 100, 257, 1000, n_hi]))
        k = int(rng.integers(1, n + 1))
        S = 10.0 ** (5 * rng.random(n))
        P = np.sort(rng.random(k))[::-1] + 0.01
        out.append((S, P))
    return out


def test_batched_equals_single_bitwise(gpu_icm):
    ts = _uneven(1, 40)
    res = gpu_icm.equity_batched(ts, Q=96)
    for (S, P), E in zip(ts, res):
        assert np.array_equal(E, gpu_icm.equity(S, P, Q=96)), (len(S), len(P))


def test_batched_against_oracle(gpu_icm, oracle):
    ts = _uneven(2, 24)
    res = gpu_icm.equity_batched(ts, Q=64)
    for (S, P), E in zip(ts, res):
        R = oracle.equity(S, P, Q=64, B=8, fft_min_deg=64)
        assert max_rel(E, R, floor=1e-300) < 1e-9, (len(S), len(P))


def test_batch_workload_sample_equals_single(gpu_icm):
    """Tournaments of the batched workload (n log-uniform in [9, 20000],
    k = ceil(0.15 n), lognormal stacks, geometric payouts 0.8)."""
    ts = W.batched(count=64)
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    assert b.info()["fallbacks"] == 0
    res = b.equity([P for _, P in ts])
    for i in range(0, 64, 7):
        S, P = ts[i]
        assert np.array_equal(res[i], gpu_icm.equity(S, P)), i
    b.close()


def test_graph_replay_and_q_change(gpu_icm):
    ts = _uneven(3, 30)
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    Ps = [P for _, P in ts]
    a = b.equity(Ps, Q=128)
    a2 = b.equity(Ps, Q=128)                       # graph replay
    for x, y in zip(a, a2):
        assert np.array_equal(x, y)
    c = b.equity([2.0 * P for P in Ps], Q=128)     # new payouts, same graph
    for x, y in zip(a, c):
        assert max_rel(y, 2.0 * x) < 1e-14
    d = b.equity(Ps, Q=40)                         # recapture for another Q
    for (S, P), y in zip(ts, d):
        assert np.array_equal(y, gpu_icm.equity(S, P, Q=40))
    b.set_options(graphs=False)
    e = b.equity(Ps, Q=128)                        # plain launches
    for x, y in zip(a, e):
        assert np.array_equal(x, y)
    b.close()


def test_fallback_members(gpu_icm):
    """Tournaments whose top levels need multi-pass transforms are solved by
    their own plans inside the batch; the others by the work lists."""
    rng = np.random.default_rng(9)
    big = (10.0 ** (3 * rng.random(40000)), np.linspace(1.0, 0.01, 40000))
    ts = _uneven(4, 6) + [big] + _uneven(5, 5)
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    info = b.info()
    assert info["fallbacks"] == 1 and info["members"] == len(ts) - 1
    res = b.equity([P for _, P in ts], Q=32)
    for (S, P), E in zip(ts, res):
        assert np.array_equal(E, gpu_icm.equity(S, P, Q=32)), len(S)
    b.close()


@pytest.mark.parametrize("coeff", [False, True])
@pytest.mark.parametrize("B,fft_min", [(4, 16), (16, 64), (8, 1 << 20)])
def test_batched_configurations(gpu_icm, B, fft_min, coeff):
    gpu_icm.configure(block_size=B, fft_min_degree=fft_min, coefficient_fft_only=coeff)
    ts = _uneven(6 + B, 16, n_hi=5000)
    res = gpu_icm.equity_batched(ts, Q=48)
    for (S, P), E in zip(ts, res):
        assert np.array_equal(E, gpu_icm.equity(S, P, Q=48)), (len(S), len(P))


def test_batch_q_chunking(gpu_icm):
    """Chunks of 5 nodes (several graph-captured chunks) give the same sums."""
    ts = _uneven(7, 12)
    ref = gpu_icm.equity_batched(ts, Q=33)
    gpu_icm.configure(q_chunk=5)
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    assert b.info()["q_chunk"] == 5
    res = b.equity([P for _, P in ts], Q=33)
    for x, y in zip(ref, res):
        assert np.array_equal(x, y)
    b.close()


def test_batch_profiling(gpu_icm):
    ts = W.batched(count=32)
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    b.set_options(profiling=True)
    b.equity([P for _, P in ts])
    ks = b.kernel_stats()
    names = {k["name"] for k in ks}
    assert {"wl_leaf", "wl_divide"} <= names
    assert all(k["ms"] > 0 and k["launches"] > 0 for k in ks)
    assert b.info()["device_ms"] > 0
    b.close()


def test_batched_closed_form(gpu_icm, oracle):
    """payout n - m with k = n in every tournament: equity = V1."""
    rng = np.random.default_rng(11)
    ts = []
    for n in (5, 64, 300, 2048, 4100):
        S = 1 + 999 * rng.random(n)
        ts.append((S, (n - np.arange(n)).astype(float)))
    res = gpu_icm.equity_batched(ts)
    for (S, _), E in zip(ts, res):
        assert max_rel(E, oracle.v1(S)) < 5e-12
