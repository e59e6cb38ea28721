"""Node chunks spread over several streams (IcmGb300Config.chunk_streams):
each chunk's nodes run as pieces of consecutive nodes on up to four streams,
each piece on its own node slots of the plan's arena, with the node sums
chained in node order.  So the equities equal the one-stream run's bit for
bit, whatever the piece count, the chunk size (several chunks, pieces of one
node, fewer nodes than streams), the level kinds (schoolbook, coefficient
FFT, spectral, multi-pass spectral), subsets, captured graphs and reuse."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def default_config(gpu_icm):
    gpu_icm.configure()
    yield
    gpu_icm.configure()


def _field(n, k, seed):
    rng = np.random.default_rng(seed)
    S = 10.0 ** (4 * rng.random(n))
    P = 0.9 ** np.arange(k)
    return S, P / P.sum()


def _run(gpu_icm, S, P, streams, q_chunk=0, Q=256, targets=None):
    gpu_icm.configure(chunk_streams=streams, q_chunk=q_chunk, small_max_n=-1)
    if targets is not None:
        return gpu_icm.gpu_equity_subset(S, P, targets, Q=Q)
    return gpu_icm.gpu_equity(S, P, Q=Q)


@pytest.mark.parametrize("n,k", [(300, 20), (5000, 120), (20000, 20000), (70000, 200)])
@pytest.mark.parametrize("streams", [2, 3, 4])
def test_streams_bitwise(gpu_icm, n, k, streams):
    S, P = _field(n, k, n + k)
    ref = _run(gpu_icm, S, P, 1)
    assert np.array_equal(_run(gpu_icm, S, P, streams), ref)


@pytest.mark.parametrize("q_chunk,Q", [(37, 256), (5, 64), (3, 16), (2, 3), (7, 2)])
def test_streams_chunking(gpu_icm, q_chunk, Q):
    """Chunks of q_chunk nodes: pieces of one node, more streams than the
    chunk's or the run's nodes, a last chunk shorter than the others."""
    S, P = _field(3000, 300, 11)
    ref = _run(gpu_icm, S, P, 1, q_chunk, Q)
    for streams in (2, 4):
        assert np.array_equal(_run(gpu_icm, S, P, streams, q_chunk, Q), ref), (streams, q_chunk, Q)


def test_streams_multipass_root(gpu_icm):
    """k = n = 40000: a spectral root too large for the one-kernel transform;
    its payout spectrum takes the multi-pass one (once, before the pieces)."""
    S, P = _field(40000, 40000, 3)
    ref = _run(gpu_icm, S, P, 1, 0, 64)
    assert np.array_equal(_run(gpu_icm, S, P, 4, 0, 64), ref)
    assert np.array_equal(_run(gpu_icm, S, P, 3, 10, 64), ref)


def test_streams_subset_and_graphs(gpu_icm):
    from icm_gb300._lib import IcmGpuOptions
    S, P = _field(9000, 900, 5)
    T = np.array([0, 17, 4500, 8999])
    ref = _run(gpu_icm, S, P, 1, targets=T)
    assert np.array_equal(_run(gpu_icm, S, P, 3, targets=T), ref)
    gpu_icm.configure(chunk_streams=1, small_max_n=-1)
    one = gpu_icm.GpuPlan(S, len(P))
    gpu_icm.configure(chunk_streams=4, q_chunk=50, small_max_n=-1)
    graphed = gpu_icm.GpuPlan(S, len(P), IcmGpuOptions(enable_graphs=1))
    P2 = np.linspace(1.0, 0.1, len(P))
    for Pr, Q in [(P, 256), (P2, 256), (P, 100), (P2, 256)]:
        assert np.array_equal(graphed.equity(Pr, Q=Q), one.equity(Pr, Q=Q)), Q
    one.close()
    graphed.close()


@pytest.mark.parametrize("n,k,q_chunk", [(3000, 400, 0), (16384, 2000, 0), (9000, 9000, 11), (700, 5, 3)])
def test_streams_vjp_bitwise(gpu_icm, n, k, q_chunk):
    """VJP plans run the forward tree and the adjoint passes of every piece on
    its stream; gradients (with and without the node terms) equal the
    one-stream run's bit for bit."""
    S, P = _field(n, k, 7 * n + k)
    cot = np.random.default_rng(n).standard_normal(n)
    gpu_icm.configure(chunk_streams=1, q_chunk=q_chunk, small_max_n=-1)
    refs = [gpu_icm.equity_vjp(S, P, cot, node_terms=t) for t in (False, True)]
    for streams in (2, 3, 4):
        gpu_icm.configure(chunk_streams=streams, q_chunk=q_chunk, small_max_n=-1)
        for t, (gS, gP) in zip((False, True), refs):
            a, b = gpu_icm.equity_vjp(S, P, cot, node_terms=t)
            assert np.array_equal(a, gS) and np.array_equal(b, gP), (streams, t)


def test_streams_random_shapes(gpu_icm):
    """Random fields, payout lengths, chunk sizes and Q: four streams equal
    one bit for bit."""
    rng = np.random.default_rng(2024)
    for _ in range(24):
        n = int(np.exp(rng.uniform(np.log(1600), np.log(30000))))
        k = int(rng.integers(1, n + 1)) if rng.random() < 0.5 else n
        Q = int(rng.choice([16, 64, 256]))
        qc = int(rng.choice([0, 0, 5, 17, 60]))
        S = 10.0 ** rng.uniform(0, float(rng.choice([2, 5, 9])), n)
        P = rng.random(k)
        ref = _run(gpu_icm, S, P, 1, qc, Q)
        assert np.array_equal(_run(gpu_icm, S, P, 4, qc, Q), ref), (n, k, Q, qc)


def test_tma_column_pass_bitwise(gpu_icm):
    """The largest levels' four-step column pass with its tile staged by a TMA
    tensor copy equals the pass with ordinary gathers bit for bit (drop-in
    field with two multi-pass levels, full and subset queries)."""
    from icm_gb300 import workloads as W
    from icm_gb300._lib import lib
    S, P, T = W.dropin(n=40000, n_targets=30)
    res, used = {}, {}
    for tma in (True, False):
        gpu_icm.configure(tma=tma)
        before = lib().icm_gb300_tma_launch_count()
        plan = gpu_icm.GpuPlan(S, len(P))
        full = plan.equity(P)
        plan.set_targets(T)
        res[tma] = (full, plan.equity(P))
        plan.close()
        used[tma] = lib().icm_gb300_tma_launch_count() - before
    gpu_icm.configure()
    assert used[True] > 0 and used[False] == 0   # the TMA pass ran, and only when asked for
    assert np.array_equal(res[True][0], res[False][0]) and np.array_equal(res[True][1], res[False][1])
