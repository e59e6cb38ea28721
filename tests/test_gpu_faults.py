"""Error paths without a device fault: the library's allocation hook makes
the n-th device allocation fail as an exhausted allocator would.  Every entry
point must report the failure (-1 / NULL with the error text, ICMError in
Python), leave nothing half-built, and give correct results on the next call.
Allocation order: small one-shot solves -- the per-thread buffer; plans --
arena, node table; batches -- arena, node tables, work lists; VJP plans --
plan arena, VJP buffers, node table."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def hook(gpu_icm):
    from icm_gb300._lib import lib
    yield lib().icm_gb300_test_fail_allocation
    lib().icm_gb300_test_fail_allocation(0)


def _tournaments(seed, sizes):
    rng = np.random.default_rng(seed)
    return [(1e4 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(max(1, n // 6))) for n in sizes]


@pytest.mark.parametrize("n,nth", [(40, 1), (5000, 1), (5000, 2)])   # one-shot small path; plan arena, node table
def test_single_solve_allocation_failure(gpu_icm, hook, n, nth):
    """Small fields run without a plan on a per-thread context that keeps its
    buffers; releasing them makes the next solve allocate again."""
    from icm_gb300._lib import lib
    (S, P), = _tournaments(n, [n])
    ref = gpu_icm.gpu_equity(S, P)
    lib().icm_gpu_release_pooled_memory()
    hook(nth)
    with pytest.raises(gpu_icm.ICMError, match="out of memory"):
        gpu_icm.gpu_equity(S, P)
    assert np.array_equal(gpu_icm.gpu_equity(S, P), ref)


@pytest.mark.parametrize("nth", [1, 2, 3])
def test_batch_allocation_failure(gpu_icm, hook, nth):
    ts = _tournaments(7, [9, 300, 4000])
    ref = gpu_icm.equity_batched(ts)
    hook(nth)
    with pytest.raises(gpu_icm.ICMError, match="out of memory"):
        gpu_icm.equity_batched(ts)
    for a, b in zip(gpu_icm.equity_batched(ts), ref):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("nth", [2, 3])
def test_reusable_batch_recovers_after_failed_run(gpu_icm, hook, nth):
    """A run that fails setting up its node tables or work lists leaves the
    batch usable: the next run prepares them again."""
    ts = _tournaments(8, [50, 2000, 7000])
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    Ps = [P for _, P in ts]
    hook(nth - 1)   # the arena exists: count from the run's first allocation
    with pytest.raises(gpu_icm.ICMError, match="out of memory"):
        b.equity(Ps)
    got = b.equity(Ps)
    b.close()
    for a, c in zip(got, gpu_icm.equity_batched(ts)):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("nth", [1, 2, 3])
def test_vjp_allocation_failure(gpu_icm, hook, nth):
    (S, P), = _tournaments(9, [3000])
    cot = np.random.default_rng(1).standard_normal(len(S))
    ref = gpu_icm.equity_vjp(S, P, cot)
    hook(nth)
    with pytest.raises(gpu_icm.ICMError, match="out of memory"):
        gpu_icm.equity_vjp(S, P, cot)
    got = gpu_icm.equity_vjp(S, P, cot)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    ts = _tournaments(10, [100, 2500])
    cots = [np.random.default_rng(2).standard_normal(len(S)) for S, _ in ts]
    refb = gpu_icm.equity_vjp_batched(ts, cots)
    hook(nth)
    with pytest.raises(gpu_icm.ICMError, match="out of memory"):
        gpu_icm.equity_vjp_batched(ts, cots)
    for (a, b), (c, d) in zip(gpu_icm.equity_vjp_batched(ts, cots), refb):
        assert np.array_equal(a, c) and np.array_equal(b, d)
