"""The linear engine (linear.cu, one warp per node, k <= 256) through the C
ABI: against the tree engine, the closed form and the oracle, across the
lane widths (k around 32, 64, 128, 256), checkpoint segments shorter than
the field, several node chunks, the zero prefix (exact shifts), subset
targets and batches.

Tolerances: 1e-12 relative between the engines (both exact; they differ in
rounding only); 1e-9 against the closed form and the oracle (quadrature
error ~1e-12 on these workloads)."""
import numpy as np
import pytest

from tests.conftest import max_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def default_config(gpu_icm):
    gpu_icm.configure()
    yield
    gpu_icm.configure()


def _both(gpu_icm, S, P, Q=256, **kw):
    gpu_icm.configure(engine="linear", **kw)
    a = gpu_icm.gpu_equity(S, P, Q=Q)
    launches = gpu_icm.last_launch_count()
    gpu_icm.configure(engine="tree", small_max_n=-1, **kw)
    b = gpu_icm.gpu_equity(S, P, Q=Q)
    gpu_icm.configure()
    return a, b, launches


@pytest.mark.parametrize("n,k", [(1, 1), (2, 1), (3, 2), (7, 7), (33, 5), (100, 31), (100, 32), (100, 33),
                                 (300, 64), (300, 65), (1000, 128), (1000, 129), (2000, 256), (5000, 17),
                                 (20000, 100)])
def test_linear_matches_tree(gpu_icm, n, k):
    rng = np.random.default_rng(n * 7 + k)
    S = 1e4 * np.exp(1.2 * rng.standard_normal(n))
    P = 0.85 ** np.arange(k)
    P /= P.sum()
    a, b, launches = _both(gpu_icm, S, P)
    assert launches == 3                       # linear, accumulate, scatter
    assert max_rel(a, b, floor=1e-300) < 1e-12


def test_linear_closed_form(gpu_icm):
    """payout n - m, k = n: equity = V1."""
    rng = np.random.default_rng(3)
    for n in (40, 200, 256):
        S = 1 + 999 * rng.random(n)
        P = (n - np.arange(n)).astype(float)
        gpu_icm.configure(engine="linear")
        E = gpu_icm.gpu_equity(S, P)
        T = S[:, None] + S[None, :]
        V1 = 1.0 + (S[:, None] / T).sum(axis=1) - 0.5
        assert max_rel(E, V1) < 1e-9


def test_linear_oracle_wide_stacks(gpu_icm, oracle):
    """1e9:1 stacks: long zero prefixes at the low nodes."""
    rng = np.random.default_rng(5)
    for n, k in [(500, 50), (3000, 200), (64, 64)]:
        S = 10.0 ** (9 * rng.random(n))
        P = (k - np.arange(k)).astype(float) ** 2
        P /= P.sum()
        gpu_icm.configure(engine="linear")
        E = gpu_icm.gpu_equity(S, P)
        assert max_rel(E, oracle.equity(S, P, Q=256), floor=1e-15) < 1e-9


def test_linear_zero_prefix_exact_and_chunks(gpu_icm):
    """Skipping the zero prefix is exact (its factors are x: shifts), and the
    node sums do not depend on the chunking."""
    rng = np.random.default_rng(6)
    S = 10.0 ** (6 * rng.random(3000))
    P = 0.9 ** np.arange(40)
    gpu_icm.configure(engine="linear")
    a = gpu_icm.gpu_equity(S, P)
    gpu_icm.configure(engine="linear", zero_prefix=False)
    b = gpu_icm.gpu_equity(S, P)
    gpu_icm.configure(engine="linear", q_chunk=37)
    c = gpu_icm.gpu_equity(S, P)
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_linear_subset_and_large_k(gpu_icm):
    rng = np.random.default_rng(9)
    S = 1e4 * np.exp(rng.standard_normal(1500))
    P = 0.8 ** np.arange(60)
    targets = np.array([0, 1, 700, 1499])
    gpu_icm.configure(engine="linear")
    full = gpu_icm.gpu_equity(S, P)
    sub = gpu_icm.gpu_equity_subset(S, P, targets)
    assert np.array_equal(sub[targets], full[targets])
    assert np.count_nonzero(sub) == len(targets)
    # k > 256: the tree engine serves the request
    P2 = 0.99 ** np.arange(400)
    E2 = gpu_icm.gpu_equity(S, P2)
    gpu_icm.configure()
    assert max_rel(E2, gpu_icm.gpu_equity(S, P2), floor=1e-300) < 1e-12


def test_linear_batched_bitwise(gpu_icm):
    rng = np.random.default_rng(10)
    ts = []
    for n in [1, 3, 40, 500, 2500, 9000]:
        k = min(n, max(1, int(np.ceil(0.02 * n))) + 3)
        ts.append((1e4 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(k)))
    gpu_icm.configure(engine="linear")
    res = gpu_icm.equity_batched(ts)
    for (S, P), E in zip(ts, res):
        assert np.array_equal(E, gpu_icm.gpu_equity(S, P)), len(S)
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    b.set_options(graphs=False, profiling=True)
    r = b.equity([P for _, P in ts])
    assert any(s["name"] == "wl_linear" for s in b.kernel_stats())
    b.close()
    for x, y in zip(r, res):
        assert np.array_equal(x, y)
