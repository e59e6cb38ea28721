"""The one-CTA-per-node small path (small.cu) through the C ABI: against the
level-by-level path (small_max_n=-1), the closed forms and the oracle, with
several node chunks (the in-kernel ordered node sum across launches), subset
targets and batches whose small members run through the same kernel.

Tolerances: 1e-12 relative between the two GPU paths (both exact; they
differ only in rounding, FFT against schoolbook products); 1e-9 against the
closed forms and the oracle (quadrature error ~1e-12 on these workloads)."""
import numpy as np
import pytest

from tests.conftest import max_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def default_config(gpu_icm):
    gpu_icm.configure()
    yield
    gpu_icm.configure()


def _paths(gpu_icm, S, P, Q=256, **kw):
    gpu_icm.configure(**kw)
    a = gpu_icm.gpu_equity(S, P, Q=Q)
    launches = gpu_icm.last_launch_count()
    gpu_icm.configure(small_max_n=-1, **kw)
    b = gpu_icm.gpu_equity(S, P, Q=Q)
    gpu_icm.configure()
    return a, b, launches


@pytest.mark.parametrize("n,k", [(1, 1), (2, 1), (2, 2), (3, 3), (9, 3), (10, 10), (45, 9), (64, 64), (100, 15),
                                 (128, 128), (200, 40), (256, 64), (500, 30), (512, 64), (500, 200), (512, 256),
                                 (352, 300), (336, 336)])
def test_small_path_matches_level_path(gpu_icm, oracle, n, k):
    rng = np.random.default_rng(n * 1000 + k)
    S = 1e4 * np.exp(1.5 * rng.standard_normal(n))
    P = 0.8 ** np.arange(k)
    P /= P.sum()
    a, b, launches = _paths(gpu_icm, S, P)
    assert launches == 1                      # one launch per solve (one node chunk)
    assert max_rel(a, b, floor=1e-300) < 1e-12
    assert max_rel(a, oracle.equity(S, P, Q=256), floor=1e-15) < 1e-9


@pytest.mark.parametrize("B", [4, 8, 16, 32])
def test_small_path_block_sizes_closed_form(gpu_icm, B):
    """payout n - m, k = n: equity = V1 (closed form)."""
    rng = np.random.default_rng(B)
    n = 96
    S = 1 + 999 * rng.random(n)
    P = (n - np.arange(n)).astype(float)
    gpu_icm.configure(block_size=B)
    E = gpu_icm.gpu_equity(S, P)
    assert gpu_icm.last_launch_count() == 1
    T = S[:, None] + S[None, :]
    V1 = 1.0 + (S[:, None] / T).sum(axis=1) - 0.5
    assert max_rel(E, V1) < 1e-9


def test_small_path_oracle_wide_stacks(gpu_icm, oracle):
    """1e9:1 stacks (many leaf factors underflow to 0 at low nodes)."""
    rng = np.random.default_rng(7)
    for n, k in [(30, 30), (150, 20), (300, 300)]:
        S = 10.0 ** (9 * rng.random(n))
        P = (k - np.arange(k)).astype(float) ** 2
        P /= P.sum()
        E = gpu_icm.gpu_equity(S, P)
        ref = oracle.equity(S, P, Q=256)
        assert max_rel(E, ref, floor=1e-15) < 1e-9


def test_small_path_node_chunks(gpu_icm):
    """Several launches: the last CTA of each adds the chunk to the running sum."""
    rng = np.random.default_rng(11)
    S = 1e4 * np.exp(rng.standard_normal(77))
    P = 0.9 ** np.arange(20)
    full = gpu_icm.gpu_equity(S, P)
    gpu_icm.configure(q_chunk=37)
    chunked = gpu_icm.gpu_equity(S, P)
    assert gpu_icm.last_launch_count() == 7    # ceil(256 / 37)
    assert np.array_equal(full, chunked)       # node sums in the same order
    plan = gpu_icm.GpuPlan(S, len(P))
    r1, r2 = plan.equity(P), plan.equity(P)    # the CTA counter resets itself
    assert np.array_equal(r1, r2) and np.array_equal(r1, full)
    plan.close()


def test_small_path_subset(gpu_icm):
    rng = np.random.default_rng(12)
    S = 1e4 * np.exp(rng.standard_normal(180))
    P = 0.8 ** np.arange(30)
    targets = np.array([0, 5, 17, 90, 179])
    full = gpu_icm.gpu_equity(S, P)
    sub = gpu_icm.gpu_equity_subset(S, P, targets)
    assert np.array_equal(sub[targets], full[targets])
    mask = np.ones(len(S), bool)
    mask[targets] = False
    assert not sub[mask].any()


def test_batched_small_members_bitwise(gpu_icm):
    """Forest members on the small path equal single solves bit for bit."""
    rng = np.random.default_rng(13)
    ts = []
    for n in [1, 2, 5, 9, 30, 64, 100, 250, 400, 900, 3000, 12000]:
        k = max(1, int(np.ceil(0.15 * n)))
        ts.append((1e4 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(k)))
    res = gpu_icm.equity_batched(ts)
    for (S, P), E in zip(ts, res):
        assert np.array_equal(E, gpu_icm.gpu_equity(S, P)), len(S)
    b = gpu_icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
    r1 = b.equity([P for _, P in ts])
    b.set_options(graphs=False, profiling=True)
    r2 = b.equity([P for _, P in ts])
    assert any(s["name"] == "wl_small" for s in b.kernel_stats())
    b.close()
    for x, y, z in zip(r1, r2, res):
        assert np.array_equal(x, z) and np.array_equal(y, z)


@pytest.mark.parametrize("dist", ["uniform", "adversarial", "adv_1e9"])
def test_exhaustive_small_fields(gpu_icm, oracle, dist):
    """Every (n, k) with n <= 64, linear payouts, on the small path and on the
    level path (small_max_n = -1), each as one batch, against the oracle.
    Stacks as the reference's verify grid (bench/bench.c:65-88): uniform in
    [1, 100], one 1e4 stack among ones, one 1e9 stack among ones.  Tolerance
    1e-9 (1e-8 for the 1e9:1 field, the reference's own GPU gate)."""
    rng = np.random.default_rng(42)
    cases = []
    for n in range(1, 65):
        if dist == "uniform":
            S = rng.integers(1, 101, n).astype(float)
        else:
            S = np.ones(n)
            S[0] = 1e4 if dist == "adversarial" else 1e9
        for k in range(1, n + 1):
            cases.append((S, (k - np.arange(k)).astype(float)))
    small = gpu_icm.equity_batched(cases)
    gpu_icm.configure(small_max_n=-1)
    level = gpu_icm.equity_batched(cases)
    gpu_icm.configure()
    tol = 1e-8 if dist == "adv_1e9" else 1e-9
    for (S, P), a, b in zip(cases, small, level):
        ref = oracle.equity(S, P, Q=256)
        floor = 1e-12 * np.abs(ref).max()
        assert max_rel(a, ref, floor=floor) < tol, (len(S), len(P))
        assert max_rel(b, ref, floor=floor) < tol, (len(S), len(P))
