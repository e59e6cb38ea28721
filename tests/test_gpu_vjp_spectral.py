"""VJPs through spectral tree levels (vjp_spec.cu) against the same VJPs
with every level on coefficients (vjp_spectral_min_degree = -1).

The two compute the same derivative with different transforms, so they
agree to FFT rounding: 5e-11 of the gradient's largest entry (1e-11 to
2e-11 seen where stacks spread over e^{+-7.5}, far less otherwise).  The cases
cover a spectral band reaching the root (k = n) and one ending below it
(k < n: the band's top converts the coefficient Pbar handed down and writes
coefficient gbar), the band's bottom at the leaf level and above
coefficient levels, lone parents (odd node counts), wholly-zero nodes (wide
stacks), node terms, and levels whose transforms take several passes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 5e-11


@pytest.fixture(autouse=True)
def default_config(gpu_icm):
    gpu_icm.configure()
    yield
    gpu_icm.configure()


def _case(n, k, sig, seed):
    rng = np.random.default_rng(seed)
    S = 1e4 * np.exp(sig * rng.standard_normal(n))
    P = 0.9 ** np.arange(k)
    cot = rng.standard_normal(n)
    return S, P, cot


def _pair(gpu_icm, S, P, cot, Q, node_terms=False, **cfg):
    gpu_icm.configure(**{**cfg, "vjp_spectral_min_degree": -1})
    ref = gpu_icm.equity_vjp(S, P, cot, Q=Q, node_terms=node_terms)
    gpu_icm.configure(**cfg)
    got = gpu_icm.equity_vjp(S, P, cot, Q=Q, node_terms=node_terms)
    return got, ref


def _close(got, ref, what):
    for a, b, name in ((got[0], ref[0], "dL/dS"), (got[1], ref[1], "dL/dpayout")):
        scale = np.abs(b).max()
        assert np.all(np.isfinite(a)), (what, name)
        assert np.abs(a - b).max() <= TOL * scale, (what, name, np.abs(a - b).max() / scale)


def _kinds(gpu_icm, n, k, B, fm, flags=2):
    import ctypes
    from icm_gb300._lib import lib
    why = ctypes.create_string_buffer(512)
    assert lib().icm_gb300_check_geometry(n, k, B, fm, flags, why, 512) == 0, why.value
    return [int(x) for x in why.value.decode().split()[1:]]


@pytest.mark.parametrize("n,k,sig", [(3000, 3000, 1.0), (2047, 2047, 1.0), (1025, 1025, 2.0), (3000, 700, 1.0),
                                     (5000, 1500, 2.5), (777, 300, 1.0)])
def test_spectral_vjp_matches_coefficient_vjp(gpu_icm, n, k, sig):
    S, P, cot = _case(n, k, sig, n + k)
    cfg = dict(block_size=8, fft_min_degree=16)
    gpu_icm.configure(**cfg)
    assert 2 in _kinds(gpu_icm, n, k, 8, 16)
    got, ref = _pair(gpu_icm, S, P, cot, Q=64, **cfg)
    _close(got, ref, (n, k, sig))


@pytest.mark.parametrize("min_degree", [0, 16, 64, 256])
def test_band_bottom_above_coefficient_levels(gpu_icm, min_degree):
    """The spectral band starting above coefficient levels (its bottom
    converts coefficient gbar and writes coefficient Pbar)."""
    S, P, cot = _case(4096, 4096, 1.5, 7)
    cfg = dict(block_size=8, fft_min_degree=16, vjp_spectral_min_degree=min_degree)
    got, ref = _pair(gpu_icm, S, P, cot, Q=48, **cfg)
    _close(got, ref, min_degree)


@pytest.mark.parametrize("B", [4, 16, 32])
def test_spectral_vjp_block_sizes(gpu_icm, B):
    S, P, cot = _case(3000, 3000, 1.0, 31 + B)
    got, ref = _pair(gpu_icm, S, P, cot, Q=48, block_size=B, fft_min_degree=16)
    _close(got, ref, B)


@pytest.mark.parametrize("k", [128, 129, 130, 256, 257, 513, 1025])
def test_spectral_band_top_at_truncation_edges(gpu_icm, k):
    """k at and around deg + 1 for the children degrees 128, 256, 512, 1024:
    the band's top level moves by one level across each edge."""
    S, P, cot = _case(4000, k, 1.0, 37 + k)
    got, ref = _pair(gpu_icm, S, P, cot, Q=48, block_size=8, fft_min_degree=16)
    _close(got, ref, k)


def test_spectral_vjp_node_terms(gpu_icm):
    S, P, cot = _case(2500, 2500, 1.0, 11)
    got, ref = _pair(gpu_icm, S, P, cot, Q=64, node_terms=True, fft_min_degree=16)
    _close(got, ref, "node terms")


def test_spectral_vjp_zero_prefix_off(gpu_icm):
    """Wholly-zero nodes computed rather than pruned give the same gradients."""
    S, P, cot = _case(3000, 3000, 2.5, 13)
    got, ref = _pair(gpu_icm, S, P, cot, Q=64, fft_min_degree=16)
    gpu_icm.configure(fft_min_degree=16, zero_prefix=False)
    full = gpu_icm.equity_vjp(S, P, cot, Q=64)
    _close(got, ref, "pruned")
    _close(full, ref, "not pruned")


def test_spectral_vjp_chunks_and_streams(gpu_icm):
    """Node chunks and chunk pieces on one or four streams give the same gradients."""
    S, P, cot = _case(9000, 9000, 1.0, 17)
    gpu_icm.configure(fft_min_degree=16)
    base = gpu_icm.equity_vjp(S, P, cot, Q=96)
    for cfg in (dict(q_chunk=7), dict(chunk_streams=1), dict(chunk_streams=4, q_chunk=13)):
        gpu_icm.configure(fft_min_degree=16, **cfg)
        got = gpu_icm.equity_vjp(S, P, cot, Q=96)
        assert np.array_equal(got[0], base[0]) and np.array_equal(got[1], base[1]), cfg


@pytest.mark.parametrize("n,k", [(70000, 70000), (40000, 20000)])
def test_spectral_vjp_multipass_levels(gpu_icm, n, k):
    """k = n: children of degree 16384 and 32768, the upward step in several
    passes, the downward step in one CTA (h = 8192) and in several passes.
    k < n: the band ends below the root at children of degree 8192, the
    largest that its top converts in one CTA."""
    S, P, cot = _case(n, k, 1.0, 19)
    if k == n:
        assert max(_kinds(gpu_icm, n, k, 8, 64)) == 2
    got, ref = _pair(gpu_icm, S, P, cot, Q=8)
    _close(got, ref, (n, k))


def test_spectral_vjp_plan_reuse(gpu_icm):
    """A reusable VJP plan gives the one-shot gradients on every run."""
    S, P, cot = _case(6000, 6000, 1.0, 23)
    gpu_icm.configure(fft_min_degree=16)
    one = gpu_icm.equity_vjp(S, P, cot, Q=64)
    v = gpu_icm.VjpPlan(S, len(P))
    for _ in range(2):
        gS, gP = v.run(P, cot, Q=64)
        assert np.array_equal(gS, one[0]) and np.array_equal(gP, one[1])
    v.close()


def test_batched_vjp_against_spectral_single(gpu_icm):
    """Batched VJPs (adjoint forests, spectral levels as in single plans)
    equal the default single VJPs of the same tournaments bit for bit."""
    rng = np.random.default_rng(29)
    ts, cots = [], []
    for n in (150, 1200, 3000, 4000):
        S, P, cot = _case(n, n if n != 1200 else 500, 1.0, int(rng.integers(1 << 30)))
        ts.append((S, P))
        cots.append(cot)
    res = gpu_icm.equity_vjp_batched(ts, cots, Q=64)
    for (S, P), c, got in zip(ts, cots, res):
        one = gpu_icm.equity_vjp(S, P, c, Q=64)
        assert np.array_equal(one[0], got[0]) and np.array_equal(one[1], got[1]), len(S)
    gpu_icm.configure(fft_min_degree=16)   # spectral levels from degree 16 up, in both
    res = gpu_icm.equity_vjp_batched(ts, cots, Q=64, node_terms=True)
    for (S, P), c, got in zip(ts, cots, res):
        one = gpu_icm.equity_vjp(S, P, c, Q=64, node_terms=True)
        assert np.array_equal(one[0], got[0]) and np.array_equal(one[1], got[1]), len(S)
    # batches against the coefficient-level VJP, to rounding
    gpu_icm.configure(fft_min_degree=16, vjp_spectral_min_degree=-1)
    ref = gpu_icm.equity_vjp_batched(ts, cots, Q=64, node_terms=True)
    for got, r in zip(res, ref):
        _close(got, r, "batch")


def _schoolbook_vjp(gpu_icm, S, P, cot, Q, node_terms=False):
    """The VJP with schoolbook products only (no FFT rounding): the accurate
    reference where FFT-based gradients lose digits on outlier stacks."""
    gpu_icm.configure(fft_min_degree=1 << 24, vjp_spectral_min_degree=-1)
    ref = gpu_icm.equity_vjp(S, P, cot, Q=Q, node_terms=node_terms)
    gpu_icm.configure()
    return ref


@pytest.mark.parametrize("n", [8000, 70000])
def test_spectral_vjp_wide_stacks_against_schoolbook(gpu_icm, n):
    """Stacks spread over e^{+-7.5} (many wholly-zero nodes; at n = 70000
    multi-pass levels with cold children skipped): the few players with the
    smallest stacks have gradients that FFT rounding perturbs by about 1e-10
    of the largest entry.  Against the schoolbook VJP both the spectral VJP
    and the coefficient-FFT VJP stay within 1e-9 of the largest entry (the
    bound of the analytic VJP checks)."""
    S, P, cot = _case(n, n, 2.5, 41)
    ref = _schoolbook_vjp(gpu_icm, S, P, cot, Q=12)
    spec = gpu_icm.equity_vjp(S, P, cot, Q=12)
    scale = np.abs(ref[0]).max()
    err_spec = np.abs(spec[0] - ref[0]).max() / scale
    assert err_spec <= 1e-9, err_spec
    assert np.abs(spec[1] - ref[1]).max() <= 1e-12 * np.abs(ref[1]).max()
    if n == 8000:
        gpu_icm.configure(vjp_spectral_min_degree=-1)
        coef = gpu_icm.equity_vjp(S, P, cot, Q=12)
        gpu_icm.configure()
        err_coef = np.abs(coef[0] - ref[0]).max() / scale
        assert err_coef <= 1e-9, err_coef


def test_spectral_vjp_plan_q_changes(gpu_icm):
    """One reusable VJP plan across node counts and node terms gives the one-shot results."""
    S, P, cot = _case(12000, 12000, 1.5, 43)
    v = gpu_icm.VjpPlan(S, len(P))
    for Q, nt in ((40, False), (96, True), (40, True), (200, False)):
        got = v.run(P, cot, Q=Q, node_terms=nt)
        one = gpu_icm.equity_vjp(S, P, cot, Q=Q, node_terms=nt)
        assert np.array_equal(got[0], one[0]) and np.array_equal(got[1], one[1]), (Q, nt)
    v.close()
