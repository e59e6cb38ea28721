"""VJPs of the equities through the C ABI against analytic derivatives of
the closed forms, central finite differences of the oracle and Euler's
identity for the payout gradient.

The quadrature nodes move with max S.  With node terms the VJP is the exact
derivative of the Q-node formula and must equal finite differences in every
direction; without them (the default) it must equal finite differences in
directions that keep max S fixed, and differ from the node-term gradient
only in the largest stack's entry.

Tolerances: 1e-9 of the gradient's largest entry against the analytic
gradients (quadrature error ~1e-12 on those workloads).  Against finite
differences, on the directional derivative's absolute scale
sum_i |dL/dS_i S_i u_i|: 1e-6 at relative step 1e-6 (the oracle's rounding
noise, ~1e-13 of L, divided by the step), and 2e-8 for the Richardson
extrapolation of steps 1e-4 and 5e-5 (truncation ~1e-16, noise ~2e-9);
both plus 1e-9 of sum_i |cot_i E_i| for the rounding of L itself.  Stacks
within 1% of the largest stay unperturbed, so that no step changes which
player sets the nodes (the formula is not differentiable there)."""
import numpy as np
import pytest

from tests.conftest import max_rel
from tests.vjp_reference import fd_directional, quadratic_loss_grad, v1_loss_grad, v1_loss_grad_blocked
from icm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL_ANALYTIC = 1e-9
TOL_FD = 1e-6
TOL_FD_RICHARDSON = 2e-8


@pytest.fixture(autouse=True)
def default_config(gpu_icm):
    gpu_icm.configure()
    yield
    gpu_icm.configure()


def _fd_agrees(loss, S, u, g, floor):
    terms = g * S * u
    an = float(terms.sum())
    scale = float(np.abs(terms).sum())
    fd = fd_directional(loss, S, u)
    assert abs(fd - an) <= TOL_FD * scale + floor, (fd, an, scale)
    d1, d2 = fd_directional(loss, S, u, 1e-4), fd_directional(loss, S, u, 5e-5)
    rich = (4.0 * d2 - d1) / 3.0
    assert abs(rich - an) <= TOL_FD_RICHARDSON * scale + floor, (rich, an, scale)


def _check_fd(gpu_icm, oracle, S, P, cot, Q, rng, directions=3, B=8, fft_min=64):
    """Both VJP modes against central differences of the oracle."""
    gS, gP = gpu_icm.equity_vjp(S, P, cot, Q=Q)
    gN, gPN = gpu_icm.equity_vjp(S, P, cot, Q=Q, node_terms=True)
    imax = int(np.argmax(S))
    assert np.array_equal(np.delete(gS, imax), np.delete(gN, imax)) and np.array_equal(gP, gPN)

    def loss(Sx):
        return float(cot @ oracle.equity(Sx, P, Q=Q, B=B, fft_min_deg=fft_min))
    floor = 1e-9 * float(np.abs(cot * oracle.equity(S, P, Q=Q, B=B, fft_min_deg=fft_min)).sum())
    near = (S > 0.99 * S[imax]) & (np.arange(len(S)) != imax)
    for _ in range(directions):
        u = rng.standard_normal(len(S))
        u[near] = 0.0
        _fd_agrees(loss, S, u, gN, floor)           # exact derivative of the Q-node formula
        u[imax] = 0.0
        _fd_agrees(loss, S, u, gS, floor)           # nodes held fixed
    return gS, gP


@pytest.mark.parametrize("n,dist", [(7, "u"), (64, "u"), (300, "log"), (2048, "u"), (5000, "log")])
def test_stack_gradient_v1_closed_form(gpu_icm, n, dist):
    """payout n - m, k = n: equity = V1, gradient analytic."""
    rng = np.random.default_rng(n)
    S = 1 + 999 * rng.random(n) if dist == "u" else 10.0 ** (4 * rng.random(n))
    P = (n - np.arange(n)).astype(float)
    cot = rng.standard_normal(n)
    gS, gP = gpu_icm.equity_vjp(S, P, cot)
    ref = v1_loss_grad(S, cot)
    assert np.abs(gS - ref).max() <= TOL_ANALYTIC * np.abs(ref).max()
    E = gpu_icm.equity(S, P)
    assert abs(gP @ P - cot @ E) <= 1e-12 * np.abs(cot * E).sum()     # Euler: L is linear in payout


@pytest.mark.parametrize("n", [5, 40, 150])
def test_stack_gradient_quadratic_closed_form(gpu_icm, n):
    """payout (k - j + 1)^2, k = n: equity = 2 V2 + 3 V1 - 2."""
    rng = np.random.default_rng(100 + n)
    S = 1 + 99 * rng.random(n)
    P = (n - np.arange(n)).astype(float) ** 2
    cot = rng.standard_normal(n)
    gS, _ = gpu_icm.equity_vjp(S, P, cot)
    ref = quadratic_loss_grad(S, cot)
    assert np.abs(gS - ref).max() <= TOL_ANALYTIC * np.abs(ref).max()


@pytest.mark.parametrize("n,k", [(1, 1), (2, 1), (3, 2), (9, 4), (33, 33), (100, 7), (1000, 150), (3001, 3001),
                                 (6000, 900)])
def test_stack_gradient_against_oracle_fd(gpu_icm, oracle, n, k):
    rng = np.random.default_rng(n * 31 + k)
    S = 1e4 * np.exp(rng.standard_normal(n))
    P = 0.8 ** np.arange(k)
    P /= P.sum()
    cot = rng.standard_normal(n)
    gS, gP = _check_fd(gpu_icm, oracle, S, P, cot, 256, rng)
    # payout: exact directional derivative (linear)
    d = rng.standard_normal(k)
    L0 = cot @ oracle.equity(S, P, Q=256)
    L1 = cot @ oracle.equity(S, P + d, Q=256)
    assert abs((L1 - L0) - gP @ d) <= 1e-10 * (abs(L1) + abs(L0) + 1e-300)


@pytest.mark.parametrize("B,fft_min", [(4, 16), (16, 64), (32, 1 << 20), (8, 8)])
def test_vjp_block_size_and_fft_levels(gpu_icm, oracle, B, fft_min):
    """Schoolbook and one-kernel FFT adjoint levels, every block size."""
    gpu_icm.configure(block_size=B, fft_min_degree=fft_min)
    rng = np.random.default_rng(B * 7 + fft_min % 97)
    n = 1500
    S = 10.0 ** (3 * rng.random(n))
    for k in (n, 200, 3):
        P = (k - np.arange(k)).astype(float)
        cot = rng.standard_normal(n)
        gS, gP = _check_fd(gpu_icm, oracle, S, P, cot, 256, rng, directions=2, B=B)
        E = gpu_icm.equity(S, P)
        assert abs(gP @ P - cot @ E) <= 1e-12 * np.abs(cot * E).sum()


def test_payout_gradient_place_probabilities(gpu_icm, oracle):
    """dL/dpayout[m] = sum_i cot_i Pr(i finishes m-th): one unit payout per place."""
    rng = np.random.default_rng(3)
    n, k = 12, 5
    S = 1 + 99 * rng.random(n)
    cot = rng.standard_normal(n)
    _, gP = gpu_icm.equity_vjp(S, np.ones(k), cot)
    ref = np.array([cot @ oracle.equity(S, np.eye(k)[m], Q=256) for m in range(k)])
    assert max_rel(gP, ref, floor=1e-12) < 1e-9


def test_vjp_workload_size(gpu_icm, oracle):
    """n = 16384, k = 2000, gamma(2, 5000) stacks, linear and quadratic payouts,
    N(0, 1) cotangent: finite differences of the oracle along random directions."""
    for shape in ("linear", "quadratic"):
        S, P, cot = W.vjp(payout=shape)
        gS, gP = _check_fd(gpu_icm, oracle, S, P, cot, 256, np.random.default_rng(5), directions=2)
        E = gpu_icm.equity(S, P)
        assert abs(gP @ P - cot @ E) <= 1e-12 * np.abs(cot * E).sum()


def test_vjp_plan_reuse_and_batched(gpu_icm):
    rng = np.random.default_rng(8)
    ts, cots = [], []
    for n in (100, 700, 4000, 1):
        k = max(1, n // 3)
        ts.append((1e3 * np.exp(rng.standard_normal(n)), np.linspace(1, 0.1, k)))
        cots.append(rng.standard_normal(n))
    res = gpu_icm.equity_vjp_batched(ts, cots, Q=64)
    for (S, P), c, (gS, gP) in zip(ts, cots, res):
        a, b = gpu_icm.equity_vjp(S, P, c, Q=64)
        assert np.array_equal(a, gS) and np.array_equal(b, gP)
    S, P = ts[2]
    plan = gpu_icm.VjpPlan(S, len(P))
    a1 = plan.run(P, cots[2], Q=64)
    a2 = plan.run(P, cots[2], Q=64)
    assert np.array_equal(a1[0], a2[0]) and np.array_equal(a1[1], a2[1])
    a3 = plan.run(P, 2.0 * cots[2], Q=64)
    assert max_rel(a3[0], 2.0 * a1[0], floor=np.abs(a1[0]).max() * 1e-3) < 1e-12
    assert plan.device_ms() > 0
    plan.close()


def test_autograd_function(gpu_icm):
    torch = pytest.importorskip("torch")
    from icm_gb300.autograd import ICMEquity, equity
    rng = np.random.default_rng(12)
    S = torch.tensor(1 + 99 * rng.random(6), dtype=torch.float64, requires_grad=True)
    P = torch.tensor([0.5, 0.3, 0.2], dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda s, p: ICMEquity.apply(s, p, 256, True), (S, P), eps=1e-6, atol=1e-7,
                                    rtol=1e-5)
    S2 = torch.tensor(1e4 * np.exp(rng.standard_normal(500)), dtype=torch.float64, requires_grad=True)
    P2 = torch.tensor(0.9 ** np.arange(50), dtype=torch.float64, requires_grad=True)
    cot = torch.tensor(rng.standard_normal(500), dtype=torch.float64)
    (equity(S2, P2) * cot).sum().backward()
    gS, gP = gpu_icm.equity_vjp(S2.detach().numpy(), P2.detach().numpy(), cot.numpy())
    assert np.array_equal(S2.grad.numpy(), gS) and np.array_equal(P2.grad.numpy(), gP)


@pytest.mark.parametrize("wl", ["vjp", "lognormal_wide"])
def test_vjp_zero_prefix_pruning(gpu_icm, wl):
    """Pruning wholly-zero tree nodes leaves both gradients unchanged to rounding."""
    if wl == "vjp":
        S, P, cot = W.vjp(n=8192, k=900)
    else:
        rng = np.random.default_rng(4)
        S = 1e4 * np.exp(1.5 * rng.standard_normal(20000))
        P = np.linspace(1.0, 0.0, 20000, endpoint=False)
        cot = rng.standard_normal(20000)
    out = []
    for zp in (True, False):
        gpu_icm.configure(zero_prefix=zp)
        out.append(gpu_icm.equity_vjp(S, P, cot, node_terms=True))
    for a, b in zip(out[0], out[1]):
        assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()


def _mixed_batch(rng, count=40, big=False):
    """Uneven sizes: single-block tournaments (n <= B), schoolbook-only and
    FFT trees, truncated and full k, wide stacks (zero-prefix pruning), and
    optionally one tournament whose levels need the multi-pass transforms."""
    ts, cots = [], []
    sizes = [1, 2, 3, 5, 8, 17, 64, 100, 333, 1024, 2500, 6000] + list(rng.integers(1, 5000, count - 12))
    if big:
        sizes.append(70000)
    for i, n in enumerate(sizes):
        n = int(n)
        k = n if i % 3 == 0 or n == 70000 else max(1, int(np.ceil(n * rng.uniform(0.02, 0.6))))
        sig = 2.0 if i % 4 == 0 else 1.0
        ts.append((1e4 * np.exp(sig * rng.standard_normal(n)), 0.85 ** np.arange(k)))
        cots.append(rng.standard_normal(n))
    return ts, cots


@pytest.mark.parametrize("node_terms", [False, True])
def test_batched_vjp_forest_bitwise(gpu_icm, node_terms):
    """Every tournament's gradients from the adjoint forest equal its single
    VJP bit for bit (spectral levels in both, as configured)."""
    rng = np.random.default_rng(21 + node_terms)
    ts, cots = _mixed_batch(rng, big=node_terms)
    res = gpu_icm.equity_vjp_batched(ts, cots, Q=128, node_terms=node_terms)
    for (S, P), c, (gS, gP) in zip(ts, cots, res):
        a, b = gpu_icm.equity_vjp(S, P, c, Q=128, node_terms=node_terms)
        assert np.array_equal(a, gS) and np.array_equal(b, gP), (len(S), len(P))


def test_batched_vjp_forest_bitwise_coefficients(gpu_icm):
    """The same with every VJP level on coefficients (vjp_spectral_min_degree = -1)."""
    gpu_icm.configure(vjp_spectral_min_degree=-1)
    rng = np.random.default_rng(24)
    ts, cots = _mixed_batch(rng, count=16)
    res = gpu_icm.equity_vjp_batched(ts, cots, Q=96)
    for (S, P), c, (gS, gP) in zip(ts, cots, res):
        a, b = gpu_icm.equity_vjp(S, P, c, Q=96)
        assert np.array_equal(a, gS) and np.array_equal(b, gP), (len(S), len(P))


@pytest.mark.parametrize("B,fft_min", [(4, 16), (16, 32)])
def test_batched_vjp_forest_block_sizes(gpu_icm, B, fft_min):
    gpu_icm.configure(block_size=B, fft_min_degree=fft_min)
    rng = np.random.default_rng(B)
    ts, cots = _mixed_batch(rng, count=20)
    res = gpu_icm.equity_vjp_batched(ts, cots, Q=64)
    for (S, P), c, (gS, gP) in zip(ts, cots, res):
        a, b = gpu_icm.equity_vjp(S, P, c, Q=64)
        assert np.array_equal(a, gS) and np.array_equal(b, gP), (len(S), len(P))


def test_vjp_batch_reuse_graphs(gpu_icm):
    """Reusable batched VJP: graph replays, Q changes, node-term toggles and
    fallback members give the one-shot results; profiling changes nothing."""
    rng = np.random.default_rng(33)
    ts, cots = _mixed_batch(rng, count=16, big=True)
    vb = gpu_icm.GpuVjpBatch([S for S, _ in ts], [len(P) for _, P in ts])
    assert vb.info()["fallbacks"] == 1
    Ps = [P for _, P in ts]
    for Q, nt in [(64, False), (64, False), (96, True), (96, False), (64, True)]:
        got = vb.vjp(Ps, cots, Q=Q, node_terms=nt)
        ref = gpu_icm.equity_vjp_batched(ts, cots, Q=Q, node_terms=nt)
        for (a, b), (c, d) in zip(got, ref):
            assert np.array_equal(a, c) and np.array_equal(b, d)
    vb.set_options(graphs=False, profiling=True)
    got = vb.vjp(Ps, cots, Q=64)
    stats = vb.kernel_stats()
    assert any(s["name"].startswith("wl_adj_") for s in stats)
    ref = gpu_icm.equity_vjp_batched(ts, cots, Q=64)
    for (a, b), (c, d) in zip(got, ref):
        assert np.array_equal(a, c) and np.array_equal(b, d)
    with pytest.raises(gpu_icm.ICMError):
        vb.equity(Ps)
    vb.close()


def test_vjp_multipass_levels(gpu_icm):
    """n = k = 20000: the top two levels need transforms of 16384 and 32768
    points (beyond one CTA), so their adjoint steps run through global
    four-step FFTs.  Against the analytic V1 gradient and Euler's identity."""
    rng = np.random.default_rng(20000)
    n = 20000
    S = 1 + 999 * rng.random(n)
    P = (n - np.arange(n)).astype(float)
    cot = rng.standard_normal(n)
    gS, gP = gpu_icm.equity_vjp(S, P, cot)
    ref = v1_loss_grad_blocked(S, cot)
    assert np.abs(gS - ref).max() <= TOL_ANALYTIC * np.abs(ref).max()
    E = gpu_icm.equity(S, P)
    assert abs(gP @ P - cot @ E) <= 1e-12 * np.abs(cot * E).sum()


# ---------------------------------------------------------------------------
# against central differences of the reference itself (tests/golden/
# vjp_fd_reference.json: the reference's own icm_equity, built from its
# unmodified src/cpu/icm.c, differenced along stacks with max S fixed and
# along a payout direction, where L is linear)
def _fd_cases():
    import json
    import os
    from tests.conftest import GOLDEN
    return json.load(open(os.path.join(GOLDEN, "vjp_fd_reference.json")))["cases"]


@pytest.mark.parametrize("case", _fd_cases(), ids=lambda c: c["name"])
def test_vjp_against_reference_finite_differences(gpu_icm, case):
    from tests.golden.make_golden import stack_direction, vjp_inputs
    S, P, cot = vjp_inputs(case["gen"], case["cot_seed"])
    assert len(S) == case["n"] and len(P) == case["k"]
    gS, gP = gpu_icm.equity_vjp(S, P, cot, Q=case["Q"])
    E = gpu_icm.equity(S, P, Q=case["Q"])
    L = float(cot @ E)
    floor = 1e-9 * float(np.abs(cot * E).sum())
    assert abs(L - case["L"]) <= floor
    for d in case["stack_directions"]:
        u = stack_direction(S, d["seed"])
        terms = gS * S * u
        an, scale = float(terms.sum()), float(np.abs(terms).sum())
        assert abs(d["fd_1e-6"] - an) <= TOL_FD * scale + floor, (d, an, scale)
        assert abs(d["fd_richardson"] - an) <= TOL_FD_RICHARDSON * scale + floor, (d, an, scale)
    v = W.SplitMix64(case["payout_direction"]["seed"]).normal(len(P))
    pv = gP * v
    assert abs(float(pv.sum()) - case["payout_direction"]["derivative"]) <= 1e-10 * float(np.abs(pv).sum())
