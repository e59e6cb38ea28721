"""The tanh-sinh quadrature option (IcmGb300Config.quadrature = 1) through
the C ABI: its nodes and the engine against a direct numpy restatement of the
Q-node formula (small n: polynomial products per player), the V1 closed form
and its analytic gradient; batches (nodes of zero weight at the tails, run by
forests, skipped by single plans) equal single solves bit for bit.

Tolerances: 1e-12 against the restatement at the same nodes (rounding only);
against V1 with stacks in [1, 1000] at Q = 256 the rule's own error is ~1e-15
(restatement: 5.6e-16), so 1e-11; gradients 1e-9 of the largest entry."""
import numpy as np
import pytest
from numpy.polynomial import polynomial as Pm

from tests.conftest import max_rel
from tests.vjp_reference import v1_loss_grad

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def tanh_sinh(gpu_icm):
    gpu_icm.configure(quadrature="tanh_sinh")
    yield
    gpu_icm.configure()


def ts_nodes(Q):
    """v = (1 + tanh t) / 2, t = pi/2 sinh x, x on [-5.5, 5.5]; w = h pi/2 cosh x / (2 cosh^2 t)."""
    h = 11.0 / (Q - 1)
    x = -5.5 + np.arange(Q) * h
    t = 0.5 * np.pi * np.sinh(x)
    e = np.exp(-2.0 * np.abs(t))
    logv = np.where(t >= 0, -np.log1p(e), 2.0 * t - np.log1p(e))
    w = h * 0.5 * np.pi * np.cosh(x) * (2.0 * e / (1.0 + e) ** 2)
    return logv, np.where((logv < 0) & np.isfinite(logv), w, 0.0)


def direct_equity(S, P, logv, w):
    """sum_q w_q S_i a_i / v_q <payout, prod_{j != i} (a_j + (1 - a_j) x) mod x^k>."""
    n, k = len(S), len(P)
    E = np.zeros(n)
    for lv, ww in zip(logv, w):
        if ww == 0.0:
            continue
        arg = S * lv
        a = np.where(arg < -700.0, 0.0, np.exp(np.maximum(arg, -745.0)))
        for i in range(n):
            poly = np.array([1.0])
            for j in range(n):
                if j != i:
                    poly = Pm.polymul(poly, [a[j], 1.0 - a[j]])[:k]
            pw = ww * S[i] * a[i] * np.exp(-lv)
            if np.isfinite(pw):
                E[i] += pw * np.dot(P[: len(poly)], poly)
    return E


def test_tanh_sinh_against_restatement(gpu_icm):
    rng = np.random.default_rng(1)
    for n, k in [(12, 12), (15, 4)]:
        S = 10.0 ** (3 * rng.random(n))
        P = 0.8 ** np.arange(k)
        ref = direct_equity(S, P, *ts_nodes(128))
        assert max_rel(gpu_icm.gpu_equity(S, P, Q=128), ref, floor=1e-300) < 1e-12


@pytest.mark.parametrize("engine", ["auto", "tree"])
def test_tanh_sinh_v1_closed_form(gpu_icm, engine):
    rng = np.random.default_rng(2)
    n = 300
    S = 1 + 999 * rng.random(n)
    P = (n - np.arange(n)).astype(float)
    gpu_icm.configure(quadrature="tanh_sinh", engine=engine, small_max_n=-1 if engine == "tree" else 0)
    E = gpu_icm.gpu_equity(S, P)
    T = S[:, None] + S[None, :]
    V1 = 1.0 + (S[:, None] / T).sum(axis=1) - 0.5
    assert max_rel(E, V1) < 1e-11


def test_tanh_sinh_vjp(gpu_icm):
    """Nodes independent of the stacks: the node terms vanish; the gradient of
    the V1 loss matches its analytic form."""
    rng = np.random.default_rng(3)
    n = 200
    S = 1 + 999 * rng.random(n)
    P = (n - np.arange(n)).astype(float)
    cot = rng.standard_normal(n)
    gS, gP = gpu_icm.equity_vjp(S, P, cot)
    gN, gPN = gpu_icm.equity_vjp(S, P, cot, node_terms=True)
    assert np.array_equal(gS, gN) and np.array_equal(gP, gPN)
    ref = v1_loss_grad(S, cot)
    assert np.abs(gS - ref).max() <= 1e-9 * np.abs(ref).max()


def test_tanh_sinh_batched_bitwise(gpu_icm):
    rng = np.random.default_rng(4)
    ts = [(1e3 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(max(1, n // 5))) for n in (3, 80, 700, 5000)]
    res = gpu_icm.equity_batched(ts)
    for (S, P), E in zip(ts, res):
        assert np.array_equal(E, gpu_icm.gpu_equity(S, P))
    cots = [rng.standard_normal(len(S)) for S, _ in ts]
    for (S, P), c, (gS, gP) in zip(ts, cots, gpu_icm.equity_vjp_batched(ts, cots)):
        a, b = gpu_icm.equity_vjp(S, P, c)
        assert np.array_equal(a, gS) and np.array_equal(b, gP)
