"""The reference derivatives used by the VJP tests, checked on the CPU:
analytic gradients of the closed forms against central finite differences
of the oracle's closed forms."""
import numpy as np

from tests.vjp_reference import fd_directional, quadratic_loss_grad, v1_loss_grad


def _rich(f, S, u):
    d1, d2 = fd_directional(f, S, u, 1e-3), fd_directional(f, S, u, 5e-4)
    return (4.0 * d2 - d1) / 3.0


def test_v1_gradient_formula(oracle):
    rng = np.random.default_rng(1)
    S = 10.0 ** (3 * rng.random(200))
    cot = rng.standard_normal(200)
    g = v1_loss_grad(S, cot)
    for _ in range(3):
        u = rng.standard_normal(200)
        fd = _rich(lambda x: float(cot @ oracle.v1(x)), S, u)
        terms = g * S * u
        assert abs(fd - terms.sum()) <= 1e-9 * np.abs(terms).sum()


def test_quadratic_gradient_formula(oracle):
    rng = np.random.default_rng(2)
    n = 40
    S = 1 + 99 * rng.random(n)
    cot = rng.standard_normal(n)
    g = quadratic_loss_grad(S, cot)

    def loss(x):
        return float(cot @ (2.0 * oracle.v2(x) + 3.0 * oracle.v1(x) - 2.0))
    for _ in range(3):
        u = rng.standard_normal(n)
        terms = g * S * u
        assert abs(_rich(loss, S, u) - terms.sum()) <= 1e-9 * np.abs(terms).sum()


def test_quadratic_closed_form_matches_oracle(oracle):
    """E = 2 V2 + 3 V1 - 2 for payout (n - m)^2 (the identity the tests rely on)."""
    rng = np.random.default_rng(3)
    n = 30
    S = 1 + 99 * rng.random(n)
    E = oracle.equity(S, (n - np.arange(n)).astype(float) ** 2, Q=256)
    ref = 2.0 * oracle.v2(S) + 3.0 * oracle.v1(S) - 2.0
    assert np.max(np.abs(E - ref) / np.abs(ref)) < 1e-10
