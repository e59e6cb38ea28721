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


def test_reference_fd_fixture_matches_oracle_differences(oracle):
    """The committed central differences of the reference (vjp_fd_reference.json)
    agree with the same differences of the oracle on the small k = n case, and
    the payout-direction value equals <cot, E(S, v)> of the oracle."""
    import json
    import os
    from tests.conftest import GOLDEN
    from tests.golden.make_golden import stack_direction, vjp_inputs
    from icm_gb300 import workloads as W
    case = [c for c in json.load(open(os.path.join(GOLDEN, "vjp_fd_reference.json")))["cases"]
            if c["name"] == "dropin_2048_kn"][0]
    S, P, cot = vjp_inputs(case["gen"], case["cot_seed"])

    def loss(x, pay=P):
        return float(cot @ oracle.equity(x, pay, Q=256, B=8, fft_min_deg=64))
    floor = 1e-9 * float(np.abs(cot * oracle.equity(S, P, Q=256, B=8, fft_min_deg=64)).sum())
    assert abs(loss(S) - case["L"]) <= floor
    d = case["stack_directions"][0]
    u = stack_direction(S, d["seed"])
    rich = _rich(loss, S, u)
    assert abs(rich - d["fd_richardson"]) <= 1e-7 * abs(d["fd_richardson"]) + floor
    v = W.SplitMix64(case["payout_direction"]["seed"]).normal(len(P))
    assert abs(loss(S, v) - case["payout_direction"]["derivative"]) <= 1e-11 * abs(case["payout_direction"]["derivative"]) + floor
