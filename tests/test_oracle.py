"""The oracle itself, pinned before it is trusted: against the reference's
golden vectors (web/verify/reference.json), the reference library's outputs
on seeded workloads, and the closed-form V1/V2 equities.  CPU only."""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN, max_rel
from tests.golden.webgen import all_cases
from icm_gb300 import workloads as W
from oracle.oracle import staged

WEB = json.load(open(os.path.join(GOLDEN, "web_reference.json")))
REFW = json.load(open(os.path.join(GOLDEN, "ref_workloads.json")))
REF_JSON = staged("web/verify/reference.json") or ""


def _web_inputs():
    return {name: (n, k, Q, S, P) for name, n, k, Q, S, P in all_cases()}


@pytest.mark.skipif(not os.path.isfile(REF_JSON), reason="reference sources not staged")
def test_webgen_rebuilds_reference_inputs_bit_for_bit():
    ref = json.load(open(REF_JSON))
    for (name, n, k, Q, S, P), c in zip(all_cases(), ref):
        assert name == c["name"]
        assert np.array_equal(S, np.array(c["stacks"])), name
        assert np.array_equal(P, np.array(c["payouts"])), name


@pytest.mark.parametrize("case", [c for c in WEB["cases"] if c["n"] <= 3000], ids=lambda c: c["name"])
@pytest.mark.parametrize("B", [4, 8])
def test_oracle_matches_reference_golden(oracle, case, B):
    n, k, Q, S, P = _web_inputs()[case["name"]]
    E = oracle.equity(S, P, Q=Q, B=B, fft_min_deg=64)
    idx = np.array(case["idx"])
    assert max_rel(E[idx], case["equity"]) < 1e-12


def test_oracle_naive_engine_agrees(oracle):
    n, k, Q, S, P = _web_inputs()["mtt200"]
    a = oracle.equity(S, P, Q=Q, B=8)
    b = oracle.equity_naive(S, P, Q=Q)
    assert max_rel(a, b) < 1e-11


@pytest.mark.parametrize("case", [c for c in REFW["cases"] if c["n"] <= 8192], ids=lambda c: c["name"])
def test_oracle_matches_reference_library_fixtures(oracle, case):
    S, P = _regen(case)
    E = oracle.equity(S, P, Q=case["Q"], B=8, fft_min_deg=64)
    idx = np.array(case["idx"])
    assert max_rel(E[idx], case["equity"]) < 1e-11
    if "targets" in case:
        Es = oracle.equity(S, P, Q=case["Q"], B=8, fft_min_deg=64, targets=case["targets"])
        assert max_rel(Es[case["targets"]], case["subset_equity"]) < 1e-11
        assert np.count_nonzero(np.delete(Es, case["targets"])) == 0


def _regen(case):
    """Rebuild a fixture's inputs from its generator expression."""
    ns = {"plain_small": W.plain_small, "dropin": W.dropin, "gpu_scale": W.gpu_scale,
          "batched": W.batched, "vjp": W.vjp}
    out = eval(case["gen"], {}, ns)
    if case["gen"].startswith("batched"):
        S, P = out[case["member"]]
    else:
        S, P = out[0], out[1]
    assert abs(S.sum() - case["sum_S"]) <= 1e-9 * case["sum_S"], "generator drift"
    assert abs(P.sum() - case["sum_P"]) <= 1e-12
    return S, P


def test_oracle_closed_form_v1(oracle):
    rng = np.random.default_rng(3)
    for n, dist in [(64, "uniform"), (300, "adversarial"), (1000, "geometric")]:
        if dist == "uniform":
            S = 1 + 99 * rng.random(n)
        elif dist == "adversarial":
            S = np.ones(n); S[0] = 1e4
        else:
            S = 2.0 ** (np.arange(n) * 10.0 / n)
        P = (n - np.arange(n)).astype(float)
        assert max_rel(oracle.equity(S, P, B=8, fft_min_deg=64), oracle.v1(S)) < 5e-12


def test_oracle_closed_form_v2(oracle):
    rng = np.random.default_rng(4)
    n = 120
    S = 1 + 99 * rng.random(n)
    r = n - 1 - np.arange(n)
    P = np.where(r >= 2, r * (r - 1) / 2.0, 0.0)
    assert max_rel(oracle.equity(S, P, B=8), oracle.v2(S)) < 5e-12


def test_closed_form_fixture_against_reference_library():
    """Quadrature floor of the reference at the full drop-in size: the
    reference itself is within 1e-9 of the exact quadratic-payout equity."""
    cf = json.load(open(os.path.join(GOLDEN, "closed_form.json")))
    case = [c for c in REFW["cases"] if c["name"] == "dropin_65536"][0]
    assert case["targets"] == cf["targets"]
    assert max_rel(case["full_at_targets"], cf["equity"]) < 1e-9
    assert max_rel(case["subset_equity"], cf["equity"]) < 1e-9


def test_oracle_subset_prunes_but_matches(oracle):
    S, P = W.plain_small()
    T = [0, 7, 42, 100, 255, 500, 777, 900, 999, 1023]
    full = oracle.equity(S, P, B=8)
    sub = oracle.equity(S, P, B=8, targets=T)
    assert max_rel(sub[T], full[T]) < 1e-13
    assert np.count_nonzero(np.delete(sub, T)) == 0


def test_oracle_quadrature_nodes(oracle):
    lv, w = oracle.nodes(256, 1e9)
    assert np.all(np.diff(lv) > 0) and np.all(lv < 0) and np.all(w > 0)
    # trapezoid in probit space integrates the normal density to ~1
    assert abs(w.sum() - 1.0) < 1e-9
