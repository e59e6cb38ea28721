"""GPU-only scale: n = 2^20 players, stacks 1e4 exp(1.5 N(0,1)).
(a) k = n linear payout: closed form E = V1 / sum(n - m) on sampled players
(1e-9); (b) k = 1000 geometric payout 0.97: the oracle on sampled targets at
a reduced node count (the same Q on both sides, 1e-8), and the reference's
own subset query at Q = 256 (a committed fixture, 1e-8)."""
import numpy as np
import pytest

from tests.conftest import max_rel
from icm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_linear_full_field_closed_form(gpu_icm, oracle):
    S, P = W.gpu_scale(shape="linear")
    E = gpu_icm.equity(S, P)
    idx = np.random.default_rng(1).choice(len(S), 64, replace=False)
    ref = oracle.v1(S, idx=idx) * (P[0] / len(S))
    assert max_rel(E[idx], ref) < 1e-9
    assert abs(E.sum() - 1.0) < 1e-9


def test_geometric_k1000_against_oracle(gpu_icm, oracle):
    S, P = W.gpu_scale(shape="geometric")
    T = np.sort(np.random.default_rng(2).choice(len(S), 16, replace=False)).tolist()
    E = gpu_icm.equity(S, P, Q=24)
    R = oracle.equity(S, P, Q=24, B=8, fft_min_deg=64, targets=T)
    assert max_rel(E[T], R[T]) < 1e-8
    Es = gpu_icm.equity_subset(S, P, T, Q=24)
    assert max_rel(Es[T], E[T]) < 1e-12


def test_geometric_k1000_against_reference_at_q256(gpu_icm):
    """(b) at the full Q = 256 against the reference's own icm_equity_subset
    (tests/golden/ref_gpu_scale_geometric.json, 16 targets), full field and
    subset, within the reference's GPU gate of 1e-8."""
    import json
    import os
    from tests.conftest import GOLDEN
    fx = json.load(open(os.path.join(GOLDEN, "ref_gpu_scale_geometric.json")))
    S, P = W.gpu_scale(shape="geometric")
    assert len(S) == fx["n"] and len(P) == fx["k"]
    T = fx["targets"]
    E = gpu_icm.equity(S, P, Q=fx["Q"])
    assert max_rel(E[T], fx["subset_equity"]) < 1e-8
    Es = gpu_icm.equity_subset(S, P, T, Q=fx["Q"])
    assert max_rel(Es[T], fx["subset_equity"]) < 1e-8
    assert np.count_nonzero(np.delete(Es, T)) == 0
